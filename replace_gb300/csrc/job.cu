// libgpl_gb300: job lifecycle, device model upload, one physics evaluation,
// the Nesterov control loop (NesterovPlace, src/nesterovPlace.cpp:64-607) and
// the C ABI declared in include/gpl.h.
//
// Control stays on the host in this file: each back-track step launches the
// evaluation kernels and reads back one small result record (overflow, HPWL,
// gradient sums, step length).  All per-cell and per-bin state stays on the
// device for the whole job.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "control.h"
#include "gpl_internal.h"

namespace gpl {

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }

const char* kernel_class_name(int k) {
  static const char* names[kKClasses] = {"density_scatter", "poisson_rows_dct", "poisson_cols_solve",
                                         "poisson_rows_inverse", "wa_wirelength", "gcell_gradient",
                                         "reduce_finalize", "other"};
  return (k >= 0 && k < kKClasses) ? names[k] : "?";
}

void Timer::begin(int k) {
  (void)k;
  if (!enabled) return;
  cudaEvent_t a;
  if (!pool.empty()) { a = pool.back(); pool.pop_back(); } else cudaEventCreate(&a);
  cudaEventRecord(a, stream);
  pending = a;
}

void Timer::end(int k) {
  if (!enabled || !pending) return;
  cudaEvent_t b;
  if (!pool.empty()) { b = pool.back(); pool.pop_back(); } else cudaEventCreate(&b);
  cudaEventRecord(b, stream);
  live.push_back({k, pending, b});
  pending = nullptr;
}

int Timer::resolve() {
  if (live.empty()) return GPL_OK;
  GPL_CUDA(cudaStreamSynchronize(stream));
  for (auto& p : live) {
    float ms_ = 0.0f;
    cudaEventElapsedTime(&ms_, p.a, p.b);
    ms[p.k] += ms_;
    groups[p.k]++;
    pool.push_back(p.a);
    pool.push_back(p.b);
  }
  live.clear();
  return GPL_OK;
}

void Timer::release() {
  for (auto& p : live) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
  for (auto e : pool) cudaEventDestroy(e);
  live.clear();
  pool.clear();
}

int launch_initial_prev(DeviceModel& d, const float2* cur_slp, const float2* cur_sum, float coef,
                        float2* out, cudaStream_t s, Timer& t);

}  // namespace gpl

using namespace gpl;

// Host arrays of a job's device model (see stage_device_model).
struct DevStage {
  std::vector<int2> half;
  std::vector<uint8_t> kind;
  std::vector<float2> precond;
  std::vector<int32_t> big, big_idx;
  std::vector<int4> pins;
  std::vector<int32_t> dnet_start, g_dpins;
  std::vector<float2> tw, w4x, w4y;
  std::vector<float> wx, wy;
  int wa_bucket_start[kWaBuckets + 1] = {0};
  int wa_block_start[kWaBuckets + 1] = {0};
  std::vector<int32_t> net_rank;       // device (bucket-order) index of each net
};

struct gpl_job {
  HostModel m;
  DeviceModel d;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  Timer timer;
  char* arena = nullptr;
  HostPinned* pinned = nullptr;        // control/result staging
  bool own_pinned = false;
  cudaMemPool_t pool = nullptr;         // stream-ordered pool (server jobs)
  cudaEvent_t sync_ev = nullptr;        // blocking-sync event (server jobs)
  bool nb_ready = false, np_ready = false;
  // NesterovPlace state (src/nesterovPlace.h:76-125), the host copy; the
  // device loop works on d_state and the two are exchanged around a chunk
  NesterovState S{};
  cudaGraphExec_t graph_exec = nullptr; // one evaluation, replayed
  long long graph_kernels = 0;
  // device loop: head kernel, then WHILE { [IF tile order] evaluation, step }
  cudaGraphExec_t loop_exec = nullptr;
  bool loop_tried = false;
  NesterovState* d_state = nullptr;
  IterEntry* d_log = nullptr;
  int log_cap = 0;
  long long order_kernels = 0;
  float poisson_fft_us = 0.0f, poisson_gemm_us = 0.0f;   // auto mode's timings
  float scatter_us = 0.0f;                                // the chosen scatter shape's time
  bool poisson_chosen = false;
  // WA runs beside the Poisson passes on a second stream (fork after the
  // scatter, join before the gcell kernel)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // position-independent Nesterov setup, built beside the initial place
  std::thread prep;
  std::unique_ptr<DevStage> stage;
  int prep_rc = 0;
  std::string prep_err;
  bool static_done = false;
  // per-net weights in the netlist's net order (empty: every weight 1) and
  // the device index of each net, for uploads after the device model exists
  std::vector<float> net_w;
  std::vector<int32_t> net_rank;
};

namespace {

int upload(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (!bytes) return GPL_OK;
  GPL_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
  return GPL_OK;
}

// wall clock in ms (verbose_level >= 2 timings)
double wall_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int check_device(int dev) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    set_error("no CUDA device available: the GB300 placement core has no CPU fallback");
    return GPL_ERR_NO_DEVICE;
  }
  if (dev < 0 || dev >= n) { set_error("device ordinal out of range"); return GPL_ERR_INVALID_ARG; }
  GPL_CUDA(cudaSetDevice(dev));
  return GPL_OK;
}

struct Sizer {
  size_t bytes = 0;
  void add(size_t n, size_t sz) { size_t b = ((n * sz + 255) / 256) * 256; bytes += b ? b : 256; }
};
struct Carver {
  char* base;
  size_t off = 0;
  template <class T> T* take(size_t n) {
    size_t b = ((n * sizeof(T) + 255) / 256) * 256;
    T* p = reinterpret_cast<T*>(base + off);
    off += b ? b : 256;
    return p;
  }
};

// Bytes of a job's arena (the carving in ensure_nb follows the same order).
size_t arena_bytes(size_t ng, size_t n_pins, size_t n_nets, size_t n_gpins, size_t n_big, size_t nb,
                   int cnt_x, int cnt_y, size_t part_stride, size_t log_cap) {
  const size_t ps = (size_t)kPartSlots * part_stride;
  // tile and chunk tables sized for the smallest scatter shape
  int tw, th, tx, ty;
  tile_grid(cnt_x, cnt_y, kTileSideMin, &tw, &th, &tx, &ty);
  const size_t tiles = (size_t)tx * ty;
  Sizer S;
  S.add(ng, 4); S.add(tiles, 4); S.add(tiles + 1, 4);
  S.add(scatter_max_chunks((int)ng, (int)tiles, kScatterChunkMin), 16); S.add(1, 4);
  S.add(ng, sizeof(int2)); S.add(ng, 4); S.add(ng, 1); S.add(ng, 8); S.add(ng + 1, 4);
  S.add(n_big, 4); S.add(ng, 4); S.add(n_big, 8);
  S.add(n_pins, 16); S.add(n_nets + 1, 4);
  S.add(n_pins, 8); S.add(n_nets, 4); S.add(n_gpins, 4);
  S.add(2 * nb, 8); S.add(2 * nb, 8); S.add(nb, 8);
  S.add(nb, 4); S.add(nb, 4); S.add(nb, 4); S.add(nb, 4); S.add(nb, 8); S.add(nb, 4);
  S.add(cnt_x, 4); S.add(cnt_y, 4); S.add(cnt_x, 8); S.add(cnt_y, 8); S.add(kFftMax / 2, 8);
  for (int k = 0; k < 4; k++) { S.add(ng, 8); S.add(ng, 8); }
  S.add(ng, 8); S.add(ng, 8);                 // coordi
  S.add(ng, 8); S.add(ng, 8);                 // hook outputs: wl / density gradients
  S.add(1, sizeof(EvalCtl));
  S.add(ps, 8); S.add(1, sizeof(EvalResult)); S.add(kHpwlLanes * kHpwlStride, 8); S.add(4, 4);
  S.add(kPartSlots, 8);
  S.add(1, sizeof(NesterovState)); S.add(log_cap, sizeof(IterEntry));   // device loop
  return S.bytes;
}

// The device model's host arrays: everything but the movable gcells'
// positions, so that it can be built beside the initial place.
int stage_device_model(const HostModel& m, DevStage& st) {
  const size_t ng = m.n_g;
  st.half.resize(ng);
  st.kind.resize(ng);
  st.precond.resize(ng);
  st.big.clear();
  st.big_idx.assign(ng, -1);
  for (size_t g = 0; g < ng; g++) {
    st.half[g] = make_int2((m.gdux[g] - m.gdlx[g]) / 2, (m.gduy[g] - m.gdly[g]) / 2);
    st.kind[g] = m.gkind[g];
    // bins a cell can touch per axis: its extent in bins plus one for a straddle
    const long long bx = (2LL * st.half[g].x) / m.size_x + 2, by = (2LL * st.half[g].y) / m.size_y + 2;
    if (bx * by > 64) {
      st.kind[g] |= 4;
      st.big_idx[g] = (int)st.big.size();
      st.big.push_back((int)g);
    }
    // getWireLengthPreconditioner / getDensityPreconditioner (src/nesterovBase.cpp:1442-1454)
    st.precond[g] = make_float2((float)(m.g_pin_start[g + 1] - m.g_pin_start[g]),
                                (float)(m.gux[g] - m.glx[g]) * (float)(m.guy[g] - m.gly[g]));
  }
  // WA buckets by degree: group widths 2, 4, 8, 16, 32 lanes, then a warp per net
  std::vector<int32_t> net_order;
  {
    // key = lowest gcell index on the net (ng for nets without a movable
    // pin); a stable counting sort by key, then a stable split by bucket,
    // orders each bucket by key with ties in net order
    std::vector<int32_t> key(m.n_nets), cnt(ng + 2, 0);
    std::vector<uint8_t> bucket(m.n_nets);
    for (int n = 0; n < m.n_nets; n++) {
      const int deg = m.net_start[n + 1] - m.net_start[n];
      int b = 0;
      while (b < kWaBuckets - 1 && deg > (2 << b)) b++;
      bucket[n] = (uint8_t)b;
      int k = (int)ng;
      for (int q = m.net_start[n]; q < m.net_start[n + 1]; q++)
        if (m.pin_g[q] >= 0) k = std::min(k, m.pin_g[q]);
      key[n] = k;
      cnt[k + 1]++;
    }
    for (size_t k = 0; k <= ng; k++) cnt[k + 1] += cnt[k];
    std::vector<int32_t> by_key(m.n_nets);
    for (int n = 0; n < m.n_nets; n++) by_key[cnt[key[n]]++] = n;
    std::vector<std::vector<int32_t>> bk(kWaBuckets);
    for (int n : by_key) bk[bucket[n]].push_back(n);
    net_order.reserve(m.n_nets);
    st.wa_bucket_start[0] = 0;
    st.wa_block_start[0] = 0;
    for (int b = 0; b < kWaBuckets; b++) {
      net_order.insert(net_order.end(), bk[b].begin(), bk[b].end());
      st.wa_bucket_start[b + 1] = (int)net_order.size();
      const int per = wa_nets_per_block(b);
      st.wa_block_start[b + 1] = st.wa_block_start[b] + ((int)bk[b].size() + per - 1) / per;
    }
  }
  // device pin numbering: the bucket-ordered nets' pins, contiguous per net
  // (the pins are visited in host order, each net written at its rank's slot)
  std::vector<int32_t> dpin_of(m.n_pins, -1);
  std::vector<int4>& pins = st.pins;
  std::vector<int32_t>& dnet_start = st.dnet_start;
  pins.resize(m.n_pins);
  dnet_start.assign(m.n_nets + 1, 0);
  {
    std::vector<int32_t>& rank = st.net_rank;
    rank.assign(m.n_nets, 0);
    int w = 0;
    for (int k = 0; k < m.n_nets; k++) {
      const int n = net_order[k];
      rank[n] = k;
      dnet_start[k] = w;
      w += m.net_start[n + 1] - m.net_start[n];
    }
    dnet_start[m.n_nets] = w;
    for (int n = 0; n < m.n_nets; n++) {
      int t = dnet_start[rank[n]];
      for (int q = m.net_start[n]; q < m.net_start[n + 1]; q++, t++) {
        const int g = m.pin_g[q];
        dpin_of[q] = t;
        pins[t] = g >= 0 ? make_int4(g, m.pin_ox[q], m.pin_oy[q], 0)
                         : make_int4(-1, m.pin_x[q], m.pin_y[q], 0);
      }
    }
  }
  st.g_dpins.resize(m.g_pins.size());
  for (size_t t = 0; t < m.g_pins.size(); t++) st.g_dpins[t] = dpin_of[m.g_pins[t]];
  make_twiddle(st.tw);
  make_w4(m.cnt_x, st.w4x);
  make_w4(m.cnt_y, st.w4y);
  make_freq(m.cnt_x, m.cnt_y, m.size_x, m.size_y, st.wx, st.wy);
  return GPL_OK;
}

// Runs the position-independent setup (NesterovBase and the device model's
// host arrays); on a worker thread its error message is kept for the caller.
void prepare_static(gpl_job* j, const PlaceRects& rects) {
  int rc = GPL_OK;
  try {
    rc = build_nesterov_static(j->m, rects);
    if (!rc) {
      j->stage.reset(new DevStage());
      rc = stage_device_model(j->m, *j->stage);
    }
  } catch (const std::bad_alloc&) {
    set_error("host allocation failed in the Nesterov setup");
    rc = GPL_ERR_OUT_OF_MEMORY;
  }
  if (rc) j->prep_err = gpl_last_error();
  j->prep_rc = rc;
}

// Starts the position-independent setup beside the initial place (the
// movable instances' sizes are final once the initial place has centred
// them; only their positions change).
void start_static_prep(gpl_job* j) {
  if (j->static_done || j->prep.joinable()) return;
  PlaceRects rects = place_rects(j->m);
  j->prep = std::thread([j, rects = std::move(rects)]() { prepare_static(j, rects); });
}

// Waits for (or runs) the position-independent setup.
int finish_static_prep(gpl_job* j) {
  if (j->static_done) return GPL_OK;
  if (j->prep.joinable()) {
    j->prep.join();
  } else {
    prepare_static(j, place_rects(j->m));
  }
  if (j->prep_rc) {
    set_error(j->prep_err);
    return j->prep_rc;
  }
  j->static_done = true;
  return GPL_OK;
}

int build_graph(gpl_job* j);

// Uploads the job's net weights in device net order (stream-ordered after
// earlier evaluations) and selects the WA kernel variant; when that changes,
// the captured graphs are rebuilt (evaluation) or dropped until the next run
// (device loop).
int apply_net_weights(gpl_job* j) {
  DeviceModel& d = j->d;
  const bool on = !j->net_w.empty();
  if (on) {
    std::vector<float> w(j->net_w.size());
    for (size_t n = 0; n < w.size(); n++) w[j->net_rank[n]] = j->net_w[n];
    int rc = upload(d.net_w, w.data(), w.size() * sizeof(float), j->stream);
    if (rc) return rc;
    GPL_CUDA(cudaStreamSynchronize(j->stream));
  }
  if (on == d.net_weighted) return GPL_OK;
  d.net_weighted = on;
  GPL_CUDA(cudaStreamSynchronize(j->stream));
  if (j->loop_exec) {
    cudaGraphExecDestroy(j->loop_exec);
    j->loop_exec = nullptr;
    j->loop_tried = false;
  }
  if (j->graph_exec) {
    cudaGraphExecDestroy(j->graph_exec);
    j->graph_exec = nullptr;
    return build_graph(j);
  }
  return GPL_OK;
}

// NesterovBase, then the device model (one arena).
int ensure_nb(gpl_job* j) {
  if (j->nb_ready) return GPL_OK;
  const double t0 = wall_ms();
  int rc = finish_static_prep(j);
  if (rc) return rc;
  HostModel& m = j->m;
  place_gcells(m);
  if (m.p.verbose_level >= 2) printf("[NesterovInit] host NesterovBase (wait) %.2f ms\n", wall_ms() - t0);
  DeviceModel& d = j->d;
  const DevStage& st = *j->stage;
  GPL_CUDA(cudaSetDevice(j->device));
  if (!j->side) {
    GPL_CUDA(cudaStreamCreateWithFlags(&j->side, cudaStreamNonBlocking));
    GPL_CUDA(cudaEventCreateWithFlags(&j->ev_fork, cudaEventDisableTiming));
    GPL_CUDA(cudaEventCreateWithFlags(&j->ev_join, cudaEventDisableTiming));
  }
  d.n_g = m.n_g; d.n_place = m.n_place; d.n_pins = m.n_pins; d.n_nets = m.n_nets;
  d.cnt_x = m.cnt_x; d.cnt_y = m.cnt_y; d.size_x = m.size_x; d.size_y = m.size_y;
  d.core_lx = m.core_lx; d.core_ly = m.core_ly; d.core_ux = m.core_ux; d.core_uy = m.core_uy;
  d.target_density = m.p.target_density;
  d.n_big = (int)st.big.size();
  for (int b = 0; b <= kWaBuckets; b++) {
    d.wa_bucket_start[b] = st.wa_bucket_start[b];
    d.wa_block_start[b] = st.wa_block_start[b];
  }
  const size_t nb = (size_t)m.cnt_x * m.cnt_y;
  const size_t ng = m.n_g;
  GPL_CUDA(cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, j->device));
  d.part_stride = std::max(std::max(cell_grid(d), poisson_blocks_a(m.cnt_x, m.cnt_y)), 1);
  const size_t ps = (size_t)kPartSlots * d.part_stride;

  const size_t log_cap = (size_t)std::max(1, m.p.nesterov_place_max_iter);
  const size_t bytes = arena_bytes(ng, m.n_pins, m.n_nets, m.g_pins.size(), st.big.size(), nb, m.cnt_x,
                                   m.cnt_y, d.part_stride, log_cap);
  cudaError_t e = dev_alloc((void**)&j->arena, bytes, j->pool, j->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    j->arena = nullptr;
    set_error(std::string("device allocation of the job arena failed: ") + cudaGetErrorString(e));
    return GPL_ERR_OUT_OF_MEMORY;
  }
  d.bytes = (int64_t)bytes;
  Carver C{j->arena};
  {
    int tw, th, tx, ty;
    tile_grid(m.cnt_x, m.cnt_y, kTileSideMin, &tw, &th, &tx, &ty);
    d.tile_cap = tx * ty;
    d.chunk_cap = scatter_max_chunks((int)ng, d.tile_cap, kScatterChunkMin);
  }
  set_scatter_shape(d, 32, kScatterChunk);        // until the autotuner picks
  d.order = C.take<int32_t>(ng);
  d.tile_count = C.take<int32_t>((size_t)d.tile_cap);
  d.tile_start = C.take<int32_t>((size_t)d.tile_cap + 1);
  d.chunks = C.take<int4>(d.chunk_cap);
  d.n_chunks = C.take<int32_t>(1);
  d.g_half = C.take<int2>(ng); d.g_scale = C.take<float>(ng); d.g_kind = C.take<uint8_t>(ng);
  d.g_precond = C.take<float2>(ng); d.g_pin_start = C.take<int32_t>(ng + 1);
  d.big_cells = C.take<int32_t>(st.big.size());
  d.g_big_idx = C.take<int32_t>(ng); d.d_big = C.take<float2>(st.big.size());
  d.pins = C.take<int4>(m.n_pins);
  d.net_start = C.take<int32_t>(m.n_nets + 1);
  d.pin_grad = C.take<float2>(m.n_pins);
  d.net_w = C.take<float>(m.n_nets);
  d.g_pins = C.take<int32_t>(m.g_pins.size());
  d.area[0] = C.take<unsigned long long>(2 * nb); d.area[1] = C.take<unsigned long long>(2 * nb);
  d.nonplace = C.take<int64_t>(nb);
  d.density = C.take<float>(nb); d.spec = C.take<float>(nb); d.p1 = C.take<float>(nb);
  d.p2 = C.take<float>(nb); d.field = C.take<float2>(nb); d.phi = C.take<float>(nb);
  d.wx = C.take<float>(m.cnt_x); d.wy = C.take<float>(m.cnt_y);
  d.w4x = C.take<float2>(m.cnt_x); d.w4y = C.take<float2>(m.cnt_y);
  d.twiddle = C.take<float2>(st.tw.size());
  for (int k = 0; k < 4; k++) { d.slp[k] = C.take<float2>(ng); d.sum[k] = C.take<float2>(ng); }
  d.coordi[0] = C.take<float2>(ng); d.coordi[1] = C.take<float2>(ng);
  d.wl_out = C.take<float2>(ng); d.d_out = C.take<float2>(ng);
  d.ctl = C.take<EvalCtl>(1);
  d.part = C.take<double>(ps);
  d.result = C.take<EvalResult>(1);
  d.hpwl_total = C.take<long long>(kHpwlLanes * kHpwlStride);
  d.counters = C.take<unsigned>(4);
  d.part_total = C.take<double>(kPartSlots);
  j->d_state = C.take<NesterovState>(1);
  j->d_log = C.take<IterEntry>(log_cap);
  j->log_cap = (int)log_cap;
  cudaStream_t s = j->stream;
  int rc2 = GPL_OK;
  rc2 = rc2 ? rc2 : upload(d.g_half, st.half.data(), ng * sizeof(int2), s);
  rc2 = rc2 ? rc2 : upload(d.g_scale, m.gscale.data(), ng * 4, s);
  rc2 = rc2 ? rc2 : upload(d.g_kind, st.kind.data(), ng, s);
  rc2 = rc2 ? rc2 : upload(d.g_precond, st.precond.data(), ng * sizeof(float2), s);
  rc2 = rc2 ? rc2 : upload(d.g_pin_start, m.g_pin_start.data(), (ng + 1) * 4, s);
  rc2 = rc2 ? rc2 : upload(d.big_cells, st.big.data(), st.big.size() * 4, s);
  rc2 = rc2 ? rc2 : upload(d.g_big_idx, st.big_idx.data(), ng * 4, s);
  rc2 = rc2 ? rc2 : upload(d.pins, st.pins.data(), (size_t)m.n_pins * sizeof(int4), s);
  rc2 = rc2 ? rc2 : upload(d.g_pins, st.g_dpins.data(), st.g_dpins.size() * 4, s);
  rc2 = rc2 ? rc2 : upload(d.net_start, st.dnet_start.data(), (size_t)(m.n_nets + 1) * 4, s);
  rc2 = rc2 ? rc2 : upload(d.nonplace, m.bin_nonplace.data(), nb * 8, s);
  rc2 = rc2 ? rc2 : upload(d.wx, st.wx.data(), st.wx.size() * 4, s);
  rc2 = rc2 ? rc2 : upload(d.wy, st.wy.data(), st.wy.size() * 4, s);
  rc2 = rc2 ? rc2 : upload(d.w4x, st.w4x.data(), st.w4x.size() * sizeof(float2), s);
  rc2 = rc2 ? rc2 : upload(d.w4y, st.w4y.data(), st.w4y.size() * sizeof(float2), s);
  rc2 = rc2 ? rc2 : upload(d.twiddle, st.tw.data(), st.tw.size() * sizeof(float2), s);
  if (rc2) return rc2;
  GPL_CUDA(cudaMemsetAsync(d.area[0], 0, 2 * nb * 8, s));
  GPL_CUDA(cudaMemsetAsync(d.area[1], 0, 2 * nb * 8, s));
  GPL_CUDA(cudaMemsetAsync(d.part, 0, ps * 8, s));
  GPL_CUDA(cudaMemsetAsync(d.phi, 0, nb * 4, s));
  GPL_CUDA(cudaMemsetAsync(d.counters, 0, 4 * sizeof(unsigned), s));
  GPL_CUDA(cudaMemsetAsync(d.hpwl_total, 0, sizeof(long long) * kHpwlLanes * kHpwlStride, s));
  d.result_h = &j->pinned->result;
  d.ctl_h = &j->pinned->ctl;
  memset(d.ctl_h, 0, sizeof(EvalCtl));
  GPL_CUDA(cudaStreamSynchronize(s));
  j->net_rank.swap(j->stage->net_rank);
  j->stage.reset();     // the host copies are no longer needed
  j->nb_ready = true;
  return apply_net_weights(j);
}

EvalArgs base_args(gpl_job* j) {
  EvalArgs a;
  a.min_precond = j->m.p.min_preconditioner;
  a.min_wl_force_bar = j->m.p.min_wire_length_force_bar;
  return a;
}

// Copies the control record to the device (stream-ordered).
int put_ctl(gpl_job* j, const EvalCtl& c) {
  *j->d.ctl_h = c;
  GPL_CUDA(cudaMemcpyAsync(j->d.ctl, j->d.ctl_h, sizeof(EvalCtl), cudaMemcpyHostToDevice, j->stream));
  return GPL_OK;
}

// WA forces, per-gcell gradients and reductions again (the gcell kernel's
// last block writes the result record), then the record's copy to the host:
// a second pass over the same coordinates and bins with new coefficients.
int launch_phase2(gpl_job* j, bool want_phi, int area_set) {
  DeviceModel& d = j->d;
  int rc = launch_wa(d, base_args(j), j->stream, j->timer);
  if (rc) return rc;
  int phi_blocks = 0;
  if (want_phi) {
    rc = launch_sum_phi(d, area_set, j->stream, j->timer, &phi_blocks);
    if (rc) return rc;
  }
  rc = launch_cell(d, base_args(j), phi_blocks, j->stream, j->timer);
  if (rc) return rc;
  GPL_CUDA(cudaMemcpyAsync(d.result_h, d.result, sizeof(EvalResult), cudaMemcpyDeviceToHost, j->stream));
  return GPL_OK;
}

// One evaluation's launches: scatter (with the predictor), then the WA
// kernel on the side stream beside the Poisson passes (WA needs only the
// predicted coordinates, Poisson only the areas), joined before the gcell
// kernel, and the result record's copy to the host.  With kernel timing on,
// everything stays on the job's stream so that each class is timed alone.
int launch_eval(gpl_job* j, bool want_phi, int area_set, bool copy_result = true) {
  DeviceModel& d = j->d;
  int rc = launch_scatter(d, base_args(j), j->stream, j->timer);
  if (rc) return rc;
  const bool fork = j->side && !j->timer.enabled;
  if (fork) {
    GPL_CUDA(cudaEventRecord(j->ev_fork, j->stream));
    GPL_CUDA(cudaStreamWaitEvent(j->side, j->ev_fork, 0));
  }
  rc = launch_wa(d, base_args(j), fork ? j->side : j->stream, j->timer);
  if (rc) return rc;
  if (fork) GPL_CUDA(cudaEventRecord(j->ev_join, j->side));
  rc = launch_poisson_job(d, want_phi, j->stream, j->timer);
  if (rc) return rc;
  if (fork) GPL_CUDA(cudaStreamWaitEvent(j->stream, j->ev_join, 0));
  int phi_blocks = 0;
  if (want_phi) {
    rc = launch_sum_phi(d, area_set, j->stream, j->timer, &phi_blocks);
    if (rc) return rc;
  }
  rc = launch_cell(d, base_args(j), phi_blocks, j->stream, j->timer);
  if (rc) return rc;
  if (copy_result)
    GPL_CUDA(cudaMemcpyAsync(d.result_h, d.result, sizeof(EvalResult), cudaMemcpyDeviceToHost, j->stream));
  return GPL_OK;
}

int finish(gpl_job* j) {
  GPL_CUDA(host_wait(j->stream, j->sync_ev));
  j->S.last = *j->d.result_h;
  return GPL_OK;
}

// Mean time of `reps` Poisson solves on the job's stream (after one warm-up).
float time_poisson(gpl_job* j, int reps) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  Timer quiet;
  launch_poisson_job(j->d, false, j->stream, quiet);
  cudaEventRecord(a, j->stream);
  for (int r = 0; r < reps; r++) launch_poisson_job(j->d, false, j->stream, quiet);
  cudaEventRecord(b, j->stream);
  float ms = 0.0f;
  if (cudaEventSynchronize(b) == cudaSuccess) cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaGetLastError();
  return 1000.0f * ms / reps;
}

// The form of the Poisson solve (gpl_params.poisson_path): auto times the
// shared-memory FFT passes and the tensor-core GEMMs on this job's grid and
// keeps the faster.  Runs before the first evaluation (the areas are still
// zero, so the trial solves change nothing the evaluation reads).
int choose_poisson_path(gpl_job* j) {
  DeviceModel& d = j->d;
  if (j->poisson_chosen) return GPL_OK;
  j->poisson_chosen = true;
  const int want = j->m.p.poisson_path;
  d.poisson_path = 1;
  if (want == 1) return GPL_OK;
  if (!poisson_gemm_eligible(d.cnt_x, d.cnt_y)) {
    if (want == 2) {
      set_error("tensor-core Poisson path: both bin counts must be multiples of 128");
      return GPL_ERR_INVALID_ARG;
    }
    return GPL_OK;
  }
  // Auto mode considers the GEMM form only up to 512 bins per axis: above
  // that it is measured slower than the register-FFT form (1024^2: 196 us
  // against 59 us per solve), so larger grids set up nothing for it.  Its
  // error against the FP64 oracle is within the bars at every size (field
  // 7e-7 at 128^2, 2.6e-6 at 512^2, 5.3e-6 at 1024^2).
  const bool worth_timing = d.cnt_x <= 512 && d.cnt_y <= 512;
  if (want == 0 && !worth_timing) return GPL_OK;
  int rc = poisson_gemm_setup(d, &d.pg, j->pool, j->stream);
  if (rc) {
    if (want == 2) return rc;
    cudaGetLastError();
    return GPL_OK;                 // auto: the FFT form
  }
  EvalCtl c;
  memset(&c, 0, sizeof(c));
  rc = put_ctl(j, c);
  if (rc) return rc;
  if (want == 2) {
    d.poisson_path = 2;
    j->poisson_gemm_us = time_poisson(j, 5);
    return GPL_OK;
  }
  j->poisson_fft_us = time_poisson(j, 5);
  d.poisson_path = 2;
  j->poisson_gemm_us = time_poisson(j, 5);
  int flag = 0;
  poisson_gemm_error(d.pg, j->stream, &flag);
  if (flag || !(j->poisson_gemm_us > 0.0f) || j->poisson_gemm_us >= j->poisson_fft_us) {
    d.poisson_path = 1;
    poisson_gemm_free(d.pg, j->pool, j->stream);
    d.pg = nullptr;
  }
  return GPL_OK;
}

// The whole evaluation as one CUDA graph (control-record upload, kernels,
// result download); every evaluation of the job replays it.
int build_graph(gpl_job* j) {
  if (!j->m.p.use_graph || j->graph_exec) return GPL_OK;
  int rc0 = poisson_prepare_device();
  if (rc0) return rc0;
  const bool te = j->timer.enabled;
  j->timer.enabled = false;
  const long long k0 = j->timer.kernels;
  cudaGraph_t g = nullptr;
  int rc = GPL_OK;
  if (cudaStreamBeginCapture(j->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    j->timer.enabled = te;
    return GPL_OK;                       // stream cannot be captured: direct launches
  }
  cudaMemcpyAsync(j->d.ctl, j->d.ctl_h, sizeof(EvalCtl), cudaMemcpyHostToDevice, j->stream);
  rc = launch_eval(j, false, 0);
  cudaError_t e = cudaStreamEndCapture(j->stream, &g);
  j->graph_kernels = j->timer.kernels - k0;
  j->timer.kernels = k0;
  j->timer.enabled = te;
  if (rc || e != cudaSuccess || !g) {
    cudaGetLastError();
    if (g) cudaGraphDestroy(g);
    return GPL_OK;
  }
  if (cudaGraphInstantiate(&j->graph_exec, g, 0) != cudaSuccess) {
    cudaGetLastError();
    j->graph_exec = nullptr;
  }
  cudaGraphDestroy(g);
  return GPL_OK;
}

// One evaluation at control record c (area set chosen here).
int evaluate(gpl_job* j, EvalCtl c, bool want_phi) {
  c.area_cur = j->S.area_next;
  int rc = GPL_OK;
  if (j->graph_exec && !want_phi && !j->timer.enabled) {
    *j->d.ctl_h = c;
    GPL_CUDA(cudaGraphLaunch(j->graph_exec, j->stream));
    j->timer.count((int)j->graph_kernels);
  } else {
    rc = put_ctl(j, c);
    if (!rc) rc = launch_eval(j, want_phi, c.area_cur);
  }
  if (rc) return rc;
  j->S.last_area = c.area_cur;
  j->S.area_next = c.area_cur ^ 1;
  j->S.last_slot = c.i_eval;
  j->S.evals++;
  return finish(j);
}

// Phase 2 again with a new control record (same coordinates and bins).
int rerun_phase2(gpl_job* j, EvalCtl c) {
  c.area_cur = j->S.last_area;
  int rc = put_ctl(j, c);
  if (!rc) rc = launch_phase2(j, false, c.area_cur);
  if (rc) return rc;
  return finish(j);
}

float overflow_ratio(const gpl_job* j) { return overflow_ratio_of(j->S, j->S.last.overflow); }

void update_wl_coef(gpl_job* j, float overflow) { update_wl_coef_of(j->S, overflow); }

EvalCtl ctl_of(gpl_job* j, int i_eval, int i_ref, bool write_sum) {
  EvalCtl c;
  memset(&c, 0, sizeof(c));
  c.density_penalty = j->S.density_penalty;
  c.wl_coef_x = j->S.wl_coef_x;
  c.wl_coef_y = j->S.wl_coef_y;
  c.i_src = j->S.i_cur;
  c.i_eval = i_eval;
  c.i_ref = i_ref;
  c.c_cur = j->S.c_cur;
  c.c_next = j->S.c_next;
  c.write_sum = write_sum ? 1 : 0;
  return c;
}

bool diverged(const gpl_job* j) { return diverged_result(j->S.last); }

// The scatter's shape (tile side, gcells per chunk): every candidate is
// timed on the job's first coordinates (slot `slot`) and the fastest kept.  The trial scatters only add into
// area set 0, which is cleared afterwards; the areas do not depend on the
// shape.
int choose_scatter_shape(gpl_job* j, int slot) {
  DeviceModel& d = j->d;
  int rc = scatter_prepare_device();
  if (rc) return rc;
  // The trials run the predictor as the loop does (its loads and stores are
  // part of the scatter's cost) with step 0 and coefficient 0, so the
  // predicted coordinates equal slot `slot`'s; they go to the hook's slot 3
  // and to coordi[c_next], both unread before they are next written.
  const size_t ng = (size_t)d.n_g;
  GPL_CUDA(cudaMemsetAsync(d.sum[slot], 0, ng * sizeof(float2), j->stream));
  EvalCtl c;
  memset(&c, 0, sizeof(c));
  c.predict = 1;
  c.i_src = slot;
  c.i_eval = 3;
  c.i_ref = -1;
  c.c_cur = j->S.c_cur;
  c.c_next = j->S.c_next;
  rc = put_ctl(j, c);
  if (rc) return rc;
  Timer quiet;
  cudaEvent_t a = nullptr, b = nullptr;
  GPL_CUDA(cudaEventCreate(&a));
  GPL_CUDA(cudaEventCreate(&b));
  constexpr int kReps = 3;
  float best = 1e30f;
  int best_side = 32, best_chunk = kScatterChunk;
  int seen[16][3];
  int n_seen = 0;
  const int want_side = j->m.p.scatter_tile, want_chunk = j->m.p.scatter_chunk;
  for (int side : kTileSides) {
    for (int chunk : kScatterChunks) {
      if ((want_side && side != want_side) || (want_chunk && chunk != want_chunk)) continue;
      if (!set_scatter_shape(d, side, chunk)) continue;
      bool dup = false;
      for (int k = 0; k < n_seen; k++) dup |= seen[k][0] == d.tile_w && seen[k][1] == d.tile_h && seen[k][2] == chunk;
      if (dup || n_seen >= 16) continue;
      seen[n_seen][0] = d.tile_w; seen[n_seen][1] = d.tile_h; seen[n_seen][2] = chunk;
      n_seen++;
      rc = launch_tile_order(d, slot, j->stream, quiet);
      if (!rc) rc = launch_scatter(d, base_args(j), j->stream, quiet);    // warm-up
      if (rc) break;
      cudaEventRecord(a, j->stream);
      for (int r = 0; r < kReps && !rc; r++) rc = launch_scatter(d, base_args(j), j->stream, quiet);
      cudaEventRecord(b, j->stream);
      if (rc) break;
      float ms = 0.0f;
      if (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
        rc = GPL_ERR_CUDA;
        set_error("scatter autotuner: event timing failed");
        break;
      }
      if (ms < best) { best = ms; best_side = side; best_chunk = chunk; }
    }
    if (rc) break;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  set_scatter_shape(d, best_side, best_chunk);
  j->scatter_us = best < 1e29f ? 1000.0f * best / kReps : 0.0f;
  const size_t nb = (size_t)d.cnt_x * d.cnt_y;
  GPL_CUDA(cudaMemsetAsync(d.area[0], 0, 2 * nb * 8, j->stream));
  GPL_CUDA(cudaMemsetAsync(d.area[1], 0, 2 * nb * 8, j->stream));
  return GPL_OK;
}

// NesterovPlace::init (src/nesterovPlace.cpp:64-175)
int nesterov_init(gpl_job* j) {
  const bool tell = j->m.p.verbose_level >= 2;
  const double t0 = wall_ms();
  int rc = ensure_nb(j);
  if (rc) return rc;
  HostModel& m = j->m;
  DeviceModel& d = j->d;
  NesterovState& S = j->S;
  S.max_back_track = m.p.max_back_track;
  S.max_iter = m.p.nesterov_place_max_iter;
  S.target_overflow = m.p.target_overflow;
  S.min_phi_coef = m.p.min_phi_coef;
  S.reference_hpwl = m.p.reference_hpwl;
  S.ovf_den = (float)(m.std_area + m.macro_area * m.p.target_density);
  const size_t ng = m.n_g;
  std::vector<float2> c0(ng);
  for (size_t g = 0; g < ng; g++) {
    // updateDensityCoordiLayoutInside (src/nesterovBase.cpp:1245-1268)
    float tlx = (float)m.gdlx[g], tly = (float)m.gdly[g];
    const int ddx = m.gdux[g] - m.gdlx[g], ddy = m.gduy[g] - m.gdly[g];
    if (tlx < m.core_lx) tlx = (float)m.core_lx;
    if (tly < m.core_ly) tly = (float)m.core_ly;
    if (tlx + ddx > m.core_ux) tlx = (float)(m.core_ux - ddx);
    if (tly + ddy > m.core_uy) tly = (float)(m.core_uy - ddy);
    const int nlx = (int)tlx, nly = (int)tly;
    c0[g] = make_float2((float)((2 * nlx + ddx) / 2), (float)((2 * nly + ddy) / 2));
  }
  j->S.i_prev = 0; j->S.i_cur = 1; j->S.i_next = 2; j->S.c_cur = 0; j->S.c_next = 1;
  rc = upload(d.slp[j->S.i_cur], c0.data(), ng * sizeof(float2), j->stream);
  if (rc) return rc;
  GPL_CUDA(cudaMemcpyAsync(d.slp[j->S.i_prev], d.slp[j->S.i_cur], ng * sizeof(float2), cudaMemcpyDeviceToDevice, j->stream));
  GPL_CUDA(cudaMemcpyAsync(d.coordi[j->S.c_cur], d.slp[j->S.i_cur], ng * sizeof(float2), cudaMemcpyDeviceToDevice, j->stream));
  const double t1 = wall_ms();
  // autotuned shapes: the scatter's tile and chunk, then the Poisson form
  // (both before the evaluation graph is captured)
  rc = choose_scatter_shape(j, j->S.i_cur);
  if (rc) return rc;
  rc = choose_poisson_path(j);
  if (rc) return rc;
  const double t2 = wall_ms();
  rc = build_graph(j);
  if (rc) return rc;
  if (tell)
    printf("[NesterovInit] base, device model and centres %.2f ms, autotuning %.2f ms (scatter tile %dx%d, "
           "chunk %d), graph %.2f ms\n", t1 - t0, t2 - t1, d.tile_w, d.tile_h, d.chunk, wall_ms() - t2);
  j->S.density_penalty = 0.0f;
  j->S.max_phi_coef = m.p.max_phi_coef;
  j->S.wl_coef_x = j->S.wl_coef_y = 0.0f;
  // first evaluation at the initial centres: overflow and HPWL
  rc = launch_tile_order(d, j->S.i_cur, j->stream, j->timer);
  if (rc) return rc;
  rc = evaluate(j, ctl_of(j, j->S.i_cur, -1, false), false);
  if (rc) return rc;
  j->S.prev_hpwl = j->S.last.hpwl;
  j->S.base_wl_coef = (float)(m.p.init_wire_length_coef / ((float)(m.size_x + m.size_y) * 0.5));
  j->S.sum_overflow = overflow_ratio(j);
  update_wl_coef(j, j->S.sum_overflow);
  // the WA forces and gradients with the wire-length coefficients set
  rc = rerun_phase2(j, ctl_of(j, j->S.i_cur, -1, true));
  if (rc) return rc;
  if (diverged(j)) {
    j->S.is_diverged = true; j->S.diverge_code = GPL_ERR_DIVERGED_INIT; j->np_ready = true;
    set_error("RePlAce diverged. Please tune the parameters again");
    return GPL_ERR_DIVERGED_INIT;
  }
  // updateInitialPrevSLPCoordi (src/nesterovPlace.cpp:492-512)
  rc = launch_initial_prev(d, d.slp[j->S.i_cur], d.sum[j->S.i_cur], m.p.initial_prev_coordi_update_coef,
                           d.slp[j->S.i_prev], j->stream, j->timer);
  if (rc) return rc;
  rc = evaluate(j, ctl_of(j, j->S.i_prev, j->S.i_cur, true), false);
  if (rc) return rc;
  if (diverged(j)) {
    j->S.is_diverged = true; j->S.diverge_code = GPL_ERR_DIVERGED_INIT; j->np_ready = true;
    set_error("RePlAce diverged. Please tune the parameters again");
    return GPL_ERR_DIVERGED_INIT;
  }
  j->S.density_penalty = ((float)j->S.last.wl_sum / (float)j->S.last.d_sum) * m.p.init_density_penalty;
  j->S.sum_overflow = overflow_ratio(j);
  j->S.step_length = j->S.last.new_step_length;
  j->S.cur_a = 1.0f;
  j->S.min_sum_overflow = 1e30f;
  j->S.hpwl_with_min = 1e30f;
  j->S.max_phi_changed = false;
  j->S.iter = 0;
  j->S.finished = false;
  j->np_ready = true;
  return GPL_OK;
}

// The job's loop graph: a head kernel, then WHILE (condition set by the
// kernels) { IF (refresh) the tile order; one evaluation; the step kernel }.
// Built once per job after the evaluation graph; a failure leaves the host
// loop in charge (same kernels, same control arithmetic).
int build_loop_graph(gpl_job* j) {
  if (j->loop_tried) return GPL_OK;
  j->loop_tried = true;
  if (!j->m.p.use_graph || !j->m.p.device_loop || !j->d_state || !j->d_log) return GPL_OK;
  int rc0 = poisson_prepare_device();
  if (rc0) return rc0;
  DeviceModel& d = j->d;
  const bool te = j->timer.enabled;
  j->timer.enabled = false;
  const long long k0 = j->timer.kernels;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool ok = cudaGraphCreate(&g, 0) == cudaSuccess;
  cudaGraphConditionalHandle h_loop = 0, h_order = 0;
  ok = ok && cudaGraphConditionalHandleCreate(&h_loop, g, 0, cudaGraphCondAssignDefault) == cudaSuccess;
  ok = ok && cudaGraphConditionalHandleCreate(&h_order, g, 0, cudaGraphCondAssignDefault) == cudaSuccess;
  // head
  cudaGraphNode_t head = nullptr;
  if (ok) {
    cudaGraph_t cap = nullptr;
    ok = cudaStreamBeginCaptureToGraph(j->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
         cudaSuccess;
    int rc = ok ? launch_loop_head(j->d_state, d.ctl, h_loop, h_order, j->stream) : GPL_OK;
    if (ok) ok = cudaStreamEndCapture(j->stream, &cap) == cudaSuccess && !rc;
    size_t n = 1;
    ok = ok && cudaGraphGetNodes(g, &head, &n) == cudaSuccess && n == 1;
  }
  // WHILE node and its body
  cudaGraph_t body = nullptr;
  if (ok) {
    cudaGraphNodeParams wp = {cudaGraphNodeTypeConditional};
    wp.conditional.handle = h_loop;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode = nullptr;
    ok = cudaGraphAddNode(&wnode, g, &head, nullptr, 1, &wp) == cudaSuccess;
    if (ok) body = wp.conditional.phGraph_out[0];
  }
  cudaGraphNode_t inode = nullptr;
  long long order_kernels = 0;
  if (ok) {
    cudaGraphNodeParams ip = {cudaGraphNodeTypeConditional};
    ip.conditional.handle = h_order;
    ip.conditional.type = cudaGraphCondTypeIf;
    ip.conditional.size = 1;
    ok = cudaGraphAddNode(&inode, body, nullptr, nullptr, 0, &ip) == cudaSuccess;
    if (ok) {
      cudaGraph_t obody = ip.conditional.phGraph_out[0], cap = nullptr;
      const long long o0 = j->timer.kernels;
      ok = cudaStreamBeginCaptureToGraph(j->stream, obody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
           cudaSuccess;
      int rc = ok ? launch_tile_order(d, -1, j->stream, j->timer) : GPL_OK;
      if (ok) ok = cudaStreamEndCapture(j->stream, &cap) == cudaSuccess && !rc;
      order_kernels = j->timer.kernels - o0;
    }
  }
  if (ok) {
    cudaGraph_t cap = nullptr;
    ok = cudaStreamBeginCaptureToGraph(j->stream, body, &inode, nullptr, 1, cudaStreamCaptureModeThreadLocal) ==
         cudaSuccess;
    int rc = ok ? launch_eval(j, false, 0, false) : GPL_OK;
    if (ok && !rc)
      rc = launch_loop_step(j->d_state, d.ctl, d.result, j->d_log, j->log_cap, h_loop, h_order, j->stream);
    if (ok) ok = cudaStreamEndCapture(j->stream, &cap) == cudaSuccess && !rc;
  }
  ok = ok && cudaGraphInstantiate(&exec, g, 0) == cudaSuccess;
  j->timer.kernels = k0;
  j->timer.enabled = te;
  if (g) cudaGraphDestroy(g);
  cudaGetLastError();
  if (!ok) {
    if (exec) cudaGraphExecDestroy(exec);
    if (j->m.p.verbose_level > 0) printf("[NesterovSolve] device loop not built: the host drives the loop\n");
    return GPL_OK;
  }
  j->loop_exec = exec;
  j->order_kernels = order_kernels;
  return GPL_OK;
}

// Appends a finished iteration to the caller's log and prints the
// reference's progress line.
void record_iteration(gpl_job* j, const IterEntry& e, int iter_number, gpl_iter_log* log) {
  if (log && log->count < log->capacity) {
    const int k = log->count++;
    if (log->overflow) log->overflow[k] = e.overflow;
    if (log->hpwl) log->hpwl[k] = e.hpwl;
    if (log->step_length) log->step_length[k] = e.step_length;
    if (log->backtracks) log->backtracks[k] = e.backtracks;
  }
  if (j->m.p.verbose_level > 0 && (iter_number == 1 || iter_number % 10 == 0)) {
    printf("[NesterovSolve] Iter: %d overflow: %g HPWL: %lld\n", iter_number, e.overflow, (long long)e.hpwl);
    fflush(stdout);
  }
}

// Up to max_iters iterations (0: to the stop rule) on the device loop.
int run_device_chunk(gpl_job* j, int max_iters, gpl_iter_log* log) {
  NesterovState& S = j->S;
  const int iter0 = S.iter, evals0 = S.evals, refreshes0 = S.refreshes;
  S.chunk_limit = max_iters;
  NesterovState* hs = &j->pinned->state;
  *hs = S;
  GPL_CUDA(cudaMemcpyAsync(j->d_state, hs, sizeof(NesterovState), cudaMemcpyHostToDevice, j->stream));
  GPL_CUDA(cudaGraphLaunch(j->loop_exec, j->stream));
  GPL_CUDA(cudaMemcpyAsync(hs, j->d_state, sizeof(NesterovState), cudaMemcpyDeviceToHost, j->stream));
  GPL_CUDA(host_wait(j->stream, j->sync_ev));
  S = *hs;
  const int n_log = std::min(S.log_count, j->log_cap);
  if (n_log > 0) {
    std::vector<IterEntry> entries(n_log);
    GPL_CUDA(cudaMemcpyAsync(entries.data(), j->d_log, n_log * sizeof(IterEntry), cudaMemcpyDeviceToHost, j->stream));
    GPL_CUDA(cudaStreamSynchronize(j->stream));
    for (int k = 0; k < n_log; k++) record_iteration(j, entries[k], iter0 + k + 1, log);
  }
  // launches: the head, per evaluation its kernels and the step kernel, per
  // refresh the tile-order kernels
  j->timer.count((int)(1 + (long long)(S.evals - evals0) * (j->graph_kernels + 1) +
                       (long long)(S.refreshes - refreshes0) * j->order_kernels));
  return GPL_OK;
}

// The same loop driven from the host, one evaluation at a time.
int run_host_loop(gpl_job* j, int max_iters, gpl_iter_log* log) {
  NesterovState& S = j->S;
  int done = 0;
  while (!S.finished && S.iter < S.max_iter) {
    if (max_iters > 0 && done >= max_iters) break;
    done++;
    start_iteration(S);
    if (S.iter % kTileOrderEvery == 0) {
      int rc = launch_tile_order(j->d, S.i_cur, j->stream, j->timer);
      if (rc) return rc;
      S.refreshes++;
    }
    for (;;) {
      const EvalCtl c = next_ctl(S);
      int rc = GPL_OK;
      if (j->graph_exec && !j->timer.enabled) {
        *j->d.ctl_h = c;
        GPL_CUDA(cudaGraphLaunch(j->graph_exec, j->stream));
        j->timer.count((int)j->graph_kernels);
      } else {
        rc = put_ctl(j, c);
        if (!rc) rc = launch_eval(j, false, c.area_cur);
      }
      if (rc) return rc;
      GPL_CUDA(host_wait(j->stream, j->sync_ev));
      const EvalResult r = *j->d.result_h;
      IterEntry e;
      bool logged = false;
      const int a = after_eval(S, r, &e, &logged);
      if (logged) record_iteration(j, e, S.iter, log);
      if (a != kRetry) break;
    }
  }
  return GPL_OK;
}

int end_of_run(gpl_job* j);

// NesterovPlace::doNesterovPlace (src/nesterovPlace.cpp:275-472), resumable:
// the device loop when the job has one (no kernel timing), else the host loop.
int nesterov_run(gpl_job* j, int max_iters, gpl_iter_log* log) {
  NesterovState& S = j->S;
  if (S.diverge_code == GPL_ERR_DIVERGED_INIT) { S.finished = 1; return S.diverge_code; }
  if (!S.finished && S.iter < S.max_iter) {
    int rc = build_loop_graph(j);
    if (rc) return rc;
    const bool device = j->loop_exec && !j->timer.enabled;
    rc = device ? run_device_chunk(j, max_iters, log) : run_host_loop(j, max_iters, log);
    if (rc) return rc;
    if (S.finished && !S.diverge_code && j->m.p.verbose_level > 0) {
      printf("[NesterovSolve] Finished with Overflow: %g\n", S.sum_overflow);
      fflush(stdout);
    }
  }
  return end_of_run(j);
}

// After a chunk of iterations: the stop on the iteration limit, the
// divergence message, and the tensor-core form's time-out flag.
int end_of_run(gpl_job* j) {
  NesterovState& S = j->S;
  if (S.iter >= S.max_iter) S.finished = 1;
  switch (S.diverge_code) {
    case GPL_ERR_DIVERGED_BACKTRACK: set_error("RePlAce divergence detected. Please decrease init_density_penalty value"); break;
    case GPL_ERR_DIVERGED_NAN: set_error("RePlAce divergence detected: NaN or Inf in the gradient sums"); break;
    case GPL_ERR_DIVERGED_PHI: set_error("RePlAce divergence detected. Please decrease max_phi_cof value"); break;
    default: break;
  }
  if (j->d.poisson_path == 2) {
    int flag = 0;
    int rc = poisson_gemm_error(j->d.pg, j->stream, &flag);
    if (rc) return rc;
    if (flag) {
      set_error("tensor-core Poisson path: a pipeline wait timed out; results are invalid");
      return GPL_ERR_CUDA;
    }
  }
  return S.diverge_code;
}

// ------------------------------------------------------------ batched form
// The Nesterov loops of many jobs in lockstep: every round, each member
// job's next evaluation (its next back-tracking try, or the first try of
// its next iteration) goes into one launch per phase (batched kernels of
// density.cu, wirelength.cu, poisson.cu) driven by a table of work items
// (member slot, block of the job's own launch, that launch's grid); then
// each job's control (control.h) takes its result exactly as the host loop
// does.  A job's blocks compute what its own launches compute, in the same
// blocks, so its iterates, log and result are bit-identical to running it
// alone.  Members join and leave between rounds; the round's launches are
// one CUDA graph (persistent grids; argument tables and items in device
// memory), captured again only when the launches themselves change.
}  // namespace

namespace gpl {

enum BatchTable { kTScatter = 0, kTWa, kTPa, kTPb, kTPc, kTCell, kTables };

struct BatchRun {
  int cap = 0, device = 0, sms = 1;
  cudaStream_t s = nullptr;
  char* dev = nullptr;                 // argument tables, control and result records, counts
  char* host = nullptr;                // pinned: control and result records, counts
  char* args[kTables] = {nullptr};
  size_t stride[kTables] = {0};
  EvalCtl* ctl_d = nullptr;
  EvalResult* res_d = nullptr;
  int* counts_d = nullptr;
  EvalCtl* ctl_h = nullptr;
  EvalResult* res_h = nullptr;
  int* counts_h = nullptr;
  int4* items_d = nullptr;             // [items_cap], grown on demand
  int4* items_h = nullptr;             // pinned mirror
  int items_cap = 0;
  int item_off[kBPhases] = {0};
  bool phase_used[kBPhases] = {false};
  size_t smem_scatter = 0, smem_p[3] = {0, 0, 0};
  std::vector<std::array<int, kBPhases>> vgrid;
  std::vector<BatchMember> members;    // by slot; job == nullptr: free
  cudaGraphExec_t exec = nullptr;
  bool items_dirty = true, graph_dirty = true;
  long long launches_per_round = 0;
  ~BatchRun() {
    if (exec) cudaGraphExecDestroy(exec);
    if (s) cudaStreamSynchronize(s);
    if (dev) cudaFree(dev);
    if (items_d) cudaFree(items_d);
    if (host) cudaFreeHost(host);
    if (items_h) cudaFreeHost(items_h);
    if (s) cudaStreamDestroy(s);
  }
};

BatchRun* batch_create(int device, int capacity, int* rc_out) {
  *rc_out = GPL_OK;
  std::unique_ptr<BatchRun> B(new BatchRun());
  B->cap = capacity;
  B->device = device;
  auto fail = [&](int rc) { *rc_out = rc; return nullptr; };
  if (cudaSetDevice(device) != cudaSuccess) { set_error("batch: cudaSetDevice failed"); return fail(GPL_ERR_CUDA); }
  cudaDeviceGetAttribute(&B->sms, cudaDevAttrMultiProcessorCount, device);
  B->sms = std::max(1, B->sms);
  if (cudaStreamCreateWithFlags(&B->s, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("batch: stream creation failed");
    return fail(GPL_ERR_CUDA);
  }
  int rc = scatter_prepare_device();
  if (!rc) rc = scatter_batch_prepare_device();
  if (!rc) rc = poisson_prepare_device();
  if (!rc) rc = poisson_batch_prepare_device();
  if (rc) return fail(rc);
  B->stride[kTScatter] = scatter_batch_args_bytes();
  B->stride[kTWa] = wa_batch_args_bytes();
  B->stride[kTPa] = poisson_batch_args_bytes(0);
  B->stride[kTPb] = poisson_batch_args_bytes(1);
  B->stride[kTPc] = poisson_batch_args_bytes(2);
  B->stride[kTCell] = cell_batch_args_bytes();
  size_t off = 0;
  auto take = [&](size_t b) { const size_t o = off; off += (b + 255) / 256 * 256; return o; };
  size_t o_args[kTables];
  for (int t = 0; t < kTables; t++) o_args[t] = take(B->stride[t] * capacity);
  const size_t o_ctl = take(sizeof(EvalCtl) * capacity), o_res = take(sizeof(EvalResult) * capacity);
  const size_t o_counts = take(sizeof(int) * kBPhases);
  if (cudaMalloc(&B->dev, off) != cudaSuccess) {
    cudaGetLastError();
    set_error("batch: device tables");
    return fail(GPL_ERR_OUT_OF_MEMORY);
  }
  for (int t = 0; t < kTables; t++) B->args[t] = B->dev + o_args[t];
  B->ctl_d = reinterpret_cast<EvalCtl*>(B->dev + o_ctl);
  B->res_d = reinterpret_cast<EvalResult*>(B->dev + o_res);
  B->counts_d = reinterpret_cast<int*>(B->dev + o_counts);
  size_t hoff = 0;
  auto htake = [&](size_t b) { const size_t o = hoff; hoff += (b + 255) / 256 * 256; return o; };
  const size_t h_ctl = htake(sizeof(EvalCtl) * capacity), h_res = htake(sizeof(EvalResult) * capacity);
  const size_t h_counts = htake(sizeof(int) * kBPhases);
  if (cudaMallocHost(&B->host, hoff) != cudaSuccess) {
    cudaGetLastError();
    set_error("batch: pinned records");
    return fail(GPL_ERR_OUT_OF_MEMORY);
  }
  memset(B->host, 0, hoff);
  B->ctl_h = reinterpret_cast<EvalCtl*>(B->host + h_ctl);
  B->res_h = reinterpret_cast<EvalResult*>(B->host + h_res);
  B->counts_h = reinterpret_cast<int*>(B->host + h_counts);
  B->vgrid.assign(capacity, {});
  for (auto& v : B->vgrid) v.fill(0);
  B->members.assign(capacity, BatchMember());
  return B.release();
}

void batch_destroy(BatchRun* B) { delete B; }

// Whether the job can run in a batch: the FFT Poisson form with its
// shared-memory passes (the batched kernels' form).
bool batch_eligible(const gpl_job* j) {
  return j->np_ready && j->d.poisson_path == 1 &&
         !(j->d.cnt_x == j->d.cnt_y && (j->d.cnt_x == 512 || j->d.cnt_x == 1024));
}

// The job takes member slot `slot`: its argument tables (its control and
// result records redirected to the batch's slots) and its blocks per phase.
int batch_join(BatchRun* B, int slot, gpl_job* j, int max_iters, gpl_iter_log* log) {
  if (slot < 0 || slot >= B->cap || B->members[slot].job) { set_error("batch: slot in use"); return GPL_ERR_BAD_STATE; }
  if (!batch_eligible(j)) {
    set_error("batched Nesterov loop: the job does not run the block-form FFT Poisson passes (its grid is "
              "512 x 512 or 1024 x 1024, or it runs the tensor-core form); run it alone");
    return GPL_ERR_INVALID_ARG;
  }
  if (j->device != B->device) { set_error("batch: the job is on another device"); return GPL_ERR_INVALID_ARG; }
  DeviceModel& d = j->d;
  std::vector<char> buf;
  size_t total = 0;
  for (int t = 0; t < kTables; t++) total += B->stride[t];
  buf.assign(total, 0);
  char* part[kTables];
  size_t o = 0;
  for (int t = 0; t < kTables; t++) { part[t] = buf.data() + o; o += B->stride[t]; }
  EvalCtl* own_ctl = d.ctl;
  EvalResult* own_res = d.result;
  d.ctl = B->ctl_d + slot;
  d.result = B->res_d + slot;
  write_scatter_batch_args(d, part[kTScatter]);
  write_wa_batch_args(d, base_args(j), part[kTWa]);
  write_cell_batch_args(d, base_args(j), part[kTCell]);
  int g3[3];
  size_t sm3[3];
  const bool ok = write_poisson_batch_args(d, part[kTPa], part[kTPb], part[kTPc], g3, sm3);
  d.ctl = own_ctl;
  d.result = own_res;
  if (!ok) { set_error("batch: Poisson arguments"); return GPL_ERR_INVALID_ARG; }
  // the job's own stream may still hold work (initialisation)
  GPL_CUDA(cudaStreamSynchronize(j->stream));
  for (int t = 0; t < kTables; t++)
    GPL_CUDA(cudaMemcpyAsync(B->args[t] + (size_t)slot * B->stride[t], part[t], B->stride[t],
                             cudaMemcpyHostToDevice, B->s));
  GPL_CUDA(cudaStreamSynchronize(B->s));       // the staging buffer is local
  std::array<int, kBPhases>& v = B->vgrid[slot];
  v.fill(0);
  v[kBScatter] = d.max_chunks;
  v[kBScatterBig] = d.n_big;
  v[kBDgradBig] = d.n_big;
  v[kBCell] = cell_grid(d);
  int small = 0, large = 0;
  wa_launch_blocks(d, &small, &large);
  v[d.net_weighted ? kBWaSmallW : kBWaSmall] = small;
  v[d.net_weighted ? kBWaLargeW : kBWaLarge] = large;
  for (int q = 0; q < 3; q++) v[kBPoissonA + q] = g3[q];
  const size_t ss = scatter_smem(d);
  if (ss > B->smem_scatter) { B->smem_scatter = ss; B->graph_dirty = true; }
  for (int q = 0; q < 3; q++)
    if (sm3[q] > B->smem_p[q]) { B->smem_p[q] = sm3[q]; B->graph_dirty = true; }
  for (int p = 0; p < kBPhases; p++)
    if (v[p] && !B->phase_used[p]) { B->phase_used[p] = true; B->graph_dirty = true; }
  BatchMember& m = B->members[slot];
  m = BatchMember();
  m.job = j;
  m.limit = max_iters;
  m.log = log;
  const NesterovState& S = j->S;
  m.running = !S.finished && S.iter < S.max_iter && S.diverge_code != GPL_ERR_DIVERGED_INIT;
  B->items_dirty = true;
  return GPL_OK;
}

void batch_leave(BatchRun* B, int slot) {
  if (slot < 0 || slot >= B->cap) return;
  B->members[slot] = BatchMember();
  B->vgrid[slot].fill(0);
  B->items_dirty = true;
}

namespace {

// Work items of the running members: slot k's blocks of each phase.
int batch_items(BatchRun& B) {
  int total = 0;
  for (int p = 0; p < kBPhases; p++)
    for (int k = 0; k < B.cap; k++)
      if (B.members[k].job && B.members[k].running) total += B.vgrid[k][p];
  if (total > B.items_cap) {
    const int cap = std::max(total, 2 * B.items_cap);
    if (B.items_d) cudaFree(B.items_d);
    if (B.items_h) cudaFreeHost(B.items_h);
    B.items_d = nullptr;
    B.items_h = nullptr;
    B.items_cap = 0;
    GPL_CUDA(cudaMalloc(&B.items_d, sizeof(int4) * cap));
    GPL_CUDA(cudaMallocHost(&B.items_h, sizeof(int4) * cap));
    B.items_cap = cap;
    B.graph_dirty = true;              // the launches read the new buffer
  }
  int at = 0;
  for (int p = 0; p < kBPhases; p++) {
    B.item_off[p] = at;
    int c = 0;
    for (int k = 0; k < B.cap; k++) {
      const BatchMember& m = B.members[k];
      if (!m.job || !m.running) continue;
      const int vg = B.vgrid[k][p];
      for (int vb = 0; vb < vg; vb++) B.items_h[at + c++] = make_int4(k, vb, vg, 0);
    }
    B.counts_h[p] = c;
    at += c;
  }
  if (at) GPL_CUDA(cudaMemcpyAsync(B.items_d, B.items_h, sizeof(int4) * at, cudaMemcpyHostToDevice, B.s));
  GPL_CUDA(cudaMemcpyAsync(B.counts_d, B.counts_h, sizeof(int) * kBPhases, cudaMemcpyHostToDevice, B.s));
  // the item offsets are launch arguments: a new layout is a new graph
  static_assert(kBPhases <= 16, "phase table");
  B.graph_dirty = true;
  B.items_dirty = false;
  return GPL_OK;
}

// One round's launches: control records up, every phase in use, result
// records down.  Persistent grids of about the per-job kernels' residency.
int batch_launch_round(BatchRun& B) {
  static const int per_sm[kBPhases] = {4, 4, 5, 1, 5, 1, 4, 4, 4, 4, 4};
  long long nl = 0;
  GPL_CUDA(cudaMemcpyAsync(B.ctl_d, B.ctl_h, sizeof(EvalCtl) * B.cap, cudaMemcpyHostToDevice, B.s));
  auto items = [&](int p) { return B.items_d + B.item_off[p]; };
  auto count = [&](int p) { return B.counts_d + p; };
  auto grid = [&](int p) { return B.sms * per_sm[p]; };
  int rc = GPL_OK;
  if (B.phase_used[kBScatter]) {
    rc = launch_density_batch(kBScatter, B.args[kTScatter], items(kBScatter), count(kBScatter), grid(kBScatter),
                              B.smem_scatter, B.s);
    nl++;
  }
  if (!rc && B.phase_used[kBScatterBig]) {
    rc = launch_density_batch(kBScatterBig, B.args[kTScatter], items(kBScatterBig), count(kBScatterBig),
                              grid(kBScatterBig), 0, B.s);
    nl++;
  }
  const int wa_phase[4] = {kBWaSmall, kBWaLarge, kBWaSmallW, kBWaLargeW};
  for (int q = 0; q < 4 && !rc; q++) {
    const int p = wa_phase[q];
    if (!B.phase_used[p]) continue;
    rc = launch_wa_batch(q & 1, q >= 2, B.args[kTWa], items(p), count(p), grid(p), B.s);
    nl++;
  }
  for (int q = 0; q < 3 && !rc; q++) {
    const int p = kBPoissonA + q;
    if (!B.phase_used[p]) continue;
    rc = launch_poisson_batch(q, B.args[kTPa + q], items(p), count(p), grid(p), B.smem_p[q], B.s);
    nl++;
  }
  if (!rc && B.phase_used[kBDgradBig]) {
    rc = launch_density_batch(kBDgradBig, B.args[kTCell], items(kBDgradBig), count(kBDgradBig), grid(kBDgradBig),
                              0, B.s);
    nl++;
  }
  if (!rc && B.phase_used[kBCell]) {
    rc = launch_density_batch(kBCell, B.args[kTCell], items(kBCell), count(kBCell), grid(kBCell), 0, B.s);
    nl++;
  }
  if (rc) return rc;
  GPL_CUDA(cudaMemcpyAsync(B.res_h, B.res_d, sizeof(EvalResult) * B.cap, cudaMemcpyDeviceToHost, B.s));
  B.launches_per_round = nl;
  return GPL_OK;
}

// The round as one CUDA graph (a failure leaves direct launches).
void batch_capture(BatchRun& B) {
  if (B.exec) { cudaGraphExecDestroy(B.exec); B.exec = nullptr; }
  B.graph_dirty = false;
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(B.s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  const int rc = batch_launch_round(B);
  const cudaError_t e = cudaStreamEndCapture(B.s, &g);
  if (!rc && e == cudaSuccess && g) {
    if (cudaGraphInstantiate(&B.exec, g, 0) != cudaSuccess) B.exec = nullptr;
  }
  if (g) cudaGraphDestroy(g);
  cudaGetLastError();
}

}  // namespace

// One round over the running members: each one's next evaluation, then its
// control.  Members whose loop ended (stop rule, divergence, iteration limit
// of this run) stop running; the caller sees m.running == false.
int batch_round(BatchRun* Bp, long long* launches) {
  BatchRun& B = *Bp;
  int running = 0;
  for (const BatchMember& m : B.members) running += (m.job && m.running) ? 1 : 0;
  if (!running) return GPL_OK;
  if (B.items_dirty) {
    int rc = batch_items(B);
    if (rc) return rc;
  }
  if (B.graph_dirty) batch_capture(B);
  long long nl = 0;
  for (int k = 0; k < B.cap; k++) {
    BatchMember& m = B.members[k];
    if (!m.job || !m.running) continue;
    NesterovState& S = m.job->S;
    if (m.start) {
      start_iteration(S);
      if (S.iter % kTileOrderEvery == 0) {
        int rc = launch_tile_order(m.job->d, S.i_cur, B.s, m.job->timer);
        if (rc) return rc;
        S.refreshes++;
        nl += 3;
      }
      m.start = false;
    }
    B.ctl_h[k] = next_ctl(S);
  }
  if (B.exec) {
    GPL_CUDA(cudaGraphLaunch(B.exec, B.s));
  } else {
    int rc = batch_launch_round(B);
    if (rc) return rc;
  }
  nl += B.launches_per_round;
  GPL_CUDA(cudaStreamSynchronize(B.s));
  for (int k = 0; k < B.cap; k++) {
    BatchMember& m = B.members[k];
    if (!m.job || !m.running) continue;
    gpl_job* j = m.job;
    NesterovState& S = j->S;
    IterEntry e;
    bool logged = false;
    const int a = after_eval(S, B.res_h[k], &e, &logged);
    if (logged) record_iteration(j, e, S.iter, m.log);
    if (a == kRetry) continue;
    m.start = true;
    m.done++;
    if (S.finished || S.iter >= S.max_iter || (m.limit > 0 && m.done >= m.limit)) {
      m.running = false;
      B.items_dirty = true;
      if (S.finished && !S.diverge_code && j->m.p.verbose_level > 0) {
        printf("[NesterovSolve] Finished with Overflow: %g\n", S.sum_overflow);
        fflush(stdout);
      }
    }
  }
  if (launches) *launches += nl;
  return GPL_OK;
}

bool batch_running(const BatchRun* B, int slot) {
  return slot >= 0 && slot < B->cap && B->members[slot].job && B->members[slot].running;
}

int batch_count_running(const BatchRun* B) {
  int n = 0;
  for (const BatchMember& m : B->members) n += (m.job && m.running) ? 1 : 0;
  return n;
}

void batch_stop_member(BatchRun* B, int slot) {
  if (slot < 0 || slot >= B->cap || !B->members[slot].job) return;
  B->members[slot].running = false;
  B->items_dirty = true;
}

// A member's loop status after it stopped running (gpl_nesterov_run's).
int batch_member_status(gpl_job* j, gpl_nesterov_stats* o) {
  const int st = j->S.diverge_code == GPL_ERR_DIVERGED_INIT ? j->S.diverge_code : end_of_run(j);
  if (o) {
    o->iterations = j->S.iter;
    o->evaluations = j->S.evals;
    o->finished = j->S.finished ? 1 : 0;
    o->status = j->S.diverge_code;
    o->overflow = j->S.sum_overflow;
    o->step_length = j->S.step_length;
    o->density_penalty = j->S.density_penalty;
    o->wire_length_coef = j->S.wl_coef_x;
    o->hpwl = j->S.prev_hpwl;
  }
  return st;
}

}  // namespace gpl

namespace {

void fill_info(gpl_job* j, gpl_job_info* info) {
  if (!info) return;
  memset(info, 0, sizeof(*info));
  const HostModel& m = j->m;
  info->n_place_insts = (int)m.place_insts.size();
  info->n_gcells = m.n_g;
  info->n_fillers = m.n_fill;
  info->bin_cnt_x = m.cnt_x; info->bin_cnt_y = m.cnt_y;
  info->bin_size_x = m.size_x; info->bin_size_y = m.size_y;
  info->filler_dx = m.fill_dx; info->filler_dy = m.fill_dy;
  info->place_insts_area = m.place_area; info->std_insts_area = m.std_area;
  info->macro_insts_area = m.macro_area; info->non_place_insts_area = m.non_place_area;
  info->device_bytes = j->d.bytes;
  info->poisson_path = j->d.poisson_path;
  info->poisson_fft_us = j->poisson_fft_us;
  info->poisson_gemm_us = j->poisson_gemm_us;
  info->scatter_tile = j->d.tile_w;
  info->scatter_chunk = j->d.chunk;
  info->scatter_us = j->scatter_us;
}

}  // namespace

namespace gpl {

int job_new(const gpl_netlist_desc* nl, const gpl_params* p, gpl_job** out) {
  if (!out) { set_error("null job pointer"); return GPL_ERR_INVALID_ARG; }
  *out = nullptr;
  if (!p) { set_error("null parameters"); return GPL_ERR_INVALID_ARG; }
  gpl_job* j = new gpl_job();
  int rc = build_placer_base(j->m, nl, p);
  if (rc) { delete j; return rc; }
  if ((p->scatter_tile && p->scatter_tile != 16 && p->scatter_tile != 32 && p->scatter_tile != 64) ||
      (p->scatter_chunk && p->scatter_chunk != 1024 && p->scatter_chunk != 2048)) {
    delete j;
    set_error("scatter_tile must be 0, 16, 32 or 64 and scatter_chunk 0, 1024 or 2048");
    return GPL_ERR_INVALID_ARG;
  }
  if (p->max_back_track < 1 || p->nesterov_place_max_iter < 0) {
    delete j;
    set_error("max_back_track must be at least 1 and nesterov_place_max_iter not negative");
    return GPL_ERR_INVALID_ARG;
  }
  NesterovState& S = j->S;
  S.cur_a = 1.0f;
  S.min_sum_overflow = 1e30f;
  S.hpwl_with_min = 1e30f;
  S.max_phi_coef = p->max_phi_coef;
  S.i_prev = 0; S.i_cur = 1; S.i_next = 2; S.c_cur = 0; S.c_next = 1;
  S.last_slot = -1;
  j->device = p->device;
  rc = check_device(j->device);
  if (rc) { delete j; return rc; }
  *out = j;
  return GPL_OK;
}

void job_bind(gpl_job* j, cudaStream_t stream, HostPinned* pinned, cudaMemPool_t pool,
              cudaEvent_t sync_ev) {
  j->sync_ev = sync_ev;
  j->stream = stream;
  j->own_stream = false;
  j->pinned = pinned;
  j->own_pinned = false;
  memset(j->pinned, 0, sizeof(HostPinned));
  j->pool = pool;
  j->timer.stream = stream;
}

int job_device_bytes(gpl_job* j, int64_t* bytes, bool centred) {
  const HostModel& m = j->m;
  NbCounts c;
  // sizes as the job will see them: centring keeps 2 * (size / 2)
  PlaceRects rects = place_rects(m);
  if (centred)
    for (size_t k = 0; k < rects.lx.size(); k++) {
      rects.ux[k] = rects.lx[k] + 2 * ((rects.ux[k] - rects.lx[k]) / 2);
      rects.uy[k] = rects.ly[k] + 2 * ((rects.uy[k] - rects.ly[k]) / 2);
    }
  int rc = nb_counts(m, &c, &rects);
  if (rc) return rc;
  int sm = 0;
  GPL_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, j->device));
  size_t n_gpins = 0;
  for (int i : m.place_insts) n_gpins += m.inst_pin_start[i + 1] - m.inst_pin_start[i];
  const size_t ng = m.place_insts.size() + (size_t)c.n_fill;
  const size_t nb = (size_t)c.cnt_x * c.cnt_y;
  // upper bounds: every gcell big, the larger partial grid
  const size_t stride = std::max<size_t>((size_t)sm * 8, (size_t)c.cnt_y);
  const size_t arena = arena_bytes(ng, m.n_pins, m.n_nets, n_gpins, ng, nb, c.cnt_x, c.cnt_y, stride,
                                   (size_t)std::max(1, m.p.nesterov_place_max_iter));
  const size_t ip = m.p.initial_place_max_iter > 0 ? initial_place_bytes(m, sm) : 0;
  const size_t pg = (m.p.poisson_path != 1 && poisson_gemm_eligible(c.cnt_x, c.cnt_y))
                        ? (size_t)poisson_gemm_bytes(c.cnt_x, c.cnt_y) : 0;
  *bytes = (int64_t)std::max(arena + pg, ip);
  return GPL_OK;
}

}  // namespace gpl

// =================================================================== C ABI
extern "C" {

const char* gpl_version(void) { return "gpl_gb300 1.0 (sm_103a)"; }

const char* gpl_last_error(void) { return g_last_error.c_str(); }

void gpl_params_default(gpl_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->initial_place_max_iter = 20;
  p->initial_place_min_diff_length = 1500;
  p->initial_place_max_solver_iter = 100;
  p->initial_place_max_fanout = 200;
  p->initial_place_net_weight_scale = 800.0f;
  p->incremental_place_mode = 0;
  p->target_density = 1.0f;
  p->bin_grid_cnt_x = 0;
  p->bin_grid_cnt_y = 0;
  p->min_wire_length_force_bar = -300.0f;
  p->nesterov_place_max_iter = 2000;
  p->max_back_track = 10;
  p->init_density_penalty = 0.00008f;
  p->init_wire_length_coef = 0.25f;
  p->target_overflow = 0.1f;
  p->min_phi_coef = 0.95f;
  p->max_phi_coef = 1.05f;
  p->min_preconditioner = 1.0f;
  p->initial_prev_coordi_update_coef = 100.0f;
  p->reference_hpwl = 446000000.0f;
  p->verbose_level = 0;
  p->device = 0;
  p->stream = nullptr;
  p->use_graph = 1;
  p->ip_solver = 0;
  p->poisson_path = 0;
  p->scatter_tile = 0;
  p->scatter_chunk = 0;
  p->device_loop = 0;
}

gpl_status gpl_create(const gpl_netlist_desc* nl, const gpl_params* p, gpl_job** out) {
  gpl_job* j = nullptr;
  int rc = job_new(nl, p, &j);
  if (rc) return (gpl_status)rc;
  cudaError_t e = cudaMallocHost(&j->pinned, sizeof(HostPinned));
  if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); delete j; return GPL_ERR_CUDA; }
  j->own_pinned = true;
  memset(j->pinned, 0, sizeof(HostPinned));
  if (p->stream) {
    j->stream = (cudaStream_t)p->stream;
  } else {
    e = cudaStreamCreateWithFlags(&j->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      set_error(cudaGetErrorString(e));
      cudaFreeHost(j->pinned);
      delete j;
      return GPL_ERR_CUDA;
    }
    j->own_stream = true;
  }
  j->timer.stream = j->stream;
  *out = j;
  return GPL_OK;
}

void gpl_destroy(gpl_job* j) {
  if (!j) return;
  if (j->prep.joinable()) j->prep.join();
  cudaSetDevice(j->device);
  if (j->stream) cudaStreamSynchronize(j->stream);
  j->timer.release();
  if (j->graph_exec) cudaGraphExecDestroy(j->graph_exec);
  if (j->loop_exec) cudaGraphExecDestroy(j->loop_exec);
  if (j->d.pg) poisson_gemm_free(j->d.pg, j->pool, j->stream);
  if (j->arena) dev_free(j->arena, j->pool, j->stream);
  if (j->own_pinned && j->pinned) cudaFreeHost(j->pinned);
  if (j->side) {
    cudaStreamSynchronize(j->side);
    cudaStreamDestroy(j->side);
  }
  if (j->ev_fork) cudaEventDestroy(j->ev_fork);
  if (j->ev_join) cudaEventDestroy(j->ev_join);
  if (j->own_stream && j->stream) cudaStreamDestroy(j->stream);
  delete j;
}

gpl_status gpl_set_net_weights(gpl_job* j, const float* w, int64_t n_nets) {
  if (!j) { set_error("null job"); return GPL_ERR_INVALID_ARG; }
  if (w) {
    if (n_nets != j->m.n_nets) { set_error("net weights: n_nets differs from the netlist's"); return GPL_ERR_INVALID_ARG; }
    for (int64_t n = 0; n < n_nets; n++)
      if (!(w[n] >= 0.0f) || !std::isfinite(w[n])) {
        set_error("net weights must be finite and >= 0 (net " + std::to_string(n) + ")");
        return GPL_ERR_INVALID_ARG;
      }
    j->net_w.assign(w, w + n_nets);
  } else {
    j->net_w.clear();
  }
  if (!j->nb_ready) return GPL_OK;       // uploaded with the device model
  cudaSetDevice(j->device);
  return (gpl_status)apply_net_weights(j);
}

gpl_status gpl_nesterov_init(gpl_job* j, gpl_job_info* info) {
  if (!j) { set_error("null job"); return GPL_ERR_INVALID_ARG; }
  if (j->np_ready) { set_error("Nesterov already initialised"); return GPL_ERR_BAD_STATE; }
  cudaSetDevice(j->device);
  int rc = nesterov_init(j);
  fill_info(j, info);
  return (gpl_status)rc;
}

gpl_status gpl_nesterov_run(gpl_job* j, int32_t max_iters, gpl_nesterov_stats* st, gpl_iter_log* log) {
  if (!j) { set_error("null job"); return GPL_ERR_INVALID_ARG; }
  if (!j->np_ready) { set_error("call gpl_nesterov_init first"); return GPL_ERR_BAD_STATE; }
  cudaSetDevice(j->device);
  int rc = nesterov_run(j, max_iters, log);
  if (st) {
    st->iterations = j->S.iter;
    st->evaluations = j->S.evals;
    st->finished = j->S.finished ? 1 : 0;
    st->status = j->S.diverge_code;
    st->overflow = j->S.sum_overflow;
    st->step_length = j->S.step_length;
    st->density_penalty = j->S.density_penalty;
    st->wire_length_coef = j->S.wl_coef_x;
    st->hpwl = j->S.prev_hpwl;
  }
  return (gpl_status)rc;
}

gpl_status gpl_batch_nesterov_run(gpl_job* const* jobs, int32_t n_jobs, int32_t max_iters,
                                  gpl_nesterov_stats* stats, gpl_status* status, int64_t* kernel_launches) {
  if (!jobs || n_jobs <= 0) { set_error("gpl_batch_nesterov_run: no jobs"); return GPL_ERR_INVALID_ARG; }
  for (int k = 0; k < n_jobs; k++) {
    if (!jobs[k]) { set_error("gpl_batch_nesterov_run: null job"); return GPL_ERR_INVALID_ARG; }
    if (!jobs[k]->np_ready) { set_error("gpl_batch_nesterov_run: call gpl_nesterov_init first"); return GPL_ERR_BAD_STATE; }
    if (jobs[k]->device != jobs[0]->device) {
      set_error("gpl_batch_nesterov_run: the jobs must be on one device");
      return GPL_ERR_INVALID_ARG;
    }
    for (int q = 0; q < k; q++)
      if (jobs[q] == jobs[k]) { set_error("gpl_batch_nesterov_run: a job is listed twice"); return GPL_ERR_INVALID_ARG; }
  }
  for (int k = 0; k < n_jobs; k++)
    if (!batch_eligible(jobs[k])) {
      set_error("gpl_batch_nesterov_run: job " + std::to_string(k) +
                " does not run the block-form FFT Poisson passes (its grid is 512 x 512 or 1024 x 1024, or it "
                "runs the tensor-core form); run it alone");
      return GPL_ERR_INVALID_ARG;
    }
  int rc = GPL_OK;
  std::unique_ptr<BatchRun, void (*)(BatchRun*)> B(batch_create(jobs[0]->device, n_jobs, &rc), batch_destroy);
  if (!B) return (gpl_status)rc;
  for (int k = 0; k < n_jobs && !rc; k++) rc = batch_join(B.get(), k, jobs[k], max_iters, nullptr);
  long long nl = 0;
  for (;;) {
    if (rc) break;
    bool any = false;
    for (const BatchMember& m : B->members) any |= m.job && m.running;
    if (!any) break;
    rc = batch_round(B.get(), &nl);
  }
  if (kernel_launches) *kernel_launches = nl;
  if (rc) return (gpl_status)rc;
  for (int k = 0; k < n_jobs; k++) {
    const int st = batch_member_status(jobs[k], stats ? &stats[k] : nullptr);
    if (status) status[k] = (gpl_status)st;
  }
  return GPL_OK;
}

gpl_status gpl_get_inst_locations(gpl_job* j, int32_t* lx, int32_t* ly) {
  if (!j || !lx || !ly) { set_error("null argument"); return GPL_ERR_INVALID_ARG; }
  const HostModel& m = j->m;
  for (int i = 0; i < m.n_insts; i++) { lx[i] = m.ilx[i]; ly[i] = m.ily[i]; }
  if (j->np_ready && j->S.last_slot >= 0) {
    // NesterovPlace::updateDb: lx = dCx - dDx/2 at the last evaluated centres
    std::vector<float2> c(m.n_g);
    GPL_CUDA(cudaMemcpyAsync(c.data(), j->d.slp[j->S.last_slot], m.n_g * sizeof(float2), cudaMemcpyDeviceToHost, j->stream));
    GPL_CUDA(cudaStreamSynchronize(j->stream));
    for (int k = 0; k < m.n_place; k++) {
      const int i = m.place_insts[k];
      const int hx = (m.gdux[k] - m.gdlx[k]) / 2, hy = (m.gduy[k] - m.gdly[k]) / 2;
      lx[i] = (int)c[k].x - (2 * hx) / 2;
      ly[i] = (int)c[k].y - (2 * hy) / 2;
    }
  }
  return GPL_OK;
}

gpl_status gpl_get_gcell_coords(gpl_job* j, float* xy) {
  if (!j || !xy) { set_error("null argument"); return GPL_ERR_INVALID_ARG; }
  if (!j->np_ready) { set_error("Nesterov not initialised"); return GPL_ERR_BAD_STATE; }
  GPL_CUDA(cudaMemcpyAsync(xy, j->d.slp[j->S.i_cur], (size_t)j->m.n_g * sizeof(float2), cudaMemcpyDeviceToHost, j->stream));
  GPL_CUDA(cudaStreamSynchronize(j->stream));
  return GPL_OK;
}

gpl_status gpl_eval(gpl_job* j, const float* xy, float cx, float cy, float* wl_grad,
                    float* density_grad, gpl_eval_stats* st) {
  if (!j || !xy) { set_error("null argument"); return GPL_ERR_INVALID_ARG; }
  cudaSetDevice(j->device);
  int rc = ensure_nb(j);
  if (rc) return (gpl_status)rc;
  DeviceModel& d = j->d;
  const size_t ng = j->m.n_g;
  rc = choose_poisson_path(j);
  if (rc) return (gpl_status)rc;
  // slot 3 of the coordinate / gradient-sum buffers belongs to this hook
  rc = upload(d.slp[3], xy, ng * sizeof(float2), j->stream);
  if (rc) return (gpl_status)rc;
  EvalCtl c;
  memset(&c, 0, sizeof(c));
  c.wl_coef_x = cx; c.wl_coef_y = cy;
  c.i_src = 3; c.i_eval = 3; c.i_ref = -1;
  c.c_cur = 0; c.c_next = 1;
  c.write_sum = 1; c.write_wd = 1;
  rc = launch_tile_order(d, 3, j->stream, j->timer);
  if (rc) return (gpl_status)rc;
  rc = evaluate(j, c, true);
  if (rc) return (gpl_status)rc;
  if (wl_grad) GPL_CUDA(cudaMemcpyAsync(wl_grad, d.wl_out, ng * sizeof(float2), cudaMemcpyDeviceToHost, j->stream));
  if (density_grad) GPL_CUDA(cudaMemcpyAsync(density_grad, d.d_out, ng * sizeof(float2), cudaMemcpyDeviceToHost, j->stream));
  GPL_CUDA(cudaStreamSynchronize(j->stream));
  if (st) {
    st->overflow_area_f64 = j->S.last.overflow;
    st->overflow_area = (int64_t)j->S.last.overflow;
    st->hpwl = j->S.last.hpwl;
    st->sum_phi = j->S.last.sum_phi;
    st->wire_length_grad_sum = j->S.last.wl_sum;
    st->density_grad_sum = j->S.last.d_sum;
  }
  return GPL_OK;
}

gpl_status gpl_get_bins(gpl_job* j, int64_t* inst, int64_t* fill, int64_t* np, float* dens,
                        float* phi, float* fx, float* fy) {
  if (!j) { set_error("null job"); return GPL_ERR_INVALID_ARG; }
  if (!j->nb_ready) { set_error("no evaluation yet"); return GPL_ERR_BAD_STATE; }
  DeviceModel& d = j->d;
  const size_t nb = (size_t)d.cnt_x * d.cnt_y;
  cudaStream_t s = j->stream;
  if (inst) GPL_CUDA(cudaMemcpyAsync(inst, d.area[j->S.last_area], nb * 8, cudaMemcpyDeviceToHost, s));
  if (fill) GPL_CUDA(cudaMemcpyAsync(fill, d.area[j->S.last_area] + nb, nb * 8, cudaMemcpyDeviceToHost, s));
  if (np) GPL_CUDA(cudaMemcpyAsync(np, d.nonplace, nb * 8, cudaMemcpyDeviceToHost, s));
  if (dens) GPL_CUDA(cudaMemcpyAsync(dens, d.density, nb * 4, cudaMemcpyDeviceToHost, s));
  if (phi) GPL_CUDA(cudaMemcpyAsync(phi, d.phi, nb * 4, cudaMemcpyDeviceToHost, s));
  if (fx || fy) {
    std::vector<float2> f(nb);
    GPL_CUDA(cudaMemcpyAsync(f.data(), d.field, nb * 8, cudaMemcpyDeviceToHost, s));
    GPL_CUDA(cudaStreamSynchronize(s));
    for (size_t b = 0; b < nb; b++) {
      if (fx) fx[b] = f[b].x;
      if (fy) fy[b] = f[b].y;
    }
  }
  GPL_CUDA(cudaStreamSynchronize(s));
  return GPL_OK;
}

gpl_status gpl_get_gcells(gpl_job* j, int32_t* drect, float* scale, uint8_t* kind) {
  if (!j) { set_error("null job"); return GPL_ERR_INVALID_ARG; }
  cudaSetDevice(j->device);
  int rc = ensure_nb(j);
  if (rc) return (gpl_status)rc;
  const HostModel& m = j->m;
  for (int g = 0; g < m.n_g; g++) {
    if (drect) {
      drect[4 * g] = m.gdlx[g]; drect[4 * g + 1] = m.gdly[g];
      drect[4 * g + 2] = m.gdux[g]; drect[4 * g + 3] = m.gduy[g];
    }
    if (scale) scale[g] = m.gscale[g];
    if (kind) kind[g] = m.gkind[g];
  }
  return GPL_OK;
}

int32_t gpl_kernel_times(gpl_job* j, const char** names, double* ms, int64_t* launches, int32_t cap) {
  if (!j) return 0;
  j->timer.resolve();
  int n = 0;
  for (int k = 0; k < kKClasses && n < cap; k++) {
    if (names) names[n] = kernel_class_name(k);
    if (ms) ms[n] = j->timer.ms[k];
    if (launches) launches[n] = j->timer.groups[k];
    n++;
  }
  return n;
}

void gpl_kernel_times_reset(gpl_job* j, int32_t enable) {
  if (!j) return;
  j->timer.resolve();
  for (int k = 0; k < kKClasses; k++) { j->timer.ms[k] = 0; j->timer.groups[k] = 0; }
  j->timer.kernels = 0;
  j->timer.enabled = enable != 0;
}

int64_t gpl_kernel_launch_count(gpl_job* j) { return j ? j->timer.kernels : 0; }

gpl_status gpl_initial_place(gpl_job* j, gpl_ip_stats* st) {
  if (!j) { set_error("null job"); return GPL_ERR_INVALID_ARG; }
  if (j->nb_ready) { set_error("initial place must run before the Nesterov stage"); return GPL_ERR_BAD_STATE; }
  // InitialPlace::doBicgstabPlace (src/initialPlace.cpp:56-105): centre the
  // movable instances unless incremental, then the B2B + BiCGSTAB rounds
  const double t0 = wall_ms();
  if (!j->m.p.incremental_place_mode) host_place_center(j->m);
  if (st) memset(st, 0, sizeof(*st));
  if (j->m.p.initial_place_max_iter <= 0) return GPL_OK;
  cudaSetDevice(j->device);
  // the Nesterov setup's host part runs on a worker thread meanwhile
  start_static_prep(j);
  if (j->m.p.verbose_level >= 2) printf("[InitialPlace] centring and worker start %.2f ms\n", wall_ms() - t0);
  int sm = 0;
  GPL_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, j->device));
  return (gpl_status)run_initial_place(j->m, j->stream, sm, st, j->timer, j->pinned->ip_state, j->pool,
                                       j->sync_ev);
}

gpl_status gpl_batch_initial_place(gpl_job* const* jobs, int32_t n_jobs, gpl_ip_stats* stats, gpl_status* status,
                                   int64_t* kernel_launches) {
  if (kernel_launches) *kernel_launches = 0;
  if (!jobs || n_jobs <= 0) { set_error("gpl_batch_initial_place: no jobs"); return GPL_ERR_INVALID_ARG; }
  for (int k = 0; k < n_jobs; k++) {
    if (!jobs[k]) { set_error("gpl_batch_initial_place: null job"); return GPL_ERR_INVALID_ARG; }
    if (jobs[k]->nb_ready) {
      set_error("gpl_batch_initial_place: initial place must run before the Nesterov stage");
      return GPL_ERR_BAD_STATE;
    }
    if (jobs[k]->device != jobs[0]->device) {
      set_error("gpl_batch_initial_place: the jobs must be on one device");
      return GPL_ERR_INVALID_ARG;
    }
    for (int q = 0; q < k; q++)
      if (jobs[q] == jobs[k]) { set_error("gpl_batch_initial_place: a job is listed twice"); return GPL_ERR_INVALID_ARG; }
  }
  cudaSetDevice(jobs[0]->device);
  int sm = 0;
  GPL_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, jobs[0]->device));
  // each job as gpl_initial_place prepares it: centred (unless incremental),
  // its Nesterov setup's host part started on its worker thread
  std::vector<IpBatchJob> b(n_jobs);
  for (int k = 0; k < n_jobs; k++) {
    gpl_job* j = jobs[k];
    if (!j->m.p.incremental_place_mode) host_place_center(j->m);
    if (stats) memset(&stats[k], 0, sizeof(stats[k]));
    if (j->m.p.initial_place_max_iter > 0) start_static_prep(j);
    b[k].m = &j->m;
    b[k].s = j->stream;
    b[k].pinned = j->pinned->ip_state;
    b[k].pool = j->pool;
    b[k].sync_ev = j->sync_ev;
    b[k].stats = stats ? &stats[k] : nullptr;
  }
  const int rc = run_initial_place_batch(b.data(), n_jobs, sm, kernel_launches);
  for (int k = 0; k < n_jobs; k++)
    if (status) status[k] = (gpl_status)b[k].status;
  return (gpl_status)rc;
}

}  // extern "C"
