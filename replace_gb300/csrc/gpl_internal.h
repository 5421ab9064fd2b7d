// Internal declarations of libgpl_gb300: host model, device layout, kernels.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gpl.h"

namespace gpl {

// ------------------------------------------------------------------ errors
void set_error(const std::string& msg);

#define GPL_CUDA(call)                                                        \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      ::gpl::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));    \
      return e_ == cudaErrorMemoryAllocation ? GPL_ERR_OUT_OF_MEMORY          \
                                             : GPL_ERR_CUDA;                  \
    }                                                                         \
  } while (0)

// ------------------------------------------------------------- host model
// Everything NesterovBase / BinGrid / PlacerBase compute once per job on the
// host (src/placerBase.cpp:606-758, src/nesterovBase.cpp:631-741, 917-1155).
struct HostModel {
  gpl_params p;
  int core_lx, core_ly, core_ux, core_uy, site_w, site_h;
  int n_insts = 0, n_pins = 0, n_nets = 0;
  std::vector<int32_t> ilx, ily, iux, iuy;
  std::vector<uint8_t> ikind;
  // pin_x / pin_y: positions of pins off movable instances (IO pins, pins of
  // fixed instances); a movable instance's pin is its centre plus (pin_ox, pin_oy)
  std::vector<int32_t> pin_inst, pin_ox, pin_oy, pin_x, pin_y, net_start;
  std::vector<int32_t> inst_pin_start, inst_pins;
  std::vector<int32_t> place_insts, non_place_insts;
  int64_t place_area = 0, std_area = 0, macro_area = 0, non_place_area = 0;
  // NesterovBase
  int n_g = 0, n_place = 0, n_fill = 0, fill_dx = 0, fill_dy = 0;
  std::vector<int32_t> glx, gly, gux, guy;       // real rectangle
  std::vector<int32_t> gdlx, gdly, gdux, gduy;   // density rectangle
  std::vector<float> gscale;
  std::vector<uint8_t> gkind;                    // 0 std, 1 macro, 2 filler
  std::vector<int32_t> g_pin_start, g_pins;
  std::vector<int32_t> pin_g;                    // gcell of each pin or -1
  // BinGrid
  int cnt_x = 0, cnt_y = 0, size_x = 0, size_y = 0;
  std::vector<int64_t> bin_nonplace;
};

int build_placer_base(HostModel& m, const gpl_netlist_desc* d, const gpl_params* p);
// counts of the NesterovBase and BinGrid that size a job's device memory
struct NbCounts {
  int fill_dx = 0, fill_dy = 0, n_fill = 0;
  int cnt_x = 0, cnt_y = 0, size_x = 0, size_y = 0;
};
// the movable instances' rectangles (in place_insts order)
struct PlaceRects {
  std::vector<int32_t> lx, ly, ux, uy;
};
PlaceRects place_rects(const HostModel& m);
// rects: the movable instances' rectangles to use (default: the model's)
int nb_counts(const HostModel& m, NbCounts* c, const PlaceRects* rects = nullptr);
// NesterovBase in two parts: the position-independent part (may run beside
// an initial place, from a copy of the movable rectangles), then the movable
// gcells at the instances' current positions
int build_nesterov_static(HostModel& m, const PlaceRects& rects);
void place_gcells(HostModel& m);
int build_nesterov_base(HostModel& m);
// InitialPlace::placeInstsCenter + Instance::setCenterLocation
void host_place_center(HostModel& m);

// A heap array left uninitialised, so that its pages are first touched by
// the (parallel) pass that fills it.
template <class T>
struct RawArray {
  std::unique_ptr<T[]> p;
  size_t n;
  explicit RawArray(size_t count) : p(new T[count > 0 ? count : 1]), n(count) {}
  T* data() { return p.get(); }
  size_t size() const { return n; }
  T& operator[](size_t i) { return p[i]; }
  const T& operator[](size_t i) const { return p[i]; }
};

// Runs body(a, b) over [0, n) split into disjoint ranges on a few host
// threads (one range below 65,536 items): the per-pin host passes of a job
// setup touch tens of MB of fresh pages at a million cells.
template <class F>
void parallel_ranges(int n, F&& body) {
  const int n_thr = (int)std::max(1u, std::min(8u, std::thread::hardware_concurrency() / 2));
  if (n_thr <= 1 || n < (1 << 16)) { body(0, n); return; }
  std::vector<std::thread> th;
  for (int t = 0; t < n_thr; t++) {
    const int a = (int)((long long)n * t / n_thr), b = (int)((long long)n * (t + 1) / n_thr);
    th.emplace_back([&body, a, b]() { body(a, b); });
  }
  for (auto& x : th) x.join();
}
void host_set_inst_center(HostModel& m, int inst, int x, int y);

// WA net buckets by degree: 2, 4, 8, 16, 32 (lane groups), 64, 128 (a warp,
// two or four pins per lane), more (a warp, looping).
constexpr int kWaBuckets = 8;

// -------------------------------------------------------------- device model
struct DeviceModel {
  // static gcell data
  int n_g = 0, n_place = 0;
  int2* g_half = nullptr;          // half density size (dDx/2, dDy/2)
  float* g_scale = nullptr;
  uint8_t* g_kind = nullptr;
  float2* g_precond = nullptr;     // (#pins, real dx*dy)
  int32_t* g_pin_start = nullptr;  // CSR of each gcell's pin slots
  int32_t* g_pins = nullptr;       // device pin index of each slot
  int32_t* big_cells = nullptr;    // gcells covering many bins (macros)
  int n_big = 0;
  // pins and nets
  int n_pins = 0, n_nets = 0;
  // Pins are renumbered on the device: nets in WA-bucket order (degree <= 2,
  // 4, 8, 16, 32, 64, 128, more), each net's pins contiguous.
  int4* pins = nullptr;            // (gcell or -1, x offset or position, y ..., 0)
  int32_t* net_start = nullptr;    // pin CSR of the bucket-ordered nets
  int wa_bucket_start[kWaBuckets + 1] = {0};    // first net of each bucket
  int wa_block_start[kWaBuckets + 1] = {0};     // first block of each bucket in the WA launch
  float2* pin_grad = nullptr;      // WA gradient per device pin
  float* net_w = nullptr;          // per-net weight, bucket order
  bool net_weighted = false;       // launch the weighted WA variant
  // bin grid
  int cnt_x = 0, cnt_y = 0, size_x = 0, size_y = 0;
  int core_lx, core_ly, core_ux, core_uy;
  float target_density = 1.0f;
  unsigned long long* area[2] = {nullptr, nullptr};  // [inst | filler] x nb, double-buffered
  int area_cur = 0;
  int64_t* nonplace = nullptr;
  float* density = nullptr;
  float* spec = nullptr;           // pass A output (DCT-II along x)
  float* p1 = nullptr;             // pass B outputs
  float* p2 = nullptr;
  float2* field = nullptr;         // (Ex, Ey)
  float* phi = nullptr;
  float* wx = nullptr;             // [cnt_x]
  float* wy = nullptr;             // [cnt_y]
  float2* w4x = nullptr;           // [cnt_x]
  float2* w4y = nullptr;           // [cnt_y]
  float2* twiddle = nullptr;       // exp(-2 pi i k / kFftMax), k < kFftMax/2
  int32_t* g_big_idx = nullptr;    // index into big_cells or -1
  float2* d_big = nullptr;         // density gradient of big cells
  // Nesterov vectors (float2 per gcell): slots 0-2 rotate as prev/cur/next,
  // slot 3 holds the coordinates of the gradient-check hook (gpl_eval)
  float2* slp[4] = {nullptr, nullptr, nullptr, nullptr};   // SLP coordinates
  float2* sum[4] = {nullptr, nullptr, nullptr, nullptr};   // preconditioned sum gradients
  float2* coordi[2] = {nullptr, nullptr};                  // cur / next coordinates
  struct EvalCtl* ctl = nullptr;    // device copy of the evaluation's control record
  struct EvalCtl* ctl_h = nullptr;  // pinned host staging
  float2* wl_out = nullptr;        // optional per-gcell WL gradient (eval hook)
  float2* d_out = nullptr;         // optional per-gcell density gradient (eval hook)
  // reduction partials
  double* part = nullptr;          // [kPartSlots * part_stride]
  int part_stride = 0;
  long long* hpwl_total = nullptr; // HPWL accumulators (WA warps add, the gcell kernel sums and clears)
  double* part_total = nullptr;    // [kPartSlots] final sums
  unsigned* counters = nullptr;    // [2] last-block counters (gcell kernel, WA kernel)
  int sm_count = 0;
  // gcells ordered by bin tile for the scatter (refreshed every few
  // evaluations; any order gives the same int64 areas)
  int tile_w = 32, tile_h = 32, tiles_x = 1, tiles_y = 1, max_chunks = 1;
  int chunk = 2048;                // gcells per scatter chunk (at most)
  int tile_cap = 1, chunk_cap = 1; // capacity of the tile and chunk tables
  int32_t* order = nullptr;        // [n_g] gcell indices, tile by tile
  int32_t* tile_count = nullptr;   // [tiles] counts, then fill cursors
  int32_t* tile_start = nullptr;   // [tiles + 1]
  int4* chunks = nullptr;          // [max_chunks] (tile, first, end, 0) of <= kScatterChunk gcells
  int32_t* n_chunks = nullptr;     // [1]
  // Poisson solve: 1 = shared-memory FFT passes, 2 = tensor-core GEMMs
  int poisson_path = 1;
  struct PoissonGemm* pg = nullptr;
  struct EvalResult* result = nullptr;     // device
  struct EvalResult* result_h = nullptr;   // pinned host mirror
  int64_t bytes = 0;
};

constexpr int kFftMax = 4096;

// HPWL accumulators: kHpwlLanes int64 counters kHpwlStride apart (one
// 32-byte sector each), so the WA warps' atomics spread over them.
constexpr int kHpwlLanes = 32;
constexpr int kHpwlStride = 4;

enum PartSlot {
  kPartOverflow = 0, kPartWl, kPartD, kPartCoordDist, kPartGradDist, kPartNan,
  kPartPhi, kPartSlots
};

// Everything that changes from one evaluation to the next.  Kernels read it
// from device memory, so a single captured graph serves every evaluation.
struct EvalCtl {
  float step, coeff;            // predictor: x' = clamp(cur + step*sum), y' = clamp(x' + coeff*(x' - coordi))
  float density_penalty;
  float wl_coef_x, wl_coef_y;   // 1/gamma
  int predict;                  // 1: slp[i_eval] is predicted from slot i_src and coordi[c_cur]
  int i_src, i_eval, i_ref;     // slots of slp/sum; i_ref < 0: no step-length reference
  int c_cur, c_next;
  int area_cur;                 // area set scattered into; the other one is cleared
  int write_sum;                // write sum[i_eval]
  int write_wd;                 // write the per-gcell WL and density gradients (hook)
  int pad[2];
};

struct EvalResult {
  double overflow;        // FP64 sum of per-bin overflow
  double wl_sum, d_sum;   // sum |grad|
  double coord_dist, grad_dist;   // sum of squared differences
  double sum_phi;
  double nan_flag;
  long long hpwl;
  float new_step_length;
  int pad;
};

// Everything the Nesterov loop carries from one evaluation to the next.  The
// job keeps a host copy; the device loop works on a device copy and the two
// are exchanged around each device chunk.
struct NesterovState {
  // parameters
  int max_back_track, max_iter;
  float target_overflow, min_phi_coef, reference_hpwl;
  float ovf_den;            // std area + macro area * target density (float, as the reference)
  float base_wl_coef;
  // NesterovPlace state (src/nesterovPlace.h:76-125)
  float cur_a, coeff, step_length, density_penalty, wl_coef_x, wl_coef_y;
  float sum_overflow, min_sum_overflow, hpwl_with_min, max_phi_coef;
  int max_phi_changed, is_diverged, finished, diverge_code;
  long long prev_hpwl;
  int iter, evals, attempts;
  // buffer slots (rotated by index), area set alternation
  int i_prev, i_cur, i_next, c_cur, c_next;
  int area_next, last_area, last_slot;
  // device loop: iterations this chunk may run (0 = to the stop rule), done,
  // evaluations, log entries, tile-order refreshes
  int chunk_limit, chunk_done, chunk_evals, log_count, refreshes, pad;
  EvalResult last;          // the last evaluation's result
};

// One logged iteration.
struct IterEntry {
  long long hpwl;
  float overflow, step_length;
  int backtracks, pad;
};

// Pinned host staging of one job: the evaluation's control record and result
// and the initial place's solver scalars.  A job allocates its own, or a
// server hands each of its slots one for the life of the server (freeing
// pinned memory may synchronise the device).
struct HostPinned {
  EvalResult result;
  EvalCtl ctl;
  NesterovState state;
  alignas(16) unsigned char ip_state[1024];
};

// Device memory of a job: from a stream-ordered pool when one is given (a
// server's; allocation and release never synchronise the device), else
// cudaMalloc / cudaFree.
inline cudaError_t dev_alloc(void** p, size_t bytes, cudaMemPool_t pool, cudaStream_t s) {
  return pool ? cudaMallocFromPoolAsync(p, bytes, pool, s) : cudaMalloc(p, bytes);
}
inline void dev_free(void* p, cudaMemPool_t pool, cudaStream_t s) {
  if (!p) return;
  if (pool) cudaFreeAsync(p, s); else cudaFree(p);
}

// Waits for the stream's work so far: with a blocking-sync event when one is
// given (the host thread sleeps instead of spinning: a server runs more slot
// threads than it has cores), else cudaStreamSynchronize.
inline cudaError_t host_wait(cudaStream_t s, cudaEvent_t ev) {
  if (!ev) return cudaStreamSynchronize(s);
  cudaError_t e = cudaEventRecord(ev, s);
  return e != cudaSuccess ? e : cudaEventSynchronize(ev);
}

// kernel-class timing (CUDA events around each launch when enabled)
enum KernelClass { kKScatter = 0, kKPoissonA, kKPoissonB, kKPoissonC, kKWa, kKCell,
                   kKReduce, kKOther, kKClasses };
const char* kernel_class_name(int k);

// Optional CUDA-event timing of kernel classes on the job's stream.  Event
// pairs are recorded around each launch group and resolved later, so timing
// adds no host synchronisation to the launch sequence.
struct TimedPair { int k; cudaEvent_t a, b; };
struct Timer {
  bool enabled = false;
  cudaStream_t stream = nullptr;
  std::vector<TimedPair> live;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t pending = nullptr;
  long long kernels = 0;            // kernels launched (always counted)
  double ms[kKClasses] = {0};
  long long groups[kKClasses] = {0};
  void begin(int k);
  void end(int k);
  void count(int n) { kernels += n; }
  int resolve();                    // synchronises the stream, accumulates ms
  void release();
};

// ------------------------------------------------------------------ kernels
// Per-job constants of the evaluation kernels (the per-evaluation values
// are in EvalCtl).
struct EvalArgs {
  float min_precond = 1.0f;
  float min_wl_force_bar = -300.0f;
};

// Bin-grid geometry and transform tables used by the Poisson passes.
struct PoissonGrid {
  int nx, ny, size_x, size_y;
  int core_lx, core_ly, core_ux, core_uy;
  const float* wx;        // [nx]
  const float* wy;        // [ny]
  const float2* w4x;      // exp(-i pi k / 2nx), [nx]
  const float2* w4y;      // exp(-i pi k / 2ny), [ny]
  const float2* tw;       // exp(-2 pi i m / kFftMax), [kFftMax/2]
};

int poisson_passes(const PoissonGrid& g, unsigned long long* const* area_pair,
                   const EvalCtl* ctl, const int64_t* nonplace, float td,
                   const float* density_in, float* density, double* part_overflow,
                   float* spec, float* p1, float* p2, float2* field, float* fx, float* fy,
                   float* phi, cudaStream_t s, Timer* t);
int poisson_blocks_a(int nx, int ny);
void make_w4(int n, std::vector<float2>& w);

int launch_scatter(DeviceModel& d, const EvalArgs& a, cudaStream_t s, Timer& t);
// Orders the gcells by the bin tile of their centres in slp[slot] (counting
// sort) and builds the scatter's chunk table; slot < 0: the slot the device
// control record's predictor starts from (ctl->i_src).
int launch_tile_order(DeviceModel& d, int slot, cudaStream_t s, Timer& t);

// Device loop of the Nesterov iteration (control.cu, control.h).
int launch_loop_head(NesterovState* S, EvalCtl* ctl, cudaGraphConditionalHandle h_loop,
                     cudaGraphConditionalHandle h_order, cudaStream_t s);
int launch_loop_step(NesterovState* S, EvalCtl* ctl, const EvalResult* res, IterEntry* log, int log_cap,
                     cudaGraphConditionalHandle h_loop, cudaGraphConditionalHandle h_order, cudaStream_t s);
// Tile grid of a bin grid, and the chunk-table bound, for sizing.
// Scatter shapes: tile side in bins and gcells per chunk.  The autotuner
// (nesterov_init) times these on the job's first coordinates and keeps the
// fastest; any shape gives the same int64 areas.
constexpr int kScatterChunk = 2048;               // the default chunk
constexpr int kTileSides[] = {16, 32, 64};
constexpr int kScatterChunks[] = {1024, 2048};
constexpr int kTileSideMin = 16, kScatterChunkMin = 1024;
static_assert(kScatterChunk < 65536 && kScatterChunks[1] < 65536,
              "the scatter's 16-bit split window sums need < 2^16 gcells per chunk");
void tile_grid(int cnt_x, int cnt_y, int side, int* tw, int* th, int* tx, int* ty);
int scatter_max_chunks(int n_g, int tiles, int chunk);
// Sets the scatter shape (within the tables' capacity); false if it does not fit.
bool set_scatter_shape(DeviceModel& d, int side, int chunk);
// dynamic shared memory of the scatter kernel for the current shape, and the
// kernel's limit raised to the largest shape (outside any stream capture)
size_t scatter_smem(const DeviceModel& d);
int scatter_prepare_device();
int launch_wa(DeviceModel& d, const EvalArgs& a, cudaStream_t s, Timer& t);
int launch_cell(DeviceModel& d, const EvalArgs& a, int n_phi_blocks, cudaStream_t s, Timer& t);
// the Poisson passes of a job evaluation (area set chosen by EvalCtl)
int launch_poisson_job(DeviceModel& d, bool want_phi, cudaStream_t s, Timer& t);
// The tensor-core GEMM form of the Poisson solve (poisson_gemm.cu).
struct PoissonGemm;
bool poisson_gemm_eligible(int nx, int ny);
int64_t poisson_gemm_bytes(int nx, int ny);
int poisson_gemm_setup(DeviceModel& d, PoissonGemm** out, cudaMemPool_t pool, cudaStream_t s);
void poisson_gemm_free(PoissonGemm* pg, cudaMemPool_t pool, cudaStream_t s);
int poisson_gemm_error(const PoissonGemm* pg, cudaStream_t s, int* flag);
int launch_poisson_gemm(DeviceModel& d, PoissonGemm* pg, bool want_phi, cudaStream_t s, Timer& t);
// Sets the Poisson kernels' shared-memory limit on the current device (once
// per device); called before a stream capture, where it must not run first.
int poisson_prepare_device();
int cell_grid(const DeviceModel& d);
int launch_sum_phi(DeviceModel& d, int area_set, cudaStream_t s, Timer& t, int* n_blocks);
int cell_blocks(const DeviceModel& d);
int bin_blocks(const DeviceModel& d);
int net_blocks(const DeviceModel& d);
int wa_nets_per_block(int bucket);

// InitialPlace::doBicgstabPlace rounds on the device (initial_place.cu); on
// return the host model's movable instances are at the solution.
// `pinned` is the job's ip_state block; `pool` as for dev_alloc.
int run_initial_place(HostModel& m, cudaStream_t s, int sm_count, gpl_ip_stats* stats, Timer& t,
                      void* pinned, cudaMemPool_t pool, cudaEvent_t sync_ev);
// device bytes run_initial_place allocates for this model
size_t initial_place_bytes(const HostModel& m, int sm_count);
// One job of the batched initial place: its host model, and the stream,
// pinned block, pool and event its setup and read-back use (as
// run_initial_place's); stats may be null; status is the job's result.
struct IpBatchJob {
  HostModel* m = nullptr;
  cudaStream_t s = nullptr;
  void* pinned = nullptr;
  cudaMemPool_t pool = nullptr;
  cudaEvent_t sync_ev = nullptr;
  gpl_ip_stats* stats = nullptr;
  int status = 0;
};
// The initial place of n jobs in lockstep rounds, one launch per phase over
// all jobs (initial_place.cu); each job's result is bit-identical to
// run_initial_place's kernel-per-phase form.  *launches: kernels launched.
// Returns GPL_OK, or the error that stopped the batch as a whole (each
// job's status is in jobs[k].status either way).
int run_initial_place_batch(IpBatchJob* jobs, int n, int sm_count, int64_t* launches);

// A job's host model without a stream or staging (a server binds those when
// it admits the job), and the binding: stream, pinned staging and pool stay
// the caller's.
int job_new(const gpl_netlist_desc* nl, const gpl_params* p, gpl_job** out);
void job_bind(gpl_job* j, cudaStream_t stream, HostPinned* pinned, cudaMemPool_t pool,
              cudaEvent_t sync_ev);
// Upper bound of the device bytes the job will hold at once (initial place
// scratch or the Nesterov arena, whichever is larger).  centred: the job's
// movable instances will be centred first (InitialPlace::placeInstsCenter).
int job_device_bytes(gpl_job* j, int64_t* bytes, bool centred);

// twiddle / frequency tables (host computed, double precision)
void make_twiddle(std::vector<float2>& tw);

// ------------------------------------------------------------ batched form
// Phases of one evaluation run for many jobs at once (batch.cu): each is one
// persistent launch over a table of work items int4 (instance, block of the
// instance's own launch, that launch's grid, 0).
enum BatchPhase {
  kBScatter = 0, kBScatterBig, kBWaSmall, kBWaLarge, kBWaSmallW, kBWaLargeW,
  kBPoissonA, kBPoissonB, kBPoissonC, kBDgradBig, kBCell, kBPhases
};
// element sizes of the argument tables (the batched kernels index them as
// arrays of the per-job argument structures)
size_t scatter_batch_args_bytes();
size_t cell_batch_args_bytes();
size_t wa_batch_args_bytes();
// blocks of a job's small-net and large-net WA launches
void wa_launch_blocks(const DeviceModel& d, int* small, int* large);
size_t poisson_batch_args_bytes(int pass);     // pass 0, 1, 2 = A, B, C
void write_scatter_batch_args(const DeviceModel& d, void* dst);
void write_cell_batch_args(const DeviceModel& d, const EvalArgs& a, void* dst);
void write_wa_batch_args(const DeviceModel& d, const EvalArgs& a, void* dst);
// the block-form Poisson passes of a job's grid: arguments, grids and
// dynamic shared memory of passes A, B, C; false for the warp form
// (512 x 512 and 1024 x 1024 grids) and the tensor-core form
bool write_poisson_batch_args(const DeviceModel& d, void* dst_a, void* dst_b, void* dst_c,
                              int grid[3], size_t smem[3]);
int scatter_batch_prepare_device();
int poisson_batch_prepare_device();
int launch_density_batch(int phase, const void* args, const int4* items, const int* count, int grid,
                         size_t smem, cudaStream_t s);
int launch_wa_batch(bool large, bool weighted, const void* args, const int4* items, const int* count, int grid,
                    cudaStream_t s);
int launch_poisson_batch(int pass, const void* args, const int4* items, const int* count, int grid,
                         size_t smem, cudaStream_t s);

// The host side of the batched form (job.cu): members join and leave
// between rounds; a round runs every running member's next evaluation.
struct BatchRun;
struct BatchMember {
  gpl_job* job = nullptr;
  bool running = false;     // still iterating in this batch
  bool start = true;        // its next evaluation starts an iteration
  int done = 0;             // iterations in this batch
  int limit = 0;            // iteration limit in this batch (0: to the stop rule)
  gpl_iter_log* log = nullptr;
};
BatchRun* batch_create(int device, int capacity, int* rc);
void batch_destroy(BatchRun* b);
bool batch_eligible(const gpl_job* j);
int batch_join(BatchRun* b, int slot, gpl_job* j, int max_iters, gpl_iter_log* log);
void batch_leave(BatchRun* b, int slot);
int batch_round(BatchRun* b, long long* launches);
bool batch_running(const BatchRun* b, int slot);
int batch_count_running(const BatchRun* b);
void batch_stop_member(BatchRun* b, int slot);     // ends the member's loop here (cancel)
// the member's gpl_nesterov_run status and stats once it stopped running
int batch_member_status(gpl_job* j, gpl_nesterov_stats* stats);

// Unique id of the calling thread's current CUDA context (cuCtxGetId through
// the runtime's driver entry points; 0 when it cannot be read).  Caches of
// device addresses are keyed on it: after cudaDeviceReset the device gets a
// new primary context, whose memory and symbol addresses are new.
unsigned long long current_context_id();
void make_freq(int nx, int ny, int bsx, int bsy, std::vector<float>& wx, std::vector<float>& wy);

}  // namespace gpl
