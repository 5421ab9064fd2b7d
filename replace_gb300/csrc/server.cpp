// Placement server (gpl_server_* in include/gpl.h): continuous batching of
// independent placement jobs on one GPU.
//
// One host thread per slot.  A slot owns a CUDA stream and a pinned staging
// block for the life of the server; jobs take device memory from one
// stream-ordered pool whose release threshold is the HBM budget, so admitting
// and retiring jobs never synchronises the device.  Jobs leave the queue in
// submission order when a slot is idle and the head job's footprint fits
// next to the footprints already reserved.  While admitted, a job runs the
// ordinary job path (initial place, Nesterov init, Nesterov loop in chunks)
// on its slot's stream; its evaluations replay the job's own CUDA graph, so
// the kernels of all admitted jobs overlap on the device.
//
// Batched mode (gpl_server_params.batched): after its initial place and
// Nesterov init on its slot, a job joins one running batch (the batched
// form of the Nesterov loop, BatchRun in job.cu): a batch thread runs
// rounds in which every member's next evaluation goes into one launch per
// phase, admits new members between rounds and retires members whose loop
// ended; the slot thread then finishes the job as before.  A member's
// result is bit-identical to the same job run alone.
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "gpl_internal.h"

using namespace gpl;

namespace {

// Device bytes added to each job's footprint bound: graph, pool rounding.
constexpr int64_t kJobSlack = 4 << 20;

struct Entry {
  int64_t ticket = 0;
  gpl_job* job = nullptr;
  int64_t bytes = 0;
  std::atomic<bool> cancel{false};
  // batched mode: set by the batch thread when the job's loop ended there
  bool batch_done = false;
  int batch_rc = 0;
  bool batch_cancelled = false;
  gpl_server_result res{};
  std::vector<int32_t> lx, ly;
};

void copy_message(gpl_server_result& r, const char* msg) {
  std::strncpy(r.message, msg ? msg : "", sizeof(r.message) - 1);
  r.message[sizeof(r.message) - 1] = '\0';
}

}  // namespace

struct gpl_server {
  gpl_server_params p{};
  int64_t budget = 0, reserved = 0;
  cudaMemPool_t pool = nullptr;
  std::vector<cudaStream_t> streams;
  std::vector<HostPinned*> pinned;
  std::vector<cudaEvent_t> sync_ev;   // per slot; null = spin-waiting syncs
  std::vector<std::thread> workers;
  std::mutex mu;
  std::condition_variable cv_work;   // queue, budget or stop changed
  std::condition_variable cv_done;   // a job ended
  std::deque<std::shared_ptr<Entry>> queue;
  std::map<int64_t, std::shared_ptr<Entry>> running;
  std::map<int64_t, std::shared_ptr<Entry>> ended;   // kept until released
  std::deque<int64_t> unpolled;
  int64_t next_ticket = 1;
  bool stop = false;
  // batched mode: the batch thread, its batch, and the jobs waiting to join
  std::thread batcher;
  BatchRun* batch = nullptr;
  std::deque<std::pair<int, Entry*>> batch_in;
  std::condition_variable cv_batch;   // a job joins, a slot thread ends, or stop
  int workers_exited = 0;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

// One admitted job on slot `slot`, start to end.
void run_job(gpl_server* s, int slot, Entry& e) {
  gpl_job* j = e.job;
  job_bind(j, s->streams[slot], s->pinned[slot], s->pool, s->sync_ev[slot]);
  int rc = GPL_OK;
  gpl_ip_stats ip{};
  if (s->p.run_initial_place) rc = gpl_initial_place(j, &ip);
  if (!rc) rc = gpl_nesterov_init(j, nullptr);
  gpl_nesterov_stats st{};
  if (!rc && s->batch && batch_eligible(j)) {
    // the loop runs in the batch; this thread waits for its end
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->batch_in.emplace_back(slot, &e);
      s->cv_batch.notify_all();
      s->cv_done.wait(lk, [&] { return e.batch_done; });
    }
    if (e.batch_rc) {
      rc = e.batch_rc;
    } else if (e.batch_cancelled) {
      rc = GPL_ERR_CANCELLED;
      set_error("cancelled");
      batch_member_status(j, &st);
    } else {
      rc = batch_member_status(j, &st);
    }
  }
  while (!rc && !st.finished && !e.batch_done) {
    if (e.cancel.load()) {
      rc = GPL_ERR_CANCELLED;
      set_error("cancelled");
      break;
    }
    // a diverged loop returns its code with st filled where it stopped
    rc = gpl_nesterov_run(j, s->p.chunk_iters, &st, nullptr);
    if (st.finished) break;
  }
  e.res.status = rc;
  e.res.finished = st.finished;
  e.res.iterations = st.iterations;
  e.res.ip_rounds = ip.iterations;
  e.res.overflow = st.overflow;
  e.res.hpwl = st.hpwl;
  if (rc) copy_message(e.res, gpl_last_error());
  e.lx.assign(e.res.n_insts, 0);
  e.ly.assign(e.res.n_insts, 0);
  if (e.res.n_insts > 0) gpl_get_inst_locations(j, e.lx.data(), e.ly.data());
  gpl_destroy(j);                               // frees in stream order
  e.job = nullptr;
  host_wait(s->streams[slot], s->sync_ev[slot]); // the memory is back in the pool
}

// Batched mode: runs rounds while members run; takes joining jobs between
// rounds, retires members whose loop ended (or that were cancelled) and
// wakes their slot threads.
void batcher(gpl_server* s) {
  cudaSetDevice(s->p.device);
  std::vector<Entry*> member(s->p.max_active, nullptr);
  for (;;) {
    std::deque<std::pair<int, Entry*>> joining;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      // at stop, the batch serves until every slot thread has ended (a slot
      // may still be initialising a job that will join)
      const int n_slots = s->p.max_active;
      s->cv_batch.wait(lk, [&] {
        return (s->stop && s->workers_exited == n_slots) || !s->batch_in.empty() ||
               batch_count_running(s->batch) > 0;
      });
      joining.swap(s->batch_in);
      if (joining.empty() && batch_count_running(s->batch) == 0) return;   // stopped, slots ended
    }
    std::vector<Entry*> ended;
    for (auto& jn : joining) {
      const int rc = batch_join(s->batch, jn.first, jn.second->job, 0, nullptr);
      if (rc) {
        jn.second->batch_rc = rc;
        ended.push_back(jn.second);
      } else {
        member[jn.first] = jn.second;
      }
    }
    for (int k = 0; k < (int)member.size(); k++)
      if (member[k] && member[k]->cancel.load() && batch_running(s->batch, k)) {
        member[k]->batch_cancelled = true;
        batch_stop_member(s->batch, k);
      }
    long long nl = 0;
    int rc = batch_round(s->batch, &nl);
    for (int k = 0; k < (int)member.size(); k++) {
      if (!member[k]) continue;
      if (rc) member[k]->batch_rc = rc;
      if (rc || !batch_running(s->batch, k)) {
        batch_leave(s->batch, k);
        ended.push_back(member[k]);
        member[k] = nullptr;
      }
    }
    if (!ended.empty()) {
      std::lock_guard<std::mutex> lk(s->mu);
      for (Entry* e : ended) e->batch_done = true;
      s->cv_done.notify_all();
    }
  }
}

void worker_loop(gpl_server* s, int slot);

void worker(gpl_server* s, int slot) {
  worker_loop(s, slot);
  std::lock_guard<std::mutex> lk(s->mu);
  s->workers_exited++;
  s->cv_batch.notify_all();
}

void worker_loop(gpl_server* s, int slot) {
  cudaSetDevice(s->p.device);
  for (;;) {
    std::shared_ptr<Entry> e;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] {
        return s->stop || (!s->queue.empty() && s->reserved + s->queue.front()->bytes <= s->budget);
      });
      if (s->stop) return;
      e = s->queue.front();
      s->queue.pop_front();
      s->reserved += e->bytes;
      e->res.admit_s = s->now();
      s->running[e->ticket] = e;
    }
    s->cv_work.notify_all();   // the next queued job may fit as well
    run_job(s, slot, *e);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      e->res.finish_s = s->now();
      s->reserved -= e->bytes;
      s->running.erase(e->ticket);
      s->ended[e->ticket] = e;
      s->unpolled.push_back(e->ticket);
    }
    s->cv_work.notify_all();
    s->cv_done.notify_all();
  }
}

}  // namespace

extern "C" {

void gpl_server_params_default(gpl_server_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->device = 0;
  p->max_active = 8;
  p->hbm_budget_bytes = 0;
  p->chunk_iters = 64;
  p->run_initial_place = 1;
  p->blocking_sync = 1;
  p->batched = 0;
}

gpl_status gpl_server_create(const gpl_server_params* p, gpl_server** out) {
  if (!out || !p) { set_error("null argument"); return GPL_ERR_INVALID_ARG; }
  *out = nullptr;
  if (p->max_active < 1 || p->max_active > 256 || p->chunk_iters < 1 || p->hbm_budget_bytes < 0) {
    set_error("server parameters: max_active in [1, 256], chunk_iters >= 1, budget >= 0");
    return GPL_ERR_INVALID_ARG;
  }
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    set_error("no CUDA device available: the GB300 placement core has no CPU fallback");
    return GPL_ERR_NO_DEVICE;
  }
  if (p->device < 0 || p->device >= n) { set_error("device ordinal out of range"); return GPL_ERR_INVALID_ARG; }
  GPL_CUDA(cudaSetDevice(p->device));
  std::unique_ptr<gpl_server> s(new gpl_server());
  s->p = *p;
  size_t free_b = 0, total_b = 0;
  GPL_CUDA(cudaMemGetInfo(&free_b, &total_b));
  s->budget = p->hbm_budget_bytes > 0 ? p->hbm_budget_bytes : (int64_t)(0.8 * (double)free_b);
  cudaMemPoolProps props;
  std::memset(&props, 0, sizeof(props));
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = p->device;
  GPL_CUDA(cudaMemPoolCreate(&s->pool, &props));
  uint64_t thr = (uint64_t)s->budget;
  GPL_CUDA(cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &thr));
  for (int k = 0; k < p->max_active; k++) {
    cudaStream_t st = nullptr;
    GPL_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    s->streams.push_back(st);
    HostPinned* hp = nullptr;
    GPL_CUDA(cudaMallocHost(&hp, sizeof(HostPinned)));
    s->pinned.push_back(hp);
    cudaEvent_t ev = nullptr;
    if (p->blocking_sync)
      GPL_CUDA(cudaEventCreateWithFlags(&ev, cudaEventBlockingSync | cudaEventDisableTiming));
    s->sync_ev.push_back(ev);
  }
  if (p->batched) {
    int rc = GPL_OK;
    s->batch = batch_create(p->device, p->max_active, &rc);
    if (!s->batch) return (gpl_status)rc;
  }
  gpl_server* raw = s.release();
  if (raw->batch) raw->batcher = std::thread(batcher, raw);
  for (int k = 0; k < p->max_active; k++) raw->workers.emplace_back(worker, raw, k);
  *out = raw;
  return GPL_OK;
}

gpl_status gpl_server_submit(gpl_server* s, const gpl_netlist_desc* nl, const gpl_params* p,
                             int64_t* ticket) {
  return gpl_server_submit_weighted(s, nl, p, nullptr, 0, ticket);
}

gpl_status gpl_server_submit_weighted(gpl_server* s, const gpl_netlist_desc* nl, const gpl_params* p,
                                      const float* weights, int64_t n_nets, int64_t* ticket) {
  if (!s || !nl || !p || !ticket) { set_error("null argument"); return GPL_ERR_INVALID_ARG; }
  if (p->device != s->p.device) { set_error("job device differs from the server's"); return GPL_ERR_INVALID_ARG; }
  gpl_params prm = *p;
  if (s->p.batched && prm.poisson_path == 0) prm.poisson_path = 1;   // the batched kernels' form
  gpl_job* j = nullptr;
  int rc = job_new(nl, &prm, &j);
  if (rc) return (gpl_status)rc;
  if (weights) {
    // stored on the host now, uploaded with the job's device model
    rc = gpl_set_net_weights(j, weights, n_nets);
    if (rc) { gpl_destroy(j); return (gpl_status)rc; }
  }
  int64_t bytes = 0;
  rc = job_device_bytes(j, &bytes, s->p.run_initial_place && !prm.incremental_place_mode);
  if (rc) { gpl_destroy(j); return (gpl_status)rc; }
  bytes += kJobSlack;
  if (bytes > s->budget) {
    gpl_destroy(j);
    set_error("job footprint (" + std::to_string(bytes) + " B) exceeds the server's HBM budget (" +
              std::to_string(s->budget) + " B)");
    return GPL_ERR_OUT_OF_MEMORY;
  }
  auto e = std::make_shared<Entry>();
  e->job = j;
  e->bytes = bytes;
  e->res.n_insts = nl->n_insts;
  e->res.device_bytes = bytes;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    e->ticket = s->next_ticket++;
    e->res.ticket = e->ticket;
    e->res.submit_s = s->now();
    s->queue.push_back(e);
  }
  s->cv_work.notify_all();
  *ticket = e->ticket;
  return GPL_OK;
}

int32_t gpl_server_poll(gpl_server* s, gpl_server_result* out, int32_t capacity, int32_t wait_ms) {
  if (!s || !out || capacity <= 0) return 0;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->unpolled.empty() && wait_ms > 0)
    s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->unpolled.empty(); });
  int32_t n = 0;
  while (n < capacity && !s->unpolled.empty()) {
    const int64_t t = s->unpolled.front();
    s->unpolled.pop_front();
    auto it = s->ended.find(t);
    if (it != s->ended.end()) out[n++] = it->second->res;
  }
  return n;
}

gpl_status gpl_server_get_inst_locations(gpl_server* s, int64_t ticket, int32_t* lx, int32_t* ly) {
  if (!s || !lx || !ly) { set_error("null argument"); return GPL_ERR_INVALID_ARG; }
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->ended.find(ticket);
  if (it == s->ended.end()) { set_error("no ended job with this ticket"); return GPL_ERR_BAD_STATE; }
  const Entry& e = *it->second;
  if (!e.lx.empty()) {
    std::memcpy(lx, e.lx.data(), e.lx.size() * sizeof(int32_t));
    std::memcpy(ly, e.ly.data(), e.ly.size() * sizeof(int32_t));
  }
  return GPL_OK;
}

gpl_status gpl_server_release(gpl_server* s, int64_t ticket) {
  if (!s) { set_error("null server"); return GPL_ERR_INVALID_ARG; }
  std::lock_guard<std::mutex> lk(s->mu);
  if (!s->ended.erase(ticket)) { set_error("no ended job with this ticket"); return GPL_ERR_BAD_STATE; }
  return GPL_OK;
}

gpl_status gpl_server_cancel(gpl_server* s, int64_t ticket) {
  if (!s) { set_error("null server"); return GPL_ERR_INVALID_ARG; }
  std::shared_ptr<Entry> dropped;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
      if ((*it)->ticket == ticket) {
        dropped = *it;
        s->queue.erase(it);
        break;
      }
    }
    if (!dropped) {
      auto r = s->running.find(ticket);
      if (r != s->running.end()) {
        r->second->cancel = true;
        return GPL_OK;
      }
      if (s->ended.count(ticket)) return GPL_OK;
      set_error("unknown ticket");
      return GPL_ERR_INVALID_ARG;
    }
    dropped->res.status = GPL_ERR_CANCELLED;
    copy_message(dropped->res, "cancelled before admission");
    dropped->res.admit_s = dropped->res.finish_s = s->now();
    s->ended[ticket] = dropped;
    s->unpolled.push_back(ticket);
  }
  gpl_destroy(dropped->job);   // never bound: host memory only
  dropped->job = nullptr;
  s->cv_work.notify_all();     // the new queue head may fit
  s->cv_done.notify_all();
  return GPL_OK;
}

void gpl_server_counts(gpl_server* s, int32_t* queued, int32_t* running, int32_t* ended) {
  if (!s) return;
  std::lock_guard<std::mutex> lk(s->mu);
  if (queued) *queued = (int32_t)s->queue.size();
  if (running) *running = (int32_t)s->running.size();
  if (ended) *ended = (int32_t)s->unpolled.size();
}

void gpl_server_destroy(gpl_server* s) {
  if (!s) return;
  std::deque<std::shared_ptr<Entry>> dropped;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    dropped.swap(s->queue);
    for (auto& r : s->running) r.second->cancel = true;
  }
  s->cv_work.notify_all();
  s->cv_batch.notify_all();
  for (auto& t : s->workers) t.join();
  if (s->batcher.joinable()) s->batcher.join();
  if (s->batch) batch_destroy(s->batch);
  for (auto& e : dropped) gpl_destroy(e->job);
  cudaSetDevice(s->p.device);
  for (auto st : s->streams) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  for (auto hp : s->pinned) cudaFreeHost(hp);
  for (auto ev : s->sync_ev)
    if (ev) cudaEventDestroy(ev);
  if (s->pool) cudaMemPoolDestroy(s->pool);
  delete s;
}

}  // extern "C"
