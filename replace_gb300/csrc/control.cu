// The device loop of the Nesterov iteration: the one-thread kernels that run
// between evaluations inside the job's loop graph (a conditional WHILE node
// whose body is one evaluation followed by k_loop_step).  They apply the
// control of control.h to the device copy of the state, write the next
// evaluation's control record, log each iteration and set the graph's
// conditions: continue the loop, refresh the scatter's tile order first.
#include <cuda_runtime.h>

#include "control.h"

namespace gpl {
namespace {

__device__ __forceinline__ bool chunk_open(const NesterovState& s) {
  return !s.finished && s.iter < s.max_iter && (s.chunk_limit <= 0 || s.chunk_done < s.chunk_limit);
}

// An upper bound of one chunk's evaluations (every iteration back-tracking to
// the limit), so that the loop ends whatever the state.
__device__ __forceinline__ long long chunk_eval_cap(const NesterovState& s) {
  const long long iters = s.chunk_limit > 0 ? s.chunk_limit : (long long)s.max_iter;
  return iters * (long long)(s.max_back_track + 1) + 2;
}

// Chunk start: the first evaluation's control record, or no loop at all.
__global__ void k_loop_head(NesterovState* S, EvalCtl* ctl, cudaGraphConditionalHandle h_loop,
                            cudaGraphConditionalHandle h_order) {
  NesterovState s = *S;
  s.chunk_done = 0;
  s.chunk_evals = 0;
  s.log_count = 0;
  const bool go = chunk_open(s);
  bool order = false;
  if (go) {
    start_iteration(s);
    order = s.iter % kTileOrderEvery == 0;
    if (order) s.refreshes++;
    *ctl = next_ctl(s);
  }
  *S = s;
  cudaGraphSetConditional(h_loop, go ? 1u : 0u);
  cudaGraphSetConditional(h_order, order ? 1u : 0u);
}

// After one evaluation of the loop body.
__global__ void k_loop_step(NesterovState* S, EvalCtl* ctl, const EvalResult* res, IterEntry* log, int log_cap,
                            cudaGraphConditionalHandle h_loop, cudaGraphConditionalHandle h_order) {
  NesterovState s = *S;
  IterEntry e;
  bool logged = false;
  const int a = after_eval(s, *res, &e, &logged);
  s.chunk_evals++;
  if (logged && s.log_count < log_cap) log[s.log_count++] = e;
  bool go = false, order = false;
  if (a == kRetry) {
    go = true;
  } else if (a == kNextIteration) {
    s.chunk_done++;
    go = chunk_open(s);
    if (go) {
      start_iteration(s);
      order = s.iter % kTileOrderEvery == 0;
      if (order) s.refreshes++;
    }
  } else {
    s.chunk_done++;
  }
  if (go && s.chunk_evals >= chunk_eval_cap(s)) go = false;
  if (go) *ctl = next_ctl(s);
  *S = s;
  cudaGraphSetConditional(h_loop, go ? 1u : 0u);
  cudaGraphSetConditional(h_order, order ? 1u : 0u);
}

}  // namespace

int launch_loop_head(NesterovState* S, EvalCtl* ctl, cudaGraphConditionalHandle h_loop,
                     cudaGraphConditionalHandle h_order, cudaStream_t s) {
  k_loop_head<<<1, 1, 0, s>>>(S, ctl, h_loop, h_order);
  GPL_CUDA(cudaGetLastError());
  return GPL_OK;
}

int launch_loop_step(NesterovState* S, EvalCtl* ctl, const EvalResult* res, IterEntry* log, int log_cap,
                     cudaGraphConditionalHandle h_loop, cudaGraphConditionalHandle h_order, cudaStream_t s) {
  k_loop_step<<<1, 1, 0, s>>>(S, ctl, res, log, log_cap, h_loop, h_order);
  GPL_CUDA(cudaGetLastError());
  return GPL_OK;
}

}  // namespace gpl
