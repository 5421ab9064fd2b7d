// The Nesterov control of NesterovPlace::doNesterovPlace
// (src/nesterovPlace.cpp:275-472, updateNextIter :514-553,
// updateWireLengthCoef :474-490), written once for the host loop and for the
// device loop (a one-thread kernel between evaluations inside a CUDA graph
// with a conditional WHILE node), so that both run the same arithmetic.
//
// One iteration: start_iteration, then evaluations at next_ctl until
// after_eval reports the iteration's end (the step length is accepted,
// back-tracking ran out, or the gradients diverged); the post-iteration
// update (buffer rotation, overflow, coefficients, penalty, stop rules) runs
// inside after_eval.
#pragma once

#include <cmath>
#include <cstdint>

#include "gpl_internal.h"

#if defined(__CUDACC__)
#define GPL_HD __host__ __device__ __forceinline__
#else
#define GPL_HD inline
#endif

namespace gpl {

enum StepAction { kRetry = 0, kNextIteration = 1, kStop = 2 };

// Iterations between refreshes of the scatter's tile order (cells move
// slowly; any order gives the same int64 areas).
constexpr int kTileOrderEvery = 32;

// NaN or infinite (v - v is 0 for every finite v, NaN otherwise)
GPL_HD bool bad_value(double v) { return !(v - v == 0.0); }

GPL_HD bool diverged_result(const EvalResult& r) {
  return bad_value((float)r.wl_sum) || bad_value((float)r.d_sum) || r.nan_flag != 0.0;
}

// sumOverflow_ (src/nesterovPlace.cpp:112-115, 529-532)
GPL_HD float overflow_ratio_of(const NesterovState& S, double overflow) {
  return (float)(int64_t)overflow / S.ovf_den;
}

// NesterovPlace::updateWireLengthCoef (src/nesterovPlace.cpp:474-490)
GPL_HD void update_wl_coef_of(NesterovState& S, float overflow) {
  float c;
  if (overflow > 1.0) c = 0.1f;
  else if (overflow < 0.1) c = 10.0f;
  else c = (float)(1.0 / pow(10.0, (overflow - 0.1) * 20 / 9.0 - 1.0));
  S.wl_coef_x = c * S.base_wl_coef;
  S.wl_coef_y = c * S.base_wl_coef;
}

// Start of an iteration: the Nesterov coefficient (src/nesterovPlace.cpp:332-336).
GPL_HD void start_iteration(NesterovState& S) {
  const float prev_a = S.cur_a;
  S.cur_a = (float)((1.0 + sqrt(4.0 * prev_a * prev_a + 1.0)) * 0.5);
  S.coeff = (float)((prev_a - 1.0) / S.cur_a);
  S.attempts = 0;
}

// The control record of the iteration's next evaluation: predict slot i_next
// from i_cur with the current step length, reference slot i_cur.
GPL_HD EvalCtl next_ctl(const NesterovState& S) {
  EvalCtl c;
  c.step = S.step_length;
  c.coeff = S.coeff;
  c.density_penalty = S.density_penalty;
  c.wl_coef_x = S.wl_coef_x;
  c.wl_coef_y = S.wl_coef_y;
  c.predict = 1;
  c.i_src = S.i_cur;
  c.i_eval = S.i_next;
  c.i_ref = S.i_cur;
  c.c_cur = S.c_cur;
  c.c_next = S.c_next;
  c.area_cur = S.area_next;
  c.write_sum = 1;
  c.write_wd = 0;
  c.pad[0] = c.pad[1] = 0;
  return c;
}

// After the back-tracking loop: bt is the 0-based index of the accepted (or
// diverged) attempt, max_back_track when none was accepted.
GPL_HD int post_iteration(NesterovState& S, int bt, IterEntry* entry, bool* logged) {
  *logged = false;
  if (!S.max_phi_changed && S.sum_overflow < 0.35f) {
    S.max_phi_changed = 1;
    S.max_phi_coef = (float)(S.max_phi_coef * 0.99);
  }
  if (S.max_back_track == bt) {
    S.diverge_code = GPL_ERR_DIVERGED_BACKTRACK;
    S.is_diverged = 1;
  }
  if (S.is_diverged) {
    if (!S.diverge_code) S.diverge_code = GPL_ERR_DIVERGED_NAN;
    S.finished = 1;
    return kStop;
  }
  // updateNextIter (src/nesterovPlace.cpp:514-553)
  const int op = S.i_prev;
  S.i_prev = S.i_cur; S.i_cur = S.i_next; S.i_next = op;
  const int cc = S.c_cur; S.c_cur = S.c_next; S.c_next = cc;
  S.sum_overflow = overflow_ratio_of(S, S.last.overflow);
  update_wl_coef_of(S, S.sum_overflow);
  const long long hpwl = S.last.hpwl;
  const float sd = (float)(hpwl - S.prev_hpwl) / S.reference_hpwl;
  float pc = (sd < 0) ? S.max_phi_coef : (float)(S.max_phi_coef * pow(S.max_phi_coef, sd * -1.0));
  pc = pc < S.min_phi_coef ? S.min_phi_coef : pc;
  S.prev_hpwl = hpwl;
  S.density_penalty *= pc;
  entry->overflow = S.sum_overflow;
  entry->hpwl = S.prev_hpwl;
  entry->step_length = S.step_length;
  entry->backtracks = bt + 1;
  entry->pad = 0;
  *logged = true;
  const int it = S.iter;
  S.iter++;
  if (S.min_sum_overflow > S.sum_overflow) {
    S.min_sum_overflow = S.sum_overflow;
    S.hpwl_with_min = (float)S.prev_hpwl;
  }
  if (S.sum_overflow < 0.3f && S.sum_overflow - S.min_sum_overflow >= 0.02f && S.hpwl_with_min * 1.2f < S.prev_hpwl) {
    S.diverge_code = GPL_ERR_DIVERGED_PHI;
    S.is_diverged = 1;
    S.finished = 1;
    return kStop;
  }
  if (it > 50 && S.sum_overflow <= S.target_overflow) {
    S.finished = 1;
    return kStop;
  }
  return kNextIteration;
}

// The result of the evaluation at next_ctl(S): bookkeeping, the step-length
// test (src/nesterovPlace.cpp:381-402), and at the iteration's end the
// post-iteration update.
GPL_HD int after_eval(NesterovState& S, const EvalResult& r, IterEntry* entry, bool* logged) {
  *logged = false;
  S.last = r;
  S.last_area = S.area_next;
  S.area_next ^= 1;
  S.last_slot = S.i_next;
  S.evals++;
  S.attempts++;
  int bt = S.attempts - 1;
  if (diverged_result(r)) {
    S.is_diverged = 1;
  } else {
    const float ns = r.new_step_length;
    if (ns > S.step_length * 0.95) {
      S.step_length = ns;
    } else {
      S.step_length = ns;
      if (S.attempts < S.max_back_track) return kRetry;
      bt = S.max_back_track;
    }
  }
  return post_iteration(S, bt, entry, logged);
}

}  // namespace gpl
