// Binomial checkpoint schedule for reversing a chain of time steps
// (Griewank's treeverse: with s free state slots and every step advanced at
// most r times, C(s + r, s) steps can be reversed).  Pure host C++: the
// executor supplies the state operations, so the schedule is exercised on the
// CPU by a simulated executor and drives the GPU adjoint in vk_api.cu.
//
// Executor interface (slot -1 is the executor's working state):
//   place(dst, src, n)  slot dst receives the state n steps after the one in
//                       slot src (a copy and n steps; an executor that knows
//                       dst already holds that state may skip both)
//   reverse_step(slot)  the slot holds the state before step i (the step being
//                       reversed): recompute that step's stage inputs and
//                       apply its adjoint; the slot is left unchanged
//   ok()                false after a failure (the schedule stops issuing)
//
// The forward run that precedes the reversal can store the states of the
// schedule's first descent (spine()) as it passes them, so that the reversal
// starts without re-advancing the chain.
#pragma once

#include <cstdint>
#include <utility>
#include <vector>

namespace vk {

// C(s + r, s), saturated at 2^62 (the number of steps reversible with s free
// slots and at most r advances of each step).
inline int64_t binom_capacity(int s, int64_t r) {
  const int64_t cap = int64_t(1) << 62;
  if (s <= 0 || r <= 0) return 1;
  // C(r + i, i) = C(r + i - 1, i - 1) (r + i) / i, exact at every i
  unsigned long long c = 1;
  for (int i = 1; i <= s; ++i) {
    const unsigned long long num = (unsigned long long)(r + i);
    if (c > (unsigned long long)cap / num) return cap;
    c = c * num / (unsigned long long)i;
  }
  return c > (unsigned long long)cap ? cap : (int64_t)c;
}

// Least r >= 1 with C(s + r, s) >= n (s >= 1); without a free slot every
// step is advanced up to n - 1 times.
inline int64_t binom_sweeps(int s, int64_t n) {
  if (s <= 0) return n > 1 ? n - 1 : 1;
  int64_t r = 1;
  while (binom_capacity(s, r) < n) ++r;
  return r;
}

// Steps a treeverse call over n >= 2 steps with s >= 1 free slots advances
// before its first checkpoint: the right part [lo + m, hi) keeps s - 1 free
// slots and r sweeps, the left part [lo, lo + m) all s slots and r - 1 sweeps
// (Pascal's rule).
inline int64_t treeverse_split(int s, int64_t n) {
  const int64_t r = binom_sweeps(s, n);
  const int64_t right = binom_capacity(s - 1, r);
  return n - right > 1 ? n - right : 1;
}

// Reverse steps [lo, hi): the state before step lo is in slot_lo (never
// overwritten); free_slots lists the slots this call may use.
template <class Ex>
void treeverse(Ex& ex, int64_t lo, int64_t hi, int slot_lo, std::vector<int>& free_slots) {
  const int64_t n = hi - lo;
  if (n <= 0 || !ex.ok()) return;
  if (n == 1) {
    ex.reverse_step(slot_lo);
    return;
  }
  const int s = (int)free_slots.size();
  if (s == 0) {
    // no slot left: advance a working copy from lo for every step, last first
    for (int64_t i = hi - 1; i >= lo && ex.ok(); --i) {
      ex.place(-1, slot_lo, i - lo);
      ex.reverse_step(-1);
    }
    return;
  }
  const int64_t m = treeverse_split(s, n);
  const int t = free_slots.back();
  free_slots.pop_back();
  ex.place(t, slot_lo, m);
  treeverse(ex, lo + m, hi, t, free_slots);
  free_slots.push_back(t);
  treeverse(ex, lo, lo + m, slot_lo, free_slots);
}

// The checkpoints of the first descent of treeverse(ex, 0, nsteps, 0, free)
// with free = {nsnap - 1, ..., 1} (slot 0 holds the initial state): the
// (slot, step) pairs it places before reversing its first step, in order.
// A forward run that stores the state before step `step` into `slot` for each
// of them leaves the reversal's first descent with nothing to recompute.
inline std::vector<std::pair<int, int64_t>> treeverse_spine(int64_t nsteps, int nsnap) {
  std::vector<std::pair<int, int64_t>> out;
  int64_t lo = 0;
  // the descent pops free_slots.back(): slots 1, 2, ... while the count of
  // free slots falls from nsnap - 1
  for (int nfree = nsnap - 1; nsteps - lo > 1 && nfree >= 1; --nfree) {
    lo += treeverse_split(nfree, nsteps - lo);
    out.push_back({nsnap - nfree, lo});
  }
  return out;
}

}  // namespace vk
