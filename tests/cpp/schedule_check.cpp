// Simulated executor for vk::treeverse: states are step indices.  For each
// (nsteps, nsnap) prints
//   "ok <nsteps> <advances> <max_slots_in_use> <r> <advances_after_spine> <spine_last>"
// or "fail <nsteps> <nsnap> <reason>".  The second run prefills the slots of
// treeverse_spine as the forward run would, and counts the advances left to
// the reversal.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "vk_schedule.h"

struct SimEx {
  std::vector<long long> st;   // slot -> step index of the held state (-1: none)
  long long work = -1;
  long long next = 0;          // next step expected to be reversed
  long long advances = 0;
  int in_use = 1, max_in_use = 1;
  bool good = true;
  const char* why = "";
  long long& at(int s) { return s < 0 ? work : st[(size_t)s]; }
  void place(int d, int s, long long n) {
    if (at(s) < 0) { good = false; why = "place from an empty slot"; return; }
    const long long target = at(s) + n;
    if (d == s && n == 0) return;
    if (at(d) == target) return;   // the slot already holds that state
    if (d >= 0 && st[(size_t)d] < 0) { ++in_use; if (in_use > max_in_use) max_in_use = in_use; }
    at(d) = target;
    advances += n;
  }
  void reverse_step(int s) {
    if (at(s) != next) { good = false; why = "wrong state for the step being reversed"; return; }
    --next;
  }
  bool ok() const { return good; }
};

static bool run(long long nsteps, int nsnap, bool prefill, SimEx& ex, long long* spine_last) {
  ex.st.assign((size_t)nsnap, -1);
  ex.st[0] = 0;
  ex.next = nsteps - 1;
  *spine_last = 0;
  if (prefill) {
    for (const auto& p : vk::treeverse_spine(nsteps, nsnap)) {
      if (ex.st[(size_t)p.first] < 0) ++ex.in_use;
      ex.st[(size_t)p.first] = p.second;
      *spine_last = p.second;
    }
    ex.max_in_use = ex.in_use;
  }
  std::vector<int> free_slots;
  for (int s = nsnap - 1; s >= 1; --s) free_slots.push_back(s);
  vk::treeverse(ex, 0, nsteps, 0, free_slots);
  if (ex.good && ex.next != -1) { ex.good = false; ex.why = "not every step reversed"; }
  if (ex.good && (int)free_slots.size() != nsnap - 1) { ex.good = false; ex.why = "slots not returned"; }
  return ex.good;
}

int main(int argc, char** argv) {
  for (int a = 1; a + 1 < argc; a += 2) {
    const long long nsteps = atoll(argv[a]);
    const int nsnap = atoi(argv[a + 1]);
    SimEx plain, pre;
    long long dummy = 0, spine_last = 0;
    const bool ok1 = run(nsteps, nsnap, false, plain, &dummy);
    const bool ok2 = ok1 && run(nsteps, nsnap, true, pre, &spine_last);
    if (ok1 && ok2)
      printf("ok %lld %lld %d %lld %lld %lld\n", nsteps, plain.advances,
             plain.max_in_use > pre.max_in_use ? plain.max_in_use : pre.max_in_use,
             (long long)vk::binom_sweeps(nsnap - 1, nsteps), pre.advances, spine_last);
    else
      printf("fail %lld %d %s\n", nsteps, nsnap, ok1 ? pre.why : plain.why);
  }
  return 0;
}
