// Simulated executor for vk::treeverse: states are step indices.  Prints
// "ok <advances> <max_slots_in_use>" or "fail <reason>" for each (nsteps, nsnap).
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
  void copy(int d, int s) {
    if (at(s) < 0) { good = false; why = "copy from an empty slot"; return; }
    if (d >= 0 && st[(size_t)d] < 0) { ++in_use; if (in_use > max_in_use) max_in_use = in_use; }
    at(d) = at(s);
  }
  void advance(int s, long long n) { at(s) += n; advances += n; }
  void reverse_step(int s) {
    if (at(s) != next) { good = false; why = "wrong state for the step being reversed"; return; }
    --next;
  }
  bool ok() const { return good; }
};

int main(int argc, char** argv) {
  for (int a = 1; a + 1 < argc; a += 2) {
    const long long nsteps = atoll(argv[a]);
    const int nsnap = atoi(argv[a + 1]);
    SimEx ex;
    ex.st.assign((size_t)nsnap, -1);
    ex.st[0] = 0;
    ex.next = nsteps - 1;
    std::vector<int> free_slots;
    for (int s = nsnap - 1; s >= 1; --s) free_slots.push_back(s);
    vk::treeverse(ex, 0, nsteps, 0, free_slots);
    if (ex.good && ex.next != -1) { ex.good = false; ex.why = "not every step reversed"; }
    if (ex.good && (int)free_slots.size() != nsnap - 1) { ex.good = false; ex.why = "slots not returned"; }
    if (ex.good)
      printf("ok %lld %lld %d %lld\n", nsteps, ex.advances, ex.max_in_use,
             (long long)vk::binom_sweeps(nsnap - 1, nsteps));
    else
      printf("fail %lld %d %s\n", nsteps, nsnap, ex.why);
  }
  return 0;
}
