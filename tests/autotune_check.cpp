// The autotuner's bookkeeping (csrc/autotune.h), built by the host compiler
// against tests/fake_cuda/cuda_runtime.h: per-launch trials round robin,
// trials within one launch on shares of the work (scaled), settling small
// keys, and the choice of the fastest median.
#include <stdio.h>

#include "autotune.h"

#define CHECK(c)                                         \
  do {                                                   \
    if (!(c)) {                                          \
      printf("check failed line %d: %s\n", __LINE__, #c); \
      return 1;                                          \
    }                                                    \
  } while (0)

static void run(gpb::Autotuner& t, const std::string& key, int v, double ms, float scale = 1.f) {
  t.begin(key, v, nullptr, scale);
  fake_cuda_clock() += ms;
  t.end(nullptr);
}

int main() {
  gpb::Autotuner t;
  // per-launch trials: 3 variants x 2 reps, variant 2 fastest
  const double cost[3] = {3.0, 2.0, 1.0};
  for (int i = 0; i < 6; i++) {
    bool trial = false;
    const int v = t.pick("a", 3, 2, 1, &trial);
    CHECK(trial && v >= 0 && v < 3);
    run(t, "a", v, cost[v]);
  }
  bool trial = true;
  CHECK(t.pick("a", 3, 2, 1, &trial) == 1 && !trial);  // all in flight: the fallback, untimed
  CHECK(!t.decided("a"));
  t.collect();
  CHECK(t.decided("a"));
  CHECK(t.pick("a", 3, 2, 1, &trial) == 2 && !trial);
  // trials within one launch, each on a share of the work: variant 0 runs a
  // quarter of the items in 1 ms (4 ms whole), variant 1 three quarters in 2.7 ms
  t.entry("b", 2, 1);
  run(t, "b", 0, 1.0, 4.f);
  run(t, "b", 1, 2.7, 4.f / 3.f);
  t.collect();
  CHECK(t.decided("b") && t.pick("b", 2, 1, 0, &trial) == 1);
  // a key too small to time is settled on the default
  t.settle("c", 3, 1);
  CHECK(t.decided("c") && t.pick("c", 3, 1, 0, &trial) == 1);
  // a trial for a key never registered is dropped, not a crash
  run(t, "d", 5, 1.0);
  t.collect();
  CHECK(!t.decided("d"));
  // trials not yet timed go round again
  t.pick("e", 2, 1, 0, &trial);
  t.collect();
  CHECK(!t.decided("e"));
  int seen = 0;
  for (int i = 0; i < 2; i++) {
    const int v = t.pick("e", 2, 1, 0, &trial);
    if (trial) {
      run(t, "e", v, 1.0 + v);
      seen++;
    }
  }
  t.collect();
  CHECK(seen == 2 && t.decided("e") && t.pick("e", 2, 1, 1, &trial) == 0);
  // off: the fallback, every key decided
  gpb::Autotuner off;
  off.enabled = false;
  CHECK(off.decided("x") && off.pick("x", 3, 1, 2, &trial) == 2 && !trial);
  CHECK(t.report().find("a=2") != std::string::npos);
  printf("ok\n");
  return 0;
}
