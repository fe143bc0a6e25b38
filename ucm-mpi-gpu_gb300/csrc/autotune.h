// autotune.h -- the library's online autotuner for kernel variants.
//
// A tunable launch has several variants that compute bit-identical results
// (thread counts per tile, how a persistent kernel walks its tiles, how it
// stages an operand) but run at different speeds depending on the batch's
// shape.  For a key -- the kernel and a bucket of the launch's shape -- the
// first launches try the variants in turn on real work, each timed with a
// pair of CUDA events on the launching stream; once every variant has `reps`
// timings, the one with the smallest median wins and every later launch with
// that key uses it.  Timings are read only where the host has already
// synchronised with the stream (collect()), so tuning adds no host round
// trip.  Choices live in the context for its lifetime.
#pragma once

#include <cuda_runtime.h>
#include <stdio.h>

#include <algorithm>
#include <map>
#include <string>
#include <vector>

namespace gpb {

class Autotuner {
 public:
  struct Entry {
    int nvar = 0, reps = 1;
    int chosen = -1;
    std::vector<std::vector<float>> ms;  // timings per variant
    std::vector<int> issued;             // launches per variant, timed or in flight
  };

  bool enabled = true;

  ~Autotuner() {
    for (auto& p : pend_) {
      cudaEventDestroy(p.a);
      cudaEventDestroy(p.b);
    }
    for (cudaEvent_t e : free_) cudaEventDestroy(e);
  }

  // The entry of `key`, created with nvar variants and reps timings each.
  Entry& entry(const std::string& key, int nvar, int reps) {
    Entry& e = tab_[key];
    if (e.nvar == 0) {
      e.nvar = nvar;
      e.reps = reps;
      e.ms.assign(nvar, {});
      e.issued.assign(nvar, 0);
    }
    return e;
  }

  // The variant to launch for `key`, and whether this launch is a timed trial.
  int pick(const std::string& key, int nvar, int reps, int fallback, bool* trial) {
    *trial = false;
    if (!enabled || nvar <= 1) return fallback;
    Entry& e = entry(key, nvar, reps);
    if (e.chosen >= 0) return e.chosen;
    int v = 0;
    for (int i = 1; i < nvar; i++)
      if (e.issued[i] < e.issued[v]) v = i;
    if (e.issued[v] >= reps) return fallback;  // all trials in flight: wait for collect()
    e.issued[v]++;
    *trial = true;
    return v;
  }

  bool decided(const std::string& key) const {
    if (!enabled) return true;
    auto it = tab_.find(key);
    return it != tab_.end() && it->second.chosen >= 0;
  }

  // events around a trial launch of variant v; its time counts `scale`
  // times (a trial on 1/scale of a launch's independent work items)
  void begin(const std::string& key, int v, cudaStream_t s, float scale = 1.f) {
    Pending p{key, v, take(), take(), scale};
    cudaEventRecord(p.a, s);
    pend_.push_back(p);
  }
  // registers a key and decides it at once (no trials worth timing)
  void settle(const std::string& key, int nvar, int v) {
    Entry& e = entry(key, nvar, 1);
    if (e.chosen < 0) e.chosen = v;
  }
  void end(cudaStream_t s) {
    if (!pend_.empty()) cudaEventRecord(pend_.back().b, s);
  }

  // Reads finished trials (call only after the stream has synchronised) and
  // settles every key whose variants all have their timings.
  void collect() {
    for (auto& p : pend_) {
      float ms = 0.f;
      auto it = tab_.find(p.key);
      if (it != tab_.end() && p.v >= 0 && p.v < (int)it->second.ms.size() &&
          cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess)
        it->second.ms[p.v].push_back(ms * p.scale);
      free_.push_back(p.a);
      free_.push_back(p.b);
    }
    pend_.clear();
    (void)cudaGetLastError();
    for (auto& kv : tab_) {
      Entry& e = kv.second;
      if (e.chosen >= 0) continue;
      bool all = true;
      for (int v = 0; v < e.nvar; v++) all = all && (int)e.ms[v].size() >= e.reps;
      if (!all) {  // trials that were not timed go round again
        for (int v = 0; v < e.nvar; v++) e.issued[v] = (int)e.ms[v].size();
        continue;
      }
      int best = 0;
      float best_ms = 0.f;
      for (int v = 0; v < e.nvar; v++) {
        std::vector<float> t = e.ms[v];
        std::sort(t.begin(), t.end());
        const float med = t[t.size() / 2];
        if (v == 0 || med < best_ms) {
          best = v;
          best_ms = med;
        }
      }
      e.chosen = best;
    }
  }

  // "key=variant (median ms per variant); ..." for reports
  std::string report() const {
    std::string r;
    for (const auto& kv : tab_) {
      const Entry& e = kv.second;
      r += kv.first + "=" + std::to_string(e.chosen) + " (";
      for (int v = 0; v < e.nvar; v++) {
        std::vector<float> t = e.ms[v];
        std::sort(t.begin(), t.end());
        char buf[32];
        snprintf(buf, sizeof(buf), "%s%.3f", v ? " " : "", t.empty() ? -1.0 : (double)t[t.size() / 2]);
        r += buf;
      }
      r += "); ";
    }
    return r;
  }

 private:
  struct Pending {
    std::string key;
    int v;
    cudaEvent_t a, b;
    float scale;
  };
  cudaEvent_t take() {
    if (!free_.empty()) {
      cudaEvent_t e = free_.back();
      free_.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
  std::map<std::string, Entry> tab_;
  std::vector<Pending> pend_;
  std::vector<cudaEvent_t> free_;
};

}  // namespace gpb
