// host_pool_check.cpp -- built and run by test_host_pool.py: the host pool
// runs every item once, rethrows the first exception of an item after all
// items are done, and stays usable afterwards.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "host_pool.h"

int main() {
  gpb::HostPool pool(8);
  int fails = 0;
  // every item once
  for (int n : {0, 1, 2, 7, 64, 1000}) {
    std::vector<std::atomic<int>> hit(n);
    for (auto& h : hit) h = 0;
    pool.run(n, [&](int i) { hit[i]++; });
    for (int i = 0; i < n; i++) fails += hit[i] != 1;
  }
  // an exception of an item reaches the caller once the others are done
  for (int n : {1, 16, 200}) {
    std::atomic<int> done{0};
    bool caught = false;
    try {
      pool.run(n, [&](int i) {
        if (i == n / 2) throw std::runtime_error("item failed");
        done++;
      });
    } catch (const std::runtime_error&) {
      caught = true;
    }
    fails += !caught;
    if (n > 1) fails += done != n - 1;
  }
  // an inline item (n == 1) may run the pool itself
  std::atomic<int> inner{0};
  pool.run(1, [&](int) { pool.run(32, [&](int) { inner++; }); });
  fails += inner != 32;
  // still usable
  std::atomic<int> after{0};
  pool.run(100, [&](int) { after++; });
  fails += after != 100;
  // copies cut into pieces land exactly once
  {
    const size_t piece = 4096;
    std::vector<size_t> sizes = {0, 1, piece - 1, piece, piece + 1, 5 * piece + 123, 64 * piece};
    std::vector<std::vector<unsigned char>> src, dst;
    std::vector<gpb::CopyJob> jobs;
    unsigned v = 1;
    for (size_t b : sizes) {
      src.emplace_back(b);
      dst.emplace_back(b + 2, 0xAB);  // a guard byte on each side
      for (auto& c : src.back()) c = (unsigned char)(v = v * 1103515245u + 12345u) >> 3;
    }
    for (size_t k = 0; k < sizes.size(); k++) jobs.push_back({dst[k].data() + 1, src[k].data(), sizes[k]});
    gpb::parallel_copy(pool, jobs, piece);
    for (size_t k = 0; k < sizes.size(); k++) {
      fails += dst[k].front() != 0xAB || dst[k].back() != 0xAB;
      fails += !std::equal(src[k].begin(), src[k].end(), dst[k].begin() + 1);
    }
  }
  std::printf("host pool: %d failures\n", fails);
  return fails != 0;
}
