// gpb_damascene.cpp -- computeGPb / getCudaDeviceCount with the reference's
// C++ signatures (damascene/include/globalPb.h:35,44), on top of the C ABI.
#include <stdint.h>
#include <stdlib.h>

#include <mutex>
#include <vector>

#include "../../include/gpb.h"
#include "../../include/gpb_damascene.h"

namespace {
std::mutex g_mu;
gpb_ctx* g_ctx[64] = {};
std::vector<float> g_codebook;
int g_K = 0;

[[noreturn]] void fail() {
  // damascene/include/exception.h: customCheckCudaErrors throws int64 1
  throw (int64_t)1;
}

gpb_ctx* ctx_for(unsigned rank) {
  const int n = gpb_device_count();
  if (n <= 0) fail();
  const int dev = (int)(rank % (unsigned)n);  // damascene.cu:264
  if (dev >= 64) fail();
  if (!g_ctx[dev]) {
    gpb_params p;
    gpb_default_params(&p);
    p.device = dev;
    p.compat = GPB_COMPAT_DAMASCENE;
    if (gpb_create(&g_ctx[dev], &p) != GPB_OK) fail();
    gpb_status s = GPB_ERR_ARG;
    if (g_K > 0) {
      s = gpb_set_codebook(g_ctx[dev], g_codebook.data(), g_K);
    } else if (const char* path = getenv("GPB_TEXTON_CODEBOOK")) {
      s = gpb_load_codebook_yml(g_ctx[dev], path);
    }
    if (s != GPB_OK) {
      gpb_destroy(g_ctx[dev]);
      g_ctx[dev] = nullptr;
      fail();
    }
  }
  return g_ctx[dev];
}
}  // namespace

int gpbSetTextonCodebook(const float* codebook, int K) {
  if (!codebook || K < 1 || K > 32) return -1;
  std::lock_guard<std::mutex> lk(g_mu);
  g_codebook.assign(codebook, codebook + 13 * K);
  g_K = K;
  for (auto& c : g_ctx)
    if (c) gpb_set_codebook(c, codebook, K);
  return 0;
}

int getCudaDeviceCount() { return gpb_device_count(); }

void computeGPb(unsigned int rank, unsigned int width, unsigned int height, unsigned int* data,
                float** hostGPb, float** hostGPbAllConcat) {
  if (!data || !hostGPb || !hostGPbAllConcat) fail();
  std::lock_guard<std::mutex> lk(g_mu);
  gpb_ctx* ctx = ctx_for(rank);
  float* nmax = nullptr;
  float* orient = nullptr;
  const gpb_status s = gpb_compute(ctx, width, height, (const uint32_t*)data, &nmax, &orient);
  if (s != GPB_OK) {
    free(nmax);
    free(orient);
    fail();
  }
  *hostGPb = nmax;
  *hostGPbAllConcat = orient;
}
