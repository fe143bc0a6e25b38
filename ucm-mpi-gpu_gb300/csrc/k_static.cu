// k_static.cu -- the texton stage on a fixed device scratch area, for
// callers that must not allocate device memory (gpb_texton_labels_static).
//
// The same kernels as the batch pipeline (k_convert, k_texton,
// k_texton_repair) run on one image, with every buffer they need besides
// the caller's input and output placed in one file-scope __device__ array:
//
//   [kOffPatch]   the patch record (PatchDev) of the image
//   [kOffWork]    the 16 x 16 tile list, one int4 per tile
//   [kOffCount]   the repair counter: must be 0 when k_texton starts
//   [kOffGrey]    the 8-bit grey image, one byte per pixel
//   [kOffRepair]  the repair list, two ints per entry, one entry per pixel
//                 at most, so it cannot overflow
//
// k_static_setup, the first launch of every call, writes the patch record,
// the tile list and the zero counter, so no call depends on what an earlier
// call left behind, nor on the array's zero initialisation.
#include <stdint.h>

#include <mutex>

#include "gpb_internal.h"
#include "k_static.h"
#include "kernels.h"

namespace gpb {

namespace {
constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t kOffPatch = 0;
constexpr size_t kOffWork = 256;
constexpr size_t kOffCount = align256(kOffWork + 16 * (size_t)kStaticMaxTiles);
constexpr size_t kOffGrey = kOffCount + 256;
constexpr size_t kOffRepair = align256(kOffGrey + (size_t)kStaticMaxPix);
constexpr size_t kScratchBytes = kOffRepair + 8 * (size_t)kStaticMaxPix;
static_assert(sizeof(PatchDev) <= kOffWork, "patch record slot");
}  // namespace

static __device__ __align__(256) unsigned char g_texton_scratch[kScratchBytes];

size_t static_scratch_bytes() { return kScratchBytes; }

// the scratch address on the current device, looked up once per device
cudaError_t static_scratch(unsigned char** base) {
  constexpr int kMaxDevices = 64;
  static std::mutex mu;
  static unsigned char* cached[kMaxDevices] = {};
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(mu);
  if (!cached[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_texton_scratch);
    if (e != cudaSuccess) return e;
    cached[dev] = (unsigned char*)p;
  }
  *base = cached[dev];
  return cudaSuccess;
}

__global__ void __launch_bounds__(256) k_static_setup(PatchDev P, int tiles_x, int ntiles,
                                                      unsigned char* __restrict__ scratch) {
  int4* work = (int4*)(scratch + kOffWork);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ntiles; i += gridDim.x * blockDim.x)
    work[i] = make_int4(0, (i / tiles_x) * 16, (i % tiles_x) * 16, 0);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *(PatchDev*)(scratch + kOffPatch) = P;
    *(int*)(scratch + kOffCount) = 0;
  }
}

cudaError_t launch_texton_static(const uint32_t* packed, int W, int H, uint32_t* lab4, const double* k32_ring,
                                 const int* ring_of, int n_rings, cudaStream_t s) {
  const long long N = (long long)W * H;
  const int tiles_x = (W + 15) / 16, ntiles = tiles_x * ((H + 15) / 16);
  if (N > kStaticMaxPix || ntiles > kStaticMaxTiles) return cudaErrorInvalidValue;
  unsigned char* base = nullptr;
  cudaError_t e = static_scratch(&base);
  if (e != cudaSuccess) return e;
  PatchDev P;
  P.W = W;
  P.H = H;
  P.N = (int)N;
  for (int c = 0; c < 4; c++) P.nb[c] = 0;
  P.pix = 0;
  P.vec = 0;
  const PatchDev* dP = (const PatchDev*)(base + kOffPatch);
  const int4* work = (const int4*)(base + kOffWork);
  int* count = (int*)(base + kOffCount);
  uint8_t* grey = base + kOffGrey;
  int* repair = (int*)(base + kOffRepair);
  k_static_setup<<<(ntiles + 255) / 256, 256, 0, s>>>(P, tiles_x, ntiles, base);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = launch_convert(packed, N, grey, lab4, s)) != cudaSuccess) return e;
  if ((e = launch_texton(dP, work, ntiles, grey, lab4, repair, count, (int)N, s)) != cudaSuccess) return e;
  return launch_texton_repair(dP, grey, lab4, repair, count, (int)N, k32_ring, ring_of, n_rings, s);
}

}  // namespace gpb
