// k_spfeat.cu -- per-superpixel descriptors for GLSVM from the pipeline's
// own texton map, grey image and input colours (SPFeatures::genTextonFeatures
// pooling, genIntensityHistograms and genAverageFeatures,
// src/SPFeatures.cpp:260-275, 101-114, 380-391).
//
//   k_sp_accum  one thread per pixel: integer counts per (superpixel, texton),
//               (superpixel, grey bin) and size, 64-bit colour sums (global
//               atomics; labels outside [0, n) are skipped)
//   k_sp_final  one thread per (superpixel, column): counts / size * 10,
//               colour sums / size * (10 / 255), in FP64 in the reference's
//               order of operations; a zero column for the Harris corner
//               descriptor (genCornerDescrs) keeps the reference's layout
#include <stdint.h>

#include "gpb_internal.h"
#include "kernels.h"

namespace gpb {

__global__ void __launch_bounds__(256) k_sp_accum(const PatchDev* __restrict__ patches, int pi,
                                                  const int32_t* __restrict__ labels, int n,
                                                  const uint32_t* __restrict__ lab4, const uint8_t* __restrict__ grey,
                                                  const uint32_t* __restrict__ packed, int bin_step, int K, int nbins,
                                                  uint32_t* __restrict__ counts, unsigned long long* __restrict__ csum) {
  const PatchDev P = patches[pi];
  const int ncnt = K + nbins + 1;  // textons, grey bins, size
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < P.N; i += (long long)gridDim.x * blockDim.x) {
    const int l = labels[i];
    if (l < 0 || l >= n) continue;
    uint32_t* row = counts + (long long)l * ncnt;
    const int t = (int)(lab4[P.pix + i] >> 24);
    if (K > 0 && t < K) atomicAdd(row + t, 1u);
    atomicAdd(row + K + grey[P.pix + i] / bin_step, 1u);
    atomicAdd(row + K + nbins, 1u);
    const uint32_t px = packed[P.pix + i];
    atomicAdd(csum + 3LL * l + 0, (unsigned long long)((px >> 16) & 255));  // B
    atomicAdd(csum + 3LL * l + 1, (unsigned long long)((px >> 8) & 255));   // G
    atomicAdd(csum + 3LL * l + 2, (unsigned long long)(px & 255));          // R
  }
}

__global__ void __launch_bounds__(256) k_sp_final(int n, int K, int nbins, const uint32_t* __restrict__ counts,
                                                  const unsigned long long* __restrict__ csum, double* __restrict__ out) {
  const int ncnt = K + nbins + 1, ncol = K + nbins + 1 + 3;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < (long long)n * ncol;
       e += (long long)gridDim.x * blockDim.x) {
    const int l = (int)(e / ncol), c = (int)(e % ncol);
    const double size = (double)counts[(long long)l * ncnt + K + nbins];
    double v = 0.0;
    if (size > 0) {
      if (c < K + nbins) {
        v = (double)counts[(long long)l * ncnt + c] / size;
        v = v * 10.0;
      } else if (c > K + nbins) {
        v = (double)csum[3LL * l + (c - K - nbins - 1)] / size;
        v = v * (10.0 / 255.0);
      }
    }
    out[e] = v;
  }
}

cudaError_t launch_sp_features(const PatchDev* patches, int pi, long long npix, const int32_t* labels, int n,
                               const uint32_t* lab4, const uint8_t* grey, const uint32_t* packed, int bin_step,
                               int K, int nbins, uint32_t* counts, unsigned long long* csum, double* out,
                               cudaStream_t s) {
  const int ncnt = K + nbins + 1;
  cudaError_t e = cudaMemsetAsync(counts, 0, (size_t)n * ncnt * sizeof(uint32_t), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(csum, 0, (size_t)n * 3 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  const long long g1 = (npix + 255) / 256;
  k_sp_accum<<<(int)(g1 < 1 ? 1 : (g1 > 4096 ? 4096 : g1)), 256, 0, s>>>(patches, pi, labels, n, lab4, grey, packed,
                                                                          bin_step, K, nbins, counts, csum);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const long long g2 = ((long long)n * (ncnt + 3) + 255) / 256;
  k_sp_final<<<(int)(g2 < 1 ? 1 : (g2 > 4096 ? 4096 : g2)), 256, 0, s>>>(n, K, nbins, counts, csum, out);
  return cudaGetLastError();
}

}  // namespace gpb
