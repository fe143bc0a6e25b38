// k_stitch.cu -- whole-image gPb planes from the last batch's halo'd patches,
// on the device (replaces Pieces2Gpb, src/utilities.cpp:180-213, which
// copies every part's full box into the image in loop order so that later
// parts overwrite the overlaps).
//
//   k_stitch_copy   a sub-box of one patch into the image (LAST: the whole
//                   box, launched patch after patch on one stream, so the
//                   later patch wins as in the reference; INTERIOR: only the
//                   patch's own interior, so no pixel has two writers)
//   k_stitch_acc    BLEND: weight * value and weight accumulated per image
//                   pixel (atomics; weights fall linearly over the overlap)
//   k_stitch_norm   BLEND: value = sum / weight
//
// Patch values are read in the context's compat layout (orient planes
// row-major for GPB_COMPAT_CPU, column-major for GPB_COMPAT_DAMASCENE); the
// image planes are row-major, in the patch output's plane order.
#include <stdint.h>

#include "gpb_internal.h"
#include "kernels.h"

namespace gpb {

__device__ __forceinline__ float patch_orient(const float* orient, const PatchDev& P, int colmajor, int o, int y,
                                              int x) {
  const long long base = 8 * P.pix + (long long)o * P.N;
  return orient[base + (colmajor ? (long long)x * P.H + y : (long long)y * P.W + x)];
}

__global__ void __launch_bounds__(256) k_stitch_copy(const PatchDev* __restrict__ patches, int pi,
                                                     const float* __restrict__ nmax, const float* __restrict__ orient,
                                                     int colmajor, StitchBox bx, int img_w, int img_h,
                                                     float* __restrict__ out_nmax, float* __restrict__ out_orient) {
  const PatchDev P = patches[pi];
  const long long plane = (long long)img_w * img_h;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < (long long)bx.w * bx.h;
       i += (long long)gridDim.x * blockDim.x) {
    const int y = bx.y + (int)(i / bx.w), x = bx.x + (int)(i % bx.w);  // patch coordinates
    const int gy = bx.oy + y, gx = bx.ox + x;                           // image coordinates
    if (gy < 0 || gy >= img_h || gx < 0 || gx >= img_w) continue;
    const long long g = (long long)gy * img_w + gx;
    out_nmax[g] = nmax[P.pix + (long long)y * P.W + x];
#pragma unroll
    for (int o = 0; o < 8; o++) out_orient[o * plane + g] = patch_orient(orient, P, colmajor, o, y, x);
  }
}

// weight of patch pixel (y, x): 1 in the interior, falling linearly to
// 1 / (2 ramp) at a patch edge that lies inside the image
__device__ __forceinline__ float stitch_weight(const StitchBox& b, const PatchDev& P, int y, int x, int img_w,
                                               int img_h, float ramp) {
  float w = 1.f;
  if (b.oy > 0) w = fminf(w, (y + 0.5f) / ramp);
  if (b.ox > 0) w = fminf(w, (x + 0.5f) / ramp);
  if (b.oy + P.H < img_h) w = fminf(w, (P.H - y - 0.5f) / ramp);
  if (b.ox + P.W < img_w) w = fminf(w, (P.W - x - 0.5f) / ramp);
  return w;
}

__global__ void __launch_bounds__(256) k_stitch_acc(const PatchDev* __restrict__ patches, int pi,
                                                    const float* __restrict__ nmax, const float* __restrict__ orient,
                                                    int colmajor, StitchBox bx, int img_w, int img_h, float ramp,
                                                    float* __restrict__ acc /* [10][img] */) {
  const PatchDev P = patches[pi];
  const long long plane = (long long)img_w * img_h;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < (long long)P.N;
       i += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(i / P.W), x = (int)(i % P.W);
    const int gy = bx.oy + y, gx = bx.ox + x;
    if (gy < 0 || gy >= img_h || gx < 0 || gx >= img_w) continue;
    const long long g = (long long)gy * img_w + gx;
    const float w = stitch_weight(bx, P, y, x, img_w, img_h, ramp);
    atomicAdd(acc + g, w);
    atomicAdd(acc + plane + g, w * nmax[P.pix + i]);
#pragma unroll
    for (int o = 0; o < 8; o++) atomicAdd(acc + (2 + o) * plane + g, w * patch_orient(orient, P, colmajor, o, y, x));
  }
}

__global__ void __launch_bounds__(256) k_stitch_norm(const float* __restrict__ acc, long long plane,
                                                     float* __restrict__ out_nmax, float* __restrict__ out_orient) {
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < plane; g += (long long)gridDim.x * blockDim.x) {
    const float w = acc[g];
    if (!(w > 0.f)) continue;  // no patch covers it: left as it was
    const float r = 1.f / w;
    out_nmax[g] = acc[plane + g] * r;
#pragma unroll
    for (int o = 0; o < 8; o++) out_orient[o * plane + g] = acc[(2 + o) * plane + g] * r;
  }
}

static int grid_for(long long n) {
  long long g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g));
}

cudaError_t launch_stitch_copy(const PatchDev* patches, int pi, const float* nmax, const float* orient, int colmajor,
                               const StitchBox& bx, int img_w, int img_h, float* out_nmax, float* out_orient,
                               cudaStream_t s) {
  k_stitch_copy<<<grid_for((long long)bx.w * bx.h), 256, 0, s>>>(patches, pi, nmax, orient, colmajor, bx, img_w,
                                                                 img_h, out_nmax, out_orient);
  return cudaGetLastError();
}
cudaError_t launch_stitch_acc(const PatchDev* patches, int pi, long long npix, const float* nmax, const float* orient,
                              int colmajor, const StitchBox& bx, int img_w, int img_h, float ramp, float* acc,
                              cudaStream_t s) {
  k_stitch_acc<<<grid_for(npix), 256, 0, s>>>(patches, pi, nmax, orient, colmajor, bx, img_w, img_h, ramp, acc);
  return cudaGetLastError();
}
cudaError_t launch_stitch_norm(const float* acc, long long plane, float* out_nmax, float* out_orient, cudaStream_t s) {
  k_stitch_norm<<<grid_for(plane), 256, 0, s>>>(acc, plane, out_nmax, out_orient);
  return cudaGetLastError();
}

}  // namespace gpb
