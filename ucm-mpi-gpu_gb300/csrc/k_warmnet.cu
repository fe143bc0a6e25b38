// k_warmnet.cu -- a small learned correction of the warm-start block.
//
// The coarse-grid start (2 x 2 Galerkin problem, prolongated bilinearly)
// misses the fine structure of the eigenvectors along boundaries.  A
// two-layer convolutional net refines its first 9 columns (the wanted
// eigenvectors' approximations) before the fine block solve:
//
//   x~_j = X0_j * s_j            s_j = sqrt(N) / ||X0_j|| over the patch (RMS 1)
//   h_k  = relu(b1_k + sum_{c<10, t<9} W1[k][c][t] in_c(p + tap t))     k < 16
//          in_c = x~_c (c < 9) or mPb (c = 9), zero outside the patch
//   y~_j = x~_j + b2_j + sum_k W2[j][k] h_k                              j < 9
//   X_j  = y~_j / s_j
//
// Training (the project's own kernels; the optimiser runs on the host):
// per pixel the loss (y~_j - v~_j)^2 / (9 N_total) against the solver's
// converged eigenvectors v~ (sign-aligned with X0, RMS 1); k_wn_grad sums
// the loss and the gradient of every weight.  The layers are small
// (10 x 9 -> 16 -> 9 per pixel) and bound by memory, not by arithmetic, so
// they run in FP32 on the CUDA cores.
#include <stdint.h>

#include "k_block.h"
#include "k_warmnet.h"

namespace gpb {

namespace {

__device__ __forceinline__ void wn_forward(const float* __restrict__ w, const float (&in)[kWnIn][9],
                                           float (&h)[kWnHid], float (&dy)[kWnOut]) {
  const float* W1 = w;
  const float* b1 = w + kWnHid * kWnIn * 9;
  const float* W2 = b1 + kWnHid;
  const float* b2 = W2 + kWnOut * kWnHid;
#pragma unroll 1
  for (int k = 0; k < kWnHid; k++) {
    float a = b1[k];
    for (int c = 0; c < kWnIn; c++)
#pragma unroll
      for (int t = 0; t < 9; t++) a = fmaf(W1[(k * kWnIn + c) * 9 + t], in[c][t], a);
    h[k] = a > 0.f ? a : 0.f;
  }
  for (int j = 0; j < kWnOut; j++) {
    float a = b2[j];
    for (int k = 0; k < kWnHid; k++) a = fmaf(W2[j * kWnHid + k], h[k], a);
    dy[j] = a;
  }
}

}  // namespace

// per patch: s_j = sqrt(N) / ||X0_j|| for the first 9 columns of the block
__global__ void __launch_bounds__(256) k_wn_scale(const PatchDev* __restrict__ patches, const float* __restrict__ X,
                                                  float* __restrict__ scale) {
  const PatchDev P = patches[blockIdx.x];
  __shared__ float part[8][kWnOut];
  float acc[kWnOut];
  for (int j = 0; j < kWnOut; j++) acc[j] = 0.f;
  for (int p = threadIdx.x; p < P.N; p += blockDim.x) {
    const float* x = X + (P.vec + p) * kBlk;
    for (int j = 0; j < kWnOut; j++) acc[j] = fmaf(x[j], x[j], acc[j]);
  }
  for (int j = 0; j < kWnOut; j++)
    for (int d = 16; d; d >>= 1) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], d);
  if ((threadIdx.x & 31) == 0)
    for (int j = 0; j < kWnOut; j++) part[threadIdx.x >> 5][j] = acc[j];
  __syncthreads();
  if (threadIdx.x < kWnOut) {
    float s = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += part[w][threadIdx.x];
    scale[blockIdx.x * kWnOut + threadIdx.x] = s > 0.f ? sqrtf((float)P.N / s) : 0.f;
  }
}

// inference: Y gets the block X with its first 9 columns refined
__global__ void __launch_bounds__(128) k_wn_apply(const PatchDev* __restrict__ patches, int npatch,
                                                  const float* __restrict__ X, const float* __restrict__ mpb,
                                                  const float* __restrict__ w, const float* __restrict__ scale,
                                                  float* __restrict__ Y) {
  const PatchDev P = patches[blockIdx.y];
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.N) return;
  const int py = p / P.W, px = p % P.W;
  const float* s = scale + blockIdx.y * kWnOut;
  float in[kWnIn][9];
  for (int t = 0; t < 9; t++) {
    const int yy = py + t / 3 - 1, xx = px + t % 3 - 1;
    const bool ok = yy >= 0 && yy < P.H && xx >= 0 && xx < P.W;
    const int q = yy * P.W + xx;
    for (int c = 0; c < kWnOut; c++) in[c][t] = ok ? X[(P.vec + q) * kBlk + c] * s[c] : 0.f;
    in[kWnOut][t] = ok ? mpb[P.pix + q] : 0.f;
  }
  float h[kWnHid], dy[kWnOut];
  wn_forward(w, in, h, dy);
  const float* x = X + (P.vec + p) * kBlk;
  float* y = Y + (P.vec + p) * kBlk;
  for (int c = 0; c < kWnOut; c++) y[c] = s[c] > 0.f ? (in[c][4] + dy[c]) / s[c] : x[c];
  for (int c = kWnOut; c < kBlk; c++) y[c] = x[c];
}

// training: loss and gradient sums over a set of patches given as
// normalised inputs x~ [Ntot][9], mPb [Ntot] and targets v~ [Ntot][9]
__global__ void __launch_bounds__(128) k_wn_grad(const int4* __restrict__ geo, int npatch,
                                                 const float* __restrict__ xt, const float* __restrict__ mpb,
                                                 const float* __restrict__ vt, const float* __restrict__ w, float inv_n,
                                                 float* __restrict__ grad, double* __restrict__ loss) {
  __shared__ float g[kWnParams];
  for (int i = threadIdx.x; i < kWnParams; i += blockDim.x) g[i] = 0.f;
  __syncthreads();
  const int4 G = geo[blockIdx.y];  // W, H, first pixel, 0
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int N = G.x * G.y;
  float lsum = 0.f;
  const bool live = p < N;
  float in[kWnIn][9], h[kWnHid], dy[kWnOut], gy[kWnOut];
  if (live) {
    const int py = p / G.x, px = p % G.x;
    for (int t = 0; t < 9; t++) {
      const int yy = py + t / 3 - 1, xx = px + t % 3 - 1;
      const bool ok = yy >= 0 && yy < G.y && xx >= 0 && xx < G.x;
      const long long q = (long long)G.z + yy * G.x + xx;
      for (int c = 0; c < kWnOut; c++) in[c][t] = ok ? xt[q * kWnOut + c] : 0.f;
      in[kWnOut][t] = ok ? mpb[q] : 0.f;
    }
    wn_forward(w, in, h, dy);
    const long long q0 = (long long)G.z + p;
    for (int j = 0; j < kWnOut; j++) {
      const float r = in[j][4] + dy[j] - vt[q0 * kWnOut + j];
      lsum += r * r * inv_n;
      gy[j] = 2.f * r * inv_n;
    }
  } else {
    for (int j = 0; j < kWnOut; j++) gy[j] = 0.f;
    for (int k = 0; k < kWnHid; k++) h[k] = 0.f;
    for (int c = 0; c < kWnIn; c++)
      for (int t = 0; t < 9; t++) in[c][t] = 0.f;
  }
  const float* W2 = w + kWnHid * kWnIn * 9 + kWnHid;
  float* gW1 = g;
  float* gb1 = g + kWnHid * kWnIn * 9;
  float* gW2 = gb1 + kWnHid;
  float* gb2 = gW2 + kWnOut * kWnHid;
  const int lane = threadIdx.x & 31;
  auto add = [&](float* dst, float v) {  // warp sum, then one shared-memory add
    for (int d = 16; d; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    if (lane == 0) atomicAdd(dst, v);
  };
  for (int j = 0; j < kWnOut; j++) {
    add(gb2 + j, gy[j]);
    for (int k = 0; k < kWnHid; k++) add(gW2 + j * kWnHid + k, gy[j] * h[k]);
  }
  for (int k = 0; k < kWnHid; k++) {
    float dh = 0.f;
    for (int j = 0; j < kWnOut; j++) dh = fmaf(W2[j * kWnHid + k], gy[j], dh);
    if (h[k] <= 0.f) dh = 0.f;
    add(gb1 + k, dh);
    for (int c = 0; c < kWnIn; c++)
      for (int t = 0; t < 9; t++) add(gW1 + (k * kWnIn + c) * 9 + t, dh * in[c][t]);
  }
  for (int d = 16; d; d >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, d);
  if (lane == 0) atomicAdd(loss, (double)lsum);
  __syncthreads();
  for (int i = threadIdx.x; i < kWnParams; i += blockDim.x)
    if (g[i] != 0.f) atomicAdd(grad + i, g[i]);
}

cudaError_t wn_launch_apply(const PatchDev* patches, int npatch, int max_n, const float* X, const float* mpb,
                            const float* w, float* scale, float* Y, cudaStream_t s) {
  if (npatch <= 0) return cudaSuccess;
  k_wn_scale<<<npatch, 256, 0, s>>>(patches, X, scale);
  k_wn_apply<<<dim3((max_n + 127) / 128, npatch), 128, 0, s>>>(patches, npatch, X, mpb, w, scale, Y);
  return cudaGetLastError();
}

cudaError_t wn_launch_grad(const int4* geo, int npatch, int max_n, const float* xt, const float* mpb, const float* vt,
                           const float* w, float inv_n, float* grad, double* loss, cudaStream_t s) {
  if (npatch <= 0) return cudaSuccess;
  k_wn_grad<<<dim3((max_n + 127) / 128, npatch), 128, 0, s>>>(geo, npatch, xt, mpb, vt, w, inv_n, grad, loss);
  return cudaGetLastError();
}

}  // namespace gpb
