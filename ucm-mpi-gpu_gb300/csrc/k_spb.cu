// k_spb.cu -- spectral Pb, gPb combination and output layouts (sm_103a).
//
// Reference: src/spectralPb.cpp:269-322 (generalised eigenvectors v = D^-1/2 y
// of eigenvalues 1..nvec-1, min-max normalised, divided by sqrt(lambda),
// 8 oriented derivative-of-Gaussian filters, |.| summed into slot
// ch_per[o]), src/globalPb.cpp:97-103 and 231-235 (gPb_o = weighted cues +
// w12 sPb_o, nmax = max_o |gPb_o|), and for the Damascene layout
// damascene/src/globalPb/globalPb.cu:5-49, postprocess/skeleton.cu:229-256
// and damascene.cu:576-603 (mask mPb > 0.05, sigmoid, oriMap, column-major).
//
// One CTA owns a 16x16 output tile: each eigenvector is staged with a
// 3-pixel BORDER_REFLECT_101 halo in shared memory, all 8 orientations are
// filtered from it, and the gPb epilogue runs on the accumulated registers,
// so sPb never goes to global memory.
#include <float.h>
#include <stdint.h>

#include "gpb_internal.h"
#include "kernels.h"

namespace gpb {

__constant__ float c_oe[kNori][49];
__constant__ int c_chper[kNori];
__constant__ float c_wspb;

void upload_spb(const HostTables& t, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c_oe, t.oe, sizeof(t.oe), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_chper, t.ch_per, sizeof(t.ch_per), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_wspb, &t.w_spb, sizeof(float), 0, cudaMemcpyHostToDevice, s);
}

__device__ __forceinline__ int refl101(int i, int n) {
  for (int it = 0; it < 4 && (i < 0 || i >= n); it++) i = (i < 0) ? -i : 2 * n - 2 - i;
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

// min and max of v_i = y_i * D^-1/2 per patch and eigenvector
__global__ void __launch_bounds__(1024) k_minmax(const PatchDev* __restrict__ patches,
                                                 const float* __restrict__ evecs, long long lvec,
                                                 const float* __restrict__ dis, int nvec,
                                                 float* __restrict__ mm) {
  const int pt = blockIdx.x, i = blockIdx.y;
  const PatchDev P = patches[pt];
  float mn = FLT_MAX, mx = -FLT_MAX;
  for (int p = threadIdx.x; p < P.N; p += blockDim.x) {
    const float v = evecs[(long long)i * lvec + P.vec + p] * dis[P.vec + p];
    mn = fminf(mn, v);
    mx = fmaxf(mx, v);
  }
  __shared__ float smn[32], smx[32];
  for (int o = 16; o > 0; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if ((threadIdx.x & 31) == 0) {
    smn[threadIdx.x >> 5] = mn;
    smx[threadIdx.x >> 5] = mx;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int nw = blockDim.x >> 5;
    mn = threadIdx.x < nw ? smn[threadIdx.x] : FLT_MAX;
    mx = threadIdx.x < nw ? smx[threadIdx.x] : -FLT_MAX;
    for (int o = 16; o > 0; o >>= 1) {
      mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (threadIdx.x == 0) {
      mm[((long long)pt * nvec + i) * 2 + 0] = mn;
      mm[((long long)pt * nvec + i) * 2 + 1] = mx;
    }
  }
}

constexpr int SP_T = 16, SP_H = 3, SP_W = SP_T + 2 * SP_H;

__global__ void __launch_bounds__(256) k_spb(const PatchDev* __restrict__ patches, const int4* __restrict__ work,
                                             const float* __restrict__ evecs, long long lvec,
                                             const float* __restrict__ dis, const float* __restrict__ evals,
                                             const float* __restrict__ mm, int nvec,
                                             const float* __restrict__ go, const float* __restrict__ mpb,
                                             int compat, float* __restrict__ spb_out,
                                             float* __restrict__ gpbo_out, float* __restrict__ out_nmax,
                                             float* __restrict__ out_orient) {
  __shared__ float tile[SP_W * SP_W];
  const int4 w = work[blockIdx.x];
  const PatchDev P = patches[w.x];
  const int ty = threadIdx.x / SP_T, tx = threadIdx.x % SP_T;
  const int y = w.y + ty, x = w.z + tx;
  float acc[kNori];
#pragma unroll
  for (int o = 0; o < kNori; o++) acc[o] = 0.f;
  for (int i = 1; i < nvec; i++) {
    const float lam = evals[(long long)w.x * nvec + i];
    if (!(lam > 2.220446049250313e-16f)) continue;  // DBL_EPSILON test of spectralPb.cpp:293
    const float mn = mm[((long long)w.x * nvec + i) * 2], mx = mm[((long long)w.x * nvec + i) * 2 + 1];
    const float sc = 1.0f / ((mx - mn) * sqrtf(lam));
    __syncthreads();
    for (int idx = threadIdx.x; idx < SP_W * SP_W; idx += blockDim.x) {
      const int yy = refl101(w.y - SP_H + idx / SP_W, P.H), xx = refl101(w.z - SP_H + idx % SP_W, P.W);
      const long long q = P.vec + (long long)yy * P.W + xx;
      tile[idx] = (evecs[(long long)i * lvec + q] * dis[q] - mn) * sc;
    }
    __syncthreads();
    if (y < P.H && x < P.W) {
      const float* c = tile + ty * SP_W + tx;
#pragma unroll
      for (int o = 0; o < kNori; o++) {
        float r = 0.f;
#pragma unroll
        for (int aa = 0; aa < 7; aa++)
#pragma unroll
          for (int b = 0; b < 7; b++) r = fmaf(c_oe[o][aa * 7 + b], c[aa * SP_W + b], r);
        acc[c_chper[o]] += fabsf(r);
      }
    }
  }
  if (y >= P.H || x >= P.W) return;
  const long long p = (long long)y * P.W + x;
  const float ws = c_wspb;
  float g[kNori];
#pragma unroll
  for (int o = 0; o < kNori; o++) {
    g[o] = go[P.pix * 8 + (long long)o * P.N + p] + ws * acc[o];
    if (spb_out) spb_out[P.pix * 8 + (long long)o * P.N + p] = acc[o];
    if (gpbo_out) gpbo_out[P.pix * 8 + (long long)o * P.N + p] = g[o];
  }
  if (compat == 0) {
    float m = 0.f;
#pragma unroll
    for (int o = 0; o < kNori; o++) {
      m = fmaxf(m, fabsf(g[o]));
      out_orient[P.pix * 8 + (long long)o * P.N + p] = g[o];
    }
    out_nmax[P.pix + p] = m;
  } else {
    float m = -200.f;
#pragma unroll
    for (int o = 0; o < kNori; o++) m = fmaxf(m, g[o]);
    out_nmax[P.pix + p] = mpb[P.pix + p] > 0.05f ? m : 0.f;
    const int ori_map[8] = {4, 5, 6, 7, 0, 1, 2, 3};
#pragma unroll
    for (int i = 0; i < kNori; i++) {
      float v = g[ori_map[i]];
      v = (v * 1.2f > 1.f) ? 1.f : v * 1.2f;
      if (v < 0.f) v = 0.f;
      v = 1.0f / (1.0f + expf(2.6433f - 10.7998f * v));
      v = (v - 0.0667f) / 0.9333f;
      out_orient[P.pix * 8 + (long long)i * P.N + (long long)x * P.H + y] = v;
    }
  }
}

cudaError_t launch_minmax(const PatchDev* patches, int npatch, const float* evecs, long long lvec,
                          const float* dis, int nvec, float* mm, cudaStream_t s) {
  dim3 g(npatch, nvec);
  k_minmax<<<g, 1024, 0, s>>>(patches, evecs, lvec, dis, nvec, mm);
  return cudaGetLastError();
}

cudaError_t launch_spb(const PatchDev* patches, const int4* work, int nwork, const float* evecs,
                       long long lvec, const float* dis, const float* evals, const float* mm, int nvec,
                       const float* go, const float* mpb, int compat, float* spb_out, float* gpbo_out,
                       float* out_nmax, float* out_orient, cudaStream_t s) {
  if (nwork == 0) return cudaSuccess;
  k_spb<<<nwork, 256, 0, s>>>(patches, work, evecs, lvec, dis, evals, mm, nvec, go, mpb, compat, spb_out,
                              gpbo_out, out_nmax, out_orient);
  return cudaGetLastError();
}

}  // namespace gpb
