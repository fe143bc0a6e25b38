// k_buildw.cu -- intervening-contour affinities and the normalised Laplacian
// in symmetric stencil (DIA) form (sm_103a).
//
// Reference: Group::computeSupport / ic_walk / interveningContour
// (buildW/src/ic.cc:42-545), Group::computeAffinities2 and C_IC_SS
// (buildW/src/affinity.cc:40-156), SMatrix::symmetrize (smatrix.cc:95-117),
// driven by src/buildW.cpp:23-246; normalisation as in
// damascene/src/stencilMatrixMultiply/stencilMVM.cu:48-127.
//
// The reference walks Bresenham lines from every pixel to the border of its
// (clipped) 11x11 box.  Which mPb pixels a walk max-accumulates before it
// records each stencil offset depends only on how the box is clipped, so the
// host runs the reference walk once per clipping configuration on a symbolic
// lattice (tables.cpp) and the kernel evaluates a table-driven max over an
// mPb tile in shared memory.
//
// Storage: A = I - D^-1/2 W D^-1/2 keeps its diagonal and the 40 strictly
// upper stencil offsets, diagonal-major and in the padded vector layout, so
// the SpMV reads each coefficient once and the lower triangle as the same
// array shifted by the offset.
#include <stdint.h>

#include "gpb_internal.h"
#include "kernels.h"

namespace gpb {

__constant__ int c_sdy[kStencilN], c_sdx[kStencilN];

void upload_buildw(const HostTables& t, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c_sdy, t.sdy, sizeof(t.sdy), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_sdx, t.sdx, sizeof(t.sdx), 0, cudaMemcpyHostToDevice, s);
}

constexpr int BW_T = 16, BW_HALO = 2 * kStencilR, BW_W = BW_T + 2 * BW_HALO;

__device__ __forceinline__ int ic_config(int x, int y, int W, int H) {
  const int cl = min(x, kStencilR), cr = min(W - 1 - x, kStencilR);
  const int ct = min(y, kStencilR), cb = min(H - 1 - y, kStencilR);
  return ((cl * 6 + cr) * 6 + ct) * 6 + cb;
}

// affinity of one directed pair: W = exp(-(1 - C_IC_SS(1 - sim))/0.1) with
// sim = 1 - maxpb (affinity.cc:118-143; the reference rounds 1 - (1 - m))
__device__ __forceinline__ float directed_w(const IcPath& e, const float* tc) {
  float sim = 0.f;
  if (e.count >= 0) {
    float mp = 0.f;
    for (int i = 0; i < e.count; i++) mp = fmaxf(mp, tc[e.dy[i] * BW_W + e.dx[i]]);
    sim = 1.0f - mp;
  }
  const float ic = 1.0f - sim;
  const float val = 1.8682f + (ic / 0.3130f) * -1.3113f;
  const float post = 1.0f / (1.0f + expf(-val));
  return expf(-(1.0f - post) / 0.1f);
}

__global__ void __launch_bounds__(256) k_buildw(const PatchDev* __restrict__ patches,
                                                const int4* __restrict__ work, const float* __restrict__ mpb,
                                                const IcPath* __restrict__ ic, float* __restrict__ wsym_up,
                                                long long lvec) {
  __shared__ float tile[BW_W * BW_W];
  const int4 w = work[blockIdx.x];
  const PatchDev P = patches[w.x];
  for (int i = threadIdx.x; i < BW_W * BW_W; i += blockDim.x) {
    const int yy = w.y - BW_HALO + i / BW_W, xx = w.z - BW_HALO + i % BW_W;
    float v = 0.f;
    if (yy >= 0 && yy < P.H && xx >= 0 && xx < P.W) v = mpb[P.pix + (long long)yy * P.W + xx];
    tile[i] = v;
  }
  __syncthreads();
  const int ty = threadIdx.x / BW_T, tx = threadIdx.x % BW_T;
  const int y = w.y + ty, x = w.z + tx;
  if (y >= P.H || x >= P.W) return;
  const long long p = (long long)y * P.W + x;
  const int cfg_p = ic_config(x, y, P.W, P.H);
  const float* tp = tile + (ty + BW_HALO) * BW_W + (tx + BW_HALO);
  for (int k = kStencilN / 2 + 1; k < kStencilN; k++) {
    const int yy = y + c_sdy[k], xx = x + c_sdx[k];
    float ws = 0.f;
    if (yy >= 0 && yy < P.H && xx >= 0 && xx < P.W) {
      const float w1 = directed_w(ic[(size_t)cfg_p * kStencilN + k], tp);
      const int cfg_q = ic_config(xx, yy, P.W, P.H);
      const float* tq = tp + c_sdy[k] * BW_W + c_sdx[k];
      const float w2 = directed_w(ic[(size_t)cfg_q * kStencilN + (kStencilN - 1 - k)], tq);
      ws = 0.5f * (w1 + w2);
    }
    wsym_up[(long long)(k - kStencilN / 2 - 1) * lvec + P.vec + p] = ws;
  }
}

// degree d_p = sum of the 81 symmetric affinities (diagonal 1), D^-1/2.
// The sum is a float-float pair built by Fast2Sum (Dekker 1971; exact since
// the running sum, at least the diagonal 1, is never below a term in [0, 1]),
// so it holds the 81-term sum to about 2^-44 relative -- as close as an FP64
// accumulation at GB300's low FP64 rate would, on the FP32 pipes.  The
// unrolled offset loop issues the plane loads independently.
__global__ void __launch_bounds__(256) k_degree(const PatchDev* __restrict__ patches,
                                                const int4* __restrict__ work,
                                                const float* __restrict__ wsym_up, float* __restrict__ deg,
                                                float* __restrict__ dis, float* __restrict__ a_diag,
                                                long long lvec, float* __restrict__ wfull) {
  const int4 w = work[blockIdx.x];
  const PatchDev P = patches[w.x];
  const int y = w.y + threadIdx.x / 16, x = w.z + threadIdx.x % 16;
  if (y >= P.H || x >= P.W) return;
  const long long p = (long long)y * P.W + x;
  const float* wp = wsym_up + P.vec + p;
  float hi = 1.f, lo = 0.f;
#pragma unroll 8
  for (int j = 0; j < kUpper; j++) {
    const int k = kStencilN / 2 + 1 + j;
    const int off = c_sdy[k] * P.W + c_sdx[k];
    const float up = wp[(long long)j * lvec];
    const float lw = wp[(long long)j * lvec - off];  // zero in the pad
    // the lower entry is valid only if the neighbour lies inside the patch
    const int yy = y - c_sdy[k], xx = x - c_sdx[k];
    const float lov = (yy >= 0 && yy < P.H && xx >= 0 && xx < P.W) ? lw : 0.f;
    float sum = __fadd_rn(hi, up);
    lo = __fadd_rn(lo, __fsub_rn(up, __fsub_rn(sum, hi)));
    hi = sum;
    sum = __fadd_rn(hi, lov);
    lo = __fadd_rn(lo, __fsub_rn(lov, __fsub_rn(sum, hi)));
    hi = sum;
    if (wfull) {
      wfull[(P.pix + p) * kStencilN + k] = up;
      wfull[(P.pix + p) * kStencilN + (kStencilN - 1 - k)] = lov;
    }
  }
  if (wfull) wfull[(P.pix + p) * kStencilN + kStencilN / 2] = 1.f;
  const double d = (double)hi + (double)lo;
  deg[P.vec + p] = (float)d;
  dis[P.vec + p] = (float)(1.0 / sqrt(d));
  a_diag[P.vec + p] = (float)((d - 1.0) / d);
}

// A = I - D^-1/2 W D^-1/2 off the diagonal: a_up = -w dis_p dis_q
__global__ void __launch_bounds__(256) k_scale(const PatchDev* __restrict__ patches,
                                               const int4* __restrict__ work, const float* __restrict__ wsym_up,
                                               const float* __restrict__ dis, float* __restrict__ a_up,
                                               long long lvec) {
  const int4 w = work[blockIdx.x];
  const PatchDev P = patches[w.x];
  const int y = w.y + threadIdx.x / 16, x = w.z + threadIdx.x % 16;
  if (y >= P.H || x >= P.W) return;
  const long long p = (long long)y * P.W + x;
  const float sp = dis[P.vec + p];
  for (int j = 0; j < kUpper; j++) {
    const int k = kStencilN / 2 + 1 + j;
    const int yy = y + c_sdy[k], xx = x + c_sdx[k];
    float a = 0.f;
    if (yy >= 0 && yy < P.H && xx >= 0 && xx < P.W)
      a = -wsym_up[(long long)j * lvec + P.vec + p] * (sp * dis[P.vec + (long long)yy * P.W + xx]);
    a_up[(long long)j * lvec + P.vec + p] = a;
  }
}

cudaError_t launch_buildw(const PatchDev* patches, const int4* work, int nwork, const float* mpb,
                          const IcPath* ic, float* wsym_up, float* deg, long long lvec, cudaStream_t s) {
  (void)deg;
  if (nwork == 0) return cudaSuccess;
  k_buildw<<<nwork, 256, 0, s>>>(patches, work, mpb, ic, wsym_up, lvec);
  return cudaGetLastError();
}

cudaError_t launch_scale(const PatchDev* patches, const int4* work, int nwork, const float* wsym_up,
                         const float* deg, float* a_up, float* a_diag, float* dis, long long lvec,
                         float* wfull, cudaStream_t s) {
  if (nwork == 0) return cudaSuccess;
  k_degree<<<nwork, 256, 0, s>>>(patches, work, wsym_up, (float*)deg, dis, a_diag, lvec, wfull);
  k_scale<<<nwork, 256, 0, s>>>(patches, work, wsym_up, dis, a_up, lvec);
  return cudaGetLastError();
}

}  // namespace gpb
