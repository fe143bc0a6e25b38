// k_block.cu -- block kernels of the Chebyshev-filtered subspace iteration
// (the warm-started eigensolver) for A = I - D^-1/2 W D^-1/2 (sm_103a).
//
// A block of kBlk = 32 vectors is stored pixel-major ([vec][32] floats) in the
// padded vector layout, so every stencil neighbour of a pixel is one
// contiguous 128-byte row.  Four threads own a pixel, eight columns each
// (two float4), so a warp reads whole rows and the stencil coefficient is
// loaded once per thread.
//
//   cf_step    Y' = alpha (A Y) + beta Y + gamma X   (scaled Chebyshev
//              recurrence, Zhou & Saad 2007; with alpha=1, beta=gamma=0 it
//              is the plain block SpMV)
//   cf_gram    G = U^T V per patch (32 x 32), compensated FP32 products,
//              FP64 cross-CTA sums by the last CTA of the patch
//   cf_rotate  U <- U M (32 x 32 per patch), optionally V <- V M too
//   cf_resid   |A x_c - theta_c x_c|^2 per column
//   cf_extract the first nvec columns into separate vectors (sPb layout)
//
// Reference: the eigensolver of damascene/src/noReorthog/lanczos.cu and
// src/spectralPb.cpp:221-245 define the problem; the block method is this
// project's own.
#include <stdint.h>

#include "gpb_internal.h"
#include "k_block.h"
#include "k_eig.h"

namespace gpb {

__constant__ int c_bup_dy[kUpper], c_bup_dx[kUpper];

void upload_block(const HostTables& t, cudaStream_t s) {
  int dy[kUpper], dx[kUpper];
  for (int j = 0; j < kUpper; j++) {
    dy[j] = t.sdy[kStencilN / 2 + 1 + j];
    dx[j] = t.sdx[kStencilN / 2 + 1 + j];
  }
  cudaMemcpyToSymbolAsync(c_bup_dy, dy, sizeof(dy), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_bup_dx, dx, sizeof(dx), 0, cudaMemcpyHostToDevice, s);
}

constexpr unsigned FULLB = 0xffffffffu;

__device__ __forceinline__ void fma4(float4& acc, float a, const float4& x) {
  acc.x = fmaf(a, x.x, acc.x);
  acc.y = fmaf(a, x.y, acc.y);
  acc.z = fmaf(a, x.z, acc.z);
  acc.w = fmaf(a, x.w, acc.w);
}

// ------------------------------------------------------------ Chebyshev step
// One CTA owns an 8 x 32 pixel tile; the 32-wide rows of Y for the tile and a
// 5-pixel halo are staged transposed in shared memory (column-major planes,
// odd plane stride, so a warp reading 32 neighbouring pixels of one column
// hits 32 banks).  Lane = pixel, warp = tile row: each lane keeps its pixel's
// 32 outputs in registers, loads each stencil coefficient once (coalesced
// across the warp) and streams the neighbour's 32 values from shared memory.
constexpr int ST_H = 8, ST_W = 32, ST_R = kStencilR;
constexpr int ST_PH = ST_H + 2 * ST_R, ST_PW = ST_W + 2 * ST_R;
constexpr int ST_PLANE = ST_PH * ST_PW + 1;  // 757: odd, conflict-free transposes
constexpr size_t kStepSmem = (size_t)kBlk * ST_PLANE * sizeof(float);

__global__ void __launch_bounds__(ST_H * 32, 2) cf_step(BlkArgs a, const int4* __restrict__ work,
                                                     const float* __restrict__ Y, const float* __restrict__ X,
                                                     float* __restrict__ out, int step) {
  extern __shared__ float yt[];  // [32][ST_PLANE]
  const int4 w = work[blockIdx.x];  // (patch, y0, x0, -)
  if (!a.active[w.x]) return;
  const PatchDev P = a.patches[w.x];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // stage rows (y0-5 .. y0+12, x0-5 .. x0+36): each tile row is one
  // contiguous run of 42 x 128 bytes; threads fetch float4s, eight in flight
  // per thread, and scatter them into the transposed planes
  {
    constexpr int F4_PER_ROW = kBlk / 4;                 // 8 float4 per pixel
    constexpr int F4_PER_TROW = ST_PW * F4_PER_ROW;      // 336 per tile row
    constexpr int TOTAL = ST_PH * F4_PER_TROW;           // 6048
    constexpr int PER_THREAD = (TOTAL + ST_H * 32 - 1) / (ST_H * 32);
    float4 v[PER_THREAD];
#pragma unroll
    for (int i = 0; i < PER_THREAD; i++) {
      const int f = threadIdx.x + i * ST_H * 32;
      const int ty = f / F4_PER_TROW, rem = f % F4_PER_TROW;
      // rows below the patch's last row + radius feed no in-patch pixel
      v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (f < TOTAL && w.y - ST_R + ty < P.H + ST_R) {
        const long long q0 = P.vec + (long long)(w.y - ST_R + ty) * P.W + (w.z - ST_R);
        v[i] = ((const float4*)(Y + q0 * kBlk))[rem];
      }
    }
#pragma unroll
    for (int i = 0; i < PER_THREAD; i++) {
      const int f = threadIdx.x + i * ST_H * 32;
      if (f < TOTAL) {
        const int ty = f / F4_PER_TROW, rem = f % F4_PER_TROW;
        const int tx = rem / F4_PER_ROW, c = (rem % F4_PER_ROW) * 4;
        const int r = ty * ST_PW + tx;
        yt[(c + 0) * ST_PLANE + r] = v[i].x;
        yt[(c + 1) * ST_PLANE + r] = v[i].y;
        yt[(c + 2) * ST_PLANE + r] = v[i].z;
        yt[(c + 3) * ST_PLANE + r] = v[i].w;
      }
    }
  }
  __syncthreads();
  const int y = w.y + warp, x = w.z + lane;
  if (y >= P.H || x >= P.W) return;
  const long long q = P.vec + (long long)y * P.W + x;
  const float3 co = a.coef[(long long)w.x * a.max_steps + step];
  float acc[kBlk];
  const int ctr = (warp + ST_R) * ST_PW + (lane + ST_R);
  {
    const float d = a.a_diag[q];
#pragma unroll
    for (int c = 0; c < kBlk; c++) acc[c] = d * yt[c * ST_PLANE + ctr];
  }
#pragma unroll 1
  for (int k = 0; k < kUpper; k++) {
    const int dy = c_bup_dy[k], dx = c_bup_dx[k];
    const long long off = (long long)dy * P.W + dx;
    const float* au = a.a_up + (long long)k * a.lvec;
    const float cu = au[q], cl = au[q - off];
    const int su = ctr + dy * ST_PW + dx, sl = ctr - dy * ST_PW - dx;
#pragma unroll
    for (int c = 0; c < kBlk; c++) {
      acc[c] = fmaf(cu, yt[c * ST_PLANE + su], acc[c]);
      acc[c] = fmaf(cl, yt[c * ST_PLANE + sl], acc[c]);
    }
  }
  float4* oq = (float4*)(out + q * kBlk);
  const float4* xq = (const float4*)(X + q * kBlk);
#pragma unroll
  for (int c4 = 0; c4 < kBlk / 4; c4++) {
    float4 r;
    r.x = co.x * acc[4 * c4 + 0] + co.y * yt[(4 * c4 + 0) * ST_PLANE + ctr];
    r.y = co.x * acc[4 * c4 + 1] + co.y * yt[(4 * c4 + 1) * ST_PLANE + ctr];
    r.z = co.x * acc[4 * c4 + 2] + co.y * yt[(4 * c4 + 2) * ST_PLANE + ctr];
    r.w = co.x * acc[4 * c4 + 3] + co.y * yt[(4 * c4 + 3) * ST_PLANE + ctr];
    if (co.z != 0.f) {
      const float4 xv = xq[c4];
      r.x = fmaf(co.z, xv.x, r.x);
      r.y = fmaf(co.z, xv.y, r.y);
      r.z = fmaf(co.z, xv.z, r.z);
      r.w = fmaf(co.z, xv.w, r.w);
    }
    oq[c4] = r;
  }
}

// ------------------------------------------------------------------ Gram
__device__ __forceinline__ void ffp(float& hi, float& lo, float a, float b) {
  const float p = a * b;
  const float pe = fmaf(a, b, -p);
  const float s = hi + p;
  const float z = s - hi;
  lo += ((hi - (s - z)) + (p - z)) + pe;
  hi = s;
}

// G = U^T V: thread owns entries (i, j) = (tid / 8, 4*(tid % 8) .. +3) of the
// 32 x 32 product; rows of U and V staged through shared memory
__global__ void __launch_bounds__(256) cf_gram(BlkArgs a, const float* __restrict__ U,
                                               const float* __restrict__ V, double* __restrict__ out) {
  const EigTile t = a.tiles[blockIdx.x];
  if (!a.active[t.patch]) return;
  const PatchDev P = a.patches[t.patch];
  constexpr int CH = 64;  // pixels per stage
  __shared__ float us[CH][kBlk + 1], vs[CH][kBlk + 1];
  const int i = threadIdx.x >> 3, j0 = (threadIdx.x & 7) * 4;
  float hi[4] = {0, 0, 0, 0}, lo[4] = {0, 0, 0, 0};
  for (int p0 = t.p0; p0 < t.p1; p0 += CH) {
    __syncthreads();
    for (int idx = threadIdx.x; idx < CH * kBlk; idx += blockDim.x) {
      const int pp = idx / kBlk, c = idx % kBlk;
      const int p = p0 + pp;
      float u = 0.f, v = 0.f;
      if (p < t.p1) {
        u = U[(P.vec + p) * kBlk + c];
        v = V[(P.vec + p) * kBlk + c];
      }
      us[pp][c] = u;
      vs[pp][c] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int pp = 0; pp < CH; pp++) {
      const float ui = us[pp][i];
#pragma unroll
      for (int q = 0; q < 4; q++) ffp(hi[q], lo[q], ui, vs[pp][j0 + q]);
    }
  }
  double* part = a.part + (long long)blockIdx.x * kBlk * kBlk;
#pragma unroll
  for (int q = 0; q < 4; q++) part[i * kBlk + j0 + q] = (double)hi[q] + (double)lo[q];
  // last CTA of the patch sums the partials
  __shared__ int is_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const int prev = atomicAdd(a.counter + t.patch, 1);
    is_last = (prev == a.tile_count[t.patch] - 1);
    if (is_last) a.counter[t.patch] = 0;
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  const int tb = a.tile_begin[t.patch], tc = a.tile_count[t.patch];
  for (int e = threadIdx.x; e < kBlk * kBlk; e += blockDim.x) {
    double s = 0;
    for (int b = tb; b < tb + tc; b++) s += a.part[(long long)b * kBlk * kBlk + e];
    out[(long long)t.patch * kBlk * kBlk + e] = s;
  }
}

// U <- U M (and V <- V M if V), M = a.mat[patch] (32 x 32, FP64 on the host,
// applied in FP32: the next orthonormalisation or Rayleigh-Ritz step absorbs
// the rounding); one thread per pixel row, M in shared memory
__global__ void __launch_bounds__(256) cf_rotate(BlkArgs a, float* __restrict__ U, float* __restrict__ V,
                                                 int ncols) {
  const EigTile t = a.tiles[blockIdx.x];
  if (!a.active[t.patch]) return;
  const PatchDev P = a.patches[t.patch];
  __shared__ float mh[kBlk][kBlk];
  const double* M = a.mat + (long long)t.patch * kBlk * kBlk;
  for (int e = threadIdx.x; e < kBlk * kBlk; e += blockDim.x) mh[e / kBlk][e % kBlk] = (float)M[e];
  __syncthreads();
  for (int p = t.p0 + threadIdx.x; p < t.p1; p += blockDim.x) {
    for (int which = 0; which < (V ? 2 : 1); which++) {
      float* row = (which ? V : U) + (P.vec + p) * kBlk;
      float x[kBlk];
#pragma unroll
      for (int c = 0; c < kBlk; c += 4) {
        const float4 v = *(const float4*)(row + c);
        x[c] = v.x;
        x[c + 1] = v.y;
        x[c + 2] = v.z;
        x[c + 3] = v.w;
      }
#pragma unroll 1
      for (int c0 = 0; c0 < kBlk; c0 += 4) {
        float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int r = 0; r < kBlk; r++) {
          o.x = fmaf(x[r], mh[r][c0], o.x);
          o.y = fmaf(x[r], mh[r][c0 + 1], o.y);
          o.z = fmaf(x[r], mh[r][c0 + 2], o.z);
          o.w = fmaf(x[r], mh[r][c0 + 3], o.w);
        }
        if (c0 < ncols) *(float4*)(row + c0) = o;
      }
    }
  }
}

// per-column |A x_c - theta_c x_c|^2 (AX and X given), last CTA sums
__global__ void __launch_bounds__(256) cf_resid(BlkArgs a, const float* __restrict__ X,
                                                const float* __restrict__ AX, double* __restrict__ out) {
  const EigTile t = a.tiles[blockIdx.x];
  if (!a.active[t.patch]) return;
  const PatchDev P = a.patches[t.patch];
  const int c = threadIdx.x & 31, lanegroup = threadIdx.x >> 5;
  const float th = (float)a.theta[(long long)t.patch * kBlk + c];
  float hi = 0.f, lo = 0.f;
  for (int p = t.p0 + lanegroup; p < t.p1; p += 8) {
    const long long q = (P.vec + p) * kBlk + c;
    const float r = fmaf(-th, X[q], AX[q]);
    ffp(hi, lo, r, r);
  }
  __shared__ double red[8][kBlk];
  red[lanegroup][c] = (double)hi + (double)lo;
  __syncthreads();
  if (threadIdx.x < kBlk) {
    double s = 0;
    for (int g = 0; g < 8; g++) s += red[g][threadIdx.x];
    a.part[(long long)blockIdx.x * kBlk * kBlk + threadIdx.x] = s;
  }
  __shared__ int is_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const int prev = atomicAdd(a.counter + t.patch, 1);
    is_last = (prev == a.tile_count[t.patch] - 1);
    if (is_last) a.counter[t.patch] = 0;
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  if (threadIdx.x < kBlk) {
    const int tb = a.tile_begin[t.patch], tc = a.tile_count[t.patch];
    double s = 0;
    for (int b = tb; b < tb + tc; b++) s += a.part[(long long)b * kBlk * kBlk + threadIdx.x];
    out[(long long)t.patch * kBlk + threadIdx.x] = s;
  }
}

// columns 0..nvec-1 of X into separate vectors evec[c][vec layout]
__global__ void __launch_bounds__(256) cf_extract(BlkArgs a, const float* __restrict__ X,
                                                  float* __restrict__ evec, int nvec) {
  const EigTile t = a.tiles[blockIdx.x];
  if (!a.done[t.patch]) return;
  const PatchDev P = a.patches[t.patch];
  for (int p = t.p0 + threadIdx.x; p < t.p1; p += blockDim.x)
    for (int c = 0; c < nvec; c++) evec[(long long)c * a.lvec + P.vec + p] = X[(P.vec + p) * kBlk + c];
}

// seeded start block (a fixed hash per pixel and column)
__global__ void __launch_bounds__(256) cf_init(BlkArgs a, float* __restrict__ X) {
  const EigTile t = a.tiles[blockIdx.x];
  if (!a.active[t.patch]) return;
  const PatchDev P = a.patches[t.patch];
  for (int idx = threadIdx.x; idx < (t.p1 - t.p0) * kBlk; idx += blockDim.x) {
    const int p = t.p0 + idx / kBlk, c = idx % kBlk;
    uint32_t x = (uint32_t)p * 2654435761u ^ ((uint32_t)c * 0x9e3779b9u + 0x1234567u);
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    X[(P.vec + p) * kBlk + c] = (float)(x & 0xffffff) * (1.0f / 16777216.0f) - 0.5f;
  }
}

// ------------------------------------------------------------ coarse level
// Galerkin coarsening by 2 x 2 aggregation: W_c(P,Q) = sum of W(p,q) over
// p in P, q in Q, so (D_c - W_c) u = lambda D_c u is the projection of the
// fine generalised problem onto block-constant vectors.  Fine radius 5 gives
// coarse offsets up to 3: a full 7 x 7 stencil, stored per offset.
__global__ void __launch_bounds__(256) cf_coarsen(CoarseArgs c) {
  const int4 w = c.work[blockIdx.x];  // coarse (patch, Y0, X0)
  const PatchDev F = c.fine[w.x], C = c.coarse[w.x];
  const int Y = w.y + threadIdx.x / 16, X = w.z + threadIdx.x % 16;
  if (Y >= C.H || X >= C.W) return;
  float acc[kCN];
#pragma unroll
  for (int k = 0; k < kCN; k++) acc[k] = 0.f;
  double deg = 0.0;
  for (int sy = 0; sy < 2; sy++)
    for (int sx = 0; sx < 2; sx++) {
      const int y = 2 * Y + sy, x = 2 * X + sx;
      if (y >= F.H || x >= F.W) continue;
      const long long p = F.vec + (long long)y * F.W + x;
      acc[kCR * kCW + kCR] += 1.f;  // w_pp = 1
      deg += c.deg[p];
      for (int j = 0; j < kUpper; j++) {
        const int dy = c_bup_dy[j], dx = c_bup_dx[j];
        // upper neighbour q = p + (dy,dx) and lower neighbour q = p - (dy,dx)
        for (int sgn = -1; sgn <= 1; sgn += 2) {
          const int yy = y + sgn * dy, xx = x + sgn * dx;
          if (yy < 0 || yy >= F.H || xx < 0 || xx >= F.W) continue;
          const long long off = (long long)dy * F.W + dx;
          const float wv = sgn > 0 ? c.wsym_up[(long long)j * c.lvec_f + p] : c.wsym_up[(long long)j * c.lvec_f + p - off];
          const int dY = (yy >> 1) - Y, dX = (xx >> 1) - X;
          acc[(dY + kCR) * kCW + (dX + kCR)] += wv;
        }
      }
    }
  const long long P = C.vec + (long long)Y * C.W + X;
#pragma unroll
  for (int k = 0; k < kCN; k++) c.wc[(long long)k * c.lvec_c + P] = acc[k];
  c.degc[P] = (float)deg;
  c.disc[P] = (float)(1.0 / sqrt(deg));
}

// A_c = I - D_c^-1/2 W_c D_c^-1/2 in place on wc
__global__ void __launch_bounds__(256) cf_coarse_norm(CoarseArgs c) {
  const int4 w = c.work[blockIdx.x];
  const PatchDev C = c.coarse[w.x];
  const int Y = w.y + threadIdx.x / 16, X = w.z + threadIdx.x % 16;
  if (Y >= C.H || X >= C.W) return;
  const long long P = C.vec + (long long)Y * C.W + X;
  const float dp = c.disc[P];
  for (int k = 0; k < kCN; k++) {
    const int dY = k / kCW - kCR, dX = k % kCW - kCR;
    const int YY = Y + dY, XX = X + dX;
    float v = 0.f;
    if (YY >= 0 && YY < C.H && XX >= 0 && XX < C.W)
      v = -c.wc[(long long)k * c.lvec_c + P] * dp * c.disc[C.vec + (long long)YY * C.W + XX];
    if (k == kCR * kCW + kCR) v += 1.f;
    c.wc[(long long)k * c.lvec_c + P] = v;
  }
}

// coarse Chebyshev step: as cf_step, full 7 x 7 stencil, halo 3
constexpr int SC_PH = ST_H + 2 * kCR, SC_PW = ST_W + 2 * kCR;
constexpr int SC_PLANE = SC_PH * SC_PW + 1;  // 533: odd
constexpr size_t kStepCSmem = (size_t)kBlk * SC_PLANE * sizeof(float);

__global__ void __launch_bounds__(ST_H * 32, 2) cf_step_c(BlkArgs a, const int4* __restrict__ work,
                                                          const float* __restrict__ Y, const float* __restrict__ X,
                                                          float* __restrict__ out, int step) {
  extern __shared__ float yt[];
  const int4 w = work[blockIdx.x];
  if (!a.active[w.x]) return;
  const PatchDev P = a.patches[w.x];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  {
    constexpr int F4_PER_ROW = kBlk / 4;
    constexpr int F4_PER_TROW = SC_PW * F4_PER_ROW;
    constexpr int TOTAL = SC_PH * F4_PER_TROW;
    constexpr int PER_THREAD = (TOTAL + ST_H * 32 - 1) / (ST_H * 32);
    float4 v[PER_THREAD];
#pragma unroll
    for (int i = 0; i < PER_THREAD; i++) {
      const int f = threadIdx.x + i * ST_H * 32;
      const int ty = f / F4_PER_TROW, rem = f % F4_PER_TROW;
      v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (f < TOTAL && w.y - kCR + ty < P.H + kCR) {
        const long long q0 = P.vec + (long long)(w.y - kCR + ty) * P.W + (w.z - kCR);
        v[i] = ((const float4*)(Y + q0 * kBlk))[rem];
      }
    }
#pragma unroll
    for (int i = 0; i < PER_THREAD; i++) {
      const int f = threadIdx.x + i * ST_H * 32;
      if (f < TOTAL) {
        const int ty = f / F4_PER_TROW, rem = f % F4_PER_TROW;
        const int tx = rem / F4_PER_ROW, c = (rem % F4_PER_ROW) * 4;
        const int r = ty * SC_PW + tx;
        yt[(c + 0) * SC_PLANE + r] = v[i].x;
        yt[(c + 1) * SC_PLANE + r] = v[i].y;
        yt[(c + 2) * SC_PLANE + r] = v[i].z;
        yt[(c + 3) * SC_PLANE + r] = v[i].w;
      }
    }
  }
  __syncthreads();
  const int y = w.y + warp, x = w.z + lane;
  if (y >= P.H || x >= P.W) return;
  const long long q = P.vec + (long long)y * P.W + x;
  const float3 co = a.coef[(long long)w.x * a.max_steps + step];
  float acc[kBlk];
#pragma unroll
  for (int c = 0; c < kBlk; c++) acc[c] = 0.f;
  const int ctr = (warp + kCR) * SC_PW + (lane + kCR);
#pragma unroll 1
  for (int k = 0; k < kCN; k++) {
    const int dy = k / kCW - kCR, dx = k % kCW - kCR;
    const float cf = a.a_up[(long long)k * a.lvec + q];
    const int sidx = ctr + dy * SC_PW + dx;
#pragma unroll
    for (int c = 0; c < kBlk; c++) acc[c] = fmaf(cf, yt[c * SC_PLANE + sidx], acc[c]);
  }
  float4* oq = (float4*)(out + q * kBlk);
  const float4* xq = (const float4*)(X + q * kBlk);
#pragma unroll
  for (int c4 = 0; c4 < kBlk / 4; c4++) {
    float4 r;
    r.x = co.x * acc[4 * c4 + 0] + co.y * yt[(4 * c4 + 0) * SC_PLANE + ctr];
    r.y = co.x * acc[4 * c4 + 1] + co.y * yt[(4 * c4 + 1) * SC_PLANE + ctr];
    r.z = co.x * acc[4 * c4 + 2] + co.y * yt[(4 * c4 + 2) * SC_PLANE + ctr];
    r.w = co.x * acc[4 * c4 + 3] + co.y * yt[(4 * c4 + 3) * SC_PLANE + ctr];
    if (co.z != 0.f) {
      const float4 xv = xq[c4];
      r.x = fmaf(co.z, xv.x, r.x);
      r.y = fmaf(co.z, xv.y, r.y);
      r.z = fmaf(co.z, xv.z, r.z);
      r.w = fmaf(co.z, xv.w, r.w);
    }
    oq[c4] = r;
  }
}

// fine start block from the coarse Ritz vectors: y = D^1/2 P D_c^-1/2 y_c
__global__ void __launch_bounds__(256) cf_prolong(CoarseArgs c, const float* __restrict__ xc,
                                                  float* __restrict__ xf) {
  const int4 w = c.work_f[blockIdx.x];  // fine (patch, y0, x0)
  const PatchDev F = c.fine[w.x], C = c.coarse[w.x];
  const int y = w.y + threadIdx.x / 16, x = w.z + threadIdx.x % 16;
  if (y >= F.H || x >= F.W) return;
  const long long p = F.vec + (long long)y * F.W + x;
  const long long P = C.vec + (long long)(y >> 1) * C.W + (x >> 1);
  const float s = sqrtf(c.deg[p]) * c.disc[P];
  const float4* src = (const float4*)(xc + P * kBlk);
  float4* dst = (float4*)(xf + p * kBlk);
#pragma unroll
  for (int c4 = 0; c4 < kBlk / 4; c4++) {
    float4 v = src[c4];
    v.x *= s;
    v.y *= s;
    v.z *= s;
    v.w *= s;
    dst[c4] = v;
  }
}

cudaError_t cf_launch_coarsen(const CoarseArgs& c, int nwork_c, cudaStream_t s) {
  cf_coarsen<<<nwork_c, 256, 0, s>>>(c);
  cf_coarse_norm<<<nwork_c, 256, 0, s>>>(c);
  return cudaGetLastError();
}
cudaError_t cf_launch_prolong(const CoarseArgs& c, int nwork_f, const float* xc, float* xf, cudaStream_t s) {
  cf_prolong<<<nwork_f, 256, 0, s>>>(c, xc, xf);
  return cudaGetLastError();
}

cudaError_t cf_launch_step(const BlkArgs& a, const int4* work, int nwork, const float* Y, const float* X, float* out,
                           int step, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(cf_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStepSmem);
    attr = true;
  }
  static bool attr_c = false;
  if (!attr_c) {
    cudaFuncSetAttribute(cf_step_c, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStepCSmem);
    attr_c = true;
  }
  if (a.coarse)
    cf_step_c<<<nwork, ST_H * 32, kStepCSmem, s>>>(a, work, Y, X, out, step);
  else
    cf_step<<<nwork, ST_H * 32, kStepSmem, s>>>(a, work, Y, X, out, step);
  return cudaGetLastError();
}
cudaError_t cf_launch_gram(const BlkArgs& a, int ntiles, const float* U, const float* V, double* out,
                           cudaStream_t s) {
  cf_gram<<<ntiles, 256, 0, s>>>(a, U, V, out);
  return cudaGetLastError();
}
cudaError_t cf_launch_rotate(const BlkArgs& a, int ntiles, float* U, float* V, int ncols, cudaStream_t s) {
  cf_rotate<<<ntiles, 256, 0, s>>>(a, U, V, ncols);
  return cudaGetLastError();
}
cudaError_t cf_launch_resid(const BlkArgs& a, int ntiles, const float* X, const float* AX, double* out,
                            cudaStream_t s) {
  cf_resid<<<ntiles, 256, 0, s>>>(a, X, AX, out);
  return cudaGetLastError();
}
cudaError_t cf_launch_extract(const BlkArgs& a, int ntiles, const float* X, float* evec, int nvec,
                              cudaStream_t s) {
  cf_extract<<<ntiles, 256, 0, s>>>(a, X, evec, nvec);
  return cudaGetLastError();
}
cudaError_t cf_launch_init(const BlkArgs& a, int ntiles, float* X, cudaStream_t s) {
  cf_init<<<ntiles, 256, 0, s>>>(a, X);
  return cudaGetLastError();
}

}  // namespace gpb
