// k_eig.cu -- batched Krylov-Schur (thick-restart Lanczos) kernels for the
// smallest eigenpairs of A = I - D^-1/2 W D^-1/2 (sm_103a).
//
// Reference: the Lanczos eigensolver of
// damascene/src/noReorthog/lanczos.cu:192-752 and the stencil SpMV of
// damascene/src/stencilMatrixMultiply/stencilMVM.cu:129-182; the CPU path's
// Spectra SymGEigsSolver (src/spectralPb.cpp:221-245) defines the problem.
//
// One Lanczos step for every active patch of the batch is three launches:
//   ks_spmv   w = A v_j (FP32 symmetric stencil SpMV, the lower triangle read
//             as the upper array shifted by the offset), v_j = w_prev / beta
//             written on the fly, h = V^T w
//   ks_orth   w -= V h, h2 = V^T w          (classical Gram-Schmidt, pass 1)
//   ks_orth   w -= V h2, beta^2 = |w|^2     (pass 2)
// Dot products are FMA chains over a thread's pixels, summed across the
// warp and the CTA in float-float (a compensated FP32 pair; FP64 runs at
// 1/64 of the FP32 rate on this part); the first CGS pass's projection V h,
// whose subtraction cancels most of w on a converging step, is formed
// float-float with exact products.  The per-CTA partials are reduced in FP64
// by the last CTA of each patch to finish (threadfence + atomic counter), so
// no separate reduction launches.
// The projected matrix T lives in device memory; at the end of a restart
// cycle the host solves it (eig_host.cpp) and ks_restart assembles the kept
// Ritz vectors.
#include <stdint.h>

#include "gpb_internal.h"
#include "kernels.h"
#include "k_eig.h"

namespace gpb {

__constant__ int c_up_dy[kUpper], c_up_dx[kUpper];

void upload_eig(const HostTables& t, cudaStream_t s) {
  int dy[kUpper], dx[kUpper];
  for (int j = 0; j < kUpper; j++) {
    dy[j] = t.sdy[kStencilN / 2 + 1 + j];
    dx[j] = t.sdx[kStencilN / 2 + 1 + j];
  }
  cudaMemcpyToSymbolAsync(c_up_dy, dy, sizeof(dy), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_up_dx, dx, sizeof(dx), 0, cudaMemcpyHostToDevice, s);
}

constexpr unsigned FULLM = 0xffffffffu;

__device__ __forceinline__ void ff_add_prod(float& hi, float& lo, float a, float b) {
  // __fmul_rn / __fadd_rn: never contracted into an FMA, which would break
  // the error-free transformations
  const float p = __fmul_rn(a, b);
  const float pe = fmaf(a, b, -p);
  const float s = __fadd_rn(hi, p);
  const float z = s - hi;
  const float e = (hi - (s - z)) + (p - z);
  hi = s;
  lo += e + pe;
}
__device__ __forceinline__ void ff_add(float& hi, float& lo, float bhi, float blo) {
  const float s = hi + bhi;
  const float z = s - hi;
  const float e = (hi - (s - z)) + (bhi - z);
  hi = s;
  lo += e + blo;
}
// float-float sum over the warp, in FP32 (every lane gets it); the FP64
// pipe, about 1/64 of the FP32 rate here, is left to one conversion per CTA
__device__ __forceinline__ float2 ff_warp_reduce(float hi, float lo) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(FULLM, hi, o), l2 = __shfl_xor_sync(FULLM, lo, o);
    ff_add(hi, lo, h2, l2);
  }
  return make_float2(hi, lo);
}

// Last CTA of a patch: returns true in every thread of that CTA.
__device__ __forceinline__ bool last_cta(int* counter, int ntiles) {
  __shared__ int is_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const int prev = atomicAdd(counter, 1);
    is_last = (prev == ntiles - 1);
    if (is_last) *counter = 0;
  }
  __syncthreads();
  if (is_last) __threadfence();
  return is_last;
}

// per-warp partial sums (sred[warp][i], written by lane 0) -> one partial per
// CTA in part[cta][i]
constexpr int kRed = kMaxKrylov + 1;
__device__ __forceinline__ void cta_partials(const float2* sred, int nvals, double* part_row) {
  __syncthreads();
  for (int i = threadIdx.x; i < nvals; i += blockDim.x) {
    float hi = 0.f, lo = 0.f;
#pragma unroll
    for (int w = 0; w < kEigWarps; w++) ff_add(hi, lo, sred[w * kRed + i].x, sred[w * kRed + i].y);
    part_row[i] = (double)hi + (double)lo;
  }
}
// sum of one value over the CTAs of a patch, one warp, lanes strided
__device__ __forceinline__ double patch_sum(const double* part, int tb, int tc, int mp1, int i, int lane) {
  double s = 0;
  for (int b = tb + lane; b < tb + tc; b += 32) s += part[(long long)b * mp1 + i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULLM, s, o);
  return s;
}

// Loads are issued in batches -- the stencil by offset for all eight pixels
// of a thread, the basis by groups of kGrp vectors -- so each thread keeps
// tens of independent loads in flight; every per-pixel sum still runs in the
// same order (offsets ascending, basis vectors ascending, pixels ascending).
// Pixels are addressed by 32-bit offsets into the vector layout, which the
// host keeps below 2^31 entries.
constexpr int kGrp = 8;

// Sums kGrp = 8 float-float values over the warp at once.  Each of the first
// three xor rounds halves the values a lane carries (it keeps the half its
// lane bit selects and sends the other), the last two are plain: 18
// exchanges of a (hi, lo) pair and 9 float-float additions for the 8 values
// instead of 80 and 40.  Lane l ends with the total of value l >> 2.
__device__ __forceinline__ float2 ff_warp_reduce8(float (&hi)[kGrp], float (&lo)[kGrp], int lane) {
#pragma unroll
  for (int half = 4, o = 16; half >= 1; half >>= 1, o >>= 1) {
    const bool b = lane & o;
#pragma unroll
    for (int i = 0; i < half; i++) {
      const float kh = b ? hi[i + half] : hi[i], kl = b ? lo[i + half] : lo[i];
      const float gh = b ? hi[i] : hi[i + half], gl = b ? lo[i] : lo[i + half];
      hi[i] = kh;
      lo[i] = kl;
      ff_add(hi[i], lo[i], __shfl_xor_sync(FULLM, gh, o), __shfl_xor_sync(FULLM, gl, o));
    }
  }
#pragma unroll
  for (int o = 2; o >= 1; o >>= 1) ff_add(hi[0], lo[0], __shfl_xor_sync(FULLM, hi[0], o), __shfl_xor_sync(FULLM, lo[0], o));
  return make_float2(hi[0], lo[0]);
}

// h_i = v_i . w for i = 0..j over this thread's pixels (w is 0 at a pixel
// past the tile), reduced per warp into sred[warp][i]; v_j comes from
// registers (xj) when given.  A plain FMA chain over the thread's eight
// pixels, then float-float across threads: the error of a dot is a few
// units of rounding times |w| (Cauchy-Schwarz over the thread partials),
// which after the second pass leaves the basis orthogonal to ~1e-7 --
// two orders below what the Ritz residuals need.
__device__ __forceinline__ void basis_dots(const EigArgs& a, int j, const int (&qv)[kEigPix],
                                           const float (&wv)[kEigPix], const float* xj, float2* sred, int warp,
                                           int lane) {
  for (int i0 = 0; i0 <= j; i0 += kGrp) {
    float vv[kGrp][kEigPix];
#pragma unroll
    for (int u = 0; u < kGrp; u++) {
      const int i = i0 + u;
      const float* Vi = a.V + (long long)i * a.lvec;
#pragma unroll
      for (int r = 0; r < kEigPix; r++) vv[u][r] = (i < j || (i == j && !xj)) ? Vi[qv[r]] : (i == j ? xj[r] : 0.f);
    }
    float hi[kGrp], lo[kGrp];
#pragma unroll
    for (int u = 0; u < kGrp; u++) {
      hi[u] = lo[u] = 0.f;
#pragma unroll
      for (int r = 0; r < kEigPix; r++) hi[u] = fmaf(vv[u][r], wv[r], hi[u]);
    }
    const float2 sum = ff_warp_reduce8(hi, lo, lane);
    const int i = i0 + (lane >> 2);
    if ((lane & 3) == 0 && i <= j) sred[warp * kRed + i] = sum;
  }
}

// ------------------------------------------------------------------ SpMV
__global__ void __launch_bounds__(kEigThreads, 2) ks_spmv(EigArgs a, int j, const float* __restrict__ src,
                                                          int use_beta, float* __restrict__ dst) {
  const EigTile t = a.tiles[blockIdx.x];
  if (!a.active[t.patch]) return;
  const PatchDev P = a.patches[t.patch];
  __shared__ int off[kUpper];
  if (threadIdx.x < kUpper) off[threadIdx.x] = c_up_dy[threadIdx.x] * P.W + c_up_dx[threadIdx.x];
  __syncthreads();
  __shared__ float inv_s;
  if (threadIdx.x == 0) inv_s = use_beta ? (float)(1.0 / sqrt(a.beta2[t.patch])) : 1.f;
  __syncthreads();
  const float inv = inv_s;
  const long long base = P.vec;
  // this thread's pixels; a pixel past the tile reads the tile's first one
  // (in bounds) and its results are dropped
  int qv[kEigPix];
  bool okv[kEigPix];
#pragma unroll
  for (int r = 0; r < kEigPix; r++) {
    const int p = t.p0 + threadIdx.x + r * kEigThreads;
    okv[r] = p < t.p1;
    qv[r] = (int)(base + (okv[r] ? p : t.p0));
  }
  float acc[kEigPix];
#pragma unroll
  for (int r = 0; r < kEigPix; r++) acc[r] = 0.f;
#pragma unroll 2
  for (int k = 0; k < kUpper; k++) {
    const float* au = a.a_up + (long long)k * a.lvec;
    const int o = off[k];
    float cu[kEigPix], xu[kEigPix], cl[kEigPix], xl[kEigPix];
#pragma unroll
    for (int r = 0; r < kEigPix; r++) {
      cu[r] = au[qv[r]];
      xu[r] = src[qv[r] + o];
      cl[r] = au[qv[r] - o];
      xl[r] = src[qv[r] - o];
    }
#pragma unroll
    for (int r = 0; r < kEigPix; r++) {
      acc[r] = fmaf(cu[r], xu[r], acc[r]);
      acc[r] = fmaf(cl[r], xl[r], acc[r]);
    }
  }
  float wv[kEigPix], xv[kEigPix];
#pragma unroll
  for (int r = 0; r < kEigPix; r++) {
    const float x = src[qv[r]] * inv;
    xv[r] = okv[r] ? x : 0.f;
    wv[r] = okv[r] ? fmaf(acc[r], inv, a.a_diag[qv[r]] * x) : 0.f;
  }
  float* Vj = a.V + (long long)j * a.lvec;
#pragma unroll
  for (int r = 0; r < kEigPix; r++) {
    if (!okv[r]) continue;
    Vj[qv[r]] = xv[r];
    dst[qv[r]] = wv[r];
  }
  // h_i = v_i . w for i <= j
  __shared__ float2 sred[kEigWarps * kRed];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // the second pass measures what these dots missed (h2 = V^T (w - V h)),
  // and T takes h + h2
  basis_dots(a, j, qv, wv, xv, sred, warp, lane);
  cta_partials(sred, j + 1, a.part + (long long)blockIdx.x * a.mp1);
  if (last_cta(a.counter + t.patch, a.tile_count[t.patch])) {
    const int tb = a.tile_begin[t.patch], tc = a.tile_count[t.patch];
    double* T = a.T + (long long)t.patch * a.m * a.m;
    for (int i = warp; i <= j; i += kEigWarps) {
      const double s = patch_sum(a.part, tb, tc, a.mp1, i, lane);
      if (lane == 0) {
        a.hbuf[(long long)t.patch * a.mp1 + i] = s;
        T[i * a.m + j] = s;
        T[j * a.m + i] = s;
      }
    }
  }
}

// --------------------------------------------------------------- CGS pass
// MODE 1: w -= V h, then h2 = V^T w;  MODE 2: w -= V h2, then |w|^2.
// Pass 1 subtracts a projection of about |w|'s size (the cancellation of a
// converging step), so V h is formed in float-float and subtracted exactly;
// pass 2's V h2 is of rounding-error size and an FMA chain holds it.
template <int MODE>
__global__ void __launch_bounds__(kEigThreads, 2) ks_orth(EigArgs a, int j, float* __restrict__ w) {
  const EigTile t = a.tiles[blockIdx.x];
  if (!a.active[t.patch]) return;
  const PatchDev P = a.patches[t.patch];
  const long long base = P.vec;
  // projection coefficients as FP32 hi + lo pairs; the sum V h is formed in
  // float-float and subtracted from w before the single rounding to FP32, so
  // the cancellation of a converging step (|w - V h| << |w|) keeps its digits
  __shared__ float hs[kMaxKrylov + 1], hl[kMaxKrylov + 1];
  for (int i = threadIdx.x; i <= j; i += blockDim.x) {
    const double h = a.hbuf[(long long)t.patch * a.mp1 + i];
    hs[i] = (float)h;
    hl[i] = (float)(h - (double)hs[i]);
  }
  __syncthreads();
  int qv[kEigPix];
  bool okv[kEigPix];
  float wv[kEigPix], sh[kEigPix], sl[kEigPix];
#pragma unroll
  for (int r = 0; r < kEigPix; r++) {
    const int p = t.p0 + threadIdx.x + r * kEigThreads;
    okv[r] = p < t.p1;
    qv[r] = (int)(base + (okv[r] ? p : t.p0));
    wv[r] = okv[r] ? w[qv[r]] : 0.f;
    sh[r] = sl[r] = 0.f;
  }
  for (int i0 = 0; i0 <= j; i0 += kGrp) {
    float vv[kGrp][kEigPix];
#pragma unroll
    for (int u = 0; u < kGrp; u++) {
      const float* Vi = a.V + (long long)(i0 + u) * a.lvec;
#pragma unroll
      for (int r = 0; r < kEigPix; r++) vv[u][r] = (i0 + u <= j) ? Vi[qv[r]] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < kGrp; u++) {
      if (i0 + u > j) break;
      const float h = hs[i0 + u], h2 = hl[i0 + u];
#pragma unroll
      for (int r = 0; r < kEigPix; r++) {
        if constexpr (MODE == 1) {
          ff_add_prod(sh[r], sl[r], h, vv[u][r]);
          sl[r] = fmaf(h2, vv[u][r], sl[r]);
        } else {
          sh[r] = fmaf(h, vv[u][r], sh[r]);
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < kEigPix; r++) {
    if constexpr (MODE == 1) {
      // w - (sh + sl) with the subtraction of sh exact (two-difference)
      const float d = wv[r] - sh[r];
      const float z = d - wv[r];
      const float e = (wv[r] - (d - z)) - (sh[r] + z);
      wv[r] = okv[r] ? d + (e - sl[r]) : 0.f;
    } else {
      wv[r] = okv[r] ? wv[r] - sh[r] : 0.f;
    }
  }
#pragma unroll
  for (int r = 0; r < kEigPix; r++)
    if (okv[r]) w[qv[r]] = wv[r];
  __shared__ float2 sred[kEigWarps * kRed];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if constexpr (MODE == 1) {
    basis_dots(a, j, qv, wv, nullptr, sred, warp, lane);
    cta_partials(sred, j + 1, a.part + (long long)blockIdx.x * a.mp1);
  } else {
    float hi = 0.f, lo = 0.f;
#pragma unroll
    for (int r = 0; r < kEigPix; r++)
      if (okv[r]) ff_add_prod(hi, lo, wv[r], wv[r]);
    const float2 s = ff_warp_reduce(hi, lo);
    if (lane == 0) sred[warp * kRed] = s;
    cta_partials(sred, 1, a.part + (long long)blockIdx.x * a.mp1);
  }
  if (last_cta(a.counter + t.patch, a.tile_count[t.patch])) {
    const int tb = a.tile_begin[t.patch], tc = a.tile_count[t.patch];
    double* T = a.T + (long long)t.patch * a.m * a.m;
    if constexpr (MODE == 1) {
      for (int i = warp; i <= j; i += kEigWarps) {
        const double s = patch_sum(a.part, tb, tc, a.mp1, i, lane);
        if (lane == 0) {
          a.hbuf[(long long)t.patch * a.mp1 + i] = s;
          T[i * a.m + j] += s;
          if (i != j) T[j * a.m + i] += s;
        }
      }
    } else if (warp == 0) {
      double s = patch_sum(a.part, tb, tc, a.mp1, 0, lane);
      if (lane != 0) return;
      if (!(s > 1e-60)) s = 1e-60;
      a.beta2[t.patch] = s;
      if (j + 1 < a.m) {
        const double b = sqrt(s);
        T[(j + 1) * a.m + j] = b;
        T[j * a.m + (j + 1)] = b;
      }
    }
  }
}

// -------------------------------------------------------------- restart
// Vout[:, 0..nk) = V[:, 0..m) Y[:, 0..nk) per pixel, then Vout[nk] = w / beta
// (restart, Vout is the other basis buffer) -- or, for a converged patch
// (FINAL), the nk = nvec Ritz vectors into evec_out.
// Restart: FMA chains over the m basis vectors; the kept vectors come out
// orthonormal to a few units of rounding, which the next cycle's two CGS
// passes keep.  A thread takes one pixel and up to 32 outputs per pass over
// V, so each basis value is loaded once per pass and each 16-byte broadcast
// of Y (shared memory, zero-padded) feeds 4 FMAs; 80 registers keep three
// CTAs on an SM.
// FINAL: the eigenvectors themselves, where an FMA chain's rounding (about
// sqrt(m) units) would show in their residual: Y is split into FP32 hi + lo,
// the hi products are summed by FMA in groups of four folded into a
// float-float by TwoSum, the lo products into the low word.
template <bool FINAL>
__global__ void __launch_bounds__(kEigThreads, 2) ks_restart(EigArgs a, const float* __restrict__ w,
                                                            float* __restrict__ vout,
                                                            float* __restrict__ evec_out) {
  constexpr int COLS = 16;  // outputs per pass over V
  const EigTile t = a.tiles[blockIdx.x];
  const int mode = a.decision[t.patch];  // 0 idle, 1 restart, 2 final
  if (mode != (FINAL ? 2 : 1)) return;
  const PatchDev P = a.patches[t.patch];
  const int nk = a.nkeep[t.patch], m = a.m;
  extern __shared__ float4 ysh4[];  // [m][COLS / 4] hi, then (FINAL) lo
  float* ysh = (float*)ysh4;
  const double* Y = a.Y + (long long)t.patch * m * m;
  const int base = (int)P.vec;
  float* out = FINAL ? evec_out : vout;
  for (int c0 = 0; c0 < nk; c0 += COLS) {
    __syncthreads();
    for (int idx = threadIdx.x; idx < m * COLS; idx += blockDim.x) {
      const int i = idx / COLS, c = c0 + idx % COLS;
      const double y = c < nk ? Y[i * m + c] : 0.0;
      const float yh = (float)y;
      ysh[idx] = yh;
      ysh[m * COLS + idx] = (float)(y - (double)yh);
    }
    __syncthreads();
    for (int r = 0; r < kEigPix; r++) {
      const int p = t.p0 + threadIdx.x + r * kEigThreads;
      if (p >= t.p1) break;
      const int q = base + p;
      float acc[COLS], lo[COLS], g[COLS];
#pragma unroll
      for (int c = 0; c < COLS; c++) acc[c] = lo[c] = g[c] = 0.f;
#pragma unroll 4
      for (int i = 0; i < m; i++) {
        const float v = a.V[(long long)i * a.lvec + q];
#pragma unroll
        for (int c4 = 0; c4 < COLS / 4; c4++) {
          const float4 y = ysh4[i * (COLS / 4) + c4];
          const float yv[4] = {y.x, y.y, y.z, y.w};
          const float4 yl = ysh4[(m + i) * (COLS / 4) + c4];
          const float ylv[4] = {yl.x, yl.y, yl.z, yl.w};
#pragma unroll
          for (int j = 0; j < 4; j++) {
            g[4 * c4 + j] = fmaf(yv[j], v, g[4 * c4 + j]);
            lo[4 * c4 + j] = fmaf(ylv[j], v, lo[4 * c4 + j]);
          }
        }
        if ((i & 3) == 3 || i == m - 1) {
#pragma unroll
          for (int c = 0; c < COLS; c++) {
            const float sum = acc[c] + g[c], z = sum - acc[c];
            lo[c] += (acc[c] - (sum - z)) + (g[c] - z);
            acc[c] = sum;
            g[c] = 0.f;
          }
        }
      }
#pragma unroll
      for (int c = 0; c < COLS; c++)
        if (c0 + c < nk) out[(long long)(c0 + c) * a.lvec + q] = acc[c] + lo[c];
    }
  }
  if constexpr (!FINAL) {
    const float inv = (float)(1.0 / sqrt(a.beta2[t.patch]));
    for (int r = 0; r < kEigPix; r++) {
      const int p = t.p0 + threadIdx.x + r * kEigThreads;
      if (p < t.p1) vout[(long long)nk * a.lvec + base + p] = w[base + p] * inv;
    }
  }
}

// start vector: a fixed hash per pixel, |w|^2 into beta2 (through the same
// last-CTA reduction)
__device__ __forceinline__ float hash_unit(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return (float)(x & 0xffffff) * (1.0f / 16777216.0f) - 0.5f;
}

__global__ void __launch_bounds__(kEigThreads) ks_init(EigArgs a, float* __restrict__ w) {
  const EigTile t = a.tiles[blockIdx.x];
  if (!a.active[t.patch]) return;
  const PatchDev P = a.patches[t.patch];
  float hi = 0.f, lo = 0.f;
  for (int r = 0; r < kEigPix; r++) {
    const int p = t.p0 + threadIdx.x + r * kEigThreads;
    if (p >= t.p1) continue;
    const float v = hash_unit((uint32_t)p * 2654435761u + 12345u);
    w[P.vec + p] = v;
    ff_add_prod(hi, lo, v, v);
  }
  __shared__ float2 sred[kEigWarps * kRed];
  const float2 s = ff_warp_reduce(hi, lo);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) sred[warp * kRed] = s;
  cta_partials(sred, 1, a.part + (long long)blockIdx.x * a.mp1);
  if (last_cta(a.counter + t.patch, a.tile_count[t.patch]) && warp == 0) {
    const int tb = a.tile_begin[t.patch], tc = a.tile_count[t.patch];
    const double s2 = patch_sum(a.part, tb, tc, a.mp1, 0, lane);
    if (lane == 0) a.beta2[t.patch] = s2;
  }
}

cudaError_t ks_launch_init(const EigArgs& a, int ntiles, float* w, cudaStream_t s) {
  ks_init<<<ntiles, kEigThreads, 0, s>>>(a, w);
  return cudaGetLastError();
}
cudaError_t ks_launch_spmv(const EigArgs& a, int ntiles, int j, const float* src, int use_beta,
                           float* dst, cudaStream_t s) {
  ks_spmv<<<ntiles, kEigThreads, 0, s>>>(a, j, src, use_beta, dst);
  return cudaGetLastError();
}
cudaError_t ks_launch_orth(const EigArgs& a, int ntiles, int j, int mode, float* w, cudaStream_t s) {
  if (mode == 1)
    ks_orth<1><<<ntiles, kEigThreads, 0, s>>>(a, j, w);
  else
    ks_orth<2><<<ntiles, kEigThreads, 0, s>>>(a, j, w);
  return cudaGetLastError();
}
cudaError_t ks_launch_restart(const EigArgs& a, int ntiles, const float* w, float* vout, float* evec,
                              cudaStream_t s, bool any_restart, bool any_final) {
  if (any_restart) ks_restart<false><<<ntiles, kEigThreads, 2 * a.m * 16 * sizeof(float), s>>>(a, w, vout, evec);
  if (any_final) ks_restart<true><<<ntiles, kEigThreads, 2 * a.m * 16 * sizeof(float), s>>>(a, w, vout, evec);
  return cudaGetLastError();
}

}  // namespace gpb
