// k_block.cu -- block kernels of the Chebyshev-filtered subspace iteration
// (the warm-started eigensolver) for A = I - D^-1/2 W D^-1/2 (sm_103a).
//
// A block of kBlk = 32 vectors is stored pixel-major ([vec][32] floats) in the
// padded vector layout, so every stencil neighbour of a pixel is one
// contiguous 128-byte row; the operator of the block kernels is stored
// pixel-major too, one full stencil row per pixel (cf_full).
//
//   cf_step    Y' = alpha (A Y) + beta Y + gamma X   (scaled Chebyshev
//              recurrence, Zhou & Saad 2007; with alpha=1, beta=gamma=0 it
//              is the plain block SpMV)
//   cf_gram    G = U^T V per patch (32 x 32), FP32 FMA runs folded into
//              float-float sums, summed across CTAs by the patch's last CTA
//   cf_rotate  U <- U M (32 x 32 per patch), optionally V <- V M too
//   cf_resid   |A x_c - theta_c x_c|^2 per column
//   cf_extract the first nvec columns into separate vectors (sPb layout)
//
// Reference: the eigensolver of damascene/src/noReorthog/lanczos.cu and
// src/spectralPb.cpp:221-245 define the problem; the block method is this
// project's own.
#include <stdint.h>
#include <stdio.h>

#include <algorithm>
#include <stdlib.h>

#include "gpb_internal.h"
#include "k_block.h"
#include "k_eig.h"

namespace gpb {

// radius-5 disk offsets in scanline order (dy, then dx, ascending): the
// upper half -- after the centre -- numbered k = 0..39 as the a_up planes
__host__ __device__ constexpr bool in_disk(int dy, int dx) {
  return dy * dy + dx * dx <= kStencilR * kStencilR;
}
__host__ __device__ constexpr int disk_half_width(int dy) {  // floor(sqrt(25 - dy^2))
  return dy < 0 ? disk_half_width(-dy) : dy == 0 ? 5 : dy <= 3 ? 4 : dy == 4 ? 3 : 0;
}
__host__ __device__ constexpr int upper_rows_before(int dy) {  // offsets in rows 1..dy-1
  return dy <= 1 ? 0 : upper_rows_before(dy - 1) + 2 * disk_half_width(dy - 1) + 1;
}
__host__ __device__ constexpr int upper_k(int dy, int dx) {
  return dy == 0 ? dx - 1 : kStencilR + upper_rows_before(dy) + dx + disk_half_width(dy);
}
static_assert(upper_k(0, 1) == 0 && upper_k(1, -4) == 5 && upper_k(5, 0) == kUpper - 1, "upper offset numbering");


__constant__ int c_bup_dy[kUpper], c_bup_dx[kUpper];

void upload_block(const HostTables& t, cudaStream_t s) {
  int dy[kUpper], dx[kUpper];
  for (int j = 0; j < kUpper; j++) {
    dy[j] = t.sdy[kStencilN / 2 + 1 + j];
    dx[j] = t.sdx[kStencilN / 2 + 1 + j];
    if (upper_k(dy[j], dx[j]) != j) {  // cf_step numbers the offsets at compile time
      fprintf(stderr, "gpb: stencil offset table out of scanline order at %d\n", j);
      abort();
    }
  }
  cudaMemcpyToSymbolAsync(c_bup_dy, dy, sizeof(dy), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_bup_dx, dx, sizeof(dx), 0, cudaMemcpyHostToDevice, s);
}

__device__ __forceinline__ void fma4(float4& acc, float a, const float4& x) {
  acc.x = fmaf(a, x.x, acc.x);
  acc.y = fmaf(a, x.y, acc.y);
  acc.z = fmaf(a, x.z, acc.z);
  acc.w = fmaf(a, x.w, acc.w);
}

// ------------------------------------------------------------ Chebyshev step
// One CTA owns a kStepTileH x kStepTileW (8 x 16) pixel tile.  One thread
// issues bulk asynchronous copies (cp.async.bulk, completion counted on an
// mbarrier) of the tile's Y rows with an R-pixel halo -- each a contiguous
// (16 + 2R) x 128-byte run of the pixel-major block -- and of the tile's
// coefficient rows (pixel-major, one full stencil row per pixel).  Then lane
// = block column: a warp computes a 4 x 4 pixel block for all 32 columns, so
// a staged value (one conflict-free 128-byte shared row per warp) feeds up
// to 16 pixels and one broadcast 16-byte load brings four coefficients of a
// pixel.  About one shared-memory wavefront per output instead of 2.6.

// the radius-5 disk of the fine level (81 offsets in scanline order, rows
// padded to 84 floats = 21 x 16 bytes) and the 7 x 7 square of the coarse one
template <int NCOEF_, int R_>
struct StencilBase {
  static constexpr int R = R_, NC = NCOEF_;
};
struct DiskStencil : StencilBase<84, kStencilR> {
  static constexpr int N = kStencilN;
  __host__ __device__ static constexpr bool in(int dy, int dx) { return in_disk(dy, dx); }
  __host__ __device__ static constexpr int rows_before(int dy) {  // offsets in rows -R..dy-1
    return dy <= -R ? 0 : rows_before(dy - 1) + 2 * disk_half_width(dy - 1) + 1;
  }
  __host__ __device__ static constexpr int index(int dy, int dx) { return rows_before(dy) + dx + disk_half_width(dy); }
};
struct SquareStencil : StencilBase<52, kCR> {
  static constexpr int N = kCN;
  __host__ __device__ static constexpr bool in(int dy, int dx) {
    return dy >= -R && dy <= R && dx >= -R && dx <= R;
  }
  __host__ __device__ static constexpr int index(int dy, int dx) { return (dy + R) * (2 * R + 1) + dx + R; }
};
static_assert(DiskStencil::index(0, 0) == kStencilN / 2 && DiskStencil::index(kStencilR, 0) == kStencilN - 1,
              "disk numbering");
static_assert(SquareStencil::index(kCR, kCR) == kCN - 1, "square numbering");
static_assert(DiskStencil::NC == kFullNC && SquareStencil::NC == kCoarseNC, "row widths");

constexpr int ST_TY = kStepTileH, ST_TX = kStepTileW, ST_B = 4;  // tile and per-warp block
static_assert((ST_TY / ST_B) * (ST_TX / ST_B) == 8, "8 warps cover the tile");

template <class S>
struct StepSmem {
  static constexpr int PH = ST_TY + 2 * S::R, PW = ST_TX + 2 * S::R;
  static constexpr size_t y_bytes = (size_t)PH * PW * kBlk * sizeof(float);
  static constexpr size_t c_bytes = (size_t)ST_TY * ST_TX * S::NC * sizeof(float);
  static constexpr size_t stage = y_bytes + c_bytes;  // one pipeline stage
  static constexpr size_t bytes = 2 * stage + 256;    // two stages, tile records, mbarriers
  // the X-staging variant: one slot per consumer warp for its 4 x 4 block's X rows
  static constexpr size_t x_slot = (size_t)ST_B * ST_B * kBlk * sizeof(float);
  static constexpr size_t bytes_xs = bytes + 8 * x_slot;
  static_assert(stage % 128 == 0, "stage alignment");
  static_assert(bytes_xs <= 232448, "shared memory per CTA");
};

// what the producer warp tells the consumers about the tile in a stage
struct StepMeta {
  int end;        // 1: no more tiles for this CTA
  int W, H, y0;
  long long vec;
  int x0, pad;
  float cx, cy, cz, pad2;
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// global -> shared bulk copy: both addresses 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
// 16-byte asynchronous global -> shared copy (L2 only); src_bytes 0 writes
// zeros and reads nothing
__device__ __forceinline__ void cp_async16(void* dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// polls of the tile's barrier before a CTA gives up (each poll may suspend
// the thread for a short hardware-defined time; the copies take microseconds)
constexpr int kBarSpin = 1 << 20;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (int it = 0; it < kBarSpin; it++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

template <int K>
__device__ __forceinline__ float f4get(const float4& v) {
  if constexpr (K == 0) return v.x;
  else if constexpr (K == 1) return v.y;
  else if constexpr (K == 2) return v.z;
  else return v.w;
}

// one staged position (RY, DX) relative to the warp's block origin: the value
// of this lane's column there, times the coefficient of every block pixel
// whose stencil covers it
// C (compensated): the terms are summed by FMA in groups of four (grp) and
// each group is folded into a float-float (acc, lo) by an exact TwoSum,
// which removes the accumulation error of the 81-term sum -- the term that
// dominates near an eigenvector, where the diagonal and the off-diagonal
// sum nearly cancel -- down to the groups' own four-term rounding, at about
// a third of the cost of a TwoSum per term; used for the Rayleigh-Ritz
// products and residuals, not the filter
// a half-warp's sub-block: SB_R x SB_C pixels (the two halves of a warp
// split its 4 x 4 block by rows), two block columns per lane
constexpr int SB_R = 2, SB_C = 4, SB_N = SB_R * SB_C;

template <class S, bool C, int RY, int DX, int I>
__device__ __forceinline__ void step_pixels(const float* __restrict__ cs, float2 v, float4 (&cw)[SB_N],
                                            float2 (&acc)[SB_N], float2 (&lo)[SB_N], float2 (&grp)[SB_N]) {
  if constexpr (I < SB_N) {
    constexpr int bi = I / SB_C, bj = I % SB_C;
    if constexpr (S::in(RY - bi, DX - bj)) {
      constexpr int idx = S::index(RY - bi, DX - bj);
      // a pixel meets its offsets in scanline order, so chunk idx/4 is
      // first needed at idx % 4 == 0
      if constexpr (idx % 4 == 0) cw[I] = *(const float4*)(cs + (bi * ST_TX + bj) * S::NC + idx);
      const float cf = f4get<idx % 4>(cw[I]);
      if constexpr (C) {
        grp[I].x = fmaf(cf, v.x, grp[I].x);
        grp[I].y = fmaf(cf, v.y, grp[I].y);
        // a pixel's offsets run 0 .. N-1 in order: fold after every fourth
        if constexpr (idx % 4 == 3 || idx == S::N - 1) {
          float t = acc[I].x + grp[I].x, z = t - acc[I].x;
          lo[I].x += (acc[I].x - (t - z)) + (grp[I].x - z);
          acc[I].x = t;
          t = acc[I].y + grp[I].y;
          z = t - acc[I].y;
          lo[I].y += (acc[I].y - (t - z)) + (grp[I].y - z);
          acc[I].y = t;
          grp[I] = make_float2(0.f, 0.f);
        }
      } else {
        acc[I].x = fmaf(cf, v.x, acc[I].x);
        acc[I].y = fmaf(cf, v.y, acc[I].y);
      }
    }
    step_pixels<S, C, RY, DX, I + 1>(cs, v, cw, acc, lo, grp);
  }
}

template <class S, bool C, int P>
__device__ __forceinline__ void step_positions(const float* __restrict__ ys, const float* __restrict__ cs,
                                               float4 (&cw)[SB_N], float2 (&acc)[SB_N], float2 (&lo)[SB_N],
                                               float2 (&grp)[SB_N]) {
  constexpr int NY = SB_R + 2 * S::R, NX = SB_C + 2 * S::R;
  if constexpr (P < NY * NX) {
    constexpr int RY = P / NX - S::R, DX = P % NX - S::R;
    constexpr bool any = [] {
      for (int i = 0; i < SB_R; i++)
        for (int j = 0; j < SB_C; j++)
          if (S::in(RY - i, DX - j)) return true;
      return false;
    }();
    if constexpr (any) {
      const float2 v = *(const float2*)(ys + ((RY + S::R) * StepSmem<S>::PW + (DX + S::R)) * kBlk);
      step_pixels<S, C, RY, DX, 0>(cs, v, cw, acc, lo, grp);
    }
    step_positions<S, C, P + 1>(ys, cs, cw, acc, lo, grp);
  }
}

// Persistent, warp-specialised: one CTA per SM walks its share of the tile
// list.  Warp 8 (one lane) is the producer: for each active tile it waits
// until the consumers have released the stage, writes the tile record and
// issues the bulk copies against the stage's "full" mbarrier.  Warps 0-7
// consume: wait "full", prefetch X, run the stencil on their 4 x 4 block,
// write the outputs and arrive on the stage's "empty" mbarrier.  Two stages,
// so tile i+1 streams in while tile i is computed.  Every wait is bounded;
// a wait that gives up sets *a.err and ends the CTA.
constexpr int kStepConsumers = 8, kStepThreads = (kStepConsumers + 1) * 32;

// Q: the tiles come from a device work queue -- the producer claims the next
// unclaimed tile with an atomic ticket, so CTAs that meet partial or
// inactive tiles take more of the others -- instead of a static stride over
// the list; the last CTA to finish resets the queue for the next launch.
// XS: the previous iterate X reaches the consumers through shared memory:
// each warp issues cp.async copies of its block's X rows when a tile starts
// and waits for them only after the stencil, so their latency never stalls
// the FMAs (without XS the lanes load X into registers directly).
template <class S, bool C, bool XS, bool Q>
__global__ void __launch_bounds__(kStepThreads, 1) cf_step_t(BlkArgs a, const int4* __restrict__ work, int nwork,
                                                             const float* __restrict__ Y, const float* __restrict__ X,
                                                             float* __restrict__ out, int step) {
  using SM = StepSmem<S>;
  extern __shared__ __align__(128) unsigned char smem[];
  StepMeta* meta = (StepMeta*)(smem + 2 * SM::stage);  // [2]
  uint64_t* full = (uint64_t*)(smem + 2 * SM::stage + 128);
  uint64_t* empty = full + 2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    mbar_init(full + 0, 1);
    mbar_init(full + 1, 1);
    mbar_init(empty + 0, kStepConsumers);
    mbar_init(empty + 1, kStepConsumers);
  }
  __syncthreads();
  if (warp == kStepConsumers) {  // ------------------------------- producer
    if (lane != 0) return;
    int i = 0;
    for (int t = blockIdx.x;; t += gridDim.x, i++) {
      int4 w = make_int4(0, 0, 0, 0);
      bool have = false;
      if constexpr (Q) {
        for (;;) {
          const int tq = atomicAdd(a.queue, 1);
          if (tq >= nwork) break;
          w = work[tq];
          if (a.active[w.x]) {
            have = true;
            break;
          }
        }
      } else {
        for (; t < nwork; t += gridDim.x) {
          w = work[t];
          if (a.active[w.x]) {
            have = true;
            break;
          }
        }
      }
      const int st = i & 1;
      if (i >= 2 && !mbar_wait(empty + st, ((i >> 1) - 1) & 1)) {
        atomicExch(a.err, 1);
        return;
      }
      StepMeta& m = meta[st];
      if (!have) {
        m.end = 1;
        mbar_arrive(full + st);
        if constexpr (Q) {
          // every claim of this CTA is done; the last CTA to get here resets
          // the queue (each CTA's claims precede its count in program order)
          __threadfence();
          if (atomicAdd(a.queue + 1, 1) == (int)gridDim.x - 1) {
            a.queue[0] = 0;
            a.queue[1] = 0;
            __threadfence();
          }
        }
        return;
      }
      const PatchDev P = a.patches[w.x];
      const float3 co = a.coef[(long long)w.x * a.max_steps + step];
      m.end = 0;
      m.W = P.W;
      m.H = P.H;
      m.y0 = w.y;
      m.x0 = w.z;
      m.vec = P.vec;
      m.cx = co.x;
      m.cy = co.y;
      m.cz = co.z;
      // rows past the patch's last row (+ the radius) feed no in-patch pixel
      const int ylast = min(w.y + ST_TY - 1, P.H - 1);
      const int ny = ylast - w.y + 1 + 2 * S::R, nc = ylast - w.y + 1;
      constexpr uint32_t yrow = SM::PW * kBlk * sizeof(float), crow = ST_TX * S::NC * sizeof(float);
      float* ys = (float*)(smem + st * SM::stage);
      float* cs = (float*)(smem + st * SM::stage + SM::y_bytes);
      mbar_expect_tx(full + st, (uint32_t)ny * yrow + (uint32_t)nc * crow);
      for (int r = 0; r < ny; r++)
        bulk_g2s(ys + (size_t)r * SM::PW * kBlk,
                 Y + (P.vec + (long long)(w.y - S::R + r) * P.W + (w.z - S::R)) * kBlk, yrow, full + st);
      for (int r = 0; r < nc; r++)
        bulk_g2s(cs + (size_t)r * ST_TX * S::NC, a.afull + (P.vec + (long long)(w.y + r) * P.W + w.z) * S::NC,
                 crow, full + st);
    }
  }
  // ------------------------------------------------------------ consumers
  // warp: a 4 x 4 block of the tile; half-warp h: its rows 2h, 2h+1; lane:
  // block columns col, col + 1
  const int by = (warp / (ST_TX / ST_B)) * ST_B + SB_R * (lane >> 4), bx = (warp % (ST_TX / ST_B)) * ST_B;
  const int col = 2 * (lane & 15);
  float* xslot = (float*)(smem + SM::bytes + (size_t)(warp < kStepConsumers ? warp : 0) * SM::x_slot);
  for (int i = 0;; i++) {
    const int st = i & 1;
    if (!mbar_wait(full + st, (i >> 1) & 1)) {
      if (lane == 0) atomicExch(a.err, 1);
      return;
    }
    const StepMeta m = meta[st];
    if (m.end) return;
    const float* ys = (const float*)(smem + st * SM::stage);
    const float* cs = (const float*)(smem + st * SM::stage + SM::y_bytes);
    // the previous iterate's values for this lane's columns, fetched now so
    // the loads overlap the stencil
    float2 xr[SB_N];
    if constexpr (XS) {
      if (m.cz != 0.f) {
        // the warp's 4 x 4 block: 16 pixel rows of 128 bytes, 128 chunks of 16
        const int wy = (warp / (ST_TX / ST_B)) * ST_B;
#pragma unroll
        for (int t = 0; t < 4; t++) {
          const int c = lane + 32 * t, pix = c >> 3, sub = c & 7;
          const int y = m.y0 + wy + (pix >> 2), x = m.x0 + bx + (pix & 3);
          const bool ok = y < m.H && x < m.W;
          cp_async16(xslot + pix * kBlk + sub * 4, ok ? X + (m.vec + (long long)y * m.W + x) * kBlk + sub * 4 : X,
                     ok ? 16u : 0u);
        }
        cp_async_commit();
      }
    } else {
#pragma unroll
      for (int k = 0; k < SB_N; k++) {
        const int y = m.y0 + by + k / SB_C, x = m.x0 + bx + k % SB_C;
        const bool ok = m.cz != 0.f && y < m.H && x < m.W;
        xr[k] = ok ? *(const float2*)(X + (m.vec + (long long)y * m.W + x) * kBlk + col) : make_float2(0.f, 0.f);
      }
    }
    float2 acc[SB_N], lo[SB_N], grp[SB_N];
    float4 cw[SB_N];
#pragma unroll
    for (int k = 0; k < SB_N; k++) acc[k] = lo[k] = grp[k] = make_float2(0.f, 0.f);
    step_positions<S, C, 0>(ys + (by * SM::PW + bx) * kBlk + col, cs + (by * ST_TX + bx) * S::NC, cw, acc, lo,
                            grp);
    if constexpr (XS) {
      if (m.cz != 0.f) {
        cp_async_wait_all();
        __syncwarp();
#pragma unroll
        for (int k = 0; k < SB_N; k++)
          xr[k] = *(const float2*)(xslot + ((SB_R * (lane >> 4) + k / SB_C) * ST_B + k % SB_C) * kBlk + col);
      }
    }
#pragma unroll
    for (int k = 0; k < SB_N; k++) {
      const int y = m.y0 + by + k / SB_C, x = m.x0 + bx + k % SB_C;
      if (y >= m.H || x >= m.W) continue;
      const long long q = m.vec + (long long)y * m.W + x;
      const float2 yc = *(const float2*)(ys + ((by + k / SB_C + S::R) * SM::PW + bx + k % SB_C + S::R) * kBlk + col);
      const float2 a0 = C ? make_float2(acc[k].x + lo[k].x, acc[k].y + lo[k].y) : acc[k];
      float2 r = make_float2(m.cx * a0.x + m.cy * yc.x, m.cx * a0.y + m.cy * yc.y);
      if (m.cz != 0.f) {
        r.x = fmaf(m.cz, xr[k].x, r.x);
        r.y = fmaf(m.cz, xr[k].y, r.y);
      }
      *(float2*)(out + q * kBlk + col) = r;
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(empty + st);
  }
}

// A ROWS x 16 tile's pixel-major rows (NC floats each), staged in shared
// memory by pixel 16 * ty + tx, out to their places: a tile row's pixels are
// adjacent in the layout, so each tile row leaves as one contiguous run of
// 16-byte stores.  (A thread writing its own row would give each warp store
// 32 scattered 16-byte pieces.)  Row strides of 21 and 13 float4 put the 8
// threads of a staging store's phase in distinct banks.
template <int NC, int ROWS>
__device__ __forceinline__ void tile_rows_out(const float4* __restrict__ rows, float* __restrict__ dst, long long vec,
                                              int W, int H, int y0, int x0) {
  constexpr int Q = NC / 4;
  const int ny = min(ROWS, H - y0), nx = min(16, W - x0);
  for (int i = threadIdx.x; i < ny * 16 * Q; i += blockDim.x) {
    const int r = i / (16 * Q), j = i % (16 * Q);
    if (j < nx * Q) ((float4*)(dst + (vec + (long long)(y0 + r) * W + x0) * NC))[j] = rows[r * 16 * Q + j];
  }
}

// pixel-major full stencil rows of the fine operator from its symmetric
// storage: row p holds A(p, p + off_e) for the 81 offsets e in scanline
// order (0 where the neighbour is outside the patch), then 3 zeros
constexpr int kFullRows = 8;  // tile rows per CTA: half of a 16 x 16 work tile
__global__ void __launch_bounds__(kFullRows * 16) cf_full(const PatchDev* __restrict__ patches,
                                                          const int4* __restrict__ work,
                                                          const float* __restrict__ a_up,
                                                          const float* __restrict__ a_diag, long long lvec,
                                                          float* __restrict__ afull) {
  // one thread per pixel of a half tile (43 KB of staging, so several CTAs
  // share an SM): the plane reads are coalesced across the warp; the rows go
  // out through shared memory
  constexpr int NC = DiskStencil::NC, ctr = kStencilN / 2;
  __shared__ float4 rows[kFullRows * 16 * (NC / 4)];
  const int4 w = work[blockIdx.x >> 1];
  const PatchDev P = patches[w.x];
  const int y0 = w.y + (blockIdx.x & 1) * kFullRows;
  const int y = y0 + threadIdx.x / 16, x = w.z + threadIdx.x % 16;
  if (y < P.H && x < P.W) {
    const long long p = P.vec + (long long)y * P.W + x;
#pragma unroll 3
    for (int e4 = 0; e4 < NC / 4; e4++) {
      float v[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int e = 4 * e4 + j;
        v[j] = 0.f;
        if (e >= kStencilN) continue;
        if (e == ctr) {
          v[j] = a_diag[p];
          continue;
        }
        // upper offsets are c_bup[e - 41]; the disk is point-symmetric, so
        // lower offset e mirrors upper offset 80 - e
        const int k = e > ctr ? e - ctr - 1 : kStencilN - 1 - e - ctr - 1;
        const int dy = e > ctr ? c_bup_dy[k] : -c_bup_dy[k];
        const int dx = e > ctr ? c_bup_dx[k] : -c_bup_dx[k];
        const int yy = y + dy, xx = x + dx;
        if (yy >= 0 && yy < P.H && xx >= 0 && xx < P.W)
          v[j] = e > ctr ? a_up[(long long)k * lvec + p] : a_up[(long long)k * lvec + p + (long long)dy * P.W + dx];
      }
      rows[threadIdx.x * (NC / 4) + e4] = make_float4(v[0], v[1], v[2], v[3]);
    }
  }
  __syncthreads();
  tile_rows_out<NC, kFullRows>(rows, afull, P.vec, P.W, P.H, y0, w.z);
}

// ------------------------------------------------------------------ Gram
__device__ __forceinline__ void ffp(float& hi, float& lo, float a, float b) {
  // __fmul_rn / __fadd_rn: never contracted into an FMA, which would break
  // the error-free transformations
  const float p = __fmul_rn(a, b);
  const float pe = fmaf(a, b, -p);
  const float s = __fadd_rn(hi, p);
  const float z = s - hi;
  lo += ((hi - (s - z)) + (p - z)) + pe;
  hi = s;
}

// G = U^T V over a tile of pixels.  Chunks of 256 pixel rows of U and V are
// staged in shared memory; four groups of 64 threads take 64 rows each, a
// thread owning a 4 x 4 block of G (two broadcast 16-byte loads feed 16
// FMAs).  Each group's 64-term FP32 FMA runs are folded into a float-float
// (hi, lo) pair by an error-free TwoSum, so the sum over the tile is as
// accurate as a compensated one at about the cost of plain FMAs; the four
// groups and then the tiles are summed in FP64.
constexpr int GR_CH = 256;  // pixels per staged chunk
__device__ __forceinline__ void two_sum_into(float& hi, float& lo, float x) {
  const float s = hi + x;
  const float bb = s - hi;
  lo += (hi - (s - bb)) + (x - bb);
  hi = s;
}

// The reductions and the rotation split each eigensolver tile (kEigTile
// pixels) into kBlkSplit runs, one CTA each, so a launch has several CTAs
// per SM and no near-empty last wave.  A CTA's partial sums are float-float
// pairs in slot blockIdx.x of a.part; the last CTA of a patch adds the
// slots [tile_begin, tile_begin + tile_count) x kBlkSplit in order, in
// float-float on the FP32 pipes (one SM adding them in FP64 would take tens
// of microseconds at GB300's FP64 rate).
__device__ __forceinline__ void ff2_add(float2& s, float2 b) {
  const float t = s.x + b.x;
  const float z = t - s.x;
  s.y += ((s.x - (t - z)) + (b.x - z)) + b.y;
  s.x = t;
}
struct BlkRun {
  EigTile t;
  int p0, p1;
};
__device__ __forceinline__ BlkRun blk_run(const BlkArgs& a) {
  BlkRun r;
  r.t = a.tiles[blockIdx.x / kBlkSplit];
  const int len = (r.t.p1 - r.t.p0 + kBlkSplit - 1) / kBlkSplit;
  r.p0 = min(r.t.p1, r.t.p0 + (int)(blockIdx.x % kBlkSplit) * len);
  r.p1 = min(r.t.p1, r.p0 + len);
  return r;
}
// true in every thread of the last CTA of patch t.patch to arrive
__device__ __forceinline__ bool blk_last(const BlkArgs& a, int patch) {
  __shared__ int is_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const int prev = atomicAdd(a.counter + patch, 1);
    is_last = (prev == a.tile_count[patch] * kBlkSplit - 1);
    if (is_last) a.counter[patch] = 0;
  }
  __syncthreads();
  if (is_last) __threadfence();
  return is_last;
}
// sum of element e over the patch's CTA slots (stride floats2 per slot)
__device__ __forceinline__ double blk_sum(const BlkArgs& a, int patch, int e, int stride) {
  const float2* part = (const float2*)a.part;
  const int b0 = a.tile_begin[patch] * kBlkSplit, b1 = b0 + a.tile_count[patch] * kBlkSplit;
  float2 acc = make_float2(0.f, 0.f);
  for (int b = b0; b < b1; b++) ff2_add(acc, part[(long long)b * stride + e]);
  return (double)acc.x + (double)acc.y;
}

// TWO: one pass computes out = U^T V and out2 = U^T U (the Rayleigh-Ritz
// step's two Gram matrices), each element with the same operations in the
// same order as a pass of its own, so the results are the same to the bit.
template <bool TWO>
__global__ void __launch_bounds__(256, TWO ? 2 : 3) cf_gram(BlkArgs a, const float* __restrict__ U,
                                                            const float* __restrict__ V, double* __restrict__ out,
                                                            double* __restrict__ out2) {
  const BlkRun run = blk_run(a);
  const EigTile t = run.t;
  if (!a.active[t.patch]) return;
  const PatchDev P = a.patches[t.patch];
  extern __shared__ __align__(16) float gsm[];  // us[GR_CH][32], vs[GR_CH][32]; reused for the group sums
  float* us = gsm;
  float* vs = gsm + GR_CH * kBlk;
  const int grp = threadIdx.x >> 6, lt = threadIdx.x & 63;
  const int i0 = (lt >> 3) * 4, j0 = (lt & 7) * 4;
  constexpr int NG = TWO ? 2 : 1;  // Gram matrices formed
  float hi[NG][16], lo[NG][16];
#pragma unroll
  for (int g = 0; g < NG; g++)
#pragma unroll
    for (int k = 0; k < 16; k++) hi[g][k] = lo[g][k] = 0.f;
  for (int p0 = run.p0; p0 < run.p1; p0 += GR_CH) {
    __syncthreads();
    for (int f = threadIdx.x; f < GR_CH * kBlk / 4; f += blockDim.x) {
      const int pp = f / (kBlk / 4), c4 = f % (kBlk / 4);
      const int p = p0 + pp;
      float4 u = make_float4(0.f, 0.f, 0.f, 0.f), v = u;
      if (p < run.p1) {
        u = ((const float4*)(U + (P.vec + p) * kBlk))[c4];
        v = ((const float4*)(V + (P.vec + p) * kBlk))[c4];
      }
      ((float4*)us)[f] = u;
      ((float4*)vs)[f] = v;
    }
    __syncthreads();
    float acc[NG][16];
#pragma unroll
    for (int g = 0; g < NG; g++)
#pragma unroll
      for (int k = 0; k < 16; k++) acc[g][k] = 0.f;
    const int pbeg = grp * (GR_CH / 4);
#pragma unroll(TWO ? 2 : 4)
    for (int pp = pbeg; pp < pbeg + GR_CH / 4; pp++) {
      const float4 u4 = *(const float4*)(us + pp * kBlk + i0);
      const float4 v4 = *(const float4*)(vs + pp * kBlk + j0);
      const float uu[4] = {u4.x, u4.y, u4.z, u4.w}, vv[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
      for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[0][r * 4 + c] = fmaf(uu[r], vv[c], acc[0][r * 4 + c]);
      if constexpr (TWO) {
        const float4 w4 = *(const float4*)(us + pp * kBlk + j0);
        const float ww[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
          for (int c = 0; c < 4; c++) acc[NG - 1][r * 4 + c] = fmaf(uu[r], ww[c], acc[NG - 1][r * 4 + c]);
      }
    }
#pragma unroll
    for (int g = 0; g < NG; g++)
#pragma unroll
      for (int k = 0; k < 16; k++) two_sum_into(hi[g][k], lo[g][k], acc[g][k]);
  }
  // the four groups' blocks, summed in float-float
  __syncthreads();
  float2* red = (float2*)gsm;  // [NG][4][32 * 32] (64 KB for two)
#pragma unroll
  for (int g = 0; g < NG; g++)
#pragma unroll
    for (int k = 0; k < 16; k++)
      red[(g * 4 + grp) * kBlk * kBlk + (i0 + k / 4) * kBlk + j0 + k % 4] = make_float2(hi[g][k], lo[g][k]);
  __syncthreads();
  float2* part = (float2*)a.part + (long long)blockIdx.x * NG * kBlk * kBlk;
  for (int e = threadIdx.x; e < NG * kBlk * kBlk; e += blockDim.x) {
    const int g = e / (kBlk * kBlk), el = e % (kBlk * kBlk);
    float2 sum = red[g * 4 * kBlk * kBlk + el];
    for (int q = 1; q < 4; q++) ff2_add(sum, red[(g * 4 + q) * kBlk * kBlk + el]);
    part[e] = sum;
  }
  if (!blk_last(a, t.patch)) return;
  for (int e = threadIdx.x; e < NG * kBlk * kBlk; e += blockDim.x) {
    const int g = e / (kBlk * kBlk), el = e % (kBlk * kBlk);
    (g ? out2 : out)[(long long)t.patch * kBlk * kBlk + el] = blk_sum(a, t.patch, e, NG * kBlk * kBlk);
  }
}

// U <- U M (and V <- V M if V), M = a.mat[patch] (32 x 32, FP64 on the
// host), two pixel rows per thread.  C (the Rayleigh-Ritz rotation): M is
// split into FP32 hi + lo parts; each output sums its products with hi by
// FMA in groups of four, folded into a float-float by an exact TwoSum, and
// its products with lo by FMA into the low word, so the Ritz vectors carry
// little more than FP32 storage rounding; a plain FP32 sum (enough for the
// orthonormalisation passes, which the next Rayleigh-Ritz step corrects)
// leaves ~3e-7 relative error per element.
// Each warp stages its own 64 rows in shared memory -- coalesced 16-byte
// loads in, the rotation on each lane's two rows there, coalesced stores
// out -- synchronising only with __syncwarp, so the warps of a CTA overlap
// their load, compute and store phases.  (Threads loading their own 128-byte
// rows from global memory made every warp access touch 32 lines; staging
// behind CTA-wide barriers serialised the phases.)  Row pitch 36 floats: the
// 8 lanes of a 16-byte access phase reach 8 rows in distinct banks.
constexpr int RW_ROWS = 64, RW_PITCH = kBlk + 4;
constexpr int kRotSmem = 8 * RW_ROWS * RW_PITCH * sizeof(float);
static_assert(8 * RW_ROWS == kEigTile / kBlkSplit, "8 warps x 64 rows cover a CTA's run");
template <bool C>
__global__ void __launch_bounds__(256) cf_rotate(BlkArgs a, float* __restrict__ U, float* __restrict__ V,
                                                 int ncols) {
  const BlkRun run = blk_run(a);
  const EigTile t = run.t;
  if (!a.active[t.patch]) return;
  const PatchDev P = a.patches[t.patch];
  extern __shared__ __align__(16) float rsm[];  // [8 warps][RW_ROWS][RW_PITCH]
  __shared__ __align__(16) float mh[kBlk][kBlk], ml[kBlk][kBlk];
  const double* M = a.mat + (long long)t.patch * kBlk * kBlk;
  for (int e = threadIdx.x; e < kBlk * kBlk; e += blockDim.x) {
    const double m = M[e];
    const float h = (float)m;
    mh[e / kBlk][e % kBlk] = h;
    ml[e / kBlk][e % kBlk] = (float)(m - (double)h);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wp0 = run.p0 + warp * RW_ROWS;
  const int n = max(0, min(RW_ROWS, run.p1 - wp0));
  float* ws = rsm + warp * RW_ROWS * RW_PITCH;
  for (int which = 0; which < (V ? 2 : 1); which++) {
    float4* g4 = (float4*)((which ? V : U) + (P.vec + wp0) * kBlk);
    for (int f = lane; f < n * (kBlk / 4); f += 32) *(float4*)(ws + (f >> 3) * RW_PITCH + (f & 7) * 4) = g4[f];
    __syncwarp();
    // two rows per lane, so each broadcast load of M feeds both
    if (lane < n) {
      const bool ok1 = lane + 32 < n;
      float* rows[2];
      rows[0] = ws + lane * RW_PITCH;
      rows[1] = ok1 ? rows[0] + 32 * RW_PITCH : rows[0];
      float x[2][kBlk];
#pragma unroll
      for (int k = 0; k < 2; k++)
#pragma unroll
        for (int c = 0; c < kBlk; c += 4) {
          const float4 v = *(const float4*)(rows[k] + c);
          x[k][c] = v.x;
          x[k][c + 1] = v.y;
          x[k][c + 2] = v.z;
          x[k][c + 3] = v.w;
        }
#pragma unroll 1
      for (int c0 = 0; c0 < kBlk; c0 += 4) {
        float hi[2][4], lo[2][4], g[2][4];
#pragma unroll
        for (int k = 0; k < 2; k++)
#pragma unroll
          for (int j = 0; j < 4; j++) hi[k][j] = lo[k][j] = g[k][j] = 0.f;
#pragma unroll
        for (int r = 0; r < kBlk; r++) {
          const float4 h4 = *(const float4*)&mh[r][c0];  // broadcast: every thread reads the same row
          const float hh[4] = {h4.x, h4.y, h4.z, h4.w};
          float ll[4] = {0.f, 0.f, 0.f, 0.f};
          if constexpr (C) {
            const float4 l4 = *(const float4*)&ml[r][c0];
            ll[0] = l4.x;
            ll[1] = l4.y;
            ll[2] = l4.z;
            ll[3] = l4.w;
          }
#pragma unroll
          for (int k = 0; k < 2; k++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
              if constexpr (C) {
                g[k][j] = fmaf(x[k][r], hh[j], g[k][j]);
                lo[k][j] = fmaf(x[k][r], ll[j], lo[k][j]);
                if ((r & 3) == 3) {  // r is a compile-time constant here
                  const float sum = hi[k][j] + g[k][j], z = sum - hi[k][j];
                  lo[k][j] += (hi[k][j] - (sum - z)) + (g[k][j] - z);
                  hi[k][j] = sum;
                  g[k][j] = 0.f;
                }
              } else {
                hi[k][j] = fmaf(x[k][r], hh[j], hi[k][j]);
              }
            }
        }
        if (c0 < ncols) {
          *(float4*)(rows[0] + c0) = make_float4(hi[0][0] + lo[0][0], hi[0][1] + lo[0][1], hi[0][2] + lo[0][2],
                                                 hi[0][3] + lo[0][3]);
          if (ok1)
            *(float4*)(rows[1] + c0) = make_float4(hi[1][0] + lo[1][0], hi[1][1] + lo[1][1], hi[1][2] + lo[1][2],
                                                   hi[1][3] + lo[1][3]);
        }
      }
    }
    __syncwarp();
    for (int f = lane; f < n * (kBlk / 4); f += 32) g4[f] = *(const float4*)(ws + (f >> 3) * RW_PITCH + (f & 7) * 4);
    __syncwarp();
  }
}

// per-column |A x_c - theta_c x_c|^2 (AX and X given), last CTA sums
__global__ void __launch_bounds__(256) cf_resid(BlkArgs a, const float* __restrict__ X,
                                                const float* __restrict__ AX, double* __restrict__ out) {
  const BlkRun run = blk_run(a);
  const EigTile t = run.t;
  if (!a.active[t.patch]) return;
  const PatchDev P = a.patches[t.patch];
  const int c = threadIdx.x & 31, lanegroup = threadIdx.x >> 5;
  const float th = (float)a.theta[(long long)t.patch * kBlk + c];
  float hi = 0.f, lo = 0.f;
#pragma unroll 4
  for (int p = run.p0 + lanegroup; p < run.p1; p += 8) {
    const long long q = (P.vec + p) * kBlk + c;
    const float r = fmaf(-th, X[q], AX[q]);
    ffp(hi, lo, r, r);
  }
  __shared__ float2 red[8][kBlk];
  red[lanegroup][c] = make_float2(hi, lo);
  __syncthreads();
  if (threadIdx.x < kBlk) {
    float2 sum = red[0][threadIdx.x];
    for (int g = 1; g < 8; g++) ff2_add(sum, red[g][threadIdx.x]);
    ((float2*)a.part)[(long long)blockIdx.x * kBlk + threadIdx.x] = sum;
  }
  if (!blk_last(a, t.patch)) return;
  if (threadIdx.x < kBlk) out[(long long)t.patch * kBlk + threadIdx.x] = blk_sum(a, t.patch, threadIdx.x, kBlk);
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
// coarse degrees d_c(P) = the sum of the fine degrees of P's pixels (the
// row sums of W_c, since W_c(P, Q) sums W over P x Q), and D_c^-1/2
__global__ void __launch_bounds__(256) cf_coarse_deg(CoarseArgs c) {
  const int4 w = c.work[blockIdx.x];  // coarse (patch, Y0, X0)
  const PatchDev F = c.fine[w.x], C = c.coarse[w.x];
  const int Y = w.y + threadIdx.x / 16, X = w.z + threadIdx.x % 16;
  if (Y >= C.H || X >= C.W) return;
  double deg = 0.0;
  for (int sy = 0; sy < 2; sy++)
    for (int sx = 0; sx < 2; sx++) {
      const int y = 2 * Y + sy, x = 2 * X + sx;
      if (y < F.H && x < F.W) deg += c.deg[F.vec + (long long)y * F.W + x];
    }
  const long long P = C.vec + (long long)Y * C.W + X;
  c.degc[P] = (float)deg;
  c.disc[P] = (float)(1.0 / sqrt(deg));
}

// coarse stencil index of fine displacement (a, b) from sub-pixel (0, 0):
// coarse offset (floor(a / 2), floor(b / 2)), a, b in [-5, 6]
__host__ __device__ constexpr int cidx(int a, int b) {
  return ((a + 8) / 2 - 4 + kCR) * kCW + (b + 8) / 2 - 4 + kCR;
}
static_assert(cidx(0, 0) == kCR * kCW + kCR && cidx(-5, -5) == 0 && cidx(6, 6) == kCN - 1, "coarse offsets");

// upper offset j's displacement (the inverse of upper_k)
__host__ __device__ constexpr int upper_dy_from(int j, int dy) {
  return j < 2 * disk_half_width(dy) + 1 ? dy : upper_dy_from(j - 2 * disk_half_width(dy) - 1, dy + 1);
}
__host__ __device__ constexpr int upper_dy(int j) { return j < kStencilR ? 0 : upper_dy_from(j - kStencilR, 1); }
__host__ __device__ constexpr int upper_dx(int j) {
  return upper_dy(j) == 0 ? j + 1 : j - upper_k(upper_dy(j), 0);
}
static_assert(upper_dy(0) == 0 && upper_dx(0) == 1 && upper_dy(5) == 1 && upper_dx(5) == -4 &&
                  upper_dy(kUpper - 1) == kStencilR && upper_dx(kUpper - 1) == 0 && upper_k(upper_dy(23), upper_dx(23)) == 23,
              "upper offset inverse");

// the terms of fine sub-pixel (SY, SX) of a coarse pixel: upper offset J's
// lower neighbour q = p - (dy,dx) (its upper entry at q), then its upper
// neighbour q = p + (dy,dx); each lands on a compile-time coarse offset
template <int SY, int SX, int J>
__device__ __forceinline__ void coarsen_terms(float (&acc)[kCN], const float* __restrict__ wsym, long long lvec,
                                              long long p, int y, int x, int H, int W) {
  if constexpr (J < kUpper) {
    constexpr int dy = upper_dy(J), dx = upper_dx(J);
    const float* plane = wsym + (long long)J * lvec;
    if (y - dy >= 0 && x - dx >= 0 && x - dx < W) acc[cidx(SY - dy, SX - dx)] += plane[p - (dy * W + dx)];
    if (y + dy < H && x + dx >= 0 && x + dx < W) acc[cidx(SY + dy, SX + dx)] += plane[p];
    coarsen_terms<SY, SX, J + 1>(acc, wsym, lvec, p, y, x, H, W);
  }
}
template <int SY, int SX>
__device__ __forceinline__ void coarsen_sub(float (&acc)[kCN], const CoarseArgs& c, const PatchDev& F, int Y, int X) {
  const int y = 2 * Y + SY, x = 2 * X + SX;
  if (y < F.H && x < F.W) {
    acc[kCR * kCW + kCR] += 1.f;  // w_pp = 1
    coarsen_terms<SY, SX, 0>(acc, c.wsym_up, c.lvec_f, F.vec + (long long)y * F.W + x, y, x, F.H, F.W);
  }
}

// W_c row of one coarse pixel, then A_c = I - D_c^-1/2 W_c D_c^-1/2 on it.
// The fine offsets, the two signs and the 2 x 2 sub-pixels are unrolled at
// compile time, so every term's coarse offset -- floor((s + dy) / 2) for
// sub-pixel s -- is a constant and the 49 sums stay in registers.  Terms
// are added per sum in the order: sub-pixel, upper offset, lower before
// upper neighbour.
__global__ void __launch_bounds__(256) cf_coarsen(CoarseArgs c) {
  extern __shared__ float4 rows[];  // [256][13]
  const int4 w = c.work[blockIdx.x];
  const PatchDev F = c.fine[w.x], C = c.coarse[w.x];
  constexpr int NC = SquareStencil::NC;
  const int Y = w.y + threadIdx.x / 16, X = w.z + threadIdx.x % 16;
  if (Y < C.H && X < C.W) {
    float acc[kCN];
#pragma unroll
    for (int k = 0; k < kCN; k++) acc[k] = 0.f;
    coarsen_sub<0, 0>(acc, c, F, Y, X);
    coarsen_sub<0, 1>(acc, c, F, Y, X);
    coarsen_sub<1, 0>(acc, c, F, Y, X);
    coarsen_sub<1, 1>(acc, c, F, Y, X);
    const long long P = C.vec + (long long)Y * C.W + X;
    const float dp = c.disc[P];
    float v[NC];
#pragma unroll
    for (int k = 0; k < NC; k++) {
      v[k] = 0.f;
      if (k >= kCN) continue;
      const int dY = k / kCW - kCR, dX = k % kCW - kCR;
      const int YY = Y + dY, XX = X + dX;
      if (YY >= 0 && YY < C.H && XX >= 0 && XX < C.W)
        v[k] = -acc[k] * dp * c.disc[C.vec + (long long)YY * C.W + XX];
      if (k == kCR * kCW + kCR) v[k] += 1.f;
    }
#pragma unroll
    for (int q = 0; q < NC / 4; q++)
      rows[threadIdx.x * (NC / 4) + q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
  }
  __syncthreads();
  tile_rows_out<NC, 16>(rows, c.wc, C.vec, C.W, C.H, w.y, w.z);
}

// fine start block from the coarse Ritz vectors: the coarse generalised
// eigenvectors u_c = D_c^-1/2 y_c interpolated bilinearly to the fine pixel
// centres (clamped at the patch border), then y = D^1/2 u.  Smoother than
// the piecewise-constant P u_c of the Galerkin pair, so the fine level
// starts closer to its eigenvectors.
__global__ void __launch_bounds__(256) cf_prolong(CoarseArgs c, const float* __restrict__ xc,
                                                  float* __restrict__ xf) {
  const int4 w = c.work_f[blockIdx.x];  // fine (patch, y0, x0)
  const PatchDev F = c.fine[w.x], C = c.coarse[w.x];
  const int y = w.y + threadIdx.x / 16, x = w.z + threadIdx.x % 16;
  if (y >= F.H || x >= F.W) return;
  const long long p = F.vec + (long long)y * F.W + x;
  // fine centre in coarse pixel coordinates
  const float cy = fminf(fmaxf((y + 0.5f) * 0.5f - 0.5f, 0.f), (float)(C.H - 1));
  const float cx = fminf(fmaxf((x + 0.5f) * 0.5f - 0.5f, 0.f), (float)(C.W - 1));
  const int y0 = (int)cy, x0 = (int)cx;
  const int y1 = min(y0 + 1, C.H - 1), x1 = min(x0 + 1, C.W - 1);
  const float fy = cy - y0, fx = cx - x0;
  const long long P00 = C.vec + (long long)y0 * C.W + x0, P01 = C.vec + (long long)y0 * C.W + x1;
  const long long P10 = C.vec + (long long)y1 * C.W + x0, P11 = C.vec + (long long)y1 * C.W + x1;
  const float sq = sqrtf(c.deg[p]);
  const float w00 = (1.f - fy) * (1.f - fx) * c.disc[P00] * sq, w01 = (1.f - fy) * fx * c.disc[P01] * sq;
  const float w10 = fy * (1.f - fx) * c.disc[P10] * sq, w11 = fy * fx * c.disc[P11] * sq;
  const float4* a = (const float4*)(xc + P00 * kBlk);
  const float4* b = (const float4*)(xc + P01 * kBlk);
  const float4* cc = (const float4*)(xc + P10 * kBlk);
  const float4* d = (const float4*)(xc + P11 * kBlk);
  float4* dst = (float4*)(xf + p * kBlk);
#pragma unroll
  for (int c4 = 0; c4 < kBlk / 4; c4++) {
    const float4 va = a[c4], vb = b[c4], vc = cc[c4], vd = d[c4];
    float4 v;
    v.x = w00 * va.x + w01 * vb.x + w10 * vc.x + w11 * vd.x;
    v.y = w00 * va.y + w01 * vb.y + w10 * vc.y + w11 * vd.y;
    v.z = w00 * va.z + w01 * vb.z + w10 * vc.z + w11 * vd.z;
    v.w = w00 * va.w + w01 * vb.w + w10 * vc.w + w11 * vd.w;
    dst[c4] = v;
  }
}

constexpr int kCoarsenSmem = 256 * kCoarseNC * sizeof(float);
cudaError_t cf_launch_coarsen(const CoarseArgs& c, int nwork_c, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(cf_coarsen, cudaFuncAttributeMaxDynamicSharedMemorySize, kCoarsenSmem);
    attr = true;
  }
  cf_coarse_deg<<<nwork_c, 256, 0, s>>>(c);
  cf_coarsen<<<nwork_c, 256, kCoarsenSmem, s>>>(c);
  return cudaGetLastError();
}
cudaError_t cf_launch_prolong(const CoarseArgs& c, int nwork_f, const float* xc, float* xf, cudaStream_t s) {
  cf_prolong<<<nwork_f, 256, 0, s>>>(c, xc, xf);
  return cudaGetLastError();
}

template <class S, bool C, bool XS, bool Q>
static void step_attr() {
  cudaFuncSetAttribute(cf_step_t<S, C, XS, Q>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(XS ? StepSmem<S>::bytes_xs : StepSmem<S>::bytes));
}
template <class S, bool C>
static void step_attrs() {
  step_attr<S, C, false, false>();
  step_attr<S, C, true, false>();
  step_attr<S, C, false, true>();
  step_attr<S, C, true, true>();
}

template <class S, bool C>
static void step_go(const BlkArgs& a, const int4* work, int nwork, const float* Y, const float* X, float* out,
                    int step, int grid, int variant, cudaStream_t s) {
#define GPB_STEP(XS, Q)                                                                                  \
  cf_step_t<S, C, XS, Q><<<grid, kStepThreads, XS ? StepSmem<S>::bytes_xs : StepSmem<S>::bytes, s>>>( \
      a, work, nwork, Y, X, out, step)
  switch (variant & 3) {
    case 0: GPB_STEP(false, false); break;
    case 1: GPB_STEP(true, false); break;
    case 2: GPB_STEP(false, true); break;
    default: GPB_STEP(true, true); break;
  }
#undef GPB_STEP
}

cudaError_t cf_launch_step(const BlkArgs& a, const int4* work, int nwork, const float* Y, const float* X, float* out,
                           int step, cudaStream_t s, bool comp, int variant) {
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    step_attrs<DiskStencil, false>();
    step_attrs<DiskStencil, true>();
    step_attrs<SquareStencil, false>();
    step_attrs<SquareStencil, true>();
    if (nsm <= 0) nsm = 1;
  }
  const int grid = std::min(nwork, nsm);  // one persistent CTA per SM
  if (grid <= 0) return cudaSuccess;
  if (a.coarse) {
    if (comp) step_go<SquareStencil, true>(a, work, nwork, Y, X, out, step, grid, variant, s);
    else step_go<SquareStencil, false>(a, work, nwork, Y, X, out, step, grid, variant, s);
  } else {
    if (comp) step_go<DiskStencil, true>(a, work, nwork, Y, X, out, step, grid, variant, s);
    else step_go<DiskStencil, false>(a, work, nwork, Y, X, out, step, grid, variant, s);
  }
  return cudaGetLastError();
}
cudaError_t cf_launch_full(const PatchDev* patches, const int4* work16, int nwork, const float* a_up,
                           const float* a_diag, long long lvec, float* afull, cudaStream_t s) {
  cf_full<<<2 * nwork, kFullRows * 16, 0, s>>>(patches, work16, a_up, a_diag, lvec, afull);
  return cudaGetLastError();
}
cudaError_t cf_launch_gram(const BlkArgs& a, int ntiles, const float* U, const float* V, double* out,
                           cudaStream_t s, double* out2) {
  constexpr int smem = 2 * GR_CH * kBlk * sizeof(float);  // 64 KB; the group sums (32 or 64 KB) reuse it
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(cf_gram<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(cf_gram<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    attr = true;
  }
  if (out2)
    cf_gram<true><<<ntiles * kBlkSplit, 256, smem, s>>>(a, U, V, out, out2);
  else
    cf_gram<false><<<ntiles * kBlkSplit, 256, smem, s>>>(a, U, V, out, nullptr);
  return cudaGetLastError();
}
cudaError_t cf_launch_rotate(const BlkArgs& a, int ntiles, float* U, float* V, int ncols, cudaStream_t s,
                             bool comp) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(cf_rotate<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kRotSmem);
    cudaFuncSetAttribute(cf_rotate<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kRotSmem);
    attr = true;
  }
  if (comp)
    cf_rotate<true><<<ntiles * kBlkSplit, 256, kRotSmem, s>>>(a, U, V, ncols);
  else
    cf_rotate<false><<<ntiles * kBlkSplit, 256, kRotSmem, s>>>(a, U, V, ncols);
  return cudaGetLastError();
}
cudaError_t cf_launch_resid(const BlkArgs& a, int ntiles, const float* X, const float* AX, double* out,
                            cudaStream_t s) {
  cf_resid<<<ntiles * kBlkSplit, 256, 0, s>>>(a, X, AX, out);
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
