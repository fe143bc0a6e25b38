// k_learned.cu -- the learned warm start's network: forward, loss and
// backward kernels, BF16 operands on the tensor cores (mma.sync m16n8k16)
// with FP32 accumulation, and Adam.
//
// Tensors are per level, channel-innermost ([pixel][channel]), the patches of
// a batch back to back (LnPatch offsets).  Activations are BF16; gradients
// are FP32 and are rounded to BF16 only where a convolution feeds them to the
// tensor cores.
//
//   k_ln_conv    3 x 3 convolution as an implicit GEMM over an 8 x 16 output
//                tile: the tile's input with a 1-pixel halo and the weights
//                of a chunk of output channels are staged in shared memory;
//                each of 4 warps computes two 16-pixel rows x the chunk.
//                Forward (ReLU to BF16, or the head to FP32), and the
//                data gradient (the masked FP32 output gradient staged as
//                BF16, convolved with the flipped, transposed weights).
//   k_ln_wgrad   weight and bias gradients: per (tap, 16-channel chunk) a
//                CTA accumulates dW = dZ^T X over its share of the tiles on
//                the tensor cores, then adds it to the FP32 gradient.
//   pooling, up-sampling + concatenation and their gradients, the subspace
//   loss reductions and its gradient, Adam, the weights' BF16 copies.
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "k_block.h"
#include "k_learned.h"

namespace gpb {

const LnConv kLnNet[kLnConvs] = {
    {16, 16, 1},  {16, 16, 1},  {16, 32, 1}, {32, 32, 1}, {32, 64, 1}, {64, 64, 1}, {64, 64, 1}, {64, 64, 1},
    {128, 64, 1}, {64, 64, 1},  {96, 32, 1}, {32, 32, 1}, {48, 16, 1}, {16, 16, 1}, {16, 32, 0}};

static void conv_offsets(size_t* wo, size_t* bo, size_t* total) {
  size_t o = 0;
  for (int i = 0; i < kLnConvs; i++) {
    wo[i] = o;
    o += (size_t)kLnNet[i].cout * 9 * kLnNet[i].cin;
    bo[i] = o;
    o += kLnNet[i].cout;
  }
  *total = o;
}

size_t ln_nparams() {
  size_t wo[kLnConvs], bo[kLnConvs], t;
  conv_offsets(wo, bo, &t);
  return t;
}

namespace {

typedef __nv_bfloat16 bf16;
constexpr int TH = 8, TW = 16, HP = TH + 2, WP = TW + 2, NHALO = HP * WP;  // tile, halo tile
constexpr int kConvThreads = 128;

__device__ __forceinline__ uint32_t ld32(const bf16* p) { return *(const uint32_t*)p; }

__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *(const uint32_t*)&v;
}

// MODE 0: forward, ReLU, BF16 out.  1: forward head, FP32 out.
// 2: data gradient: `in` is the FP32 output gradient of the layer being
//    differentiated (CIN = its channels), masked by its BF16 activation
//    (mask, may be null) and rounded to BF16; w is the flipped, transposed
//    weight; FP32 out, no bias.
template <int CIN, int CO, int MODE>
__global__ void __launch_bounds__(kConvThreads) k_ln_conv(const LnPatch* __restrict__ lp,
                                                          const LnTile* __restrict__ tiles,
                                                          const void* __restrict__ in,
                                                          const bf16* __restrict__ mask,
                                                          const bf16* __restrict__ w, const float* __restrict__ bias,
                                                          void* __restrict__ out, int cout_total) {
  constexpr int SI = CIN + 8, SW = 9 * CIN + 8;  // padded shared row strides (bank spread)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  bf16* in_s = (bf16*)smem_raw;
  bf16* w_s = in_s + NHALO * SI;
  const LnTile t = tiles[blockIdx.x];
  const LnPatch P = lp[t.patch];
  const int co0 = blockIdx.y * CO;
  // stage the input tile with its halo (zeros outside the patch)
  for (int idx = threadIdx.x; idx < NHALO * (CIN / 8); idx += blockDim.x) {
    const int h = idx / (CIN / 8), q = idx % (CIN / 8);
    const int y = t.y0 - 1 + h / WP, x = t.x0 - 1 + h % WP;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (y >= 0 && y < P.H && x >= 0 && x < P.W) {
      const long long pix = P.off + (long long)y * P.W + x;
      if constexpr (MODE == 2) {
        const float* g = (const float*)in + pix * CIN + q * 8;
        const float4 g0 = *(const float4*)g, g1 = *(const float4*)(g + 4);
        float f[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
        if (mask) {
          const uint4 mk = *(const uint4*)(mask + pix * CIN + q * 8);
          const bf16* m = (const bf16*)&mk;
#pragma unroll
          for (int k = 0; k < 8; k++)
            if (!(__bfloat162float(m[k]) > 0.f)) f[k] = 0.f;
        }
        v = make_uint4(pack2(f[0], f[1]), pack2(f[2], f[3]), pack2(f[4], f[5]), pack2(f[6], f[7]));
      } else {
        v = *(const uint4*)((const bf16*)in + pix * CIN + q * 8);
      }
    }
    *(uint4*)(in_s + h * SI + q * 8) = v;
  }
  // stage this CTA's output channels of the weights
  for (int idx = threadIdx.x; idx < CO * (9 * CIN / 8); idx += blockDim.x) {
    const int r = idx / (9 * CIN / 8), q = idx % (9 * CIN / 8);
    *(uint4*)(w_s + r * SW + q * 8) = *(const uint4*)(w + (long long)(co0 + r) * 9 * CIN + q * 8);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tg = lane & 3;
  float acc[2][CO / 8][4];
#pragma unroll
  for (int mt = 0; mt < 2; mt++)
#pragma unroll
    for (int nt = 0; nt < CO / 8; nt++)
#pragma unroll
      for (int k = 0; k < 4; k++) acc[mt][nt][k] = 0.f;
#pragma unroll 1
  for (int tap = 0; tap < 9; tap++) {
    const int dy = tap / 3, dx = tap % 3;
#pragma unroll
    for (int kc = 0; kc < CIN / 16; kc++) {
      uint32_t a[2][4];
#pragma unroll
      for (int mt = 0; mt < 2; mt++) {
        const bf16* r0 = in_s + ((2 * warp + mt + dy) * WP + dx + g) * SI + kc * 16 + 2 * tg;
        a[mt][0] = ld32(r0);
        a[mt][1] = ld32(r0 + 8 * SI);
        a[mt][2] = ld32(r0 + 8);
        a[mt][3] = ld32(r0 + 8 * SI + 8);
      }
#pragma unroll
      for (int nt = 0; nt < CO / 8; nt++) {
        const bf16* wr = w_s + (nt * 8 + g) * SW + tap * CIN + kc * 16 + 2 * tg;
        const uint32_t b0 = ld32(wr), b1 = ld32(wr + 8);
#pragma unroll
        for (int mt = 0; mt < 2; mt++) mma_bf16(acc[mt][nt], a[mt][0], a[mt][1], a[mt][2], a[mt][3], b0, b1);
      }
    }
  }
  // epilogue: accumulator rows are tile pixels x = g (c0, c1) and g + 8
  // (c2, c3) of tile row 2 warp + mt; columns are channels 2 tg, 2 tg + 1
#pragma unroll
  for (int mt = 0; mt < 2; mt++) {
    const int y = t.y0 + 2 * warp + mt;
    if (y >= P.H) continue;
#pragma unroll
    for (int half = 0; half < 2; half++) {
      const int x = t.x0 + g + 8 * half;
      if (x >= P.W) continue;
      const long long pix = P.off + (long long)y * P.W + x;
#pragma unroll
      for (int nt = 0; nt < CO / 8; nt++) {
        const int ch = co0 + nt * 8 + 2 * tg;
        float v0 = acc[mt][nt][2 * half], v1 = acc[mt][nt][2 * half + 1];
        if constexpr (MODE == 0) {
          v0 = fmaxf(v0 + bias[ch], 0.f);
          v1 = fmaxf(v1 + bias[ch + 1], 0.f);
          *(uint32_t*)((bf16*)out + pix * cout_total + ch) = pack2(v0, v1);
        } else if constexpr (MODE == 1) {
          *(float2*)((float*)out + pix * cout_total + ch) = make_float2(v0 + bias[ch], v1 + bias[ch + 1]);
        } else {
          *(float2*)((float*)out + pix * cout_total + ch) = make_float2(v0, v1);
        }
      }
    }
  }
}

// dW[n][tap][c] += sum over pixels of dZ[p][n] X[p + tap][c] for the CTA's
// tap and 16-channel chunk c0 (blockIdx.y = chunk * 9 + tap), over the tiles
// blockIdx.x, + gridDim.x, ...; db[n] += sum dZ[p][n] in the centre-tap,
// first-chunk CTAs.  dZ = BF16(dA * (mask > 0)).
template <int CIN, int COUT>
__global__ void __launch_bounds__(kConvThreads) k_ln_wgrad(const LnPatch* __restrict__ lp,
                                                           const LnTile* __restrict__ tiles, int ntiles,
                                                           const float* __restrict__ dA,
                                                           const bf16* __restrict__ mask, const bf16* __restrict__ X,
                                                           float* __restrict__ dW, float* __restrict__ db) {
  constexpr int SP = TH * TW + 8;  // pixels per shared row (+ pad)
  constexpr int PAIRS = (COUT / 16) * 2, PW = (PAIRS + 3) / 4;
  __shared__ __align__(16) bf16 dz_s[COUT * SP];
  __shared__ __align__(16) bf16 x_s[16 * SP];
  const int tap = blockIdx.y % 9, c0 = (blockIdx.y / 9) * 16, dy = tap / 3 - 1, dx = tap % 3 - 1;
  const bool bias_cta = (tap == 4 && c0 == 0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tg = lane & 3;
  float acc[PW][4];
#pragma unroll
  for (int i = 0; i < PW; i++)
#pragma unroll
    for (int k = 0; k < 4; k++) acc[i][k] = 0.f;
  float dbacc = 0.f;
  for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x) {
    const LnTile t = tiles[ti];
    const LnPatch P = lp[t.patch];
    __syncthreads();
    for (int idx = threadIdx.x; idx < TH * TW * (COUT / 8); idx += blockDim.x) {
      const int px = idx / (COUT / 8), q = idx % (COUT / 8);
      const int y = t.y0 + px / TW, x = t.x0 + px % TW;
      float f[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      if (y < P.H && x < P.W) {
        const long long pix = P.off + (long long)y * P.W + x;
        const float4 g0 = *(const float4*)(dA + pix * COUT + q * 8), g1 = *(const float4*)(dA + pix * COUT + q * 8 + 4);
        f[0] = g0.x, f[1] = g0.y, f[2] = g0.z, f[3] = g0.w, f[4] = g1.x, f[5] = g1.y, f[6] = g1.z, f[7] = g1.w;
        if (mask) {
          const uint4 mk = *(const uint4*)(mask + pix * COUT + q * 8);
          const bf16* m = (const bf16*)&mk;
#pragma unroll
          for (int k = 0; k < 8; k++)
            if (!(__bfloat162float(m[k]) > 0.f)) f[k] = 0.f;
        }
      }
#pragma unroll
      for (int k = 0; k < 8; k++) dz_s[(q * 8 + k) * SP + px] = __float2bfloat16_rn(f[k]);
    }
    for (int idx = threadIdx.x; idx < TH * TW * 2; idx += blockDim.x) {
      const int px = idx >> 1, q = idx & 1;
      const int y = t.y0 + px / TW + dy, x = t.x0 + px % TW + dx;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      // only output pixels inside the patch contribute (their dZ is zero
      // otherwise); the input pixel must exist too (zero padding)
      const int yo = t.y0 + px / TW, xo = t.x0 + px % TW;
      if (yo < P.H && xo < P.W && y >= 0 && y < P.H && x >= 0 && x < P.W)
        v = *(const uint4*)(X + (P.off + (long long)y * P.W + x) * CIN + c0 + q * 8);
      const bf16* e = (const bf16*)&v;
#pragma unroll
      for (int k = 0; k < 8; k++) x_s[(q * 8 + k) * SP + px] = e[k];
    }
    __syncthreads();
    if (bias_cta && threadIdx.x < COUT) {
      float s = 0.f;
      for (int px = 0; px < TH * TW; px++) s += __bfloat162float(dz_s[threadIdx.x * SP + px]);
      dbacc += s;
    }
#pragma unroll
    for (int ks = 0; ks < TH * TW / 16; ks++) {
#pragma unroll
      for (int i = 0; i < PW; i++) {
        const int pair = warp + 4 * i;
        if (pair >= PAIRS) break;
        const int mt = pair >> 1, nt = pair & 1;
        const bf16* ar = dz_s + (mt * 16 + g) * SP + ks * 16 + 2 * tg;
        const bf16* br = x_s + (nt * 8 + g) * SP + ks * 16 + 2 * tg;
        mma_bf16(acc[i], ld32(ar), ld32(ar + 8 * SP), ld32(ar + 8), ld32(ar + 8 * SP + 8), ld32(br), ld32(br + 8));
      }
    }
  }
#pragma unroll
  for (int i = 0; i < PW; i++) {
    const int pair = warp + 4 * i;
    if (pair >= PAIRS) break;
    const int mt = pair >> 1, nt = pair & 1;
    const int n = mt * 16 + g, c = c0 + nt * 8 + 2 * tg;
    float* d0 = dW + ((long long)n * 9 + tap) * CIN + c;
    float* d1 = dW + ((long long)(n + 8) * 9 + tap) * CIN + c;
    atomicAdd(d0, acc[i][0]);
    atomicAdd(d0 + 1, acc[i][1]);
    atomicAdd(d1, acc[i][2]);
    atomicAdd(d1 + 1, acc[i][3]);
  }
  if (bias_cta && threadIdx.x < COUT) atomicAdd(db + threadIdx.x, dbacc);
}

// ---------------------------------------------------------- resampling
// 2 x 2 mean over the pixels that exist, BF16, C channels
__global__ void k_ln_pool(const LnPatch* __restrict__ lo, const LnPatch* __restrict__ hi, int npatch, int C,
                          const bf16* __restrict__ in, bf16* __restrict__ out) {
  const int p = blockIdx.y;
  const LnPatch S = lo[p], D = hi[p];  // source (fine), destination (coarse)
  const int nq = C / 8;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)D.H * D.W * nq;
       i += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(i % nq);
    const long long px = i / nq;
    const int y = (int)(px / D.W), x = (int)(px % D.W);
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int n = 0;
    for (int a = 0; a < 2; a++)
      for (int b = 0; b < 2; b++) {
        const int yy = 2 * y + a, xx = 2 * x + b;
        if (yy >= S.H || xx >= S.W) continue;
        const uint4 v = *(const uint4*)(in + (S.off + (long long)yy * S.W + xx) * C + q * 8);
        const bf16* e = (const bf16*)&v;
#pragma unroll
        for (int k = 0; k < 8; k++) s[k] += __bfloat162float(e[k]);
        n++;
      }
    const float r = 1.f / (float)n;
    *(uint4*)(out + (D.off + px) * C + q * 8) =
        make_uint4(pack2(s[0] * r, s[1] * r), pack2(s[2] * r, s[3] * r), pack2(s[4] * r, s[5] * r),
                   pack2(s[6] * r, s[7] * r));
  }
}

// dS[y][x] += dP[y/2][x/2] / count(y/2, x/2), FP32
__global__ void k_ln_pool_bwd(const LnPatch* __restrict__ lo, const LnPatch* __restrict__ hi, int C,
                              const float* __restrict__ dP, float* __restrict__ dS) {
  const int p = blockIdx.y;
  const LnPatch S = lo[p], D = hi[p];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)S.H * S.W * C;
       i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const long long px = i / C;
    const int y = (int)(px / S.W), x = (int)(px % S.W);
    const int cy = y >> 1, cx = x >> 1;
    const int n = (min(2 * cy + 2, S.H) - 2 * cy) * (min(2 * cx + 2, S.W) - 2 * cx);
    dS[(S.off + px) * C + c] += dP[(D.off + (long long)cy * D.W + cx) * C + c] / (float)n;
  }
}

// concatenation [up(coarse), skip] at the fine level, BF16
__global__ void k_ln_upcat(const LnPatch* __restrict__ lo, const LnPatch* __restrict__ hi, int C1, int C2,
                           const bf16* __restrict__ coarse, const bf16* __restrict__ skip, bf16* __restrict__ out) {
  const int p = blockIdx.y;
  const LnPatch F = lo[p], Q = hi[p];
  const int C = C1 + C2, nq = C / 8;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)F.H * F.W * nq;
       i += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(i % nq);
    const long long px = i / nq;
    const int y = (int)(px / F.W), x = (int)(px % F.W);
    uint4 v;
    if (q * 8 < C1)
      v = *(const uint4*)(coarse + (Q.off + (long long)(y >> 1) * Q.W + (x >> 1)) * C1 + q * 8);
    else
      v = *(const uint4*)(skip + (F.off + px) * C2 + (q * 8 - C1));
    *(uint4*)(out + (F.off + px) * C + q * 8) = v;
  }
}

// gradient of k_ln_upcat: the coarse part summed over each 2 x 2 block, the
// skip part copied, FP32
__global__ void k_ln_upcat_bwd_coarse(const LnPatch* __restrict__ lo, const LnPatch* __restrict__ hi, int C1,
                                      int C2, const float* __restrict__ dC, float* __restrict__ dcoarse) {
  const int p = blockIdx.y;
  const LnPatch F = lo[p], Q = hi[p];
  const int C = C1 + C2;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)Q.H * Q.W * C1;
       i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % C1);
    const long long px = i / C1;
    const int y = (int)(px / Q.W), x = (int)(px % Q.W);
    float s = 0.f;
    for (int a = 0; a < 2; a++)
      for (int b = 0; b < 2; b++) {
        const int yy = 2 * y + a, xx = 2 * x + b;
        if (yy < F.H && xx < F.W) s += dC[(F.off + (long long)yy * F.W + xx) * C + c];
      }
    dcoarse[(Q.off + px) * C1 + c] = s;
  }
}
__global__ void k_ln_upcat_bwd_skip(const LnPatch* __restrict__ lo, int C1, int C2, const float* __restrict__ dC,
                                    float* __restrict__ dskip) {
  const int p = blockIdx.y;
  const LnPatch F = lo[p];
  const int C = C1 + C2;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)F.H * F.W * C2;
       i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % C2);
    const long long px = i / C2;
    dskip[(F.off + px) * C2 + c] = dC[(F.off + px) * C + C1 + c];
  }
}

// ------------------------------------------------------------ features
__global__ void k_ln_features(const LnPatch* __restrict__ lp, const float* __restrict__ mpb,
                              const float* __restrict__ deg, bf16* __restrict__ x) {
  const LnPatch P = lp[blockIdx.y];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)P.H * P.W;
       i += (long long)gridDim.x * blockDim.x) {
    const long long q = P.off + i;
    uint4 v0 = make_uint4(pack2(mpb[q], deg[q] * (1.f / 81.f)), 0u, 0u, 0u);
    *(uint4*)(x + q * kLnIn) = v0;
    *(uint4*)(x + q * kLnIn + 8) = make_uint4(0u, 0u, 0u, 0u);
  }
}
__global__ void k_ln_features_from(const LnPatch* __restrict__ lp, const PatchDev* __restrict__ pd,
                                   const float* __restrict__ mpb, const float* __restrict__ deg,
                                   bf16* __restrict__ x) {
  const LnPatch P = lp[blockIdx.y];
  const PatchDev D = pd[blockIdx.y];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)P.H * P.W;
       i += (long long)gridDim.x * blockDim.x) {
    const long long q = P.off + i;
    *(uint4*)(x + q * kLnIn) = make_uint4(pack2(mpb[D.pix + i], deg[D.vec + i] * (1.f / 81.f)), 0u, 0u, 0u);
    *(uint4*)(x + q * kLnIn + 8) = make_uint4(0u, 0u, 0u, 0u);
  }
}

// ------------------------------------------------------------------ loss
// per patch: G = Y^T Y (32 x 32) and B = V^T Y (9 x 32), FP64 sums of FP32
// per-warp partials; lane j owns column j
constexpr int kGramLen = kLnOut * kLnOut + kLnTargets * kLnOut;
__global__ void __launch_bounds__(256) k_ln_gram(const LnPatch* __restrict__ lp, const float* __restrict__ y,
                                                 const float* __restrict__ v, double* __restrict__ gb) {
  const LnPatch P = lp[blockIdx.y];
  const long long N = (long long)P.H * P.W;
  const int lane = threadIdx.x & 31;
  const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  float G[kLnOut], B[kLnTargets];
#pragma unroll
  for (int k = 0; k < kLnOut; k++) G[k] = 0.f;
#pragma unroll
  for (int i = 0; i < kLnTargets; i++) B[i] = 0.f;
  for (long long p = w0; p < N; p += nw) {
    const long long q = P.off + p;
    const float yj = y[q * kLnOut + lane];
    const float vl = lane < kLnTargets ? v[q * kLnTargets + lane] : 0.f;
#pragma unroll
    for (int k = 0; k < kLnOut; k++) G[k] = fmaf(yj, __shfl_sync(0xffffffffu, yj, k), G[k]);
#pragma unroll
    for (int i = 0; i < kLnTargets; i++) B[i] = fmaf(__shfl_sync(0xffffffffu, vl, i), yj, B[i]);
  }
  double* o = gb + (long long)blockIdx.y * kGramLen;
#pragma unroll
  for (int k = 0; k < kLnOut; k++) atomicAdd(o + lane * kLnOut + k, (double)G[k]);
#pragma unroll
  for (int i = 0; i < kLnTargets; i++) atomicAdd(o + kLnOut * kLnOut + i * kLnOut + lane, (double)B[i]);
}

// dY[p][j] = -2 (sum_i V[p][i] C1[i][j] - sum_k Y[p][k] C2[k][j])
__global__ void __launch_bounds__(256) k_ln_dy(const LnPatch* __restrict__ lp, const float* __restrict__ y,
                                               const float* __restrict__ v, const float* __restrict__ cm,
                                               float* __restrict__ dy) {
  const LnPatch P = lp[blockIdx.y];
  const long long N = (long long)P.H * P.W;
  const int lane = threadIdx.x & 31;
  const float* C1 = cm + (long long)blockIdx.y * kGramLen;  // [9][32]
  const float* C2 = C1 + kLnTargets * kLnOut;                  // [32][32]
  float c1[kLnTargets], c2[kLnOut];
#pragma unroll
  for (int i = 0; i < kLnTargets; i++) c1[i] = C1[i * kLnOut + lane];
#pragma unroll
  for (int k = 0; k < kLnOut; k++) c2[k] = C2[k * kLnOut + lane];
  const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long p = w0; p < N; p += nw) {
    const long long q = P.off + p;
    const float yj = y[q * kLnOut + lane];
    const float vl = lane < kLnTargets ? v[q * kLnTargets + lane] : 0.f;
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < kLnTargets; i++) s = fmaf(__shfl_sync(0xffffffffu, vl, i), c1[i], s);
#pragma unroll
    for (int k = 0; k < kLnOut; k++) s = fmaf(-__shfl_sync(0xffffffffu, yj, k), c2[k], s);
    dy[q * kLnOut + lane] = -2.f * s;
  }
}

// --------------------------------------------------------------- weights
// BF16 copies of every convolution's weights: wb [cout][9][cin] and the
// flipped, transposed wt [cin][9][cout] (wt[c][8 - tap][n] = W[n][tap][c]),
// both at the parameter vector's weight offsets
struct ConvOff {
  long long wo[kLnConvs];
  int cin[kLnConvs], cout[kLnConvs];
};
__global__ void k_ln_wprep(ConvOff co, const float* __restrict__ w32, bf16* __restrict__ wb,
                           bf16* __restrict__ wt) {
  const int l = blockIdx.y;
  const int ci = co.cin[l], cn = co.cout[l];
  const long long n9 = (long long)cn * 9 * ci;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n9; i += (long long)gridDim.x * blockDim.x) {
    const float v = w32[co.wo[l] + i];
    const int c = (int)(i % ci), tap = (int)((i / ci) % 9), n = (int)(i / (9 * (long long)ci));
    wb[co.wo[l] + i] = __float2bfloat16_rn(v);
    wt[co.wo[l] + ((long long)c * 9 + (8 - tap)) * cn + n] = __float2bfloat16_rn(v);
  }
}

__global__ void k_ln_adam(long long n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                          float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// start block: X[vec + p][j] = y[p][j] + 1e-2 * (mean |y[p][.]| + 1e-6) * u(p, j)
__device__ __forceinline__ float ln_hash(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return (float)(x & 0xffffff) * (1.0f / 16777216.0f) - 0.5f;
}
__global__ void k_ln_start(const LnPatch* __restrict__ lp, const PatchDev* __restrict__ pd,
                           const float* __restrict__ y, float* __restrict__ X) {
  const LnPatch P = lp[blockIdx.y];
  const PatchDev D = pd[blockIdx.y];
  const int lane = threadIdx.x & 31;
  const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long p = w0; p < (long long)P.H * P.W; p += nw) {
    const float v = y[(P.off + p) * kLnOut + lane];
    float a = fabsf(v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    const float amp = 1e-2f * (a * (1.f / 32.f) + 1e-6f);
    X[(D.vec + p) * kBlk + lane] = v + amp * ln_hash((uint32_t)(p * 32 + lane) * 2654435761u + 977u);
  }
}

template <int CIN, int CO, int MODE>
cudaError_t conv_go(const LnPatch* lp, const LnTile* tiles, int ntiles, int cout, const void* in, const bf16* mask,
                    const bf16* w, const float* bias, void* out, cudaStream_t s) {
  constexpr size_t smem = ((size_t)NHALO * (CIN + 8) + (size_t)CO * (9 * CIN + 8)) * sizeof(bf16);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_ln_conv<CIN, CO, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  if (ntiles == 0) return cudaSuccess;
  k_ln_conv<CIN, CO, MODE><<<dim3(ntiles, cout / CO), kConvThreads, smem, s>>>(lp, tiles, in, mask, w, bias, out,
                                                                               cout);
  return cudaGetLastError();
}

// the instantiations the network uses: forward (mode 0 / 1) and data
// gradient (mode 2, cin = the layer's cout, cout = its cin)
cudaError_t conv_launch(int cin, int cout, int mode, const LnPatch* lp, const LnTile* tiles, int ntiles,
                        const void* in, const bf16* mask, const bf16* w, const float* bias, void* out,
                        cudaStream_t s) {
  const bool c16 = (cout % 32) != 0;
#define GO(CI, CO, M) return conv_go<CI, CO, M>(lp, tiles, ntiles, cout, in, mask, w, bias, out, s)
  if (mode == 0) {
    if (c16) {
      if (cin == 16) GO(16, 16, 0);
      if (cin == 48) GO(48, 16, 0);
    } else {
      if (cin == 16) GO(16, 32, 0);
      if (cin == 32) GO(32, 32, 0);
      if (cin == 64) GO(64, 32, 0);
      if (cin == 96) GO(96, 32, 0);
      if (cin == 128) GO(128, 32, 0);
    }
  } else if (mode == 1) {
    if (cin == 16 && !c16) GO(16, 32, 1);
  } else {
    if (c16) {
      if (cin == 16) GO(16, 16, 2);
      if (cin == 32) GO(32, 16, 2);
    } else {
      if (cin == 32) GO(32, 32, 2);
      if (cin == 64) GO(64, 32, 2);
    }
  }
#undef GO
  return cudaErrorInvalidValue;
}

cudaError_t wgrad_launch(int cin, int cout, const LnPatch* lp, const LnTile* tiles, int ntiles, const float* dA,
                         const bf16* mask, const bf16* X, float* dW, float* db, cudaStream_t s) {
  if (ntiles == 0) return cudaSuccess;
  const dim3 grid(std::min(ntiles, 64), 9 * (cin / 16));
#define GO(CI, CO)                                                                                \
  do {                                                                                            \
    k_ln_wgrad<CI, CO><<<grid, kConvThreads, 0, s>>>(lp, tiles, ntiles, dA, mask, X, dW, db); \
    return cudaGetLastError();                                                                    \
  } while (0)
  if (cin == 16 && cout == 16) GO(16, 16);
  if (cin == 16 && cout == 32) GO(16, 32);
  if (cin == 32 && cout == 32) GO(32, 32);
  if (cin == 32 && cout == 64) GO(32, 64);
  if (cin == 64 && cout == 64) GO(64, 64);
  if (cin == 128 && cout == 64) GO(128, 64);
  if (cin == 96 && cout == 32) GO(96, 32);
  if (cin == 48 && cout == 16) GO(48, 16);
#undef GO
  return cudaErrorInvalidValue;
}

dim3 pix_grid(long long maxpix, int npatch) {
  return dim3((unsigned)std::max(1LL, std::min((maxpix + 255) / 256, 4096LL)), npatch);
}

}  // namespace

// ----------------------------------------------------------------- host
struct LearnedNet::Impl {
  size_t wo[kLnConvs], bo[kLnConvs], np = 0;
  float* w32 = nullptr;  // master weights
  float* grad = nullptr;
  float *am = nullptr, *av = nullptr;  // Adam moments
  bf16 *wb = nullptr, *wt = nullptr;   // BF16 weights, flipped-transposed BF16 weights
  bool have = false;
  std::vector<LnPatch> lp[kLnLevels];
  std::vector<LnTile> lt[kLnLevels];
  long long npix[kLnLevels] = {0, 0, 0, 0}, maxpix[kLnLevels] = {0, 0, 0, 0};
  LnPatch* d_lp[kLnLevels] = {};
  LnTile* d_lt[kLnLevels] = {};
  size_t cap_lp[kLnLevels] = {}, cap_lt[kLnLevels] = {};
  // activations (BF16) and gradients (FP32), one arena each, carved per level
  bf16* act = nullptr;
  size_t cap_act = 0;
  float* gr = nullptr;
  size_t cap_gr = 0;
  float* y = nullptr;
  size_t cap_y = 0;
  double* gram = nullptr;
  float* cm = nullptr;
  size_t cap_gram = 0, cap_cm = 0;
  std::vector<double> h_gram;
  std::vector<float> h_cm;
  // named tensors
  bf16 *X0, *A0a, *S0, *C0, *A0c, *A0d, *P0, *A1a, *S1, *C1, *A1c, *A1d, *P1, *A2a, *S2, *C2, *A2c, *A2d, *P2,
      *A3a, *A3b;
  float *dY, *dA0d, *dA0c, *dC0, *dS0, *dA0a, *dA1d, *dA1c, *dC1, *dS1, *dA1a, *dP0, *dA2d, *dA2c, *dC2, *dS2,
      *dA2a, *dP1, *dA3b, *dA3a, *dP2;
  int launches = 0;

  Impl() { conv_offsets(wo, bo, &np); }
  ~Impl() {
    void* ps[] = {w32, grad, am, av, wb, wt, act, gr, y, gram, cm};
    for (void* p : ps)
      if (p) cudaFree(p);
    for (int l = 0; l < kLnLevels; l++) {
      if (d_lp[l]) cudaFree(d_lp[l]);
      if (d_lt[l]) cudaFree(d_lt[l]);
    }
  }
  cudaError_t wprep(cudaStream_t s) {
    ConvOff co;
    for (int l = 0; l < kLnConvs; l++) {
      co.wo[l] = (long long)wo[l];
      co.cin[l] = kLnNet[l].cin;
      co.cout[l] = kLnNet[l].cout;
    }
    k_ln_wprep<<<dim3(64, kLnConvs), 256, 0, s>>>(co, w32, wb, wt);
    launches++;
    return cudaGetLastError();
  }
  cudaError_t conv(int l, int level, const void* in, void* out, cudaStream_t s) {
    launches++;
    return conv_launch(kLnNet[l].cin, kLnNet[l].cout, kLnNet[l].relu ? 0 : 1, d_lp[level], d_lt[level],
                       (int)lt[level].size(), in, nullptr, wb + wo[l], w32 + bo[l], out, s);
  }
  // backward of convolution l: dA (FP32 gradient of its output), mask (its
  // BF16 output; null for the head), X (its input); the data gradient into
  // dX unless null
  cudaError_t conv_bwd(int l, int level, const float* dA, const bf16* mask, const bf16* X, float* dX,
                       cudaStream_t s) {
    cudaError_t e = wgrad_launch(kLnNet[l].cin, kLnNet[l].cout, d_lp[level], d_lt[level], (int)lt[level].size(), dA,
                                 mask, X, grad + wo[l], grad + bo[l], s);
    launches++;
    if (e != cudaSuccess || !dX) return e;
    launches++;
    return conv_launch(kLnNet[l].cout, kLnNet[l].cin, 2, d_lp[level], d_lt[level], (int)lt[level].size(), dA, mask,
                       wt + wo[l], nullptr, dX, s);
  }
};

LearnedNet::LearnedNet() : im_(new Impl()) {}
LearnedNet::~LearnedNet() = default;
bool LearnedNet::has_params() const { return im_->have; }
const std::vector<LnPatch>& LearnedNet::patches0() const { return im_->lp[0]; }
const LnPatch* LearnedNet::patches0_dev() const { return im_->d_lp[0]; }
long long LearnedNet::npix0() const { return im_->npix[0]; }
float* LearnedNet::y() { return im_->y; }
float* LearnedNet::grad() { return im_->grad; }
int LearnedNet::launches() const { return im_->launches; }

template <class T>
static cudaError_t grow_buf(T*& p, size_t& cap, size_t need) {
  if (need <= cap && p) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  cudaError_t e = cudaMalloc(&p, std::max<size_t>(need, 1) * sizeof(T));
  if (e == cudaSuccess) cap = need;
  return e;
}

cudaError_t LearnedNet::set_params(const float* hp, cudaStream_t s) {
  Impl& m = *im_;
  cudaError_t e;
  if (!m.w32) {
    size_t c = 0;
    if ((e = grow_buf(m.w32, c, m.np)) != cudaSuccess) return e;
    c = 0;
    if ((e = grow_buf(m.grad, c, m.np)) != cudaSuccess) return e;
    c = 0;
    if ((e = grow_buf(m.am, c, m.np)) != cudaSuccess) return e;
    c = 0;
    if ((e = grow_buf(m.av, c, m.np)) != cudaSuccess) return e;
    c = 0;
    if ((e = grow_buf(m.wb, c, m.np)) != cudaSuccess) return e;
    c = 0;
    if ((e = grow_buf(m.wt, c, m.np)) != cudaSuccess) return e;
  }
  if ((e = cudaMemcpyAsync(m.w32, hp, m.np * sizeof(float), cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(m.am, 0, m.np * sizeof(float), s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(m.av, 0, m.np * sizeof(float), s)) != cudaSuccess) return e;
  if ((e = m.wprep(s)) != cudaSuccess) return e;
  m.have = true;
  return cudaSuccess;
}

cudaError_t LearnedNet::get_params(float* hp, cudaStream_t s) {
  if (!im_->have) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemcpyAsync(hp, im_->w32, im_->np * sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(s);
}

cudaError_t LearnedNet::layout(const std::vector<int>& H, const std::vector<int>& W, cudaStream_t s) {
  Impl& m = *im_;
  const int n = (int)H.size();
  for (int l = 0; l < kLnLevels; l++) {
    m.lp[l].clear();
    m.lt[l].clear();
    long long off = 0, mx = 0;
    for (int i = 0; i < n; i++) {
      int h = H[i], w = W[i];
      for (int k = 0; k < l; k++) {
        h = (h + 1) / 2;
        w = (w + 1) / 2;
      }
      m.lp[l].push_back({h, w, off});
      for (int y = 0; y < h; y += TH)
        for (int x = 0; x < w; x += TW) m.lt[l].push_back({i, y, x, 0});
      off += (long long)h * w;
      mx = std::max(mx, (long long)h * w);
    }
    m.npix[l] = off;
    m.maxpix[l] = mx;
    cudaError_t e;
    if ((e = grow_buf(m.d_lp[l], m.cap_lp[l], m.lp[l].size())) != cudaSuccess) return e;
    if ((e = grow_buf(m.d_lt[l], m.cap_lt[l], std::max<size_t>(1, m.lt[l].size()))) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(m.d_lp[l], m.lp[l].data(), m.lp[l].size() * sizeof(LnPatch), cudaMemcpyHostToDevice,
                             s)) != cudaSuccess)
      return e;
    if (!m.lt[l].empty() && (e = cudaMemcpyAsync(m.d_lt[l], m.lt[l].data(), m.lt[l].size() * sizeof(LnTile),
                                                 cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return e;
  }
  // channel counts of the BF16 activations per level, then of the FP32
  // gradients; each tensor is its level's pixel count times its channels
  const long long N0 = m.npix[0], N1 = m.npix[1], N2 = m.npix[2], N3 = m.npix[3];
  const size_t act_need = N0 * (16 + 16 + 16 + 48 + 16 + 16) + N1 * (16 + 32 + 32 + 96 + 32 + 32) +
                          N2 * (32 + 64 + 64 + 128 + 64 + 64) + N3 * (64 + 64 + 64);
  const size_t gr_need = N0 * (32 + 16 + 16 + 48 + 16 + 16) + N1 * (32 + 32 + 96 + 32 + 32 + 16) +
                         N2 * (64 + 64 + 128 + 64 + 64 + 32) + N3 * (64 + 64 + 64);
  cudaError_t e;
  if ((e = grow_buf(m.act, m.cap_act, act_need)) != cudaSuccess) return e;
  if ((e = grow_buf(m.gr, m.cap_gr, gr_need)) != cudaSuccess) return e;
  if ((e = grow_buf(m.y, m.cap_y, (size_t)N0 * kLnOut)) != cudaSuccess) return e;
  if ((e = grow_buf(m.gram, m.cap_gram, (size_t)n * kGramLen)) != cudaSuccess) return e;
  if ((e = grow_buf(m.cm, m.cap_cm, (size_t)n * kGramLen)) != cudaSuccess) return e;
  bf16* a = m.act;
  auto A = [&](long long N, int C) {
    bf16* r = a;
    a += N * C;
    return r;
  };
  m.X0 = A(N0, 16), m.A0a = A(N0, 16), m.S0 = A(N0, 16), m.C0 = A(N0, 48), m.A0c = A(N0, 16), m.A0d = A(N0, 16);
  m.P0 = A(N1, 16), m.A1a = A(N1, 32), m.S1 = A(N1, 32), m.C1 = A(N1, 96), m.A1c = A(N1, 32), m.A1d = A(N1, 32);
  m.P1 = A(N2, 32), m.A2a = A(N2, 64), m.S2 = A(N2, 64), m.C2 = A(N2, 128), m.A2c = A(N2, 64), m.A2d = A(N2, 64);
  m.P2 = A(N3, 64), m.A3a = A(N3, 64), m.A3b = A(N3, 64);
  float* g = m.gr;
  auto G = [&](long long N, int C) {
    float* r = g;
    g += N * C;
    return r;
  };
  m.dY = G(N0, 32), m.dA0d = G(N0, 16), m.dA0c = G(N0, 16), m.dC0 = G(N0, 48), m.dS0 = G(N0, 16), m.dA0a = G(N0, 16);
  m.dA1d = G(N1, 32), m.dA1c = G(N1, 32), m.dC1 = G(N1, 96), m.dS1 = G(N1, 32), m.dA1a = G(N1, 32), m.dP0 = G(N1, 16);
  m.dA2d = G(N2, 64), m.dA2c = G(N2, 64), m.dC2 = G(N2, 128), m.dS2 = G(N2, 64), m.dA2a = G(N2, 64), m.dP1 = G(N2, 32);
  m.dA3b = G(N3, 64), m.dA3a = G(N3, 64), m.dP2 = G(N3, 64);
  return cudaSuccess;
}

cudaError_t LearnedNet::features(const float* d_mpb, const float* d_deg, cudaStream_t s) {
  Impl& m = *im_;
  k_ln_features<<<pix_grid(m.maxpix[0], (int)m.lp[0].size()), 256, 0, s>>>(m.d_lp[0], d_mpb, d_deg, m.X0);
  m.launches++;
  return cudaGetLastError();
}

cudaError_t LearnedNet::features_from(const PatchDev* patches, const float* d_mpb, const float* d_deg,
                                      cudaStream_t s) {
  Impl& m = *im_;
  k_ln_features_from<<<pix_grid(m.maxpix[0], (int)m.lp[0].size()), 256, 0, s>>>(m.d_lp[0], patches, d_mpb, d_deg,
                                                                                m.X0);
  m.launches++;
  return cudaGetLastError();
}

cudaError_t LearnedNet::forward(cudaStream_t s) {
  Impl& m = *im_;
  if (!m.have) return cudaErrorInvalidValue;
  const int np = (int)m.lp[0].size();
  cudaError_t e;
#define CKE(x)                              \
  do {                                      \
    if ((e = (x)) != cudaSuccess) return e; \
  } while (0)
  auto pool = [&](int l, int C, const bf16* in, bf16* out) {
    k_ln_pool<<<pix_grid(m.maxpix[l + 1] * (C / 8), np), 256, 0, s>>>(m.d_lp[l], m.d_lp[l + 1], np, C, in, out);
    m.launches++;
    return cudaGetLastError();
  };
  auto upcat = [&](int l, int C1, int C2, const bf16* coarse, const bf16* skip, bf16* out) {
    k_ln_upcat<<<pix_grid(m.maxpix[l] * ((C1 + C2) / 8), np), 256, 0, s>>>(m.d_lp[l], m.d_lp[l + 1], C1, C2, coarse,
                                                                           skip, out);
    m.launches++;
    return cudaGetLastError();
  };
  CKE(m.conv(0, 0, m.X0, m.A0a, s));
  CKE(m.conv(1, 0, m.A0a, m.S0, s));
  CKE(pool(0, 16, m.S0, m.P0));
  CKE(m.conv(2, 1, m.P0, m.A1a, s));
  CKE(m.conv(3, 1, m.A1a, m.S1, s));
  CKE(pool(1, 32, m.S1, m.P1));
  CKE(m.conv(4, 2, m.P1, m.A2a, s));
  CKE(m.conv(5, 2, m.A2a, m.S2, s));
  CKE(pool(2, 64, m.S2, m.P2));
  CKE(m.conv(6, 3, m.P2, m.A3a, s));
  CKE(m.conv(7, 3, m.A3a, m.A3b, s));
  CKE(upcat(2, 64, 64, m.A3b, m.S2, m.C2));
  CKE(m.conv(8, 2, m.C2, m.A2c, s));
  CKE(m.conv(9, 2, m.A2c, m.A2d, s));
  CKE(upcat(1, 64, 32, m.A2d, m.S1, m.C1));
  CKE(m.conv(10, 1, m.C1, m.A1c, s));
  CKE(m.conv(11, 1, m.A1c, m.A1d, s));
  CKE(upcat(0, 32, 16, m.A1d, m.S0, m.C0));
  CKE(m.conv(12, 0, m.C0, m.A0c, s));
  CKE(m.conv(13, 0, m.A0c, m.A0d, s));
  CKE(m.conv(14, 0, m.A0d, m.y, s));
  return cudaSuccess;
}

// dense symmetric positive definite inverse by Cholesky (n <= 32)
static bool spd_inverse(const double* A, int n, double* X) {
  std::vector<double> L((size_t)n * n, 0.0);
  for (int j = 0; j < n; j++) {
    double d = A[j * n + j];
    for (int k = 0; k < j; k++) d -= L[j * n + k] * L[j * n + k];
    if (!(d > 0)) return false;
    L[j * n + j] = std::sqrt(d);
    for (int i = j + 1; i < n; i++) {
      double v = A[i * n + j];
      for (int k = 0; k < j; k++) v -= L[i * n + k] * L[j * n + k];
      L[i * n + j] = v / L[j * n + j];
    }
  }
  for (int c = 0; c < n; c++) {  // solve L L^T x = e_c
    std::vector<double> z(n, 0.0);
    for (int i = 0; i < n; i++) {
      double v = (i == c) ? 1.0 : 0.0;
      for (int k = 0; k < i; k++) v -= L[i * n + k] * z[k];
      z[i] = v / L[i * n + i];
    }
    for (int i = n - 1; i >= 0; i--) {
      double v = z[i];
      for (int k = i + 1; k < n; k++) v -= L[k * n + i] * X[k * n + c];
      X[i * n + c] = v / L[i * n + i];
    }
  }
  return true;
}

cudaError_t LearnedNet::loss_backward(const float* d_v, double* loss, cudaStream_t s) {
  Impl& m = *im_;
  if (!m.have) return cudaErrorInvalidValue;
  const int np = (int)m.lp[0].size();
  cudaError_t e;
  // the subspace loss and its gradient with respect to y
  CKE(cudaMemsetAsync(m.gram, 0, (size_t)np * kGramLen * sizeof(double), s));
  k_ln_gram<<<dim3((unsigned)std::max(1LL, std::min(m.maxpix[0] / 2048 + 1, 512LL)), np), 256, 0, s>>>(
      m.d_lp[0], m.y, d_v, m.gram);
  m.launches++;
  CKE(cudaGetLastError());
  m.h_gram.resize((size_t)np * kGramLen);
  CKE(cudaMemcpyAsync(m.h_gram.data(), m.gram, m.h_gram.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  CKE(cudaStreamSynchronize(s));
  m.h_cm.assign((size_t)np * kGramLen, 0.f);
  double total = 0;
  constexpr int K = kLnOut, T = kLnTargets;
  std::vector<double> Gm(K * K), Gi(K * K), C1(T * K), Bt(T * K);
  for (int p = 0; p < np; p++) {
    const double* g = m.h_gram.data() + (size_t)p * kGramLen;
    double tr = 0;
    for (int i = 0; i < K; i++) tr += g[i * K + i];
    for (int i = 0; i < K * K; i++) Gm[i] = g[i];
    for (int i = 0; i < K; i++) Gm[i * K + i] += 1e-4 * tr / K + 1e-30;
    const double* B = g + K * K;  // [9][32]
    if (!spd_inverse(Gm.data(), K, Gi.data())) return cudaErrorInvalidValue;
    for (int i = 0; i < T; i++)
      for (int j = 0; j < K; j++) {
        double v = 0;
        for (int k = 0; k < K; k++) v += B[i * K + k] * Gi[k * K + j];
        C1[i * K + j] = v;
      }
    double cap = 0;
    for (int i = 0; i < T; i++)
      for (int j = 0; j < K; j++) cap += C1[i * K + j] * B[i * K + j];
    total += T - cap;
    // C2 = C1^T C1' where C2 = Gi B^T B Gi = (B Gi)^T (B Gi) = C1^T C1
    float* cm = m.h_cm.data() + (size_t)p * kGramLen;
    for (int i = 0; i < T * K; i++) cm[i] = (float)C1[i];
    for (int a = 0; a < K; a++)
      for (int b = 0; b < K; b++) {
        double v = 0;
        for (int i = 0; i < T; i++) v += C1[i * K + a] * C1[i * K + b];
        cm[T * K + a * K + b] = (float)v;
      }
  }
  *loss = total;
  CKE(cudaMemcpyAsync(m.cm, m.h_cm.data(), m.h_cm.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  k_ln_dy<<<dim3((unsigned)std::max(1LL, std::min(m.maxpix[0] / 2048 + 1, 512LL)), np), 256, 0, s>>>(
      m.d_lp[0], m.y, d_v, m.cm, m.dY);
  m.launches++;
  CKE(cudaGetLastError());
  // backward through the network
  CKE(cudaMemsetAsync(m.grad, 0, m.np * sizeof(float), s));
  auto pool_bwd = [&](int l, int C, const float* dP, float* dS) {
    k_ln_pool_bwd<<<pix_grid(m.maxpix[l] * C / 8, np), 256, 0, s>>>(m.d_lp[l], m.d_lp[l + 1], C, dP, dS);
    m.launches++;
    return cudaGetLastError();
  };
  auto upcat_bwd = [&](int l, int C1c, int C2c, const float* dC, float* dcoarse, float* dskip) {
    k_ln_upcat_bwd_coarse<<<pix_grid(m.maxpix[l + 1] * C1c / 8, np), 256, 0, s>>>(m.d_lp[l], m.d_lp[l + 1], C1c,
                                                                                   C2c, dC, dcoarse);
    k_ln_upcat_bwd_skip<<<pix_grid(m.maxpix[l] * C2c / 8, np), 256, 0, s>>>(m.d_lp[l], C1c, C2c, dC, dskip);
    m.launches += 2;
    return cudaGetLastError();
  };
  CKE(m.conv_bwd(14, 0, m.dY, nullptr, m.A0d, m.dA0d, s));
  CKE(m.conv_bwd(13, 0, m.dA0d, m.A0d, m.A0c, m.dA0c, s));
  CKE(m.conv_bwd(12, 0, m.dA0c, m.A0c, m.C0, m.dC0, s));
  CKE(upcat_bwd(0, 32, 16, m.dC0, m.dA1d, m.dS0));
  CKE(m.conv_bwd(11, 1, m.dA1d, m.A1d, m.A1c, m.dA1c, s));
  CKE(m.conv_bwd(10, 1, m.dA1c, m.A1c, m.C1, m.dC1, s));
  CKE(upcat_bwd(1, 64, 32, m.dC1, m.dA2d, m.dS1));
  CKE(m.conv_bwd(9, 2, m.dA2d, m.A2d, m.A2c, m.dA2c, s));
  CKE(m.conv_bwd(8, 2, m.dA2c, m.A2c, m.C2, m.dC2, s));
  CKE(upcat_bwd(2, 64, 64, m.dC2, m.dA3b, m.dS2));
  CKE(m.conv_bwd(7, 3, m.dA3b, m.A3b, m.A3a, m.dA3a, s));
  CKE(m.conv_bwd(6, 3, m.dA3a, m.A3a, m.P2, m.dP2, s));
  CKE(pool_bwd(2, 64, m.dP2, m.dS2));
  CKE(m.conv_bwd(5, 2, m.dS2, m.S2, m.A2a, m.dA2a, s));
  CKE(m.conv_bwd(4, 2, m.dA2a, m.A2a, m.P1, m.dP1, s));
  CKE(pool_bwd(1, 32, m.dP1, m.dS1));
  CKE(m.conv_bwd(3, 1, m.dS1, m.S1, m.A1a, m.dA1a, s));
  CKE(m.conv_bwd(2, 1, m.dA1a, m.A1a, m.P0, m.dP0, s));
  CKE(pool_bwd(0, 16, m.dP0, m.dS0));
  CKE(m.conv_bwd(1, 0, m.dS0, m.S0, m.A0a, m.dA0a, s));
  CKE(m.conv_bwd(0, 0, m.dA0a, m.A0a, m.X0, nullptr, s));
#undef CKE
  return cudaSuccess;
}

cudaError_t LearnedNet::adam(float lr, float b1, float b2, float eps, int t, cudaStream_t s) {
  Impl& m = *im_;
  if (!m.have) return cudaErrorInvalidValue;
  const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
  k_ln_adam<<<256, 256, 0, s>>>((long long)m.np, m.w32, m.grad, m.am, m.av, lr, b1, b2, eps, c1, c2);
  m.launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return m.wprep(s);
}

cudaError_t ln_launch_start(const LnPatch* lp, const PatchDev* patches, int npatch, int maxN, const float* y,
                            float* X, cudaStream_t s) {
  k_ln_start<<<pix_grid((long long)maxN * 32 / 8, npatch), 256, 0, s>>>(lp, patches, y, X);
  return cudaGetLastError();
}

}  // namespace gpb
