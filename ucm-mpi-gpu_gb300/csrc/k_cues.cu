// k_cues.cu -- oriented half-disc histogram gradients, mPb combination and
// oriented non-maximum suppression (sm_103a).
//
// Reference: lib_image::hist_gradient_2D / compute_hist_gradient_2D
// (globalPb/src/math/libraries/lib_image.cc:3120-3235, 3575-3686) as called by
// mex_pb_parts_final_selected.cpp:157-227, the weighted sum of
// multiscalePb.cpp:217-245 and nonmax_channels + nonmax_oriented_2D
// (src/nonmax_channels.cpp:8-80, lib_image.cc:4083-4197).
//
// One warp computes one pixel.  The four label images (L, a, b bins and the
// texton) are packed into one u32 per pixel and staged, reflect-padded by 20,
// in shared memory.  The radius-20 disc is walked in four nested annuli
// (r <= 3, 5, 10, 20); slice membership does not depend on r, so the counts
// are cumulative and one walk serves every (cue, radius) pair.  Lane
// l = half*16 + slice owns one counter row per cue (8-bit counters, row stride
// 36 bytes so rows fall in distinct banks), so no atomics are needed.  After
// each annulus the lanes switch role to histogram bins: per-slice sums, the
// Gaussian bin smoothing, L1 normalisation, the 8-step spin and the
// chi-squared distance all run across the warp with shuffles.  Smoothing is
// linear and applied after the per-slice scaling, so 9 convolutions (the
// half-disc total and 8 left-right differences) replace the 16 per-slice ones.
#include <float.h>
#include <stdint.h>

#include "gpb_internal.h"
#include "kernels.h"

namespace gpb {

constexpr int kAnnMax = 1400;
__constant__ int16_t c_ann_dy[kAnnMax];
__constant__ int16_t c_ann_dx[kAnnMax];
__constant__ int c_ann_start[kNannulus][32];
__constant__ int c_ann_count[kNannulus][32];
__constant__ int c_ann_total;
__constant__ float c_slice_pix[kNannulus][16];
__constant__ float c_kbg[17];
__constant__ float c_kcg[9];
__constant__ float c_wm[kNcue], c_wg[kNcue];
__constant__ int c_nms_nb[kNori][4][2];
__constant__ float c_nms_d[kNori];
__constant__ float c_nms_cos[kNori][kNori];

void upload_cues(const HostTables& t, cudaStream_t s) {
  int16_t dy[kAnnMax] = {}, dx[kAnnMax] = {};
  const int n = (int)t.ann_dy.size();
  for (int i = 0; i < n && i < kAnnMax; i++) {
    dy[i] = t.ann_dy[i];
    dx[i] = t.ann_dx[i];
  }
  float sp[kNannulus][16];
  for (int a = 0; a < kNannulus; a++)
    for (int q = 0; q < 16; q++) sp[a][q] = (float)t.slice_pixels[a][q];
  cudaMemcpyToSymbolAsync(c_ann_dy, dy, sizeof(dy), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_ann_dx, dx, sizeof(dx), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_ann_start, t.ann_start, sizeof(t.ann_start), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_ann_count, t.ann_count, sizeof(t.ann_count), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_ann_total, &n, sizeof(int), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_slice_pix, sp, sizeof(sp), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_kbg, t.kbg, sizeof(t.kbg), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_kcg, t.kcg, sizeof(t.kcg), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_wm, t.w_mpb, sizeof(t.w_mpb), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_wg, t.w_g, sizeof(t.w_g), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_nms_nb, t.nms_nb, sizeof(t.nms_nb), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_nms_d, t.nms_d, sizeof(t.nms_d), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_nms_cos, t.nms_cos, sizeof(t.nms_cos), 0, cudaMemcpyHostToDevice, s);
}

__device__ __forceinline__ int reflect_c(int i, int n) {
  for (int it = 0; it < 4 && (i < 0 || i >= n); it++) i = (i < 0) ? -i - 1 : 2 * n - 1 - i;
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

constexpr unsigned FULL = 0xffffffffu;
constexpr int CT_H = kCueTileH, CT_W = kCueTileW;
constexpr int CT_PH = CT_H + 2 * kMaxRadius, CT_PW = CT_W + 2 * kMaxRadius;
constexpr int HROW = 36;                    // bytes per counter row
constexpr int DROW = 12;                    // floats per bin row of the convolution scratch
constexpr int HWARP = 4 * 32 * HROW;        // bytes per warp
constexpr int CT_WARPS = CT_H;              // one warp per tile row
constexpr size_t kCueSmem =
    (size_t)CT_PH * CT_PW * 4 + kAnnMax * 2 + (size_t)CT_WARPS * HWARP + (size_t)CT_WARPS * 32 * DROW * 4;

// Sum of 16 per-lane values over the warp, for all 16 at once: each exchange
// step halves the number of live values (8+4+2+1+1 shuffles), then the 16
// totals are broadcast.  Result in v[0..15] on every lane.
__device__ __forceinline__ void warp_sum16(float (&v)[16], int lane) {
  const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4, b1 = lane & 2;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const float keep = b4 ? v[i + 8] : v[i], give = b4 ? v[i] : v[i + 8];
    v[i] = keep + __shfl_xor_sync(FULL, give, 16);
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const float keep = b3 ? v[i + 4] : v[i], give = b3 ? v[i] : v[i + 4];
    v[i] = keep + __shfl_xor_sync(FULL, give, 8);
  }
#pragma unroll
  for (int i = 0; i < 2; i++) {
    const float keep = b2 ? v[i + 2] : v[i], give = b2 ? v[i] : v[i + 2];
    v[i] = keep + __shfl_xor_sync(FULL, give, 4);
  }
  {
    const float keep = b1 ? v[1] : v[0], give = b1 ? v[0] : v[1];
    v[0] = keep + __shfl_xor_sync(FULL, give, 2);
  }
  v[0] += __shfl_xor_sync(FULL, v[0], 1);
  // lane l now holds the total of index l >> 1
  const float t = v[0];
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __shfl_sync(FULL, t, 2 * i);
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

// this lane's taps of a K-tap bin smoothing (zero where the source bin
// lane + K/2 - j lies outside [0, nb), or the lane itself does) and the
// kernel mass that source bin `lane` keeps in range; per patch, so computed
// once per warp
template <int K>
__device__ __forceinline__ float bin_taps(const float* kern, int lane, int nb, float (&kw)[K]) {
  float m = 0.f;
#pragma unroll
  for (int j = 0; j < K; j++) {
    const int src = lane + K / 2 - j;
    kw[j] = (lane < nb && src >= 0 && src < nb) ? kern[j] : 0.f;
    const int n = lane + j - K / 2;
    if (n >= 0 && n < nb) m += kern[j];
  }
  return m;
}

// per-warp scratch (DROW floats per bin): the 8 orientation differences and
// the total; 12 floats so that 16-byte loads of neighbouring bins are
// conflict-free

// one (cue, radius): counts of bin `lane` in the 16 slices -> 8 chi-squared
// terms of this bin accumulated with the two weight sets.  The truncated
// 'same' bin convolution (conv_in_place_1D, lib_image.cc:3084-3115) of all 8
// orientation differences and of the total runs on the warp's scratch rows.
template <int K>
__device__ __forceinline__ void cue_combo(const uint8_t* hist, int c, int lane, int nb, int ann,
                                          const float (&kw)[K > 0 ? K : 1], float m, float wm, float wg,
                                          float (&accm)[8], float (&accg)[8], float* raw, long long raw_stride,
                                          float* dsm) {
  float cs[16];
#pragma unroll
  for (int q = 0; q < 16; q++)
    cs[q] = lane < nb ? (float)(hist[(c * 32 + q) * HROW + lane] + hist[(c * 32 + 16 + q) * HROW + lane]) : 0.f;
  float S[16];
  if (K > 0) {
#pragma unroll
    for (int q = 0; q < 16; q++) S[q] = cs[q] * m;
    warp_sum16(S, lane);
  } else {
#pragma unroll
    for (int q = 0; q < 16; q++) S[q] = c_slice_pix[ann][q];
  }
  float ch[16];
  float T = 0.f, D = 0.f;
#pragma unroll
  for (int q = 0; q < 16; q++) {
    ch[q] = S[q] != 0.f ? cs[q] * __frcp_rn(S[q]) : 0.f;
    T += ch[q];
    D += q < 8 ? ch[q] : -ch[q];
  }
  float Dv[8];
#pragma unroll
  for (int o = 0; o < 8; o++) {
    Dv[o] = D;
    D += 2.f * (ch[o + 8] - ch[o]);
  }
  if (K > 0) {
    float* row = dsm + lane * DROW;
    *(float4*)(row + 0) = make_float4(Dv[0], Dv[1], Dv[2], Dv[3]);
    *(float4*)(row + 4) = make_float4(Dv[4], Dv[5], Dv[6], Dv[7]);
    row[8] = T;
    __syncwarp();
    float cd[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, ct = 0.f;
#pragma unroll
    for (int j = 0; j < K; j++) {
      const float* src = dsm + ((lane + K / 2 - j) & 31) * DROW;
      const float4 d0 = *(const float4*)(src + 0), d1 = *(const float4*)(src + 4);
      const float kj = kw[j];
      cd[0] = fmaf(d0.x, kj, cd[0]);
      cd[1] = fmaf(d0.y, kj, cd[1]);
      cd[2] = fmaf(d0.z, kj, cd[2]);
      cd[3] = fmaf(d0.w, kj, cd[3]);
      cd[4] = fmaf(d1.x, kj, cd[4]);
      cd[5] = fmaf(d1.y, kj, cd[5]);
      cd[6] = fmaf(d1.z, kj, cd[6]);
      cd[7] = fmaf(d1.w, kj, cd[7]);
      ct = fmaf(src[8], kj, ct);
    }
    __syncwarp();
#pragma unroll
    for (int o = 0; o < 8; o++) Dv[o] = cd[o];
    T = ct;
  }
  const float rT = (T != 0.f && lane < nb) ? __frcp_rn(T) : 0.f;
#pragma unroll
  for (int o = 0; o < 8; o++) {
    const float term = Dv[o] * Dv[o] * rT;
    accm[o] = fmaf(wm, term, accm[o]);
    accg[o] = fmaf(wg, term, accg[o]);
    if (raw) {
      const float chi = 0.5f * warp_sum(term);
      if (lane == 0) raw[o * raw_stride] = chi;
    }
  }
}

template <bool kRaw>
__global__ void __launch_bounds__(CT_WARPS * 32, 3) k_cues(const PatchDev* __restrict__ patches,
                                                        const int4* __restrict__ work,
                                                        const uint32_t* __restrict__ lab4,
                                                        const int* __restrict__ nbins,
                                                        float* __restrict__ mpbo, float* __restrict__ go,
                                                        float* __restrict__ raw, uint8_t* __restrict__ counts) {
  extern __shared__ __align__(16) uint8_t smem[];
  uint32_t* tile = (uint32_t*)smem;
  int16_t* offs = (int16_t*)(smem + (size_t)CT_PH * CT_PW * 4);
  uint8_t* hist_all = smem + (size_t)CT_PH * CT_PW * 4 + kAnnMax * 2;
  const int4 w = work[blockIdx.x];
  const PatchDev P = patches[w.x];
  const uint32_t* lb = lab4 + P.pix;
  for (int i = threadIdx.x; i < CT_PH * CT_PW; i += blockDim.x) {
    const int yy = reflect_c(w.y - kMaxRadius + i / CT_PW, P.H);
    const int xx = reflect_c(w.z - kMaxRadius + i % CT_PW, P.W);
    tile[i] = lb[(long long)yy * P.W + xx];
  }
  const int ntot = c_ann_total;
  for (int i = threadIdx.x; i < ntot; i += blockDim.x) offs[i] = (int16_t)(c_ann_dy[i] * CT_PW + c_ann_dx[i]);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint8_t* hist = hist_all + warp * HWARP;
  float* dsm = (float*)(hist_all + (size_t)CT_WARPS * HWARP) + warp * 32 * DROW;
  const int nbL = nbins[4 * w.x + 0] + 1, nbA = nbins[4 * w.x + 1] + 1, nbB = nbins[4 * w.x + 2] + 1,
            nbT = nbins[4 * w.x + 3] + 1;
  float kwL[17], kwA[9], kwB[9];
  const float mL = bin_taps<17>(c_kbg, lane, nbL, kwL);
  const float mA = bin_taps<9>(c_kcg, lane, nbA, kwA);
  const float mB = bin_taps<9>(c_kcg, lane, nbB, kwB);
  const float kw0[1] = {0.f};
  const int y = w.y + warp;
  if (y >= P.H) return;
  uint8_t* r0 = hist + (0 * 32 + lane) * HROW;
  uint8_t* r1 = hist + (1 * 32 + lane) * HROW;
  uint8_t* r2 = hist + (2 * 32 + lane) * HROW;
  uint8_t* r3 = hist + (3 * 32 + lane) * HROW;
  for (int px = 0; px < CT_W; px++) {
    const int x = w.z + px;
    if (x >= P.W) break;
    const long long p = (long long)y * P.W + x;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      uint32_t* row = (uint32_t*)(hist + (c * 32 + lane) * HROW);
#pragma unroll
      for (int q = 0; q < HROW / 4; q++) row[q] = 0u;
    }
    __syncwarp();
    const uint32_t* ctr = tile + (warp + kMaxRadius) * CT_PW + (px + kMaxRadius);
    float accm[8], accg[8];
#pragma unroll
    for (int o = 0; o < 8; o++) accm[o] = accg[o] = 0.f;
    float* rawp = nullptr;
    const long long rs = P.N;
    for (int a = 0; a < kNannulus; a++) {
      const int st = c_ann_start[a][lane], cnt = c_ann_count[a][lane];
      if (a < 3) {
        for (int i = 0; i < cnt; i++) {
          const uint32_t v = ctr[offs[st + i]];
          r0[v & 255]++;
          r1[(v >> 8) & 255]++;
          r2[(v >> 16) & 255]++;
          r3[v >> 24]++;
        }
      } else {
        for (int i = 0; i < cnt; i++) {
          const uint32_t v = ctr[offs[st + i]];
          r1[(v >> 8) & 255]++;
          r2[(v >> 16) & 255]++;
          r3[v >> 24]++;
        }
      }
      __syncwarp();
      if (kRaw && counts) {
        // debug: this lane's counter rows (half = lane / 16, slice = lane % 16)
        uint8_t* cp = counts + (((P.pix + p) * kNannulus + a) * 4) * 32 * 32;
#pragma unroll
        for (int c = 0; c < 4; c++)
          for (int bb = 0; bb < 32; bb++) cp[(c * 32 + lane) * 32 + bb] = hist[(c * 32 + lane) * HROW + bb];
      }
      // cue index wi = cue*3 + scale (bg1 bg2 bg3 cga1 .. tg3)
      if (kRaw) rawp = raw + P.pix * 96 + p;
      if (a == 0) {
        cue_combo<17>(hist, 0, lane, nbL, a, kwL, mL, c_wm[0], c_wg[0], accm, accg,
                      kRaw ? rawp + 0 * 8 * rs : nullptr, rs, dsm);
      } else {
        const int s = a - 1;  // scale of cga/cgb/tg
        if (a < 3)
          cue_combo<17>(hist, 0, lane, nbL, a, kwL, mL, c_wm[a], c_wg[a], accm, accg,
                        kRaw ? rawp + (long long)a * 8 * rs : nullptr, rs, dsm);
        cue_combo<9>(hist, 1, lane, nbA, a, kwA, mA, c_wm[3 + s], c_wg[3 + s], accm, accg,
                     kRaw ? rawp + (long long)(3 + s) * 8 * rs : nullptr, rs, dsm);
        cue_combo<9>(hist, 2, lane, nbB, a, kwB, mB, c_wm[6 + s], c_wg[6 + s], accm, accg,
                     kRaw ? rawp + (long long)(6 + s) * 8 * rs : nullptr, rs, dsm);
        cue_combo<0>(hist, 3, lane, nbT, a, kw0, 0.f, c_wm[9 + s], c_wg[9 + s], accm, accg,
                     kRaw ? rawp + (long long)(9 + s) * 8 * rs : nullptr, rs, dsm);
      }
      __syncwarp();
    }
    float v[16];
#pragma unroll
    for (int o = 0; o < 8; o++) {
      v[o] = accm[o];
      v[8 + o] = accg[o];
    }
    warp_sum16(v, lane);
    if (lane < 8) mpbo[P.pix * 8 + (long long)lane * P.N + p] = 0.5f * v[lane];
    else if (lane < 16) go[P.pix * 8 + (long long)(lane - 8) * P.N + p] = 0.5f * v[lane];
  }
}

// max label per patch and cue (the histogram length of hist_gradient_2D is
// max(label)+1, lib_image.cc:3665-3670)
__global__ void k_maxlabel(const PatchDev* __restrict__ patches, const uint32_t* __restrict__ lab4,
                           int* __restrict__ nbins) {
  const PatchDev P = patches[blockIdx.y];
  int m0 = 0, m1 = 0, m2 = 0, m3 = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < P.N; i += (long long)gridDim.x * blockDim.x) {
    const uint32_t v = lab4[P.pix + i];
    m0 = max(m0, (int)(v & 255));
    m1 = max(m1, (int)((v >> 8) & 255));
    m2 = max(m2, (int)((v >> 16) & 255));
    m3 = max(m3, (int)(v >> 24));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    m0 = max(m0, __shfl_xor_sync(FULL, m0, o));
    m1 = max(m1, __shfl_xor_sync(FULL, m1, o));
    m2 = max(m2, __shfl_xor_sync(FULL, m2, o));
    m3 = max(m3, __shfl_xor_sync(FULL, m3, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&nbins[4 * blockIdx.y + 0], m0);
    atomicMax(&nbins[4 * blockIdx.y + 1], m1);
    atomicMax(&nbins[4 * blockIdx.y + 2], m2);
    atomicMax(&nbins[4 * blockIdx.y + 3], m3);
  }
}

// ---------------------------------------------------------------- NMS
__device__ __forceinline__ void argmax8(const float* __restrict__ mo, long long N, long long p,
                                        float& a, int& ind) {
  float mv = -FLT_MAX;
  int mi = 0;
#pragma unroll
  for (int o = 0; o < 8; o++) {
    const float d = mo[o * N + p];
    if (d > mv) {
      mv = d;
      mi = o;
    }
  }
  a = mv < 0.f ? 0.f : mv;
  ind = mi;
}

__global__ void __launch_bounds__(256) k_nms(const PatchDev* __restrict__ patches,
                                             const int4* __restrict__ work, const float* __restrict__ mpbo,
                                             float* __restrict__ mpb) {
  const int4 w = work[blockIdx.x];
  const PatchDev P = patches[w.x];
  const int y = w.y + threadIdx.x / 16, x = w.z + threadIdx.x % 16;
  if (y >= P.H || x >= P.W) return;
  const float* mo = mpbo + P.pix * 8;
  const long long N = P.N, p = (long long)y * P.W + x;
  float v;
  int i;
  argmax8(mo, N, p, v, i);
  // x of lib_image is the row, y the column
  float out = 0.f;
  bool ok = true;
  int nr[4], nc[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    nr[k] = y + c_nms_nb[i][k][0];
    nc[k] = x + c_nms_nb[i][k][1];
    ok = ok && nr[k] >= 0 && nr[k] < P.H && nc[k] >= 0 && nc[k] < P.W;
  }
  if (ok) {
    float va[4];
    int ia[4];
#pragma unroll
    for (int k = 0; k < 4; k++) argmax8(mo, N, (long long)nr[k] * P.W + nc[k], va[k], ia[k]);
    const float d = c_nms_d[i];
    const float v0 = (1.0f - d) * va[0] * c_nms_cos[i][ia[0]] + d * va[1] * c_nms_cos[i][ia[1]];
    const float v1 = (1.0f - d) * va[2] * c_nms_cos[i][ia[2]] + d * va[3] * c_nms_cos[i][ia[3]];
    if (v > v0 && v > v1) out = v;
  }
  // clip of multiscalePb.cpp:249-261 with the x1.2 of MATLAB's max(0,min(1,1.2 v)) (D7)
  out = (1.2f * out > 1.f) ? 1.f : 1.2f * out;
  if (out < 0.f) out = 0.f;
  mpb[P.pix + p] = out;
}

cudaError_t launch_maxlabel(const PatchDev* patches, int npatch, const uint32_t* lab4, int* nbins,
                            cudaStream_t s) {
  cudaMemsetAsync(nbins, 0, sizeof(int) * 4 * npatch, s);
  dim3 g(16, npatch);
  k_maxlabel<<<g, 256, 0, s>>>(patches, lab4, nbins);
  return cudaGetLastError();
}

cudaError_t launch_cues(const PatchDev* patches, const int4* work, int nwork, const uint32_t* lab4,
                        const int* nbins, float* mpbo, float* go, float* raw, uint8_t* counts, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_cues<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCueSmem);
    cudaFuncSetAttribute(k_cues<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCueSmem);
    attr = true;
  }
  if (nwork == 0) return cudaSuccess;
  if (raw)
    k_cues<true><<<nwork, CT_WARPS * 32, kCueSmem, s>>>(patches, work, lab4, nbins, mpbo, go, raw, counts);
  else
    k_cues<false><<<nwork, CT_WARPS * 32, kCueSmem, s>>>(patches, work, lab4, nbins, mpbo, go, raw, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_nms(const PatchDev* patches, const int4* work, int nwork, const float* mpbo,
                       float* mpb, cudaStream_t s) {
  if (nwork == 0) return cudaSuccess;
  k_nms<<<nwork, 256, 0, s>>>(patches, work, mpbo, mpb);
  return cudaGetLastError();
}

}  // namespace gpb
