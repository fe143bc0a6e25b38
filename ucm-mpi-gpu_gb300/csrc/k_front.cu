// k_front.cu -- colour conversion and Schmid textons (sm_103a).
//
// (1) convert: packed B<<16|G<<8|R (src/globalPb.cpp:264-276) -> 8-bit grey
//     (CV_BGR2GRAY, src/SPFeatures.cpp:27) and the 25-bin L, a, b labels of
//     mex_pb_parts_final_selected.cpp:97-134 (lib_image.cc:123-343).
// (2) texton: the 13 S filters (49x49, src/SPFeatures.cpp:117-183) correlated
//     with the reflect-padded grey image and the nearest of K codewords
//     (src/SPFeatures.cpp:277-360, argmin fixed).  The S filters are radial,
//     so the window folds into 325 symmetric groups (|dy|,|dx|) whose integer
//     pixel sums are exact; the 13 responses and the 32 distances run in FP32
//     with an a-priori error bound.  A pixel whose best and second-best
//     distances are closer than the bound goes to (3).
// (3) texton_repair: one warp per flagged pixel recomputes the responses in
//     FP64 over radius rings in ascending order with unfused multiply/add --
//     the exact arithmetic of the FP64 restatement -- so labels are identical.
#include <stdint.h>

#include "gpb_internal.h"
#include "kernels.h"

namespace gpb {

__constant__ float c_k32[kNschmid][kSchmidGroups];
__constant__ int c_goff_start[kSchmidGroups + 1];
__constant__ int16_t c_goff_off[2401];  // dy * 64 + dx: the displacement in the 64-wide staged tile
__constant__ float c_codebook[kNschmid][kMaxCodewords];
__constant__ float c_errb[kNschmid];
__constant__ double c_gamma[256];
__constant__ int c_K;

void upload_front(const HostTables& t, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c_k32, t.k32_group, sizeof(t.k32_group), 0, cudaMemcpyHostToDevice, s);
  int start[kSchmidGroups + 1];
  int8_t dy[2401], dx[2401];
  int n = 0;
  for (int g = 0; g < kSchmidGroups; g++) {
    start[g] = n;
    const int a = t.group_a[g], b = t.group_b[g];
    int cand[8][2] = {{a, b}, {a, -b}, {-a, b}, {-a, -b}, {b, a}, {b, -a}, {-b, a}, {-b, -a}};
    for (int i = 0; i < 8; i++) {
      bool dup = false;
      for (int j = start[g]; j < n; j++)
        if (dy[j] == cand[i][0] && dx[j] == cand[i][1]) dup = true;
      if (dup) continue;
      dy[n] = (int8_t)cand[i][0];
      dx[n] = (int8_t)cand[i][1];
      n++;
    }
  }
  start[kSchmidGroups] = n;
  cudaMemcpyToSymbolAsync(c_goff_start, start, sizeof(start), 0, cudaMemcpyHostToDevice, s);
  int16_t off[2401];
  for (int j = 0; j < n; j++) off[j] = (int16_t)(dy[j] * 64 + dx[j]);
  cudaMemcpyToSymbolAsync(c_goff_off, off, sizeof(int16_t) * n, 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_errb, t.err_bound, sizeof(t.err_bound), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_gamma, t.gamma_lut, sizeof(t.gamma_lut), 0, cudaMemcpyHostToDevice, s);
}

void upload_codebook(const float* cb, int K, cudaStream_t s) {
  float tmp[kNschmid][kMaxCodewords] = {};
  for (int f = 0; f < kNschmid; f++)
    for (int k = 0; k < K; k++) tmp[f][k] = cb[f * K + k];
  cudaMemcpyToSymbolAsync(c_codebook, tmp, sizeof(tmp), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_K, &K, sizeof(int), 0, cudaMemcpyHostToDevice, s);
}

__device__ __forceinline__ int reflect(int i, int n) {
  // BORDER_REFLECT (edge repeated); patches are >= 32 px so one fold suffices
  // for every padding used here, the loop is bounded by the two folds
  for (int it = 0; it < 4 && (i < 0 || i >= n); it++) i = (i < 0) ? -i - 1 : 2 * n - 1 - i;
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

// ---------------------------------------------------------------- convert
// Lab chain with no fused multiply-add, in the order of the reference:
// gamma (table of pow(u/255, 2.5)), rgb_to_xyz, xyz_to_lab, lab_normalize,
// quantize_values (floor(v*25), 25 -> 24).
__device__ __forceinline__ int quant25(double v, int nbins) {
  if (v < 0) v = 0;
  else if (v > 1) v = 1;
  int q = (int)floor(__dmul_rn(v, (double)nbins));
  return q == nbins ? nbins - 1 : q;
}

// Lab bins (L | a << 8 | b << 16) of one BGR colour
__device__ __forceinline__ uint32_t lab_bins_of(int R, int G, int B) {
  // D1 fixed: r = R, b = B
  const double r = c_gamma[R], g = c_gamma[G], b = c_gamma[B];
  const double X = __dadd_rn(__dadd_rn(__dmul_rn(0.412453, r), __dmul_rn(0.357580, g)), __dmul_rn(0.180423, b));
  const double Y = __dadd_rn(__dadd_rn(__dmul_rn(0.212671, r), __dmul_rn(0.715160, g)), __dmul_rn(0.072169, b));
  const double Z = __dadd_rn(__dadd_rn(__dmul_rn(0.019334, r), __dmul_rn(0.119193, g)), __dmul_rn(0.950227, b));
  const double x = __ddiv_rn(X, 0.950456), y = __ddiv_rn(Y, 1.000000), z = __ddiv_rn(Z, 1.088754);
  const double th = 0.008856, third = 1.0 / 3.0, c16 = 16.0 / 116.0;
  const double fx = (x > th) ? pow(x, third) : __dadd_rn(__dmul_rn(7.787, x), c16);
  const double fy = (y > th) ? pow(y, third) : __dadd_rn(__dmul_rn(7.787, y), c16);
  const double fz = (z > th) ? pow(z, third) : __dadd_rn(__dmul_rn(7.787, z), c16);
  const double L = (y > th) ? __dsub_rn(__dmul_rn(116.0, pow(y, third)), 16.0) : __dmul_rn(903.3, y);
  const double A = __dmul_rn(500.0, __dsub_rn(fx, fy));
  const double Bb = __dmul_rn(200.0, __dsub_rn(fy, fz));
  const int qL = quant25(__ddiv_rn(L, 100.0), 25);
  const int qa = quant25(__ddiv_rn(__dsub_rn(A, -73.0), 168.0), 25);
  const int qb = quant25(__ddiv_rn(__dsub_rn(Bb, -73.0), 168.0), 25);
  return (uint32_t)qL | ((uint32_t)qa << 8) | ((uint32_t)qb << 16);
}

__device__ __forceinline__ uint8_t grey_of(int R, int G, int B) {
  return (uint8_t)((R * 4899 + G * 9617 + B * 1868 + (1 << 13)) >> 14);
}

__global__ void __launch_bounds__(256) k_convert(const uint32_t* __restrict__ packed, long long n,
                                                 uint8_t* __restrict__ grey,
                                                 uint32_t* __restrict__ lab4) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t px = packed[i];
  const int B = (px >> 16) & 255, G = (px >> 8) & 255, R = px & 255;
  grey[i] = grey_of(R, G, B);
  lab4[i] = lab_bins_of(R, G, B);
}

// The Lab bins of all 2^24 colours, indexed by the packed value B<<16|G<<8|R:
// the pipeline's convert step then gathers from this table (FP64 cube roots
// run at a small fraction of the FP32 rate on this part).
__global__ void __launch_bounds__(256) k_lab_table(uint32_t* __restrict__ table) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < (1u << 24); c += gridDim.x * blockDim.x)
    table[c] = lab_bins_of(c & 255, (c >> 8) & 255, c >> 16);
}

__global__ void __launch_bounds__(256) k_convert_lut(const uint32_t* __restrict__ packed, long long n,
                                                     const uint32_t* __restrict__ table,
                                                     uint8_t* __restrict__ grey, uint32_t* __restrict__ lab4) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t px = packed[i];
  grey[i] = grey_of(px & 255, (px >> 8) & 255, (px >> 16) & 255);
  lab4[i] = __ldg(table + (px & 0xffffffu));
}

// ----------------------------------------------------------------- texton
constexpr int TX_T = 16;              // 16 x 16 outputs per block
constexpr int TX_W = TX_T + 2 * 24;   // 64
static_assert(TX_W == 64, "c_goff_off is built for a 64-wide staged tile");

// TX_THREADS threads per 16 x 16 tile: a thread owns the TX_PIX pixels
// (ty0 + ROWSTEP k, tx), so every offset-table and filter-weight load from
// constant memory serves TX_PIX pixels (the kernel is bound by those loads,
// not by arithmetic).  Each pixel's arithmetic is the same for every thread
// count, so the variants (32, 64 or 128 threads) give identical labels and
// the autotuner picks among them.
template <int TX_THREADS>
__global__ void __launch_bounds__(TX_THREADS) k_texton(const PatchDev* __restrict__ patches,
                                                       const int4* __restrict__ work,
                                                       const uint8_t* __restrict__ grey,
                                                       uint32_t* __restrict__ lab4, int* __restrict__ repair_list,
                                                       int* __restrict__ repair_count, int repair_cap) {
  constexpr int TX_PIX = TX_T * TX_T / TX_THREADS;
  __shared__ uint8_t tile[TX_W * TX_W];
  const int4 w = work[blockIdx.x];  // (patch, ty0, tx0, -)
  const PatchDev P = patches[w.x];
  const uint8_t* g = grey + P.pix;
  for (int i = threadIdx.x; i < TX_W * TX_W; i += blockDim.x) {
    const int yy = reflect(w.y - 24 + i / TX_W, P.H), xx = reflect(w.z - 24 + i % TX_W, P.W);
    tile[i] = g[(long long)yy * P.W + xx];
  }
  __syncthreads();
  const int ty0 = threadIdx.x / TX_T, tx = threadIdx.x % TX_T;
  constexpr int ROWSTEP = TX_THREADS / TX_T;  // 4
  // FMA accumulation: |error of R_f| <= u * sum_k |partial sum_k| (each step
  // rounds once), tracked at run time in E_f
  float R[TX_PIX][kNschmid], E[TX_PIX][kNschmid];
#pragma unroll
  for (int k = 0; k < TX_PIX; k++)
#pragma unroll
    for (int f = 0; f < kNschmid; f++) R[k][f] = E[k][f] = 0.f;
  const uint8_t* c = tile + (ty0 + 24) * TX_W + (tx + 24);
  for (int gi = 0; gi < kSchmidGroups; gi++) {
    int sum[TX_PIX];
#pragma unroll
    for (int k = 0; k < TX_PIX; k++) sum[k] = 0;
    const int e = c_goff_start[gi + 1];
    for (int j = c_goff_start[gi]; j < e; j++) {
      const int off = c_goff_off[j];
#pragma unroll
      for (int k = 0; k < TX_PIX; k++) sum[k] += c[off + k * ROWSTEP * TX_W];
    }
#pragma unroll
    for (int f = 0; f < kNschmid; f++) {
      const float kf = c_k32[f][gi];
#pragma unroll
      for (int k = 0; k < TX_PIX; k++) {
        R[k][f] = fmaf(kf, (float)sum[k], R[k][f]);
        E[k][f] += fabsf(R[k][f]);
      }
    }
  }
  const int K = c_K;
#pragma unroll
  for (int k = 0; k < TX_PIX; k++) {
    const int y = w.y + ty0 + k * ROWSTEP, x = w.z + tx;
    if (y >= P.H || x >= P.W) continue;
#pragma unroll
    for (int f = 0; f < kNschmid; f++) E[k][f] = E[k][f] * 6.0e-8f * 1.01f + 1e-6f;
    float d1 = 3.4e38f, d2 = 3.4e38f;
    int k1 = 0, k2 = 0;
    for (int q = 0; q < K; q++) {
      float d = 0.f;
#pragma unroll
      for (int f = 0; f < kNschmid; f++) {
        const float t = R[k][f] - c_codebook[f][q];
        d = fmaf(t, t, d);
      }
      if (d < d1) {
        d2 = d1;
        k2 = k1;
        d1 = d;
        k1 = q;
      } else if (d < d2) {
        d2 = d;
        k2 = q;
      }
    }
    // error bound of d(k1) and d(k2): responses off by at most E_f each, plus
    // the FP32 rounding of the distance sums themselves
    float margin = 0.f;
#pragma unroll
    for (int f = 0; f < kNschmid; f++) {
      const float eb = E[k][f];
      margin += 2.f * eb * (fabsf(R[k][f] - c_codebook[f][k1]) + fabsf(R[k][f] - c_codebook[f][k2]) + eb);
    }
    margin = 2.f * margin + 4e-6f * (d1 + d2) + 1e-6f;
    const long long pix = P.pix + (long long)y * P.W + x;
    uint32_t v = lab4[pix] & 0x00ffffffu;
    lab4[pix] = v | ((uint32_t)k1 << 24);
    if (K > 1 && d2 - d1 <= margin) {
      const int slot = atomicAdd(repair_count, 1);
      if (slot < repair_cap) {
        repair_list[2 * slot] = w.x;
        repair_list[2 * slot + 1] = y * P.W + x;
      }
    }
  }
}

// FP64 repair: ring sums in integers, then sum_r K32[f][r] * S[r] in
// ascending ring order and the squared distances, all without contraction.
__global__ void __launch_bounds__(128) k_texton_repair(const PatchDev* __restrict__ patches,
                                                       const uint8_t* __restrict__ grey,
                                                       uint32_t* __restrict__ lab4,
                                                       const int* __restrict__ repair_list,
                                                       const int* __restrict__ repair_count,
                                                       int repair_cap, const double* __restrict__ k32_ring,
                                                       const int* __restrict__ ring_of, int n_rings) {
  extern __shared__ int sh[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  int* S = sh + warp * n_rings;
  __shared__ double Rsh[4][kNschmid];
  const int total = min(*repair_count, repair_cap);
  for (int item = blockIdx.x * nw + warp; item < total; item += gridDim.x * nw) {
    const PatchDev P = patches[repair_list[2 * item]];
    const int p = repair_list[2 * item + 1];
    const int y = p / P.W, x = p % P.W;
    for (int r = lane; r < n_rings; r += 32) S[r] = 0;
    __syncwarp();
    const uint8_t* g = grey + P.pix;
    for (int o = lane; o < 2401; o += 32) {
      const int dy = o / 49 - 24, dx = o % 49 - 24;
      const int v = g[(long long)reflect(y + dy, P.H) * P.W + reflect(x + dx, P.W)];
      atomicAdd(&S[ring_of[o]], v);
    }
    __syncwarp();
    if (lane < kNschmid) {
      double acc = 0;
      for (int r = 0; r < n_rings; r++)
        acc = __dadd_rn(acc, __dmul_rn(k32_ring[lane * n_rings + r], (double)S[r]));
      Rsh[warp][lane] = acc;
    }
    __syncwarp();
    const int K = c_K;
    double d = 1e300;
    if (lane < K) {
      d = 0;
      for (int f = 0; f < kNschmid; f++) {
        const double t = __dsub_rn(Rsh[warp][f], (double)c_codebook[f][lane]);
        d = __dadd_rn(d, __dmul_rn(t, t));
      }
    }
    // argmin, first index on ties
    int best = lane;
    for (int off = 16; off > 0; off >>= 1) {
      const double od = __shfl_xor_sync(0xffffffffu, d, off);
      const int ob = __shfl_xor_sync(0xffffffffu, best, off);
      if (od < d || (od == d && ob < best)) {
        d = od;
        best = ob;
      }
    }
    if (lane == 0) {
      const long long pix = P.pix + p;
      lab4[pix] = (lab4[pix] & 0x00ffffffu) | ((uint32_t)best << 24);
    }
    __syncwarp();
  }
}

cudaError_t launch_convert(const uint32_t* packed, long long n, uint8_t* grey, uint32_t* lab4,
                           cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_convert<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(packed, n, grey, lab4);
  return cudaGetLastError();
}
cudaError_t launch_lab_table(uint32_t* table, cudaStream_t s) {
  k_lab_table<<<4096, 256, 0, s>>>(table);
  return cudaGetLastError();
}
cudaError_t launch_convert_lut(const uint32_t* packed, long long n, const uint32_t* table, uint8_t* grey,
                               uint32_t* lab4, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_convert_lut<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(packed, n, table, grey, lab4);
  return cudaGetLastError();
}

cudaError_t launch_texton(const PatchDev* patches, const int4* work, int nwork, const uint8_t* grey,
                          uint32_t* lab4, int* repair_list, int* repair_count, int repair_cap,
                          cudaStream_t s, int variant) {
  if (nwork == 0) return cudaSuccess;
  if (variant == 0)
    k_texton<32><<<nwork, 32, 0, s>>>(patches, work, grey, lab4, repair_list, repair_count, repair_cap);
  else if (variant == 2)
    k_texton<128><<<nwork, 128, 0, s>>>(patches, work, grey, lab4, repair_list, repair_count, repair_cap);
  else
    k_texton<64><<<nwork, 64, 0, s>>>(patches, work, grey, lab4, repair_list, repair_count, repair_cap);
  return cudaGetLastError();
}

cudaError_t launch_texton_repair(const PatchDev* patches, const uint8_t* grey, uint32_t* lab4,
                                 const int* repair_list, const int* repair_count, int repair_cap,
                                 const double* k32_ring, const int* ring_of, int n_rings,
                                 cudaStream_t s) {
  k_texton_repair<<<304, 128, 4 * n_rings * sizeof(int), s>>>(patches, grey, lab4, repair_list, repair_count,
                                                             repair_cap, k32_ring, ring_of, n_rings);
  return cudaGetLastError();
}

}  // namespace gpb
