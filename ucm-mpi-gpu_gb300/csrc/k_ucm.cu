// k_ucm.cu -- the data-parallel stages of the oriented watershed transform
// and the ultrametric contour map (Contours2Ucm, src/contours2ucm.cpp).
//
//   k_ucm_pbmax    max over the 8 orientation planes, per-image min / max
//                  (contours2ucm.cpp:255-270)
//   k_ucm_quant    8-bit quantisation, FP64 alpha/beta and round-half-even
//                  saturation as OpenCV's convertTo (contours2ucm.cpp:272-278)
//   k_ws_rowsort   per row, the columns stably sorted by grey level
//   k_ws_flood     the level-by-level, raster-order flooding of
//                  watershed_yupeng (src/watershed.cpp:28-108) as a wavefront:
//                  level l of row x is processed at step t = 2l + x, when
//                  every pixel it reads (rows x-1..x+1 at lower levels, row
//                  x-1 at the same level, its own row to the left) is final
//                  and no other thread of the step writes a row it reads
//   k_ucm_paint    contour-strength painting along the fitted edges
//                  (contours2ucm.cpp:374-399)
//   k_ucm_super    SuperContour4C (contours2ucm.cpp:24-78) on the doubled grid
//   k_art_*        CleanWatersheds (contours2ucm.cpp:80-189): isolated zeros
//                  of the doubled grid, fixed in row-major order
//   k_ccl_*        8-connected labelling of the zeros of the cleaned grid,
//                  numbered in row-major order of each component's first
//                  cell (bwlabelManu, src/MATLAB_functions.cpp:164-217)
//   k_ucm_finish   region labels of the pixels and the padded strength grid
//                  ws_wt2 (contours2ucm.cpp:439-458)
//
// The flooding runs one CTA per image over a batch; the other stages run
// per image, grid-stride over it (the artefact fixes in one thread).
#include <stdint.h>

#include "ucm_dev.h"

namespace gpb {

namespace {

__device__ __forceinline__ unsigned f2ord(float f) {  // order-preserving float -> uint
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

}  // namespace

// ---------------------------------------------------------------- pb, u8

__global__ void __launch_bounds__(256) k_ucm_pbmax(const float* __restrict__ orient, long long N,
                                                   float* __restrict__ pb, unsigned* __restrict__ mm) {
  unsigned lo = 0xffffffffu, hi = 0u;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    float m = orient[i];
    for (int o = 1; o < 8; o++) {
      const float v = orient[(long long)o * N + i];
      if (m < v) m = v;  // the later plane wins only when strictly larger
    }
    pb[i] = m;
    lo = min(lo, f2ord(m));
    hi = max(hi, f2ord(m));
  }
  for (int d = 16; d; d >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, d));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, d));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(mm, lo);
    atomicMax(mm + 1, hi);
  }
}

__global__ void __launch_bounds__(256) k_ucm_quant(const float* __restrict__ pb, long long N,
                                                   const unsigned* __restrict__ mm, uint8_t* __restrict__ q) {
  const double lo = (double)ord2f(mm[0]), hi = (double)ord2f(mm[1]);
  const double alpha = 255.0 / (hi - lo), beta = __ddiv_rn(-255.0 * lo, hi - lo);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const double v = __dadd_rn(__dmul_rn((double)pb[i], alpha), beta);
    uint8_t r = 0;
    if (v == v) {  // NaN (a constant image) saturates to 0
      const double t = rint(v);
      r = (uint8_t)(t < 0.0 ? 0.0 : (t > 255.0 ? 255.0 : t));
    }
    q[i] = r;
  }
}

// ---------------------------------------------------------------- flooding

// One warp per row: a stable counting sort of the row's columns by level.
// off[row * 257 + l] is the first position of level l; cols[row * W + k]
// the k-th column in (level, column) order.
__global__ void __launch_bounds__(32) k_ws_rowsort(const uint8_t* __restrict__ q, int H, int W,
                                                   int32_t* __restrict__ off, uint16_t* __restrict__ cols) {
  __shared__ int cnt[256];
  const int row = blockIdx.x, lane = threadIdx.x;
  if (row >= H) return;
  for (int v = lane; v < 256; v += 32) cnt[v] = 0;
  __syncwarp();
  const uint8_t* r = q + (size_t)row * W;
  const unsigned lt = (1u << lane) - 1u;
  for (int c0 = 0; c0 < W; c0 += 32) {
    const int c = c0 + lane;
    const bool in = c < W;
    const int v = in ? r[c] : 256 + lane;  // out-of-row lanes match nobody
    const unsigned peers = __match_any_sync(0xffffffffu, v);
    if (in && (peers & lt) == 0) cnt[v] += __popc(peers);
    __syncwarp();
  }
  // exclusive scan of the 256 counts: 8 per lane
  int loc[8], s = 0;
  for (int k = 0; k < 8; k++) {
    loc[k] = s;
    s += cnt[lane * 8 + k];
  }
  int inc = s;
  for (int d = 1; d < 32; d <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += t;
  }
  const int base = inc - s;
  __syncwarp();
  for (int k = 0; k < 8; k++) {
    cnt[lane * 8 + k] = base + loc[k];
    off[(size_t)row * 257 + lane * 8 + k] = base + loc[k];
  }
  if (lane == 0) off[(size_t)row * 257 + 256] = W;
  __syncwarp();
  for (int c0 = 0; c0 < W; c0 += 32) {
    const int c = c0 + lane;
    const bool in = c < W;
    const int v = in ? r[c] : 256 + lane;
    const unsigned peers = __match_any_sync(0xffffffffu, v);
    if (in) cols[(size_t)row * W + cnt[v] + __popc(peers & lt)] = (uint16_t)c;
    __syncwarp();
    if (in && (peers & lt) == 0) cnt[v] += __popc(peers);
    __syncwarp();
  }
}

// One CTA of 1024 threads per image; warp w owns grey levels w, w + 32, ...
// At step t a warp takes, level by level, the row t - 2l of its level l
// and walks that row's pixels of level l in column order, 32 at a time:
// every lane gathers the labels of its pixel's 8 neighbours at once, then
// runs of adjacent pixels are resolved lane by lane, and most lanes settle
// without waiting because their label cannot depend on the left one.  The
// next 32 pixels' neighbours are loaded before the current ones resolve;
// the one of them that the current 32 may still write (the left neighbour
// of the next first pixel) is taken from the current last pixel instead.
// ws is -1 (not reached), 0 (watershed pixel) or a region label (> 0): a
// new region takes the label 1 + its pixel index.
__global__ void __launch_bounds__(1024) k_ws_flood(const UcmImage* __restrict__ imgs, const int32_t* __restrict__ off,
                                                   const uint16_t* __restrict__ cols, int32_t* __restrict__ ws) {
  const UcmImage I = imgs[blockIdx.x];
  const int H = I.H, W = I.W, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int32_t* L = ws + I.pix;
  const int32_t* O = off + I.row0 * 257;
  const uint16_t* C = cols + I.pix;
  for (long long p = threadIdx.x; p < (long long)H * W; p += blockDim.x) L[p] = -1;
  __syncthreads();
  constexpr int kLeft = 3;  // index of (0, -1) in the neighbour order below
  const int steps = 2 * 255 + H;
  for (int t = 0; t < steps; t++) {
    for (int lvl = warp; lvl < 256; lvl += 32) {
      const int x = t - 2 * lvl;
      if (x < 0 || x >= H) continue;
      const int b = O[x * 257 + lvl], e = O[x * 257 + lvl + 1];
      if (b >= e) continue;
      // the labels around the k-th pixel of the segment (-1 outside the image or the segment)
      auto gather = [&](int k, int& y, int (&nbv)[8]) {
        y = k < e ? (int)C[(size_t)x * W + k] : -4;
        int idx = 0;
        for (int i = -1; i <= 1; i++)
          for (int j = -1; j <= 1; j++) {
            if (i == 0 && j == 0) continue;
            const int xi = x + i, yj = y + j;
            nbv[idx++] = (k < e && xi >= 0 && xi < H && yj >= 0 && yj < W) ? L[(size_t)xi * W + yj] : -1;
          }
      };
      int y, nbv[8];
      gather(b + lane, y, nbv);
      int carry = -1, ylast = -10;  // final label and column of the previous chunk's last pixel
      for (int k0 = b; k0 < e; k0 += 32) {
        const int k = k0 + lane;
        const bool in = k < e;
        int yn, nbn[8];
        gather(k0 + 32 + lane, yn, nbn);  // the next chunk, in flight while this one resolves
        const int yl = __shfl_up_sync(0xffffffffu, y, 1);
        const bool cross = in && lane == 0 && y - 1 == ylast;          // left pixel in the previous chunk
        const bool dep = in && (cross || (lane > 0 && yl == y - 1));  // left pixel is this level's, unresolved here
        int s = -1;  // -1: no labelled neighbour, 0: two different labels, else the one label
        for (int idx = 0; idx < 8; idx++) {
          if (idx == kLeft && dep) continue;
          const int v = nbv[idx];
          if (v > 0) s = (s == -1) ? v : (v != s ? 0 : s);
        }
        const int sl = __shfl_up_sync(0xffffffffu, s, 1);
        const int mine = x * W + y + 1;
        auto after = [&](int pv) {  // this pixel's label given the left pixel's
          return (s == -1) ? (pv > 0 ? pv : mine) : ((pv > 0 && pv != s) ? 0 : s);
        };
        int done, val;
        if (cross) {
          val = after(carry);
          done = 1;
        } else {
          // final without the left lane: no dependence, a conflict already, or
          // a label the left pixel can only repeat or have lost to a conflict
          done = !in || !dep || s == 0 || (s > 0 && (sl == s || sl == 0));
          val = !dep ? (s >= 0 ? s : mine) : s;
        }
        while (!__all_sync(0xffffffffu, done)) {
          const int pv = __shfl_up_sync(0xffffffffu, val, 1);
          const int pd = __shfl_up_sync(0xffffffffu, done, 1);
          if (!done && pd) {
            val = after(pv);
            done = 1;
          }
        }
        if (in) L[(size_t)x * W + y] = val;
        const int last = min(31, e - 1 - k0);
        carry = __shfl_sync(0xffffffffu, val, last);
        ylast = __shfl_sync(0xffffffffu, y, last);
        __syncwarp();
        y = yn;
        for (int idx = 0; idx < 8; idx++) nbv[idx] = nbn[idx];
      }
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) k_ws_bw(const int32_t* __restrict__ ws, long long N, uint8_t* __restrict__ bw) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
    bw[i] = ws[i] == 0;
}

// ---------------------------------------------------------------- painting

// One thread per painted pixel: the edge's orientation plane at that pixel,
// max-ed into the strength map (which starts at 0, so negatives leave 0).
__global__ void __launch_bounds__(256) k_ucm_paint(const int32_t* __restrict__ pix, const uint8_t* __restrict__ ori,
                                                   int n, const float* __restrict__ orient, long long N,
                                                   unsigned* __restrict__ wswt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int p = pix[i];
    const float v = orient[(long long)ori[i] * N + p];
    if (v > 0.0f) atomicMax(wswt + p, __float_as_uint(v));  // non-negative floats order as their bits
  }
}

// ---------------------------------------------------------------- super contour

// pb2 (2H x 2W): even-even = ws_wt, even-odd = min of horizontal pairs,
// odd-even = min of vertical pairs, odd-odd = 0; the last row repeats the
// one before, the last column is max(itself, the one before).
__device__ __forceinline__ float super_base(const float* w, int H, int W, int r, int c) {
  const int i = r >> 1, j = c >> 1;
  if (!(r & 1) && !(c & 1)) return w[(size_t)i * W + j];
  if (!(r & 1) && (c & 1)) return c == 2 * W - 1 ? 0.0f : fminf(w[(size_t)i * W + j], w[(size_t)i * W + j + 1]);
  if ((r & 1) && !(c & 1)) return r == 2 * H - 1 ? 0.0f : fminf(w[(size_t)i * W + j], w[(size_t)(i + 1) * W + j]);
  return 0.0f;
}

__global__ void __launch_bounds__(256) k_ucm_super(const float* __restrict__ wswt, int H, int W,
                                                   float* __restrict__ pb2) {
  const long long n = 4LL * H * W;
  const int W2 = 2 * W;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    int r = (int)(k / W2);
    const int c = (int)(k % W2);
    if (r == 2 * H - 1) r = 2 * H - 2;
    float v = super_base(wswt, H, W, r, c);
    if (c == W2 - 1) {
      const float a = v, b = super_base(wswt, H, W, r, c - 1);
      v = a < b ? b : a;
    }
    pb2[k] = v;
  }
}

// ---------------------------------------------------------------- artefacts

__device__ __forceinline__ bool isolated_zero(const float* g, int R, int C, int r, int c) {
  if (g[(size_t)r * C + c] != 0.0f) return false;
  for (int i = -1; i <= 1; i++)
    for (int j = -1; j <= 1; j++) {
      if (i == 0 && j == 0) continue;
      const int rr = r + i, cc = c + j;
      if (rr < 0 || rr >= R || cc < 0 || cc >= C) continue;
      if (g[(size_t)rr * C + cc] == 0.0f) return false;
    }
  return true;
}

// one warp per row: the row's isolated zeros, counted / written in column order
__global__ void __launch_bounds__(32) k_art_rows(const float* __restrict__ g, int R, int C, int32_t* __restrict__ cnt,
                                                 const int32_t* __restrict__ base, int32_t* __restrict__ list) {
  const int r = blockIdx.x, lane = threadIdx.x;
  if (r >= R) return;
  int k = base ? base[r] : 0;
  for (int c0 = 0; c0 < C; c0 += 32) {
    const int c = c0 + lane;
    const bool hit = c < C && isolated_zero(g, R, C, r, c);
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if (base && hit) list[k + __popc(m & ((1u << lane) - 1u))] = r * C + c;
    k += __popc(m);
  }
  if (!base && lane == 0) cnt[r] = k;
}

// exclusive scan of n ints, in place, by one CTA; total to *sum
__global__ void __launch_bounds__(1024) k_scan_small(int32_t* __restrict__ a, int n, int32_t* __restrict__ sum) {
  __shared__ int32_t part[1024];
  const int per = (n + 1023) / 1024, t = threadIdx.x, b = t * per;
  int32_t s = 0;
  for (int i = b; i < b + per && i < n; i++) s += a[i];
  part[t] = s;
  __syncthreads();
  for (int d = 1; d < 1024; d <<= 1) {
    const int32_t v = t >= d ? part[t - d] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int32_t run = part[t] - s;
  for (int i = b; i < b + per && i < n; i++) {
    const int32_t v = a[i];
    a[i] = run;
    run += v;
  }
  if (t == 1023) *sum = part[1023];
}

// The fixes of CleanWatersheds in list order, one thread.  Reads outside
// the grid (artefacts within two cells of the border) read 0; writes there
// are dropped.
__global__ void k_art_fix(float* __restrict__ g, int R, int C, const int32_t* __restrict__ list,
                          const int32_t* __restrict__ n) {
  if (threadIdx.x || blockIdx.x) return;
  const long long tot = (long long)R * C;
  auto rd = [&](int r, int c) -> float {
    const long long k = (long long)r * C + c;  // a continuous matrix: columns wrap into the next row
    return (k >= 0 && k < tot) ? g[k] : 0.0f;
  };
  auto wr = [&](int r, int c, float v) {
    const long long k = (long long)r * C + c;
    if (k >= 0 && k < tot) g[k] = v;
  };
  for (int a = 0; a < *n; a++) {
    const int xc = list[a] / C, yc = list[a] % C;
    float vec[4];
    vec[0] = fmaxf(rd(xc - 2, yc - 1), rd(xc - 1, yc - 2));
    vec[1] = fmaxf(rd(xc + 2, yc - 1), rd(xc + 1, yc - 2));
    vec[2] = fmaxf(rd(xc + 2, yc + 1), rd(xc + 1, yc + 2));
    vec[3] = fmaxf(rd(xc - 2, yc + 1), rd(xc - 1, yc + 2));
    int id = 0;
    float nd = vec[0];
    for (int i = 1; i < 4; i++)
      if (vec[i] < nd) nd = vec[i], id = i;
    const int sx = (id == 1 || id == 2) ? 1 : -1, sy = (id >= 2) ? 1 : -1;
    const float p = rd(xc + 2 * sx, yc + sy), q = rd(xc + sx, yc + 2 * sy);
    if (p < q) {
      wr(xc, yc + sy, 0.0f);
      wr(xc + sx, yc, vec[id]);
    } else {
      wr(xc, yc + sy, vec[id]);
      wr(xc + sx, yc, 0.0f);
    }
    wr(xc + sx, yc + sy, vec[id]);
  }
}

// ---------------------------------------------------------------- labelling

__device__ __forceinline__ int ccl_find(const int32_t* p, int a) {
  int b = p[a];
  while (b != a) {
    a = b;
    b = p[a];
  }
  return a;
}

__device__ __forceinline__ void ccl_union(int32_t* p, int a, int b) {
  bool done = false;
  while (!done) {
    a = ccl_find(p, a);
    b = ccl_find(p, b);
    if (a == b) break;
    if (a < b) {
      const int t = a;
      a = b;
      b = t;
    }
    const int old = atomicMin(p + a, b);  // hang the larger root under the smaller
    done = (old == a);
    a = old;
  }
}

__global__ void __launch_bounds__(256) k_ccl_init(const float* __restrict__ g, long long n, int32_t* __restrict__ p) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    p[k] = g[k] == 0.0f ? (int32_t)k : -1;
}

__global__ void __launch_bounds__(256) k_ccl_hook(const float* __restrict__ g, int R, int C, int32_t* __restrict__ p) {
  const long long n = (long long)R * C;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    if (g[k] != 0.0f) continue;
    const int r = (int)(k / C), c = (int)(k % C);
    if (c > 0 && g[k - 1] == 0.0f) ccl_union(p, (int)k, (int)k - 1);
    if (r > 0) {
      if (g[k - C] == 0.0f) ccl_union(p, (int)k, (int)(k - C));
      if (c > 0 && g[k - C - 1] == 0.0f) ccl_union(p, (int)k, (int)(k - C - 1));
      if (c + 1 < C && g[k - C + 1] == 0.0f) ccl_union(p, (int)k, (int)(k - C + 1));
    }
  }
}

// flatten to roots; rank[k] = 1 where k is a root (the component's first cell)
__global__ void __launch_bounds__(256) k_ccl_flat(int32_t* __restrict__ p, long long n, int32_t* __restrict__ root) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    if (p[k] < 0) {
      root[k] = 0;
      continue;
    }
    const int r = ccl_find(p, (int)k);
    p[k] = r;
    root[k] = r == k;
  }
}

// region labels of the pixels (0-based; cells that are not zeros give -1)
// and ws_wt2, the grid padded by its last row and column
__global__ void __launch_bounds__(256) k_ucm_finish(const float* __restrict__ g, const int32_t* __restrict__ p,
                                                    const int32_t* __restrict__ rank, int H, int W,
                                                    int32_t* __restrict__ labels, float* __restrict__ wswt2) {
  const int R = 2 * H, C = 2 * W;
  const long long n2 = (long long)(R + 1) * (C + 1);
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n2; k += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(k / (C + 1)), c = (int)(k % (C + 1));
    wswt2[k] = g[(size_t)(r == R ? R - 1 : r) * C + (c == C ? C - 1 : c)];
    if (r < H && c < W) {
      const long long cell = (long long)(2 * r + 1) * C + 2 * c + 1;
      const int32_t root = p[cell];
      labels[(size_t)r * W + c] = root < 0 ? -1 : rank[root];  // rank is the exclusive count of roots before
    }
  }
}

// exclusive scan of n (up to 2^31) ints through blocks of 1024 x 4
__global__ void __launch_bounds__(1024) k_scan_blocks(int32_t* __restrict__ a, long long n, int32_t* __restrict__ bsum) {
  __shared__ int32_t part[1024];
  const long long b0 = (long long)blockIdx.x * 4096;
  const int t = threadIdx.x;
  int32_t v[4], s = 0;
  for (int k = 0; k < 4; k++) {
    const long long i = b0 + t * 4 + k;
    v[k] = i < n ? a[i] : 0;
    s += v[k];
  }
  part[t] = s;
  __syncthreads();
  for (int d = 1; d < 1024; d <<= 1) {
    const int32_t u = t >= d ? part[t - d] : 0;
    __syncthreads();
    part[t] += u;
    __syncthreads();
  }
  int32_t run = part[t] - s;
  for (int k = 0; k < 4; k++) {
    const long long i = b0 + t * 4 + k;
    if (i < n) a[i] = run;
    run += v[k];
  }
  if (t == 1023) bsum[blockIdx.x] = part[1023];
}

__global__ void __launch_bounds__(256) k_scan_add(int32_t* __restrict__ a, long long n, const int32_t* __restrict__ bsum) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] += bsum[i / 4096];
}

// ---------------------------------------------------------------- launchers

static int grid_for(long long n) {
  const long long g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g));
}

cudaError_t ucm_prepare(const float* d_orient, int H, int W, UcmScratch& s, cudaStream_t st) {
  const long long N = (long long)H * W;
  cudaError_t e = cudaMemsetAsync(s.mm, 0, 2 * sizeof(unsigned), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(s.mm, 0xff, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  k_ucm_pbmax<<<grid_for(N), 256, 0, st>>>(d_orient, N, s.pb, s.mm);
  k_ucm_quant<<<grid_for(N), 256, 0, st>>>(s.pb, N, s.mm, s.q);
  k_ws_rowsort<<<H, 32, 0, st>>>(s.q, H, W, s.off, s.cols);
  return cudaGetLastError();
}

cudaError_t ucm_flood(int nimg, long long total_pix, const UcmScratch& base, cudaStream_t st) {
  k_ws_flood<<<nimg, 1024, 0, st>>>(base.img, base.off, base.cols, base.ws);
  k_ws_bw<<<grid_for(total_pix), 256, 0, st>>>(base.ws, total_pix, base.bw);
  return cudaGetLastError();
}

cudaError_t ucm_paint(const float* d_orient, int H, int W, int npaint, UcmScratch& s, cudaStream_t st) {
  const long long N = (long long)H * W;
  cudaError_t e = cudaMemsetAsync(s.wswt, 0, N * sizeof(float), st);
  if (e != cudaSuccess) return e;
  if (npaint > 0)
    k_ucm_paint<<<grid_for(npaint), 256, 0, st>>>(s.paint_pix, s.paint_ori, npaint, d_orient, N, (unsigned*)s.wswt);
  return cudaGetLastError();
}

cudaError_t ucm_mid(int H, int W, UcmScratch& s, cudaStream_t st) {
  const int R = 2 * H, C = 2 * W;
  const long long n = (long long)R * C;
  k_ucm_super<<<grid_for(n), 256, 0, st>>>(s.wswt, H, W, s.pb2);
  k_art_rows<<<R, 32, 0, st>>>(s.pb2, R, C, s.rowcnt, nullptr, nullptr);
  k_scan_small<<<1, 1024, 0, st>>>(s.rowcnt, R, s.nart);
  k_art_rows<<<R, 32, 0, st>>>(s.pb2, R, C, nullptr, s.rowcnt, s.art);
  k_art_fix<<<1, 32, 0, st>>>(s.pb2, R, C, s.art, s.nart);
  k_ccl_init<<<grid_for(n), 256, 0, st>>>(s.pb2, n, s.par);
  k_ccl_hook<<<grid_for(n), 256, 0, st>>>(s.pb2, R, C, s.par);
  k_ccl_flat<<<grid_for(n), 256, 0, st>>>(s.par, n, s.rank);
  const int nb = (int)((n + 4095) / 4096);
  k_scan_blocks<<<nb, 1024, 0, st>>>(s.rank, n, s.bsum);
  k_scan_small<<<1, 1024, 0, st>>>(s.bsum, nb, s.nreg);
  k_scan_add<<<grid_for(n), 256, 0, st>>>(s.rank, n, s.bsum);
  k_ucm_finish<<<grid_for((long long)(R + 1) * (C + 1)), 256, 0, st>>>(s.pb2, s.par, s.rank, H, W, s.labels, s.wswt2);
  return cudaGetLastError();
}

}  // namespace gpb
