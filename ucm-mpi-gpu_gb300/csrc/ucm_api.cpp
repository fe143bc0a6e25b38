// ucm_api.cpp -- the C ABI of the OWT-UCM stage: device stages (k_ucm.cu)
// around the host stages (ucm_host.cpp), in the order of Contours2Ucm
// (src/contours2ucm.cpp:405-490).
//
// A call takes a batch of images, the pieces that the reference gives to
// one MPI rank each (src/main.cpp:456-459): the images are flooded together
// (one CTA each), their contour fitting and merging run on the context's
// host thread pool, one image per thread, and the data-parallel stages run
// image after image on the context's stream.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <vector>

#include "../../include/gpb.h"
#include "gpb_internal.h"
#include "ucm_dev.h"
#include "ucm_host.h"

using namespace gpb;

namespace {

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// where image i's slices start in the batch's concatenated arrays
struct Offsets {
  size_t pix, pix4, rows, rows2, grid2, bsum;
};

struct UcmState {
  void* base = nullptr;
  size_t cap = 0;           // bytes of base
  int32_t* paint_pix = nullptr;
  size_t cap_pix = 0;       // entries of the paint list
  uint8_t* paint_ori = nullptr;
  size_t cap_ori = 0;
  float* orient = nullptr;  // staging of host planes
  size_t cap_orient = 0;
  std::vector<UcmScratch> views;  // image i's slices of the batch arrays
  std::vector<int> H, W;          // the last call's images
};

void ucm_release(void* p) {
  UcmState* u = (UcmState*)p;
  if (!u) return;
  cudaFree(u->base);
  cudaFree(u->paint_pix);
  cudaFree(u->paint_ori);
  cudaFree(u->orient);
  delete u;
}

template <class T>
cudaError_t grow_dev(T*& p, size_t& cap, size_t need) {
  if (need <= cap && p) return cudaSuccess;
  cudaFree(p);
  p = nullptr;
  cap = 0;
  cudaError_t e = cudaMalloc(&p, std::max<size_t>(need, 1) * sizeof(T));
  if (e == cudaSuccess) cap = need;
  return e;
}

// one allocation for the batch; every per-image array is a slice of a
// concatenated array, so one kernel can sweep several images at once
cudaError_t ucm_reserve(UcmState& u, const std::vector<int>& H, const std::vector<int>& W) {
  const size_t n = H.size();
  std::vector<Offsets> off(n + 1);
  off[0] = {0, 0, 0, 0, 0, 0};
  for (size_t i = 0; i < n; i++) {
    const size_t N = (size_t)H[i] * W[i];
    off[i + 1].pix = off[i].pix + N;
    off[i + 1].pix4 = off[i].pix4 + 4 * N;
    off[i + 1].rows = off[i].rows + H[i];
    off[i + 1].rows2 = off[i].rows2 + 2 * H[i] + 1;
    off[i + 1].grid2 = off[i].grid2 + (size_t)(2 * H[i] + 1) * (2 * W[i] + 1);
    off[i + 1].bsum = off[i].bsum + 4 * N / 4096 + 2;
  }
  const Offsets& T = off[n];
  // slots: mm, pb, q, off, cols, img, ws, bw, wswt, pb2, rowcnt, nart, art, par, rank, bsum, nreg, labels, wswt2
  const size_t sizes[] = {2 * n * 4, T.pix * 4, T.pix, T.rows * 257 * 4, T.pix * 2, n * sizeof(UcmImage), T.pix * 4,
                          T.pix, T.pix * 4, T.pix4 * 4, T.rows2 * 4, n * 4, T.pix4 * 4, T.pix4 * 4, T.pix4 * 4,
                          T.bsum * 4, n * 4, T.pix * 4, T.grid2 * 4};
  constexpr size_t kSlots = sizeof(sizes) / sizeof(sizes[0]);
  size_t need = 0;
  for (size_t b : sizes) need += align256(b);
  if (need > u.cap) {
    cudaFree(u.base);
    u.base = nullptr;
    u.cap = 0;
    cudaError_t e = cudaMalloc(&u.base, need);
    if (e != cudaSuccess) return e;
    u.cap = need;
  }
  char* base[kSlots];
  char* p = (char*)u.base;
  for (size_t k = 0; k < kSlots; k++) {
    base[k] = p;
    p += align256(sizes[k]);
  }
  u.views.assign(n, UcmScratch{});
  for (size_t i = 0; i < n; i++) {
    const Offsets& o = off[i];
    UcmScratch& v = u.views[i];
    v.mm = (unsigned*)base[0] + 2 * i;
    v.pb = (float*)base[1] + o.pix;
    v.q = (uint8_t*)base[2] + o.pix;
    v.off = (int32_t*)base[3] + o.rows * 257;
    v.cols = (uint16_t*)base[4] + o.pix;
    v.img = (UcmImage*)base[5] + i;
    v.ws = (int32_t*)base[6] + o.pix;
    v.bw = (uint8_t*)base[7] + o.pix;
    v.wswt = (float*)base[8] + o.pix;
    v.pb2 = (float*)base[9] + o.pix4;
    v.rowcnt = (int32_t*)base[10] + o.rows2;
    v.nart = (int32_t*)base[11] + i;
    v.art = (int32_t*)base[12] + o.pix4;
    v.par = (int32_t*)base[13] + o.pix4;
    v.rank = (int32_t*)base[14] + o.pix4;
    v.bsum = (int32_t*)base[15] + o.bsum;
    v.nreg = (int32_t*)base[16] + i;
    v.labels = (int32_t*)base[17] + o.pix;
    v.wswt2 = (float*)base[18] + o.grid2;
  }
  return cudaSuccess;
}

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

#define UCK(x)                                                               \
  do {                                                                       \
    cudaError_t e_ = (x);                                                    \
    if (e_ != cudaSuccess) {                                                 \
      ctx_set_error(ctx, cudaGetErrorString(e_));                            \
      return e_ == cudaErrorMemoryAllocation ? GPB_ERR_NOMEM : GPB_ERR_CUDA; \
    }                                                                        \
  } while (0)

extern "C" gpb_status gpb_ucm_batch(gpb_ctx* ctx, size_t n, const uint32_t* widths, const uint32_t* heights,
                                    const float* const* orient, int orient_on_device, int double_size,
                                    double* const* ucm_out, gpb_ucm_info* info) {
  return guarded(ctx, [&]() -> gpb_status {
    if (!ctx || n == 0 || n > 65535 || !widths || !heights || !orient || !ucm_out) return GPB_ERR_ARG;
    size_t total2 = 0;
    for (size_t i = 0; i < n; i++) {
      const uint32_t w = widths[i], h = heights[i];
      if (!orient[i] || !ucm_out[i] || w < 2 || h < 2 || w > 65535 || h > 65535) return GPB_ERR_ARG;
      total2 += (2ull * h + 1) * (2ull * w + 1);
    }
    if (total2 >= (1ull << 31)) return GPB_ERR_ARG;  // int32 indices of the doubled grids
    const auto t0 = std::chrono::steady_clock::now();
    const int ni = (int)n;
    std::vector<int> H(n), W(n);
    std::vector<size_t> N(n), pix(n + 1, 0);
    for (size_t i = 0; i < n; i++) {
      H[i] = (int)heights[i];
      W[i] = (int)widths[i];
      N[i] = (size_t)H[i] * W[i];
      pix[i + 1] = pix[i] + N[i];
    }
    UCK(cudaSetDevice(ctx_device(ctx)));
    cudaStream_t st = ctx_stream(ctx);
    void*& slot = ctx_ucm_state(ctx, ucm_release);
    if (!slot) slot = new UcmState();
    UcmState& u = *(UcmState*)slot;
    u.H.clear();
    u.W.clear();
    UCK(ucm_reserve(u, H, W));
    std::vector<const float*> d_orient(n);
    if (orient_on_device) {
      for (size_t i = 0; i < n; i++) d_orient[i] = orient[i];
    } else {
      UCK(grow_dev(u.orient, u.cap_orient, 8 * pix[n]));
      for (size_t i = 0; i < n; i++) {
        d_orient[i] = u.orient + 8 * pix[i];
        UCK(cudaMemcpyAsync(u.orient + 8 * pix[i], orient[i], 8 * N[i] * sizeof(float), cudaMemcpyHostToDevice, st));
      }
    }
    std::vector<UcmImage> imgs(n);
    for (size_t i = 0; i < n; i++)
      imgs[i] = {H[i], W[i], (long long)pix[i], (int)((u.views[i].off - u.views[0].off) / 257)};
    UCK(cudaMemcpyAsync(u.views[0].img, imgs.data(), n * sizeof(UcmImage), cudaMemcpyHostToDevice, st));
    // device: orientation max, quantisation and row sort per image, then one flooding launch for all
    for (size_t i = 0; i < n; i++) UCK(ucm_prepare(d_orient[i], H[i], W[i], u.views[i], st));
    UCK(ucm_flood(ni, (long long)pix[n], u.views[0], st));
    std::vector<uint8_t> bw(pix[n]);
    UCK(cudaMemcpyAsync(bw.data(), u.views[0].bw, pix[n], cudaMemcpyDeviceToHost, st));
    UCK(cudaStreamSynchronize(st));
    const double ms_front = ms_since(t0);
    // host: contour fitting and the painted pixels, one image per thread
    const auto t1 = std::chrono::steady_clock::now();
    std::vector<ucm::FitResult> fit(n);
    std::vector<char> ok(n);
    std::vector<std::vector<int32_t>> ppix(n);
    std::vector<std::vector<uint8_t>> pori(n);
    std::vector<double> ms_fit_i(n);
    const ucm::ParFor pool = [&](int k, const std::function<void(int)>& f) { ctx_parallel_for(ctx, k, f); };
    ctx_parallel_for(ctx, ni, [&](int i) {
      const auto ti = std::chrono::steady_clock::now();
      // one image alone uses the pool inside its contour fitting and paint list instead
      ok[i] = ucm::fit_contours(bw.data() + pix[i], H[i], W[i], fit[i], n == 1 ? &pool : nullptr);
      ucm::paint_list(fit[i], W[i], ppix[i], pori[i], n == 1 ? &pool : nullptr);
      ms_fit_i[i] = ms_since(ti);
    });
    const double ms_fit = ms_since(t1);
    // device: painting, super contour, cleaning, labelling, image after image
    const auto t2 = std::chrono::steady_clock::now();
    std::vector<size_t> poff(n + 1, 0);
    for (size_t i = 0; i < n; i++) poff[i + 1] = poff[i] + ppix[i].size();
    UCK(grow_dev(u.paint_pix, u.cap_pix, poff[n]));
    UCK(grow_dev(u.paint_ori, u.cap_ori, poff[n]));
    for (size_t i = 0; i < n; i++) {
      const int np = (int)ppix[i].size();
      if (np) {
        UCK(cudaMemcpyAsync(u.paint_pix + poff[i], ppix[i].data(), (size_t)np * sizeof(int32_t),
                            cudaMemcpyHostToDevice, st));
        UCK(cudaMemcpyAsync(u.paint_ori + poff[i], pori[i].data(), (size_t)np, cudaMemcpyHostToDevice, st));
      }
      UcmScratch v = u.views[i];
      v.paint_pix = u.paint_pix + poff[i];
      v.paint_ori = u.paint_ori + poff[i];
      UCK(ucm_paint(d_orient[i], H[i], W[i], np, v, st));
      UCK(ucm_mid(H[i], W[i], v, st));
    }
    std::vector<size_t> g2(n + 1, 0);
    for (size_t i = 0; i < n; i++) g2[i + 1] = g2[i] + (size_t)(2 * H[i] + 1) * (2 * W[i] + 1);
    std::vector<float> w2(g2[n]);
    std::vector<int32_t> lab(pix[n]), counts(2 * n);
    UCK(cudaMemcpyAsync(w2.data(), u.views[0].wswt2, g2[n] * sizeof(float), cudaMemcpyDeviceToHost, st));
    UCK(cudaMemcpyAsync(lab.data(), u.views[0].labels, pix[n] * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    UCK(cudaMemcpyAsync(counts.data(), u.views[0].nreg, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    UCK(cudaMemcpyAsync(counts.data() + n, u.views[0].nart, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    UCK(cudaStreamSynchronize(st));
    const double ms_mid = ms_since(t2);
    // host: mean-boundary merge, calibration, output grid, one image per thread
    const auto t3 = std::chrono::steady_clock::now();
    ctx_parallel_for(ctx, ni, [&](int i) {
      // one image alone uses the pool inside the merge's setup and output
      ucm::mean_pb_ucm(w2.data() + g2[i], lab.data() + pix[i], H[i], W[i], !double_size, ucm_out[i],
                       n == 1 ? &pool : nullptr);
    });
    const double ms_merge = ms_since(t3);
    u.H = H;
    u.W = W;
    if (info)
      for (size_t i = 0; i < n; i++) {
        gpb_ucm_info& f = info[i];
        f.n_regions = (uint32_t)counts[i];
        f.n_vertices = (uint32_t)fit[i].vx.size();
        f.n_edges = (uint32_t)fit[i].es.size();
        f.n_artefacts = (uint32_t)counts[n + i];
        f.fit_ok = ok[i] ? 1 : 0;
        f.ms_front = ms_front;
        f.ms_fit = n == 1 ? ms_fit : ms_fit_i[i];
        f.ms_mid = ms_mid;
        f.ms_merge = ms_merge;
        f.ms_total = ms_since(t0);
      }
    return GPB_OK;
  });
}

extern "C" gpb_status gpb_ucm(gpb_ctx* ctx, uint32_t width, uint32_t height, const float* orient,
                              int orient_on_device, int double_size, double* ucm_out, gpb_ucm_info* info) {
  return gpb_ucm_batch(ctx, 1, &width, &height, &orient, orient_on_device, double_size, &ucm_out, info);
}

extern "C" gpb_status gpb_ucm_fetch(gpb_ctx* ctx, size_t image, int what, void* host, size_t bytes) {
  return guarded(ctx, [&]() -> gpb_status {
    if (!ctx || !host) return GPB_ERR_ARG;
    void*& slot = ctx_ucm_state(ctx, ucm_release);
    UcmState* u = (UcmState*)slot;
    if (!u || image >= u->H.size()) return GPB_ERR_ARG;
    const int H = u->H[image], W = u->W[image];
    const UcmScratch& v = u->views[image];
    const size_t N = (size_t)H * W, N2 = (size_t)(2 * H + 1) * (2 * W + 1);
    const void* src = nullptr;
    size_t need = 0;
    switch (what) {
      case GPB_UCM_QUANT: src = v.q; need = N; break;
      case GPB_UCM_ARCS: src = v.bw; need = N; break;
      case GPB_UCM_WSWT: src = v.wswt; need = N * sizeof(float); break;
      case GPB_UCM_WSWT2: src = v.wswt2; need = N2 * sizeof(float); break;
      case GPB_UCM_REGIONS: src = v.labels; need = N * sizeof(int32_t); break;
      default: return GPB_ERR_ARG;
    }
    if (bytes < need) return GPB_ERR_ARG;
    UCK(cudaSetDevice(ctx_device(ctx)));
    UCK(cudaMemcpyAsync(host, src, need, cudaMemcpyDeviceToHost, ctx_stream(ctx)));
    UCK(cudaStreamSynchronize(ctx_stream(ctx)));
    return GPB_OK;
  });
}

extern "C" int32_t gpb_ucm_fit_contours(const uint8_t* bw, uint32_t width, uint32_t height, int32_t cap_vertices,
                                        int32_t cap_edges, int32_t cap_pixels, int32_t* n_vertices,
                                        int32_t* vertices, int32_t* edges, int32_t* off, int32_t* pixels) {
  try {
    if (!bw || !n_vertices || width == 0 || height == 0) return -1;
    if ((uint64_t)width * height >= (1ull << 31)) return -1;  // pixel indices are 32-bit
    ucm::FitResult f;
    if (!ucm::fit_contours(bw, (int)height, (int)width, f)) return -2;
    const int nv = (int)f.vx.size(), ne = (int)f.es.size(), np = (int)f.px.size();
    *n_vertices = nv;
    if (nv > cap_vertices || ne > cap_edges || np > cap_pixels) return -1;
    for (int v = 0; v < nv; v++) {
      vertices[2 * v] = f.vx[v];
      vertices[2 * v + 1] = f.vy[v];
    }
    for (int e = 0; e < ne; e++) {
      edges[2 * e] = f.es[e];
      edges[2 * e + 1] = f.ee[e];
      off[e] = f.off[e];
    }
    off[ne] = np;
    for (int k = 0; k < np; k++) {
      pixels[2 * k] = f.px[k] / (int)width;
      pixels[2 * k + 1] = f.px[k] % (int)width;
    }
    return ne;
  } catch (...) {  // host memory ran out
    return -3;
  }
}

extern "C" gpb_status gpb_ucm_mean_pb(const double* ws_wt2, const int32_t* labels, uint32_t width, uint32_t height,
                                      double* ucm) {
  return guarded(nullptr, [&]() -> gpb_status {
    if (!ws_wt2 || !labels || !ucm || width == 0 || height == 0) return GPB_ERR_ARG;
    // grid indices are 32-bit
    if ((2 * (uint64_t)height + 1) * (2 * (uint64_t)width + 1) >= (1ull << 31)) return GPB_ERR_ARG;
    ucm::mean_pb_merge(ws_wt2, labels, (int)height, (int)width, ucm);
    return GPB_OK;
  });
}

extern "C" int32_t gpb_ucm_labels_at_scale(const double* ucm2, uint32_t width, uint32_t height, double k,
                                           int32_t* labels) {
  if (!ucm2 || !labels || width == 0 || height == 0) return -1;
  if ((2 * (uint64_t)height + 1) * (2 * (uint64_t)width + 1) >= (1ull << 31)) return -1;
  try {
    const int GH = 2 * (int)height + 1, GW = 2 * (int)width + 1;
    std::vector<uint8_t> bw((size_t)GH * GW);
    for (size_t i = 0; i < bw.size(); i++) bw[i] = ucm2[i] <= k;
    std::vector<uint32_t> l2;
    const uint32_t n = ucm::components8(bw.data(), GH, GW, l2);
    for (uint32_t i = 0; i < height; i++)
      for (uint32_t j = 0; j < width; j++)
        labels[(size_t)i * width + j] = (int32_t)l2[(size_t)(2 * i + 1) * GW + 2 * j + 1] - 1;
    return (int32_t)n;
  } catch (...) {  // host memory ran out
    return -1;
  }
}
