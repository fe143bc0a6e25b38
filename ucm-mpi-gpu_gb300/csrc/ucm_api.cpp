// ucm_api.cpp -- the C ABI of the OWT-UCM stage: device stages (k_ucm.cu)
// around the host stages (ucm_host.cpp), in the order of Contours2Ucm
// (src/contours2ucm.cpp:405-490).
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <chrono>
#include <vector>

#include "../../include/gpb.h"
#include "gpb_internal.h"
#include "ucm_dev.h"
#include "ucm_host.h"

using namespace gpb;

namespace {

struct UcmState {
  UcmScratch s{};
  void* base = nullptr;
  size_t cap = 0;          // bytes of base
  size_t cap_paint = 0;    // entries of the paint list
  float* orient = nullptr; // staging of host planes
  size_t cap_orient = 0;
  int H = 0, W = 0;        // the last call's image
};

void ucm_release(void* p) {
  UcmState* u = (UcmState*)p;
  if (!u) return;
  cudaFree(u->base);
  cudaFree(u->s.paint_pix);
  cudaFree(u->s.paint_ori);
  cudaFree(u->orient);
  delete u;
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// carve the fixed-size scratch of an H x W image out of one allocation
cudaError_t ucm_reserve(UcmState& u, int H, int W) {
  const size_t N = (size_t)H * W, N4 = 4 * N, N2 = (size_t)(2 * H + 1) * (2 * W + 1);
  const size_t sizes[] = {2 * sizeof(unsigned), N * 4, N, (size_t)H * 257 * 4, N * 2, sizeof(UcmImage), N * 4, N,
                          N * 4, N4 * 4, (size_t)(2 * H + 1) * 4, 4, N4 * 4, N4 * 4, N4 * 4,
                          (N4 / 4096 + 2) * 4, 4, N * 4, N2 * 4};
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
  char* p = (char*)u.base;
  void** slots[] = {(void**)&u.s.mm,   (void**)&u.s.pb,     (void**)&u.s.q,      (void**)&u.s.off,
                    (void**)&u.s.cols, (void**)&u.s.img,    (void**)&u.s.ws,     (void**)&u.s.bw,
                    (void**)&u.s.wswt, (void**)&u.s.pb2,    (void**)&u.s.rowcnt, (void**)&u.s.nart,
                    (void**)&u.s.art,  (void**)&u.s.par,    (void**)&u.s.rank,   (void**)&u.s.bsum,
                    (void**)&u.s.nreg, (void**)&u.s.labels, (void**)&u.s.wswt2};
  for (size_t k = 0; k < sizeof(sizes) / sizeof(sizes[0]); k++) {
    *slots[k] = p;
    p += align256(sizes[k]);
  }
  return cudaSuccess;
}

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

#define UCK(x)                                      \
  do {                                              \
    cudaError_t e_ = (x);                           \
    if (e_ != cudaSuccess) {                        \
      ctx_set_error(ctx, cudaGetErrorString(e_));   \
      return e_ == cudaErrorMemoryAllocation ? GPB_ERR_NOMEM : GPB_ERR_CUDA; \
    }                                               \
  } while (0)

extern "C" gpb_status gpb_ucm(gpb_ctx* ctx, uint32_t width, uint32_t height, const float* orient,
                              int orient_on_device, int double_size, double* ucm_out, gpb_ucm_info* info) {
  if (!ctx || !orient || !ucm_out || width < 2 || height < 2 || width > 65535 || height > 65535) return GPB_ERR_ARG;
  if (4ull * width * height >= (1ull << 31)) return GPB_ERR_ARG;  // int32 indices of the doubled grid
  const auto t0 = std::chrono::steady_clock::now();
  const int H = (int)height, W = (int)width;
  const size_t N = (size_t)H * W;
  UCK(cudaSetDevice(ctx_device(ctx)));
  cudaStream_t st = ctx_stream(ctx);
  void*& slot = ctx_ucm_state(ctx, ucm_release);
  if (!slot) slot = new UcmState();
  UcmState& u = *(UcmState*)slot;
  UCK(ucm_reserve(u, H, W));
  u.H = 0;
  u.W = 0;
  const float* d_orient = orient;
  if (!orient_on_device) {
    if (u.cap_orient < 8 * N) {
      cudaFree(u.orient);
      u.orient = nullptr;
      u.cap_orient = 0;
      UCK(cudaMalloc(&u.orient, 8 * N * sizeof(float)));
      u.cap_orient = 8 * N;
    }
    UCK(cudaMemcpyAsync(u.orient, orient, 8 * N * sizeof(float), cudaMemcpyHostToDevice, st));
    d_orient = u.orient;
  }
  const UcmImage img{H, W, 0, 0};
  UCK(cudaMemcpyAsync(u.s.img, &img, sizeof(img), cudaMemcpyHostToDevice, st));
  // device: orientation max, quantisation, flooding
  UCK(ucm_front(d_orient, H, W, u.s, st));
  std::vector<uint8_t> bw(N);
  UCK(cudaMemcpyAsync(bw.data(), u.s.bw, N, cudaMemcpyDeviceToHost, st));
  UCK(cudaStreamSynchronize(st));
  const double ms_front = ms_since(t0);
  // host: contour fitting, then the list of painted pixels
  const auto t1 = std::chrono::steady_clock::now();
  ucm::FitResult fit;
  const bool ok = ucm::fit_contours(bw.data(), H, W, fit);
  const int ne = (int)fit.es.size();
  std::vector<int32_t> ppix;
  std::vector<uint8_t> pori;
  ppix.reserve(fit.px.size() + 2 * ne);
  pori.reserve(fit.px.size() + 2 * ne);
  for (int e = 0; e < ne; e++) {
    const int a = fit.es[e], b = fit.ee[e];
    const uint8_t o = (uint8_t)ucm::edge_orientation(fit.vx[a], fit.vy[a], fit.vx[b], fit.vy[b]);
    for (int k = fit.off[e]; k < fit.off[e + 1]; k++) ppix.push_back(fit.px[k]), pori.push_back(o);
    ppix.push_back(fit.vx[a] * W + fit.vy[a]), pori.push_back(o);
    ppix.push_back(fit.vx[b] * W + fit.vy[b]), pori.push_back(o);
  }
  const double ms_fit = ms_since(t1);
  // device: painting, super contour, cleaning, labelling
  const auto t2 = std::chrono::steady_clock::now();
  const int np = (int)ppix.size();
  if ((size_t)np > u.cap_paint) {
    cudaFree(u.s.paint_pix);
    cudaFree(u.s.paint_ori);
    u.s.paint_pix = nullptr;
    u.s.paint_ori = nullptr;
    u.cap_paint = 0;
    UCK(cudaMalloc(&u.s.paint_pix, (size_t)np * sizeof(int32_t)));
    UCK(cudaMalloc(&u.s.paint_ori, (size_t)np));
    u.cap_paint = (size_t)np;
  }
  if (np) {
    UCK(cudaMemcpyAsync(u.s.paint_pix, ppix.data(), (size_t)np * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    UCK(cudaMemcpyAsync(u.s.paint_ori, pori.data(), (size_t)np, cudaMemcpyHostToDevice, st));
  }
  UCK(ucm_paint(d_orient, H, W, np, u.s, st));
  UCK(ucm_mid(H, W, u.s, st));
  const size_t N2 = (size_t)(2 * H + 1) * (2 * W + 1);
  std::vector<float> w2(N2);
  std::vector<int32_t> lab(N);
  int32_t counts[2] = {0, 0};
  UCK(cudaMemcpyAsync(w2.data(), u.s.wswt2, N2 * sizeof(float), cudaMemcpyDeviceToHost, st));
  UCK(cudaMemcpyAsync(lab.data(), u.s.labels, N * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  UCK(cudaMemcpyAsync(counts, u.s.nreg, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  UCK(cudaMemcpyAsync(counts + 1, u.s.nart, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  UCK(cudaStreamSynchronize(st));
  const double ms_mid = ms_since(t2);
  // host: mean-boundary merge, calibration, output grid
  const auto t3 = std::chrono::steady_clock::now();
  std::vector<double> um(double_size ? 0 : N2);
  double* full = double_size ? ucm_out : um.data();  // the doubled grid is the caller's buffer where asked
  ucm::mean_pb_merge(w2.data(), lab.data(), H, W, full);
  ucm::normalize(full, N2);
  if (!double_size) {
    const int GW = 2 * W + 1;
    for (int i = 0; i <= H; i++)
      for (int j = 0; j <= W; j++)
        ucm_out[(size_t)i * (W + 1) + j] = (i < H && j < W) ? um[(size_t)(2 * i + 2) * GW + 2 * j + 2] : 0.0;
  }
  u.H = H;
  u.W = W;
  if (info) {
    info->n_regions = (uint32_t)counts[0];
    info->n_vertices = (uint32_t)fit.vx.size();
    info->n_edges = (uint32_t)ne;
    info->n_artefacts = (uint32_t)counts[1];
    info->fit_ok = ok ? 1 : 0;
    info->ms_front = ms_front;
    info->ms_fit = ms_fit;
    info->ms_mid = ms_mid;
    info->ms_merge = ms_since(t3);
    info->ms_total = ms_since(t0);
  }
  return GPB_OK;
}

extern "C" int32_t gpb_ucm_fit_contours(const uint8_t* bw, uint32_t width, uint32_t height, int32_t cap_vertices,
                                        int32_t cap_edges, int32_t cap_pixels, int32_t* n_vertices,
                                        int32_t* vertices, int32_t* edges, int32_t* off, int32_t* pixels) {
  if (!bw || !n_vertices || width == 0 || height == 0) return -1;
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
}

extern "C" gpb_status gpb_ucm_mean_pb(const double* ws_wt2, const int32_t* labels, uint32_t width, uint32_t height,
                                      double* ucm) {
  if (!ws_wt2 || !labels || !ucm || width == 0 || height == 0) return GPB_ERR_ARG;
  ucm::mean_pb_merge(ws_wt2, labels, (int)height, (int)width, ucm);
  return GPB_OK;
}

extern "C" int32_t gpb_ucm_labels_at_scale(const double* ucm2, uint32_t width, uint32_t height, double k,
                                           int32_t* labels) {
  if (!ucm2 || !labels || width == 0 || height == 0) return -1;
  const int GH = 2 * (int)height + 1, GW = 2 * (int)width + 1;
  std::vector<uint8_t> bw((size_t)GH * GW);
  for (size_t i = 0; i < bw.size(); i++) bw[i] = ucm2[i] <= k;
  std::vector<uint32_t> l2;
  const uint32_t n = ucm::components8(bw.data(), GH, GW, l2);
  for (uint32_t i = 0; i < height; i++)
    for (uint32_t j = 0; j < width; j++)
      labels[(size_t)i * width + j] = (int32_t)l2[(size_t)(2 * i + 1) * GW + 2 * j + 1] - 1;
  return (int32_t)n;
}

extern "C" gpb_status gpb_ucm_fetch(gpb_ctx* ctx, int what, void* host, size_t bytes) {
  if (!ctx || !host) return GPB_ERR_ARG;
  void*& slot = ctx_ucm_state(ctx, ucm_release);
  UcmState* u = (UcmState*)slot;
  if (!u || !u->H) return GPB_ERR_ARG;
  const size_t N = (size_t)u->H * u->W, N2 = (size_t)(2 * u->H + 1) * (2 * u->W + 1);
  const void* src = nullptr;
  size_t need = 0;
  switch (what) {
    case GPB_UCM_QUANT: src = u->s.q; need = N; break;
    case GPB_UCM_ARCS: src = u->s.bw; need = N; break;
    case GPB_UCM_WSWT: src = u->s.wswt; need = N * sizeof(float); break;
    case GPB_UCM_WSWT2: src = u->s.wswt2; need = N2 * sizeof(float); break;
    case GPB_UCM_REGIONS: src = u->s.labels; need = N * sizeof(int32_t); break;
    default: return GPB_ERR_ARG;
  }
  if (bytes < need) return GPB_ERR_ARG;
  UCK(cudaSetDevice(ctx_device(ctx)));
  UCK(cudaMemcpyAsync(host, src, need, cudaMemcpyDeviceToHost, ctx_stream(ctx)));
  UCK(cudaStreamSynchronize(ctx_stream(ctx)));
  return GPB_OK;
}
