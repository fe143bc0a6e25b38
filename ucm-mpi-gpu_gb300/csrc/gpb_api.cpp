// gpb_api.cpp -- the C ABI of libgpb (include/gpb.h): context, batch layout,
// the per-batch pipeline and the eigensolver drivers.
//
// Pipeline per batch, on one stream:
//   H2D -> convert -> texton (+ FP64 repair) -> max label -> local cues ->
//   NMS -> buildW -> degree/scale -> eigensolver -> min/max -> sPb/gPb -> D2H
// It replaces computeGPb (damascene/src/damascene.cu:249-661): same inputs
// and, in GPB_COMPAT_DAMASCENE, the same output layout.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <exception>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gpb.h"
#include "autotune.h"
#include "gpb_internal.h"
#include "host_pool.h"
#include "k_block.h"
#include "k_learned.h"
#include "k_warmnet.h"
#include "k_eig.h"
#include "k_static.h"
#include "kernels.h"

namespace gpb {
void sym_eig(double* A, int n, double* w, double* Z);
void lowdin(const double* G, int n, double* M);
void mat_mul(const double* A, const double* B, double* C, int n, bool at);
}

using namespace gpb;

#define CK(x)                                   \
  do {                                          \
    cudaError_t e_ = (x);                       \
    if (e_ != cudaSuccess) {                    \
      ctx->last_error = cudaGetErrorString(e_); \
      return GPB_ERR_CUDA;                      \
    }                                           \
  } while (0)

template <class T>
static cudaError_t grow(T*& p, size_t& cap, size_t need) {
  if (need <= cap && p) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  cudaError_t e = cudaMalloc((void**)&p, need * sizeof(T) + 256);
  if (e != cudaSuccess) return e;
  cap = need;
  return cudaMemset(p, 0, need * sizeof(T) + 256);
}

struct Buf {
  // image-level
  uint32_t* packed = nullptr; size_t c_packed = 0;
  uint8_t* grey = nullptr; size_t c_grey = 0;
  uint32_t* lab4 = nullptr; size_t c_lab4 = 0;
  int* nbins = nullptr; size_t c_nbins = 0;
  int* repair = nullptr; size_t c_repair = 0;
  int* repair_count = nullptr; size_t c_rc = 0;
  float* mpbo = nullptr; size_t c_mpbo = 0;
  float* go = nullptr; size_t c_go = 0;
  float* mpb = nullptr; size_t c_mpb = 0;
  float* raw = nullptr; size_t c_raw = 0;
  float* wfull = nullptr; size_t c_wfull = 0;
  uint8_t* counts = nullptr; size_t c_counts = 0;
  // padded vector layout
  float* wup = nullptr; size_t c_wup = 0;
  float* aup = nullptr; size_t c_aup = 0;
  float* deg = nullptr; size_t c_deg = 0;
  float* dis = nullptr; size_t c_dis = 0;
  float* adiag = nullptr; size_t c_adiag = 0;
  float* V[2] = {nullptr, nullptr}; size_t c_V[2] = {0, 0};
  float* W[2] = {nullptr, nullptr}; size_t c_W[2] = {0, 0};
  float* evec = nullptr; size_t c_evec = 0;
  // solver state
  double* part = nullptr; size_t c_part = 0;
  double* hbuf = nullptr; size_t c_hbuf = 0;
  double* T = nullptr; size_t c_T = 0;
  double* Y = nullptr; size_t c_Y = 0;
  double* beta2 = nullptr; size_t c_beta2 = 0;
  int* counter = nullptr; size_t c_counter = 0;
  int* active = nullptr; size_t c_active = 0;
  int* decision = nullptr; size_t c_decision = 0;
  int* nkeep = nullptr; size_t c_nkeep = 0;
  float* evals = nullptr; size_t c_evals = 0;
  float* mm = nullptr; size_t c_mm = 0;
  float* spb = nullptr; size_t c_spb = 0;
  float* gpbo = nullptr; size_t c_gpbo = 0;
  // outputs
  float* nmax = nullptr; size_t c_nmax = 0;
  float* orient = nullptr; size_t c_orient = 0;
  // tables
  PatchDev* patches = nullptr; size_t c_patches = 0;
  int4* work_tex = nullptr; size_t c_wt = 0;
  int4* work_cue = nullptr; size_t c_wc = 0;
  int4* work16 = nullptr; size_t c_w16 = 0;
  int4* work_blk = nullptr; size_t c_wb = 0;
  EigTile* tiles = nullptr; size_t c_tiles = 0;
  int* tile_begin = nullptr; size_t c_tb = 0;
  int* tile_count = nullptr; size_t c_tc = 0;
  // block solver
  float* blk[4] = {nullptr, nullptr, nullptr, nullptr}; size_t c_blk[4] = {0, 0, 0, 0};
  double* bpart = nullptr; size_t c_bpart = 0;
  double* bgram = nullptr; size_t c_bgram = 0;
  double* bgram2 = nullptr; size_t c_bgram2 = 0;
  double* bmat = nullptr; size_t c_bmat = 0;
  double* btheta = nullptr; size_t c_btheta = 0;
  double* bres = nullptr; size_t c_bres = 0;
  float3* bcoef = nullptr; size_t c_bcoef = 0;
  int* bdone = nullptr; size_t c_bdone = 0;
  // coarse level of the warm start
  PatchDev* cpatches = nullptr; size_t c_cpatches = 0;
  EigTile* ctiles = nullptr; size_t c_ctiles = 0;
  int* ctile_begin = nullptr; size_t c_ctb = 0;
  int* ctile_count = nullptr; size_t c_ctc = 0;
  int4* cwork_blk = nullptr; size_t c_cwb = 0;
  int4* cwork16 = nullptr; size_t c_cw16 = 0;
  float* cwc = nullptr; size_t c_cwc = 0;
  float* cdeg = nullptr; size_t c_cdeg = 0;
  float* cdis = nullptr; size_t c_cdis = 0;
  float* cblk[4] = {nullptr, nullptr, nullptr, nullptr}; size_t c_cblk[4] = {0, 0, 0, 0};
  float* afull = nullptr; size_t c_afull = 0;  // pixel-major fine stencil rows
  int4* work_act = nullptr; size_t c_wact = 0;  // block-step tiles of the still active patches
  float* stitch = nullptr; size_t c_stitch = 0;  // BLEND accumulators [10][image]
  uint32_t* spcount = nullptr; size_t c_spcount = 0;          // superpixel histograms
  unsigned long long* spcsum = nullptr; size_t c_spcsum = 0;  // superpixel colour sums
  int* berr = nullptr; size_t c_berr = 0;
};

struct gpb_ctx {
  gpb_params prm;
  int device = 0;
  cudaStream_t st = nullptr;
  HostTables tab;
  IcPath* d_ic = nullptr;
  double* d_k32_ring = nullptr;
  int* d_ring_of = nullptr;
  int K = 0;
  std::vector<float> cb_host;  // 13 x K, the codebook last set
  uint64_t token = 0;          // identifies this context's constant tables
  Buf b;
  std::string last_error;
  // learned correction of the warm start (k_warmnet.cu): weights, per-patch
  // scales, and the captured start block of the last batch
  float* d_wn = nullptr;
  float* d_wn_scale = nullptr; size_t c_wn_scale = 0;
  float* d_wn_x0 = nullptr; size_t c_wn_x0 = 0;
  bool wn_capture = false;
  int wn_epochs = 0;  // informational, carried with the weights
  // device scratch of the OWT-UCM stage (ucm_api.cpp), freed with the context
  void* ucm_state = nullptr;
  void (*ucm_free)(void*) = nullptr;
  // last call
  std::vector<PatchDev> patches;
  long long total_pix = 0, lvec = 0;
  std::string layout_key;
  std::vector<float> evals_host;  // npatch * nvec
  gpb_stats stats;
  int launches = 0;
  // pinned staging
  uint32_t* h_packed = nullptr; size_t c_hpacked = 0;
  float* h_out = nullptr; size_t c_hout = 0;
  // pinned host staging of the block solvers' small per-patch matrices
  void* h_small = nullptr; size_t c_hsmall = 0;
  cudaEvent_t ev[12];
  // optional per-kernel timing of the eigensolver launches
  bool profile = false;
  bool trace = false;
  std::vector<cudaEvent_t> pev;
  std::vector<int> pkind;      // 0 spmv, 1 orth
  std::vector<double> pbytes;  // algorithmic bytes of that launch
  size_t pn = 0;
  // CUDA graphs of fixed launch chains (the stages before and after the
  // eigensolver, a block solver's filter, a Lanczos restart cycle), keyed by
  // everything their launches bake in: buffer addresses, sizes, grids
  struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    int launches = 0;
  };
  std::map<std::string, GraphEntry> graphs;
  bool use_graphs = true;
  // kernel variants chosen per shape bucket (autotune.h)
  Autotuner tuner;
  // the Lab bins of every colour (k_lab_table), built at the first batch
  uint32_t* d_lab_lut = nullptr;
  // the learned warm start's network (k_learned.cu), and the device staging
  // of a training minibatch
  std::unique_ptr<LearnedNet> net;
  float *d_tr = nullptr;
  size_t c_tr = 0;
  int learned_launches = 0;
  std::unique_ptr<HostPool> pool;
  HostPool& host_pool() {
    if (!pool) pool.reset(new HostPool(std::max(1u, std::min(16u, std::thread::hardware_concurrency()))));
    return *pool;
  }
};

static void drop_graphs(gpb_ctx* ctx) {
  for (auto& kv : ctx->graphs)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  ctx->graphs.clear();
}

// Runs body() -- stream work on the context's stream, returning the first
// CUDA error -- as a CUDA graph.  A key seen for the first time runs
// directly (which also does any one-time set-up of the kernels it launches);
// the second call with that key captures the work into a graph and launches
// it; later calls replay the graph.  A capture that fails switches graphs off
// for the context and runs the work directly.  Off while per-kernel timing
// is on, and while `allow` is false (a launch in the chain is an autotuner
// trial).
template <class F>
static cudaError_t graph_run(gpb_ctx* ctx, const std::string& key, F&& body, bool allow = true) {
  cudaStream_t s = ctx->st;
  if (!ctx->use_graphs || ctx->profile || !allow) return body();
  auto it = ctx->graphs.find(key);
  if (it == ctx->graphs.end()) {
    if (ctx->graphs.size() >= 64) drop_graphs(ctx);
    ctx->graphs.emplace(key, gpb_ctx::GraphEntry());
    return body();
  }
  gpb_ctx::GraphEntry& g = it->second;
  if (g.exec) {
    ctx->launches += g.launches;
    ctx->stats.graph_replays++;
    return cudaGraphLaunch(g.exec, s);
  }
  const int l0 = ctx->launches;
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  const cudaError_t eb = body();
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(s, &graph);
  cudaGraphExec_t exec = nullptr;
  if (eb == cudaSuccess && e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (eb != cudaSuccess || e != cudaSuccess || !exec) {
    (void)cudaGetLastError();
    ctx->use_graphs = false;
    ctx->launches = l0;
    return body();
  }
  g.exec = exec;
  g.launches = ctx->launches - l0;
  return cudaGraphLaunch(exec, s);
}

// an event record that is also a node of the graph being captured, so stage
// timings hold for replayed graphs
static cudaError_t stage_mark(cudaEvent_t ev, cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &cs);
  return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal)
                                             : cudaEventRecord(ev, s);
}

// a graph key: a tag and the values the captured launches bake in
template <class... T>
static std::string gkey(const char* tag, T... v) {
  std::string k(tag);
  const long long vals[] = {(long long)v...};
  for (long long x : vals) k += "," + std::to_string(x);
  return k;
}

static int ilog2(long long v) {
  int r = 0;
  while (v > 1) {
    v >>= 1;
    r++;
  }
  return r;
}

// events around one eigensolver launch (kind 0 = SpMV, 1 = CGS pass)
static void prof_begin(gpb_ctx* ctx, int kind, double bytes) {
  if (!ctx->profile) return;
  if (ctx->pn + 2 > ctx->pev.size()) {
    for (int i = 0; i < 256; i++) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      ctx->pev.push_back(e);
    }
    ctx->pkind.resize(ctx->pev.size());
    ctx->pbytes.resize(ctx->pev.size());
  }
  ctx->pkind[ctx->pn] = kind;
  ctx->pbytes[ctx->pn] = bytes;
  cudaEventRecord(ctx->pev[ctx->pn++], ctx->st);
}
static void prof_end(gpb_ctx* ctx) {
  if (!ctx->profile) return;
  cudaEventRecord(ctx->pev[ctx->pn++], ctx->st);
}
static void prof_collect(gpb_ctx* ctx) {
  if (!ctx->profile) return;
  cudaStreamSynchronize(ctx->st);
  for (size_t i = 0; i + 1 < ctx->pn; i += 2) {
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->pev[i], ctx->pev[i + 1]);
    if (ctx->pkind[i] == 0) {
      ctx->stats.spmv_ms += ms;
      ctx->stats.spmv_launches++;
      ctx->stats.spmv_bytes += ctx->pbytes[i];
    } else {
      ctx->stats.orth_ms += ms;
      ctx->stats.orth_launches++;
      ctx->stats.orth_bytes += ctx->pbytes[i];
    }
  }
  ctx->pn = 0;
}

// The __constant__ tables (Schmid groups, codebook, slice and stencil
// offsets, sPb filters, the compat-mode weights) live once per device and
// are shared by every context of the process.  Each compute call holds its
// device's lock and reloads the tables when another context loaded the
// bank last, so contexts with different codebooks or compat modes can be
// used in any order from any thread.
namespace {
struct ConstBank {
  std::mutex mu;
  uint64_t owner = 0;
  // Recorded on the caller's stream after gpb_texton_labels_static's kernels,
  // which read the constant tables outside the context's own stream; a
  // reload of the tables waits for it first.  Created with the bank's first
  // context, on its device.
  cudaEvent_t static_done = nullptr;
  bool static_pending = false;
};
std::mutex g_banks_mu;
std::map<int, ConstBank*> g_banks;
std::atomic<uint64_t> g_next_token{1};

ConstBank& bank_of(int device) {
  std::lock_guard<std::mutex> lk(g_banks_mu);
  ConstBank*& b = g_banks[device];
  if (!b) b = new ConstBank();  // lives for the process
  return *b;
}
}  // namespace

// caller holds bank_of(ctx->device).mu; ctx's device is current
static cudaError_t load_tables(gpb_ctx* ctx) {
  ConstBank& bk = bank_of(ctx->device);
  if (bk.owner == ctx->token) return cudaSuccess;
  cudaStream_t s = ctx->st;
  // the uploads report through cudaGetLastError: clear an earlier,
  // unrelated non-sticky error first so it is not taken for theirs
  (void)cudaGetLastError();
  if (bk.static_pending) {  // texton kernels queued on another stream still read the tables
    cudaStreamWaitEvent(s, bk.static_done, 0);
    bk.static_pending = false;
  }
  upload_front(ctx->tab, s);
  upload_cues(ctx->tab, s);
  upload_buildw(ctx->tab, s);
  upload_eig(ctx->tab, s);
  upload_spb(ctx->tab, s);
  upload_block(ctx->tab, s);
  if (ctx->K) upload_codebook(ctx->cb_host.data(), ctx->K, s);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) bk.owner = ctx->token;
  return e;
}

extern "C" void gpb_default_params(gpb_params* p) {
  p->device = -1;
  p->compat = GPB_COMPAT_CPU;
  p->nvec = 9;
  p->eig_tol = 1e-6f;
  p->eig_max_matvecs = 200000;
  p->krylov_dim = 40;
  p->krylov_keep = 26;
  p->eig_mode = GPB_EIG_LANCZOS;
  p->keep_intermediates = 0;
  p->cheb_degree = 40;
  p->warm_tol = 3e-3f;
  p->eig_gap_frac = 0.1f;
}

extern "C" const char* gpb_status_str(gpb_status s) {
  switch (s) {
    case GPB_OK: return "ok";
    case GPB_ERR_ARG: return "invalid argument";
    case GPB_ERR_TOO_LARGE: return "image or batch larger than the entry point allows";
    case GPB_ERR_CUDA: return "CUDA error";
    case GPB_ERR_NOMEM: return "out of memory";
    case GPB_ERR_NOCONV: return "eigensolver did not converge";
    case GPB_ERR_TIMEOUT: return "device wait timed out";
    default: return "internal error";
  }
}

extern "C" void gpb_free(void* p) { free(p); }

extern "C" const char* gpb_last_error(const gpb_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

extern "C" int gpb_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}

extern "C" gpb_status gpb_create(gpb_ctx** out, const gpb_params* p) {
  if (!out) return GPB_ERR_ARG;
  *out = nullptr;
  gpb_ctx* ctx = nullptr;
  try {
    ctx = new (std::nothrow) gpb_ctx();
    if (!ctx) return GPB_ERR_NOMEM;
    if (p) ctx->prm = *p;
    else gpb_default_params(&ctx->prm);
    gpb_params& q = ctx->prm;
    if (q.nvec < 2 || q.nvec > kMaxNvec || q.krylov_dim > kMaxKrylov || q.krylov_keep >= q.krylov_dim ||
        q.krylov_keep < q.nvec || !(q.eig_tol > 0) || q.eig_mode < GPB_EIG_LANCZOS || q.eig_mode > GPB_EIG_LEARNED ||
        (q.eig_mode != GPB_EIG_LANCZOS && q.nvec > kBlk) || (q.eig_mode == GPB_EIG_WARM && !(q.warm_tol > 0))) {
      delete ctx;
      return GPB_ERR_ARG;
    }
    if (q.device >= 0) {
      if (cudaSetDevice(q.device) != cudaSuccess) {
        delete ctx;
        return GPB_ERR_CUDA;
      }
    }
    cudaGetDevice(&ctx->device);
    if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess) {
      delete ctx;
      return GPB_ERR_CUDA;
    }
    for (int i = 0; i < 12; i++) cudaEventCreate(&ctx->ev[i]);
    {
      const char* pe = getenv("GPB_PROFILE");
      ctx->profile = pe && pe[0] == '1';
      const char* tr = getenv("GPB_TRACE");
      ctx->trace = tr && tr[0] == '1';
      const char* ng = getenv("GPB_NO_GRAPHS");  // launch every chain directly
      ctx->use_graphs = !(ng && ng[0] == '1');
      const char* nt = getenv("GPB_NO_TUNE");  // the default variant of every tunable kernel
      ctx->tuner.enabled = !(nt && nt[0] == '1');
    }
    build_tables(ctx->tab, q.compat);
    cudaStream_t s = ctx->st;
    ctx->token = g_next_token++;
    bool loaded;
    {
      ConstBank& bk = bank_of(ctx->device);
      std::lock_guard<std::mutex> lk(bk.mu);
      if (!bk.static_done) cudaEventCreateWithFlags(&bk.static_done, cudaEventDisableTiming);
      loaded = load_tables(ctx) == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess;
    }
    if (!loaded) {
      gpb_destroy(ctx);
      return GPB_ERR_CUDA;
    }
    // global tables: IC paths, FP64 ring coefficients and the offset->ring map
    size_t nic = ctx->tab.ic.size();
    std::vector<int> ring_of(2401);
    {
      int rid[2 * 24 * 24 + 1];
      for (int t = 0; t <= 2 * 24 * 24; t++) rid[t] = -1;
      for (int a = 0; a <= 24; a++)
        for (int bb = 0; bb <= 24; bb++) rid[a * a + bb * bb] = 0;
      int nr = 0;
      for (int t = 0; t <= 2 * 24 * 24; t++)
        if (rid[t] == 0) rid[t] = nr++;
      for (int o = 0; o < 2401; o++) {
        const int dy = o / 49 - 24, dx = o % 49 - 24;
        ring_of[o] = rid[dy * dy + dx * dx];
      }
    }
    if (cudaMalloc(&ctx->d_ic, nic * sizeof(IcPath)) != cudaSuccess ||
        cudaMalloc(&ctx->d_k32_ring, ctx->tab.k32_ring.size() * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&ctx->d_ring_of, 2401 * sizeof(int)) != cudaSuccess) {
      gpb_destroy(ctx);
      return GPB_ERR_NOMEM;
    }
    cudaMemcpyAsync(ctx->d_ic, ctx->tab.ic.data(), nic * sizeof(IcPath), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ctx->d_k32_ring, ctx->tab.k32_ring.data(), ctx->tab.k32_ring.size() * sizeof(double),
                    cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ctx->d_ring_of, ring_of.data(), 2401 * sizeof(int), cudaMemcpyHostToDevice, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) {
      gpb_destroy(ctx);
      return GPB_ERR_CUDA;
    }
    *out = ctx;
    return GPB_OK;
  } catch (const std::bad_alloc&) {  // a host table could not be allocated
    gpb_destroy(ctx);
    return GPB_ERR_NOMEM;
  } catch (...) {
    gpb_destroy(ctx);
    return GPB_ERR_INTERNAL;
  }
}

extern "C" void gpb_destroy(gpb_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->ucm_free) ctx->ucm_free(ctx->ucm_state);
  cudaFree(ctx->d_wn);
  cudaFree(ctx->d_wn_scale);
  cudaFree(ctx->d_wn_x0);
  if (ctx->st) cudaStreamSynchronize(ctx->st);
  drop_graphs(ctx);
  ctx->net.reset();
  if (ctx->d_tr) cudaFree(ctx->d_tr);
  if (ctx->d_lab_lut) cudaFree(ctx->d_lab_lut);
  {
    ConstBank& bk = bank_of(ctx->device);
    std::lock_guard<std::mutex> lk(bk.mu);
    if (bk.owner == ctx->token) bk.owner = 0;
  }
  Buf& b = ctx->b;
  void* ptrs[] = {b.packed, b.grey, b.lab4, b.nbins, b.repair, b.repair_count, b.mpbo, b.go, b.mpb, b.raw,
                  b.wfull, b.counts, b.wup, b.aup, b.deg, b.dis, b.adiag, b.V[0], b.V[1], b.W[0], b.W[1], b.evec,
                  b.part, b.hbuf, b.T, b.Y, b.beta2, b.counter, b.active, b.decision, b.nkeep, b.evals,
                  b.mm, b.spb, b.gpbo, b.nmax, b.orient, b.patches, b.work_tex, b.work_cue, b.work16, b.work_blk,
                  b.tiles, b.tile_begin, b.tile_count, ctx->d_ic, ctx->d_k32_ring, ctx->d_ring_of,
                  b.blk[0], b.blk[1], b.blk[2], b.blk[3], b.bpart, b.bgram, b.bgram2, b.bmat, b.btheta, b.bres,
                  b.bcoef, b.bdone, b.cpatches, b.ctiles, b.ctile_begin, b.ctile_count, b.cwork_blk,
                  b.cwork16, b.cwc, b.cdeg, b.cdis, b.cblk[0], b.cblk[1], b.cblk[2], b.cblk[3], b.afull, b.berr, b.work_act, b.stitch, b.spcount, b.spcsum};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (ctx->h_packed) cudaFreeHost(ctx->h_packed);
  if (ctx->h_out) cudaFreeHost(ctx->h_out);
  if (ctx->h_small) cudaFreeHost(ctx->h_small);
  for (int i = 0; i < 12; i++) cudaEventDestroy(ctx->ev[i]);
  for (cudaEvent_t e : ctx->pev) cudaEventDestroy(e);
  if (ctx->st) cudaStreamDestroy(ctx->st);
  delete ctx;
}

extern "C" gpb_status gpb_set_codebook(gpb_ctx* ctx, const float* cb, int K) {
  return guarded(ctx, [&]() -> gpb_status {
    if (!ctx || !cb || K < 1 || K > kMaxCodewords) return GPB_ERR_ARG;
    cudaSetDevice(ctx->device);
    ConstBank& bk = bank_of(ctx->device);
    std::lock_guard<std::mutex> lk(bk.mu);
    ctx->cb_host.assign(cb, cb + (size_t)kNschmid * K);
    ctx->K = K;
    bk.owner = 0;  // reload everything under this context's token
    if (load_tables(ctx) != cudaSuccess || cudaStreamSynchronize(ctx->st) != cudaSuccess) return GPB_ERR_CUDA;
    return GPB_OK;
  });
}

// minimal reader for an OpenCV FileStorage YAML matrix named texton_codebook
extern "C" gpb_status gpb_load_codebook_yml(gpb_ctx* ctx, const char* path) {
  return guarded(ctx, [&]() -> gpb_status {
    if (!ctx || !path) return GPB_ERR_ARG;
    FILE* f = fopen(path, "rb");
    if (!f) return GPB_ERR_ARG;
    std::string s;
    char buf[4096];
    size_t n;
    while ((n = fread(buf, 1, sizeof(buf), f)) > 0) s.append(buf, n);
    fclose(f);
    size_t at = s.find("texton_codebook");
    if (at == std::string::npos) return GPB_ERR_ARG;
    auto num_after = [&](const char* key, size_t from) -> long {
      size_t k = s.find(key, from);
      if (k == std::string::npos) return -1;
      return strtol(s.c_str() + k + strlen(key), nullptr, 10);
    };
    const long rows = num_after("rows:", at), cols = num_after("cols:", at);
    size_t d = s.find("data:", at);
    if (rows != kNschmid || cols < 1 || cols > kMaxCodewords || d == std::string::npos) return GPB_ERR_ARG;
    d = s.find('[', d);
    if (d == std::string::npos) return GPB_ERR_ARG;
    std::vector<float> v;
    const char* c = s.c_str() + d + 1;
    while ((long)v.size() < rows * cols) {
      char* e;
      const double x = strtod(c, &e);
      if (e == c) {
        if (*c == 0) break;
        c++;
        continue;
      }
      v.push_back((float)x);
      c = e;
    }
    if ((long)v.size() != rows * cols) return GPB_ERR_ARG;
    return gpb_set_codebook(ctx, v.data(), (int)cols);
  });
}

// ------------------------------------------------------------------ batch
namespace {

struct Layout {
  std::vector<PatchDev> patches;
  std::vector<int4> work_tex, work_cue, work16, work_blk;
  std::vector<EigTile> tiles;
  std::vector<int> tile_begin, tile_count;
  long long total_pix = 0, lvec = 0;
  int max_side = 0;
};

Layout make_layout(size_t n, const uint32_t* ws, const uint32_t* hs) {
  Layout L;
  int wmax = 0;
  for (size_t i = 0; i < n; i++) wmax = std::max(wmax, (int)ws[i]);
  // the gap before and after every patch: a stencil neighbour lies at most
  // kStencilR rows + kStencilR pixels away, and a block-step tile's staged
  // row runs kStepTileW + 2 kStencilR pixels from its left halo column
  const long long pad =
      (((long long)kStencilR * wmax + kStencilR + kStepTileW + 2 * kStencilR) + 63) / 64 * 64;
  long long pix = 0, vec = pad;
  for (size_t i = 0; i < n; i++) {
    PatchDev P;
    P.W = (int)ws[i];
    P.H = (int)hs[i];
    P.N = P.W * P.H;
    for (int c = 0; c < 4; c++) P.nb[c] = 0;
    P.pix = pix;
    P.vec = vec;
    pix += ((long long)P.N + 31) / 32 * 32;
    vec += ((long long)P.N + 31) / 32 * 32 + pad;
    L.patches.push_back(P);
    const int pi = (int)i;
    for (int y = 0; y < P.H; y += 16)
      for (int x = 0; x < P.W; x += 16) {
        L.work_tex.push_back(make_int4(pi, y, x, 0));
        L.work16.push_back(make_int4(pi, y, x, 0));
      }
    for (int y = 0; y < P.H; y += kCueTileH)
      for (int x = 0; x < P.W; x += kCueTileW) L.work_cue.push_back(make_int4(pi, y, x, 0));
    for (int y = 0; y < P.H; y += kStepTileH)
      for (int x = 0; x < P.W; x += kStepTileW) L.work_blk.push_back(make_int4(pi, y, x, 0));
    L.tile_begin.push_back((int)L.tiles.size());
    for (int p0 = 0; p0 < P.N; p0 += kEigTile) {
      EigTile t;
      t.patch = pi;
      t.p0 = p0;
      t.p1 = std::min(P.N, p0 + kEigTile);
      t.pad = 0;
      L.tiles.push_back(t);
    }
    L.tile_count.push_back((int)L.tiles.size() - L.tile_begin.back());
  }
  L.total_pix = pix;
  L.lvec = vec;
  return L;
}

// the 2 x 2 aggregated layout of a fine layout
Layout make_coarse_layout(const Layout& F) {
  std::vector<uint32_t> ws, hs;
  for (const PatchDev& P : F.patches) {
    ws.push_back((uint32_t)((P.W + 1) / 2));
    hs.push_back((uint32_t)((P.H + 1) / 2));
  }
  return make_layout(ws.size(), ws.data(), hs.data());
}

}  // namespace

static gpb_status ensure_buffers(gpb_ctx* ctx, const Layout& L, bool layout_changed, const Layout* C) {
  Buf& b = ctx->b;
  const gpb_params& q = ctx->prm;
  const size_t P = L.total_pix, V = L.lvec, np = L.patches.size(), nt = L.tiles.size();
  const int m = q.krylov_dim;
  std::vector<cudaError_t> es;
  es.push_back(grow(b.packed, b.c_packed, P));
  es.push_back(grow(b.grey, b.c_grey, P));
  es.push_back(grow(b.lab4, b.c_lab4, P));
  es.push_back(grow(b.nbins, b.c_nbins, 4 * np));
  es.push_back(grow(b.repair, b.c_repair, 2 * (P / 4 + 1024)));
  es.push_back(grow(b.repair_count, b.c_rc, 1));
  es.push_back(grow(b.mpbo, b.c_mpbo, 8 * P));
  es.push_back(grow(b.go, b.c_go, 8 * P));
  es.push_back(grow(b.mpb, b.c_mpb, P));
  if (q.keep_intermediates) {
    es.push_back(grow(b.raw, b.c_raw, 96 * P));
    es.push_back(grow(b.wfull, b.c_wfull, 81 * P));
    es.push_back(grow(b.spb, b.c_spb, 8 * P));
    es.push_back(grow(b.gpbo, b.c_gpbo, 8 * P));
    if (q.keep_intermediates >= 2) es.push_back(grow(b.counts, b.c_counts, (size_t)kNannulus * 4 * 32 * 32 * P));
  }
  const size_t old_wup = b.c_wup;
  es.push_back(grow(b.wup, b.c_wup, (size_t)kUpper * V));
  es.push_back(grow(b.aup, b.c_aup, (size_t)kUpper * V));
  es.push_back(grow(b.deg, b.c_deg, V));
  es.push_back(grow(b.dis, b.c_dis, V));
  es.push_back(grow(b.adiag, b.c_adiag, V));
  for (int i = 0; i < 2; i++) {
    es.push_back(grow(b.V[i], b.c_V[i], (size_t)(m + 1) * V));
    es.push_back(grow(b.W[i], b.c_W[i], V));
  }
  es.push_back(grow(b.evec, b.c_evec, (size_t)q.nvec * V));
  es.push_back(grow(b.part, b.c_part, nt * kEigWarps * (size_t)(m + 1)));
  es.push_back(grow(b.hbuf, b.c_hbuf, np * (m + 1)));
  es.push_back(grow(b.T, b.c_T, np * m * m));
  es.push_back(grow(b.Y, b.c_Y, np * m * m));
  es.push_back(grow(b.beta2, b.c_beta2, np));
  es.push_back(grow(b.counter, b.c_counter, np));
  es.push_back(grow(b.active, b.c_active, np));
  es.push_back(grow(b.decision, b.c_decision, np));
  es.push_back(grow(b.nkeep, b.c_nkeep, np));
  es.push_back(grow(b.evals, b.c_evals, np * q.nvec));
  es.push_back(grow(b.mm, b.c_mm, np * q.nvec * 2));
  es.push_back(grow(b.nmax, b.c_nmax, P));
  es.push_back(grow(b.orient, b.c_orient, 8 * P));
  es.push_back(grow(b.patches, b.c_patches, np));
  es.push_back(grow(b.work_tex, b.c_wt, L.work_tex.size()));
  es.push_back(grow(b.work_cue, b.c_wc, L.work_cue.size()));
  es.push_back(grow(b.work16, b.c_w16, L.work16.size()));
  es.push_back(grow(b.work_blk, b.c_wb, L.work_blk.size()));
  es.push_back(grow(b.tiles, b.c_tiles, nt));
  es.push_back(grow(b.tile_begin, b.c_tb, np));
  es.push_back(grow(b.tile_count, b.c_tc, np));
  if (q.eig_mode != GPB_EIG_LANCZOS) {
    for (int i = 0; i < 4; i++) es.push_back(grow(b.blk[i], b.c_blk[i], (size_t)kBlk * V));
    es.push_back(grow(b.afull, b.c_afull, (size_t)kFullNC * V));
    es.push_back(grow(b.work_act, b.c_wact, L.work_blk.size()));
    es.push_back(grow(b.berr, b.c_berr, 4));  // error word, spare, block-step queue [2]
    es.push_back(grow(b.bpart, b.c_bpart, nt * kBlkSplit * 2 * kBlk * kBlk));  // two Gram matrices per slot
    es.push_back(grow(b.bgram, b.c_bgram, np * kBlk * kBlk));
    es.push_back(grow(b.bgram2, b.c_bgram2, np * kBlk * kBlk));
    es.push_back(grow(b.bmat, b.c_bmat, np * kBlk * kBlk));
    es.push_back(grow(b.btheta, b.c_btheta, np * kBlk));
    es.push_back(grow(b.bres, b.c_bres, np * kBlk));
    es.push_back(grow(b.bcoef, b.c_bcoef, np * (size_t)kMaxCheb));
    es.push_back(grow(b.bdone, b.c_bdone, np));
  }
  if (q.eig_mode == GPB_EIG_WARM && C) {
    const size_t Vc = C->lvec, ntc = C->tiles.size();
    es.push_back(grow(b.cpatches, b.c_cpatches, np));
    es.push_back(grow(b.ctiles, b.c_ctiles, ntc));
    es.push_back(grow(b.ctile_begin, b.c_ctb, np));
    es.push_back(grow(b.ctile_count, b.c_ctc, np));
    es.push_back(grow(b.cwork_blk, b.c_cwb, C->work_blk.size()));
    es.push_back(grow(b.cwork16, b.c_cw16, C->work16.size()));
    es.push_back(grow(b.cwc, b.c_cwc, (size_t)kCoarseNC * Vc));
    es.push_back(grow(b.cdeg, b.c_cdeg, Vc));
    es.push_back(grow(b.cdis, b.c_cdis, Vc));
    for (int i = 0; i < 4; i++) es.push_back(grow(b.cblk[i], b.c_cblk[i], (size_t)kBlk * Vc));
  }
  for (cudaError_t e : es)
    if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? GPB_ERR_NOMEM : GPB_ERR_CUDA;
  (void)old_wup;
  if (layout_changed) {
    // the padded layout relies on zero pads: clear every padded array
    cudaStream_t s = ctx->st;
    cudaMemsetAsync(b.wup, 0, (size_t)kUpper * V * sizeof(float), s);
    cudaMemsetAsync(b.aup, 0, (size_t)kUpper * V * sizeof(float), s);
    cudaMemsetAsync(b.deg, 0, V * sizeof(float), s);
    cudaMemsetAsync(b.dis, 0, V * sizeof(float), s);
    cudaMemsetAsync(b.adiag, 0, V * sizeof(float), s);
    for (int i = 0; i < 2; i++) {
      cudaMemsetAsync(b.V[i], 0, (size_t)(m + 1) * V * sizeof(float), s);
      cudaMemsetAsync(b.W[i], 0, V * sizeof(float), s);
    }
    cudaMemsetAsync(b.evec, 0, (size_t)q.nvec * V * sizeof(float), s);
    cudaMemsetAsync(b.counter, 0, np * sizeof(int), s);
    if (q.eig_mode != GPB_EIG_LANCZOS) {
      for (int i = 0; i < 4; i++) cudaMemsetAsync(b.blk[i], 0, (size_t)kBlk * V * sizeof(float), s);
      cudaMemsetAsync(b.afull, 0, (size_t)kFullNC * V * sizeof(float), s);
    }
    if (q.eig_mode == GPB_EIG_WARM && C) {
      cudaMemsetAsync(b.cwc, 0, (size_t)kCoarseNC * C->lvec * sizeof(float), s);
      cudaMemsetAsync(b.cdis, 0, C->lvec * sizeof(float), s);
      for (int i = 0; i < 4; i++) cudaMemsetAsync(b.cblk[i], 0, (size_t)kBlk * C->lvec * sizeof(float), s);
    }
  }
  return GPB_OK;
}

// the Krylov-Schur driver (plain cold-start Lanczos with thick restart)
static gpb_status solve_lanczos(gpb_ctx* ctx, const Layout& L) {
  Buf& b = ctx->b;
  const gpb_params& q = ctx->prm;
  cudaStream_t s = ctx->st;
  const int np = (int)L.patches.size(), nt = (int)L.tiles.size();
  const int m = q.krylov_dim, keep = q.krylov_keep, nev = q.nvec;
  EigArgs a;
  memset(&a, 0, sizeof(a));  // its bytes key the restart cycle's graph
  a.patches = b.patches;
  a.tiles = b.tiles;
  a.tile_begin = b.tile_begin;
  a.tile_count = b.tile_count;
  a.a_up = b.aup;
  a.a_diag = b.adiag;
  a.part = b.part;
  a.hbuf = b.hbuf;
  a.T = b.T;
  a.Y = b.Y;
  a.beta2 = b.beta2;
  a.counter = b.counter;
  a.active = b.active;
  a.decision = b.decision;
  a.nkeep = b.nkeep;
  a.lvec = L.lvec;
  a.m = m;
  a.mp1 = m + 1;
  std::vector<int> active(np, 1), decision(np, 0), nkeep(np, 0), mv(np, 0);
  std::vector<double> T((size_t)np * m * m), Y((size_t)np * m * m), beta2(np);
  std::vector<float> evals((size_t)np * nev, 0.f);
  float* Vc = b.V[0];
  float* Va = b.V[1];
  float* cur = b.W[0];
  float* nxt = b.W[1];
  CK(cudaMemcpyAsync(b.active, active.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b.decision, decision.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(b.T, 0, (size_t)np * m * m * sizeof(double), s));
  a.V = Vc;
  CK(ks_launch_init(a, nt, cur, s));
  ctx->launches++;
  int k = 0;
  bool first = true;
  int restarts = 0;
  float maxres = 0.f;
  bool noconv = false;
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  for (;;) {
    a.V = Vc;
    long long active_px = 0;
    for (int i = 0; i < np; i++)
      if (active[i]) active_px += L.patches[i].N;
    // one restart cycle: Lanczos steps k .. m-1, three launches each
    auto cycle = [&]() -> cudaError_t {
      float* c = cur;
      float* nx = nxt;
      for (int j = k; j < m; j++) {
        const bool from_v = (j == k && !first);
        // algorithmic bytes per pixel: SpMV reads 40 upper coefficients, the
        // diagonal and x, writes v_j and w, and reads j basis vectors for the
        // dots; a CGS pass reads w and j+1 basis vectors and writes w
        const double npx = (double)active_px;
        cudaError_t e;
        prof_begin(ctx, 0, npx * 4.0 * (kUpper + 1 + 1 + 2 + j));
        if ((e = ks_launch_spmv(a, nt, j, from_v ? Vc + (long long)k * L.lvec : c, from_v ? 0 : 1, nx, s)) !=
            cudaSuccess)
          return e;
        prof_end(ctx);
        prof_begin(ctx, 1, npx * 4.0 * (j + 1 + 2));
        if ((e = ks_launch_orth(a, nt, j, 1, nx, s)) != cudaSuccess) return e;
        prof_end(ctx);
        prof_begin(ctx, 1, npx * 4.0 * (j + 1 + 2));
        if ((e = ks_launch_orth(a, nt, j, 2, nx, s)) != cudaSuccess) return e;
        prof_end(ctx);
        ctx->launches += 3;
        std::swap(c, nx);
      }
      return cudaSuccess;
    };
    CK(graph_run(ctx, gkey("lanczos", k, first, m, nt, cur, nxt) + std::string((const char*)&a, sizeof(a)), cycle));
    if ((m - k) % 2) std::swap(cur, nxt);
    CK(cudaMemcpyAsync(T.data(), b.T, T.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(beta2.data(), b.beta2, np * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    // host: dense eigensolve per active patch (threads over patches)
    int active_count = 0;
    for (int i = 0; i < np; i++) active_count += active[i];
    std::atomic<int> next(0);
    std::vector<float> res((size_t)np, 0.f);
    auto worker = [&]() {
      std::vector<double> A((size_t)m * m), w(m), Z((size_t)m * m);
      for (int i; (i = next.fetch_add(1)) < np;) {
        if (!active[i]) continue;
        mv[i] += m - k;
        const double* Ti = T.data() + (size_t)i * m * m;
        for (int r = 0; r < m; r++)
          for (int c = 0; c < m; c++) A[r * m + c] = 0.5 * (Ti[r * m + c] + Ti[c * m + r]);
        gpb::sym_eig(A.data(), m, w.data(), Z.data());
        const double beta = sqrt(beta2[i]);
        double worst = 0;
        for (int c = 0; c < nev; c++) worst = std::max(worst, fabs(beta * Z[(m - 1) * m + c]));
        res[i] = (float)worst;
        const bool conv = worst <= q.eig_tol;
        const bool cap = mv[i] + (m - keep) > q.eig_max_matvecs;
        double* Yi = Y.data() + (size_t)i * m * m;
        for (int r = 0; r < m; r++)
          for (int c = 0; c < m; c++) Yi[r * m + c] = Z[r * m + c];
        if (conv || cap) {
          decision[i] = 2;
          nkeep[i] = nev;
          for (int c = 0; c < nev; c++) evals[(size_t)i * nev + c] = (float)w[c];
          if (!conv) noconv = true;
        } else {
          decision[i] = 1;
          nkeep[i] = keep;
          double* Tn = T.data() + (size_t)i * m * m;
          std::fill(Tn, Tn + (size_t)m * m, 0.0);
          for (int c = 0; c < keep; c++) {
            Tn[c * m + c] = w[c];
            Tn[c * m + keep] = Tn[keep * m + c] = beta * Z[(m - 1) * m + c];
          }
        }
      }
    };
    {
      // one dense solve takes ~0.1 ms: threads only pay off for many patches
      const unsigned nth = std::min<unsigned>(hw, (unsigned)((active_count + 3) / 4));
      std::vector<std::thread> th;
      for (unsigned t = 1; t < nth; t++) th.emplace_back(worker);
      worker();
      for (auto& t : th) t.join();
    }
    restarts++;
    bool any_restart = false;
    for (int i = 0; i < np; i++) {
      if (decision[i] == 2 && active[i]) {
        active[i] = 0;
        maxres = std::max(maxres, res[i]);
      }
      if (decision[i] == 1) any_restart = true;
    }
    CK(cudaMemcpyAsync(b.Y, Y.data(), Y.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.T, T.data(), T.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.decision, decision.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.nkeep, nkeep.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.active, active.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
    a.V = Vc;
    const bool any_final = std::count(decision.begin(), decision.end(), 2) > 0;
    CK(ks_launch_restart(a, nt, cur, Va, b.evec, s, any_restart, any_final));
    ctx->launches += (int)any_restart + (int)any_final;
    std::swap(Vc, Va);
    std::fill(decision.begin(), decision.end(), 0);
    CK(cudaMemcpyAsync(b.decision, decision.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
    if (!any_restart) break;
    k = keep;
    first = false;
  }
  CK(cudaMemcpyAsync(b.evals, evals.data(), evals.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  CK(cudaStreamSynchronize(s));
  prof_collect(ctx);
  ctx->evals_host = evals;
  long tot = 0, mx = 0;
  for (int i = 0; i < np; i++) {
    tot += mv[i];
    mx = std::max(mx, (long)mv[i]);
  }
  ctx->stats.matvecs_total = tot;
  ctx->stats.matvecs_max = mx;
  ctx->stats.restarts = restarts;
  ctx->stats.max_residual = maxres;
  return noconv ? GPB_ERR_NOCONV : GPB_OK;
}

// ------------------------------------------------------------------------
// Warm-startable block eigensolver: Chebyshev-filtered subspace iteration
// (Zhou & Saad, J. Comput. Phys. 219 (2006) and Numer. Linear Algebra Appl.
// 14 (2007)) on a block of 32 vectors.  Each outer iteration applies a
// degree-d scaled Chebyshev filter that damps [theta_max, 2] (the spectrum of
// the normalised Laplacian ends at 2), orthonormalises the block twice on its
// Gram matrix (symmetric orthonormalisation, FP64 on the host) and performs a
// Rayleigh-Ritz step; the host solves the 32 x 32 problems.  The start block
// is the warm start; without one it is seeded noise.
// one level of the block solver: its layout, device tables, operator and
// the four block buffers
struct Level {
  const Layout* L;
  const PatchDev* patches;
  const EigTile* tiles;
  const int* tile_begin;
  const int* tile_count;
  const int4* work_blk;
  const float* afull;  // pixel-major stencil rows of the level's operator
  int coarse;
  float* blk[4];
};

// Solves one level; on return *Xout is the buffer holding the 32 Ritz
// vectors (ascending).  extract: write the first nvec into b.evec.
static gpb_status solve_block(gpb_ctx* ctx, const Level& lv, bool have_start, double tol, bool extract,
                              float** Xout) {
  const Layout& L = *lv.L;
  Buf& b = ctx->b;
  const gpb_params& q = ctx->prm;
  cudaStream_t s = ctx->st;
  const int np = (int)L.patches.size(), nt = (int)L.tiles.size(), nev = q.nvec;
  // the persistent block step walks a tile list; once patches converge it
  // gets only the tiles of the active ones (L.work_blk is patch-major)
  std::vector<int> tb_begin(np + 1, 0);
  for (const int4& t : L.work_blk) tb_begin[t.x + 1]++;
  for (int i = 0; i < np; i++) tb_begin[i + 1] += tb_begin[i];
  int nwb = (int)L.work_blk.size();
  const int4* work_blk = lv.work_blk;
  std::vector<int4> act_tiles;
  std::vector<int> listed(np, 1);  // the patches the current list holds
  // a multiple of 3, so the three-buffer Chebyshev rotation ends where it
  // started and every patch's vectors stay in X, converged or not
  const int deg = std::min((std::max(3, q.cheb_degree) + 2) / 3 * 3, kMaxCheb / 3 * 3);
  BlkArgs a;
  memset(&a, 0, sizeof(a));  // its bytes key the filter's graph
  a.patches = lv.patches;
  a.tiles = lv.tiles;
  a.tile_begin = lv.tile_begin;
  a.tile_count = lv.tile_count;
  a.a_up = nullptr;
  a.a_diag = nullptr;
  a.afull = lv.afull;
  a.err = b.berr;
  a.queue = b.berr + 2;
  a.coarse = lv.coarse;
  a.lvec = L.lvec;
  a.coef = b.bcoef;
  a.max_steps = kMaxCheb;
  a.part = b.bpart;
  a.counter = b.counter;
  a.active = b.active;
  a.done = b.bdone;
  a.mat = b.bmat;
  a.theta = b.btheta;
  const size_t BB = (size_t)kBlk * kBlk;
  // block-step variant per level and tile-count bucket
  auto step_key = [&](int nw) {
    return std::string(lv.coarse ? "step/coarse" : "step/fine") + "/tiles2^" + std::to_string(ilog2(nw));
  };
  auto step_variant = [&](int nw) {
    bool trial = false;
    return ctx->tuner.decided(step_key(nw)) ? ctx->tuner.pick(step_key(nw), kStepVariants, 3, kStepDefault, &trial)
                                            : kStepDefault;
  };
  std::vector<int> active(np, 1), done(np, 0);
  // G, M, G2 (32 x 32 per patch), theta, res and the filter coefficients
  // live in one pinned block, so their copies are direct DMA
  const size_t nG = np * BB, nT = np * (size_t)kBlk, nC = np * (size_t)kMaxCheb;
  const size_t need = (3 * nG + 2 * nT) * sizeof(double) + nC * sizeof(float3);
  if (ctx->c_hsmall < need) {
    if (ctx->h_small) cudaFreeHost(ctx->h_small);
    ctx->h_small = nullptr;
    ctx->c_hsmall = 0;
    CK(cudaMallocHost(&ctx->h_small, need));
    ctx->c_hsmall = need;
  }
  struct HostArr {  // a span with the operator[] and data() the code below uses
    double* p;
    size_t n;
    double& operator[](size_t i) { return p[i]; }
    double* data() { return p; }
    size_t size() const { return n; }
    double* begin() { return p; }
  };
  double* hb = (double*)ctx->h_small;
  HostArr G{hb, nG}, M{hb + nG, nG}, theta{hb + 2 * nG, nT}, res{hb + 2 * nG + nT, nT},
      G2{hb + 2 * nG + 2 * nT, nG};
  for (size_t i = 0; i < nT; i++) theta[i] = 0.0;
  struct CoefArr {
    float3* p;
    size_t n;
    float3& operator[](size_t i) { return p[i]; }
    float3* data() { return p; }
    size_t size() const { return n; }
  } coef{(float3*)(hb + 3 * nG + 2 * nT), nC};
  std::vector<float> evals((size_t)np * nev, 0.f);
  std::vector<long> mv(np, 0);
  // stagnation: the best worst-residual of each patch and the outer
  // iteration that last improved it by 2%; FP32 vectors put a floor of a
  // few 1e-7 under the residual, and a tolerance below it would otherwise
  // run to the matvec cap (a clustered spectrum still converging slowly
  // gains a few % per outer iteration, so the window is 6)
  std::vector<double> best_res(np, 1e300);
  std::vector<int> best_at(np, 0);
  constexpr int kStagnant = 6, kMaxOuter = 400;
  float* X = lv.blk[0];
  float* Y = lv.blk[1];
  float* Z = lv.blk[2];
  float* AX = lv.blk[3];
  CK(cudaMemcpyAsync(b.active, active.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b.bdone, done.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
  if (!have_start) {
    CK(cf_launch_init(a, nt, X, s));
    ctx->launches++;
  }
  auto upload_unit = [&]() -> cudaError_t {  // coefficient (1, 0, 0) at step 0: plain SpMV
    for (int i = 0; i < np; i++) coef[(size_t)i * kMaxCheb] = make_float3(1.f, 0.f, 0.f);
    return cudaMemcpyAsync(b.bcoef, coef.data(), coef.size() * sizeof(float3), cudaMemcpyHostToDevice, s);
  };
  // orthonormalise F (symmetric orthonormalisation), then Rayleigh-Ritz on
  // span(F) in the metric of F's Gram matrix, which folds a second
  // orthonormalisation into the same host step; AF receives A F.
  // comp: compensated Rayleigh-Ritz product and rotation (see cf_step_t, cf_rotate)
  auto rr = [&](float* F, float* AF, bool comp) -> gpb_status {
    CK(cf_launch_gram(a, nt, F, F, b.bgram, s));
    CK(cudaMemcpyAsync(G.data(), b.bgram, np * BB * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    ctx->tuner.collect();
    ctx->host_pool().run(np, [&](int i) {
      if (active[i]) gpb::lowdin(G.data() + i * BB, kBlk, M.data() + i * BB);
    });
    if (ctx->trace && active[0])
      fprintf(stderr, "[gpb] gram patch 0: G00 %.3e G11 %.3e G3131 %.3e M00 %.3e\n", G[0], G[kBlk + 1], G[BB - 1],
              M[0]);
    CK(cudaMemcpyAsync(b.bmat, M.data(), np * BB * sizeof(double), cudaMemcpyHostToDevice, s));
    CK(cf_launch_rotate(a, nt, F, nullptr, kBlk, s));
    CK(upload_unit());
    CK(cf_launch_step(a, work_blk, nwb, F, F, AF, 0, s, comp, step_variant(nwb)));
    CK(cf_launch_gram(a, nt, F, AF, b.bgram, s, b.bgram2));  // G = F^T AF and G2 = F^T F in one pass
    CK(cudaMemcpyAsync(G2.data(), b.bgram2, np * BB * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(G.data(), b.bgram, np * BB * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    ctx->launches += 4;
    ctx->host_pool().run(np, [&](int i) {
      if (!active[i]) return;
      mv[i] += kBlk;
      // M1 = G2^-1/2; the Ritz pairs of M1 H M1 give the rotation M1 Z
      std::vector<double> M1(BB), Hs(BB), T(BB), C(BB), w(kBlk), Zm(BB);
      gpb::lowdin(G2.data() + i * BB, kBlk, M1.data());
      for (int r = 0; r < kBlk; r++)
        for (int c = 0; c < kBlk; c++)
          Hs[r * kBlk + c] = 0.5 * (G[i * BB + r * kBlk + c] + G[i * BB + c * kBlk + r]);
      gpb::mat_mul(Hs.data(), M1.data(), T.data(), kBlk, false);  // T = Hs M1
      gpb::mat_mul(M1.data(), T.data(), C.data(), kBlk, true);    // C = M1^T T
      for (int r = 0; r < kBlk; r++)
        for (int c = r + 1; c < kBlk; c++) C[r * kBlk + c] = C[c * kBlk + r] = 0.5 * (C[r * kBlk + c] + C[c * kBlk + r]);
      gpb::sym_eig(C.data(), kBlk, w.data(), Zm.data());
      for (int c = 0; c < kBlk; c++) theta[(size_t)i * kBlk + c] = w[c];
      gpb::mat_mul(M1.data(), Zm.data(), M.data() + i * BB, kBlk, false);  // M = M1 Zm
    });
    CK(cudaMemcpyAsync(b.bmat, M.data(), np * BB * sizeof(double), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.btheta, theta.data(), theta.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    CK(cf_launch_rotate(a, nt, F, AF, kBlk, s, comp));
    CK(cf_launch_resid(a, nt, F, AF, b.bres, s));
    CK(cudaMemcpyAsync(res.data(), b.bres, res.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    ctx->launches += 2;
    return GPB_OK;
  };
  gpb_status st = rr(X, AX, false);
  if (st != GPB_OK) return st;
  int outer = 0;
  float maxres = 0.f;
  bool noconv = false;
  for (;;) {
    // convergence and per-patch filter coefficients
    int nactive = 0;
    bool tight = false;  // an active patch is gap-limited and near its target
    for (int i = 0; i < np; i++) {
      if (!active[i]) continue;
      double worst = 0;
      bool finite = true;
      for (int c = 0; c < nev; c++) {
        const double r2 = res[(size_t)i * kBlk + c];
        if (!std::isfinite(r2)) finite = false;
        worst = std::max(worst, sqrt(std::max(r2, 0.0)));
      }
      if (ctx->trace)
        fprintf(stderr, "[gpb] block patch %d outer %d theta0 %.3e theta8 %.3e theta31 %.3e worst %.3e%s\n", i,
                outer, theta[(size_t)i * kBlk], theta[(size_t)i * kBlk + 8], theta[(size_t)i * kBlk + kBlk - 1], worst,
                finite ? "" : " NON-FINITE");
      if (!finite) {
        ctx->last_error = "non-finite residual in the block eigensolver";
        return GPB_ERR_INTERNAL;
      }
      // eigenvector error ~ residual / gap: on the final level a patch whose
      // wanted eigenvalues nearly coincide must also reach eig_gap_frac times
      // its smallest gap (not below 1e-7, about what FP32 vectors hold)
      double tol_i = tol;
      if (extract && q.eig_gap_frac > 0) {
        double gmin = 1e300;
        const double* th = &theta[(size_t)i * kBlk];
        for (int c = 1; c < nev; c++) gmin = std::min(gmin, std::min(th[c] - th[c - 1], th[c + 1] - th[c]));
        tol_i = std::min(tol, std::max(1e-7, q.eig_gap_frac * gmin));
      }
      const bool conv = worst <= tol_i;
      if (worst < 0.98 * best_res[i]) {
        best_res[i] = worst;
        best_at[i] = outer;
      }
      const bool stalled = outer - best_at[i] >= kStagnant;
      if (conv || stalled || outer >= kMaxOuter || mv[i] + (long)(deg + 1) * kBlk > q.eig_max_matvecs) {
        active[i] = 0;
        done[i] = 1;
        maxres = std::max(maxres, (float)worst);
        // the gap target is pursued as far as FP32 allows.  FP32 vectors put
        // a floor under the residual that grows with the patch (about 6e-7
        // at 0.3 Mpix, 1e-6 at 1.6 Mpix): a patch that stops improving
        // within 4x the requested tolerance has converged as far as it can;
        // only a residual above that is a failure to converge
        if (!conv && worst > 4 * tol) noconv = true;
        for (int c = 0; c < nev; c++) evals[(size_t)i * nev + c] = (float)theta[(size_t)i * kBlk + c];
        continue;
      }
      nactive++;
      if (tol_i < tol && worst < 10 * tol) tight = true;
      // the normalised Laplacian's spectrum lies in [0, 2]: normalising the
      // filter at 0 (not at the smallest Ritz value, which a random start
      // puts near 1) keeps every component of the block bounded in FP32
      const double ub = 2.0, lo0 = -1e-3, cut = theta[(size_t)i * kBlk + kBlk - 1];
      const double e = (ub - cut) / 2, c = (ub + cut) / 2;
      double sigma = e / (lo0 - c);
      const double tau = 2 / sigma;
      coef[(size_t)i * kMaxCheb] = make_float3((float)(sigma / e), (float)(-c * sigma / e), 0.f);
      for (int k = 1; k < deg; k++) {
        const double s2 = 1 / (tau - sigma);
        coef[(size_t)i * kMaxCheb + k] = make_float3((float)(2 * s2 / e), (float)(-2 * c * s2 / e), (float)(-sigma * s2));
        sigma = s2;
      }
      mv[i] += (long)deg * kBlk;
    }
    CK(cudaMemcpyAsync(b.active, active.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
    if (nactive == 0) break;
    if (active != listed) {
      act_tiles.clear();
      for (int i = 0; i < np; i++)
        if (active[i]) act_tiles.insert(act_tiles.end(), L.work_blk.begin() + tb_begin[i], L.work_blk.begin() + tb_begin[i + 1]);
      CK(cudaMemcpyAsync(b.work_act, act_tiles.data(), act_tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
      work_blk = b.work_act;
      nwb = (int)act_tiles.size();
      listed = active;
    }
    CK(cudaMemcpyAsync(b.bcoef, coef.data(), coef.size() * sizeof(float3), cudaMemcpyHostToDevice, s));
    // filter: buffers rotate X -> Y -> Z -> X ...
    long long apx = 0;
    for (int i = 0; i < np; i++)
      if (active[i]) apx += L.patches[i].N;
    float* buf[3] = {X, Y, Z};
    int cur = 0;
    const bool decided = ctx->tuner.decided(step_key(nwb));
    const int chosen = step_variant(nwb);
    auto filter = [&]() -> cudaError_t {
      int c = 0;
      for (int k = 0; k < deg; k++) {
        const int nxt = (c + 1) % 3, prv = (c + 2) % 3;
        // algorithmic bytes per pixel: the stencil row's coefficients, the
        // 32-wide rows of Y (and of the previous iterate after the first
        // step), the output row
        prof_begin(ctx, 0, (double)apx * (4.0 * (lv.coarse ? kCN : kStencilN) + 4.0 * kBlk * (k ? 3 : 2)));
        bool trial = false;
        const int v = decided ? chosen : ctx->tuner.pick(step_key(nwb), kStepVariants, 3, chosen, &trial);
        if (trial) ctx->tuner.begin(step_key(nwb), v, s);
        const cudaError_t e = cf_launch_step(a, work_blk, nwb, buf[c], buf[prv], buf[nxt], k, s, false, v);
        if (trial) ctx->tuner.end(s);
        if (e != cudaSuccess) return e;
        prof_end(ctx);
        c = nxt;
      }
      ctx->launches += deg;
      return cudaSuccess;
    };
    CK(graph_run(ctx,
                 gkey("filter", deg, nwb, work_blk, X, Y, Z, chosen) + std::string((const char*)&a, sizeof(a)),
                 filter, decided));
    cur = deg % 3;
    if (buf[cur] != X) {
      ctx->last_error = "block filter rotation out of step";
      return GPB_ERR_INTERNAL;
    }
    st = rr(X, AX, tight);
    if (st != GPB_OK) return st;
    outer++;
  }
  *Xout = X;
  if (extract) {
    CK(cudaMemcpyAsync(b.bdone, done.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cf_launch_extract(a, nt, X, b.evec, nev, s));
    ctx->launches++;
    CK(cudaMemcpyAsync(b.evals, evals.data(), evals.size() * sizeof(float), cudaMemcpyHostToDevice, s));
    ctx->evals_host = evals;
  }
  CK(cudaStreamSynchronize(s));
  prof_collect(ctx);
  long tot = 0, mx = 0;
  for (int i = 0; i < np; i++) {
    tot += mv[i];
    mx = std::max(mx, mv[i]);
  }
  if (ctx->trace)
    fprintf(stderr, "[gpb] block level %s: outer %d, matvecs max %ld total %ld\n", lv.coarse ? "coarse" : "fine",
            outer, mx, tot);
  ctx->stats.matvecs_total += tot;
  ctx->stats.matvecs_max += mx;
  ctx->stats.restarts += outer;
  if (extract) ctx->stats.max_residual = maxres;
  return (noconv && extract) ? GPB_ERR_NOCONV : GPB_OK;
}

// warm-started block solve: the coarse (2 x 2 aggregated) problem from a
// seeded start to a loose tolerance, its Ritz vectors prolongated to the fine
// level as the start block, then the fine problem to the full tolerance
static gpb_status solve_warm(gpb_ctx* ctx, const Layout& L, const Layout& Lc) {
  Buf& b = ctx->b;
  cudaStream_t s = ctx->st;
  const size_t np = L.patches.size();
  CK(cudaMemcpyAsync(b.cpatches, Lc.patches.data(), np * sizeof(PatchDev), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b.ctiles, Lc.tiles.data(), Lc.tiles.size() * sizeof(EigTile), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b.ctile_begin, Lc.tile_begin.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b.ctile_count, Lc.tile_count.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b.cwork_blk, Lc.work_blk.data(), Lc.work_blk.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b.cwork16, Lc.work16.data(), Lc.work16.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
  CoarseArgs c;
  c.fine = b.patches;
  c.coarse = b.cpatches;
  c.work = b.cwork16;
  c.work_f = b.work16;
  c.wsym_up = b.wup;
  c.deg = b.deg;
  c.lvec_f = L.lvec;
  c.lvec_c = Lc.lvec;
  c.wc = b.cwc;
  c.degc = b.cdeg;
  c.disc = b.cdis;
  CK(cf_launch_coarsen(c, (int)Lc.work16.size(), s));
  ctx->launches += 2;
  Level lc = {&Lc, b.cpatches, b.ctiles, b.ctile_begin, b.ctile_count, b.cwork_blk, b.cwc, 1,
              {b.cblk[0], b.cblk[1], b.cblk[2], b.cblk[3]}};
  float* Xc = nullptr;
  gpb_status st = solve_block(ctx, lc, false, ctx->prm.warm_tol, false, &Xc);
  if (st != GPB_OK) return st;
  CK(cf_launch_prolong(c, (int)L.work16.size(), Xc, b.blk[0], s));
  ctx->launches++;
  const size_t blk_bytes = (size_t)kBlk * L.lvec * sizeof(float);
  if (ctx->wn_capture) {  // the start block before any correction, for training
    CK(grow(ctx->d_wn_x0, ctx->c_wn_x0, (size_t)kBlk * L.lvec));
    CK(cudaMemcpyAsync(ctx->d_wn_x0, b.blk[0], blk_bytes, cudaMemcpyDeviceToDevice, s));
  }
  if (ctx->d_wn) {  // the learned correction of the first 9 columns
    int max_n = 0;
    for (const PatchDev& P : L.patches) max_n = std::max(max_n, P.N);
    CK(grow(ctx->d_wn_scale, ctx->c_wn_scale, np * (size_t)kWnOut));
    CK(wn_launch_apply(b.patches, (int)np, max_n, b.blk[0], b.mpb, ctx->d_wn, ctx->d_wn_scale, b.blk[1], s));
    CK(cudaMemcpyAsync(b.blk[0], b.blk[1], blk_bytes, cudaMemcpyDeviceToDevice, s));
    ctx->launches += 2;
  }
  Level lf = {&L, b.patches, b.tiles, b.tile_begin, b.tile_count, b.work_blk, b.afull, 0,
              {b.blk[0], b.blk[1], b.blk[2], b.blk[3]}};
  float* Xf = nullptr;
  return solve_block(ctx, lf, true, ctx->prm.eig_tol, true, &Xf);
}

// block solve started from the learned network's fields
static gpb_status solve_learned(gpb_ctx* ctx, const Layout& L) {
  Buf& b = ctx->b;
  cudaStream_t s = ctx->st;
  if (!ctx->net || !ctx->net->has_params()) {
    ctx->last_error = "GPB_EIG_LEARNED needs the network's weights (gpb_learned_set)";
    return GPB_ERR_ARG;
  }
  std::vector<int> H, W;
  int maxn = 0;
  for (const PatchDev& P : L.patches) {
    H.push_back(P.H);
    W.push_back(P.W);
    maxn = std::max(maxn, P.N);
  }
  const int l0 = ctx->net->launches();
  CK(ctx->net->layout(H, W, s));
  CK(ctx->net->features_from(b.patches, b.mpb, b.deg, s));
  CK(ctx->net->forward(s));
  CK(ln_launch_start(ctx->net->patches0_dev(), b.patches, (int)L.patches.size(), maxn, ctx->net->y(), b.blk[0], s));
  ctx->launches += ctx->net->launches() - l0 + 1;
  Level lf = {&L, b.patches, b.tiles, b.tile_begin, b.tile_count, b.work_blk, b.afull, 0,
              {b.blk[0], b.blk[1], b.blk[2], b.blk[3]}};
  float* Xf = nullptr;
  return solve_block(ctx, lf, true, ctx->prm.eig_tol, true, &Xf);
}

static gpb_status run_batch(gpb_ctx* ctx, size_t n, const uint32_t* ws, const uint32_t* hs,
                            const uint32_t* const* host_in, const size_t* host_stride, const uint32_t* dev_in,
                            const size_t* dev_off, float* dev_nmax, float* dev_orient, gpb_result* host_out) {
  if (n == 0) return GPB_ERR_ARG;
  if (ctx->K == 0) return GPB_ERR_ARG;  // no codebook
  for (size_t i = 0; i < n; i++)
    if (ws[i] < (uint32_t)kMinSide || hs[i] < (uint32_t)kMinSide || ws[i] > 8192 || hs[i] > 8192)
      return GPB_ERR_ARG;
  cudaSetDevice(ctx->device);
  std::lock_guard<std::mutex> bank_lock(bank_of(ctx->device).mu);
  CK(load_tables(ctx));
  cudaStream_t s = ctx->st;
  Buf& b = ctx->b;
  ctx->launches = 0;
  memset(&ctx->stats, 0, sizeof(ctx->stats));
  Layout L = make_layout(n, ws, hs);
  // the eigensolver kernels index the vector layout with 32-bit offsets
  if (L.lvec >= (1LL << 31)) {
    ctx->last_error = "batch too large: its padded vector layout exceeds 2^31 entries; split it";
    return GPB_ERR_TOO_LARGE;
  }
  std::string key;
  for (size_t i = 0; i < n; i++) key += std::to_string(ws[i]) + "x" + std::to_string(hs[i]) + ",";
  const bool changed = key != ctx->layout_key;
  Layout Lc;
  const bool warm = ctx->prm.eig_mode == GPB_EIG_WARM;
  if (warm) Lc = make_coarse_layout(L);
  gpb_status st = ensure_buffers(ctx, L, changed, warm ? &Lc : nullptr);
  if (st != GPB_OK) return st;
  ctx->layout_key = key;
  const size_t np = L.patches.size();
  CK(cudaEventRecord(ctx->ev[0], s));
  CK(cudaMemcpyAsync(b.patches, L.patches.data(), np * sizeof(PatchDev), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b.work_tex, L.work_tex.data(), L.work_tex.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b.work_cue, L.work_cue.data(), L.work_cue.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b.work16, L.work16.data(), L.work16.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b.work_blk, L.work_blk.data(), L.work_blk.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b.tiles, L.tiles.data(), L.tiles.size() * sizeof(EigTile), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b.tile_begin, L.tile_begin.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b.tile_count, L.tile_count.data(), np * sizeof(int), cudaMemcpyHostToDevice, s));
  // input
  if (host_in) {
    if (ctx->c_hpacked < (size_t)L.total_pix) {
      if (ctx->h_packed) cudaFreeHost(ctx->h_packed);
      CK(cudaMallocHost(&ctx->h_packed, L.total_pix * sizeof(uint32_t)));
      ctx->c_hpacked = L.total_pix;
    }
    std::vector<CopyJob> jobs;  // the caller's rows to the staging, on the host pool
    for (size_t i = 0; i < n; i++) {
      const PatchDev& P = L.patches[i];
      if (host_stride[i] == (size_t)P.W) {
        jobs.push_back({ctx->h_packed + P.pix, host_in[i], (size_t)P.N * sizeof(uint32_t)});
      } else {
        for (int y = 0; y < P.H; y++)
          jobs.push_back({ctx->h_packed + P.pix + (size_t)y * P.W, host_in[i] + (size_t)y * host_stride[i],
                          (size_t)P.W * sizeof(uint32_t)});
      }
    }
    parallel_copy(ctx->host_pool(), jobs);
    CK(cudaMemcpyAsync(b.packed, ctx->h_packed, L.total_pix * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
  } else {
    for (size_t i = 0; i < n; i++) {
      const PatchDev& P = L.patches[i];
      CK(cudaMemcpyAsync(b.packed + P.pix, dev_in + dev_off[i], (size_t)P.N * sizeof(uint32_t),
                         cudaMemcpyDeviceToDevice, s));
    }
  }
  if (!ctx->d_lab_lut) {  // once per context; the gamma table it reads is constant
    CK(cudaMalloc(&ctx->d_lab_lut, sizeof(uint32_t) << 24));
    CK(launch_lab_table(ctx->d_lab_lut, s));
  }
  CK(cudaEventRecord(ctx->ev[1], s));
  // (a)-(c): textons, local cues, NMS, buildW and the operator rows, one
  // fixed chain per batch layout
  const int repair_cap = (int)(b.c_repair / 2);
  const bool blockm = ctx->prm.eig_mode != GPB_EIG_LANCZOS;
  // texton variant for this shape bucket: batch pixels and largest side, log2
  int side = 0;
  for (size_t i = 0; i < n; i++) side = std::max(side, (int)std::max(ws[i], hs[i]));
  const std::string tx_key = "texton/px2^" + std::to_string(ilog2(L.total_pix)) + "/side2^" + std::to_string(ilog2(side));
  // an undecided bucket tries every variant within this one launch, each on
  // a third of the tile list (the tiles are independent and the labels the
  // same), timed and scaled to the whole list
  const int ntex = (int)L.work_tex.size();
  if (ctx->tuner.enabled && !ctx->tuner.decided(tx_key) && ntex < 16 * kTextonVariants)
    ctx->tuner.settle(tx_key, kTextonVariants, 1);  // too few tiles to time
  const bool tx_trial = !ctx->tuner.decided(tx_key);
  if (tx_trial) ctx->tuner.entry(tx_key, kTextonVariants, 1);
  bool tx_unused = false;
  const int tx_var = tx_trial ? 1 : ctx->tuner.pick(tx_key, kTextonVariants, 1, 1, &tx_unused);
  auto pre_chain = [&]() -> cudaError_t {
    cudaError_t e;
#define GK(x)                               \
  do {                                      \
    if ((e = (x)) != cudaSuccess) return e; \
  } while (0)
    // (a) textons
    GK(launch_convert_lut(b.packed, L.total_pix, ctx->d_lab_lut, b.grey, b.lab4, s));
    GK(cudaMemsetAsync(b.repair_count, 0, sizeof(int), s));
    if (tx_trial) {
      for (int v = 0; v < kTextonVariants; v++) {
        const int t0 = ntex * v / kTextonVariants, t1 = ntex * (v + 1) / kTextonVariants;
        ctx->tuner.begin(tx_key, v, s, (float)ntex / (float)(t1 - t0));
        GK(launch_texton(b.patches, b.work_tex + t0, t1 - t0, b.grey, b.lab4, b.repair, b.repair_count, repair_cap,
                         s, v));
        ctx->tuner.end(s);
      }
      ctx->launches += kTextonVariants - 1;
    } else {
      GK(launch_texton(b.patches, b.work_tex, ntex, b.grey, b.lab4, b.repair, b.repair_count, repair_cap, s,
                       tx_var));
    }
    GK(launch_texton_repair(b.patches, b.grey, b.lab4, b.repair, b.repair_count, repair_cap, ctx->d_k32_ring,
                            ctx->d_ring_of, ctx->tab.n_rings, s));
    GK(stage_mark(ctx->ev[2], s));
    // (b) local cues + NMS
    GK(launch_maxlabel(b.patches, (int)np, b.lab4, b.nbins, s));
    GK(launch_cues(b.patches, b.work_cue, (int)L.work_cue.size(), b.lab4, b.nbins, b.mpbo, b.go,
                   ctx->prm.keep_intermediates ? b.raw : nullptr,
                   ctx->prm.keep_intermediates >= 2 ? b.counts : nullptr, s));
    GK(stage_mark(ctx->ev[3], s));
    GK(launch_nms(b.patches, b.work16, (int)L.work16.size(), b.mpbo, b.mpb, s));
    GK(stage_mark(ctx->ev[4], s));
    // (c) buildW
    GK(launch_buildw(b.patches, b.work16, (int)L.work16.size(), b.mpb, ctx->d_ic, b.wup, b.deg, L.lvec, s));
    GK(launch_scale(b.patches, b.work16, (int)L.work16.size(), b.wup, b.deg, b.aup, b.adiag, b.dis, L.lvec,
                    ctx->prm.keep_intermediates ? b.wfull : nullptr, s));
    if (blockm) {
      GK(cf_launch_full(b.patches, b.work16, (int)L.work16.size(), b.aup, b.adiag, L.lvec, b.afull, s));
      GK(cudaMemsetAsync(b.berr, 0, 4 * sizeof(int), s));  // error word and the block step's queue
      ctx->launches++;
    }
    GK(stage_mark(ctx->ev[5], s));
    ctx->launches += 10;
    return cudaSuccess;
  };
  CK(graph_run(ctx,
               gkey("pre", L.total_pix, L.lvec, np, L.work_tex.size(), L.work_cue.size(), L.work16.size(),
                    repair_cap, ctx->tab.n_rings, blockm, ctx->prm.keep_intermediates, tx_var) +
                   gkey("", b.packed, b.grey, b.lab4, b.repair, b.repair_count, b.patches, b.work_tex, b.work_cue,
                        b.work16, b.nbins, b.mpbo, b.go, b.raw, b.counts, b.mpb, b.wup, b.deg, b.aup, b.adiag,
                        b.dis, b.wfull, b.afull, b.berr, ctx->d_ic, ctx->d_k32_ring, ctx->d_ring_of,
                        ctx->d_lab_lut),
               pre_chain, !tx_trial));
  // (d) eigensolver
  gpb_status es;
  if (warm) {
    es = solve_warm(ctx, L, Lc);
  } else if (ctx->prm.eig_mode == GPB_EIG_LEARNED) {
    es = solve_learned(ctx, L);
  } else if (ctx->prm.eig_mode == GPB_EIG_BLOCK) {
    Level lf = {&L, b.patches, b.tiles, b.tile_begin, b.tile_count, b.work_blk, b.afull, 0,
                {b.blk[0], b.blk[1], b.blk[2], b.blk[3]}};
    float* Xf = nullptr;
    es = solve_block(ctx, lf, false, ctx->prm.eig_tol, true, &Xf);
  } else {
    es = solve_lanczos(ctx, L);
  }
  if (es == GPB_ERR_NOCONV && ctx->prm.eig_mode != GPB_EIG_LANCZOS) {
    // the plain cold-start Lanczos solver is the fallback of the block
    // solvers: the whole batch again, its own residual test and cap
    ctx->stats.eig_fallback = 1;
    es = solve_lanczos(ctx, L);
  }
  if (es != GPB_OK && es != GPB_ERR_NOCONV) return es;
  if (ctx->prm.eig_mode != GPB_EIG_LANCZOS) {
    int berr = 0;
    CK(cudaMemcpyAsync(&berr, b.berr, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (berr) {
      ctx->last_error = "a block-step tile gave up waiting for its staged data";
      return GPB_ERR_TIMEOUT;
    }
  }
  CK(cudaEventRecord(ctx->ev[6], s));
  // (e) sPb + gPb, and the results to the pinned staging
  float* o_nmax = dev_nmax ? dev_nmax : b.nmax;
  float* o_orient = dev_orient ? dev_orient : b.orient;
  if (host_out) {
    const size_t need = 9 * (size_t)L.total_pix;
    if (ctx->c_hout < need) {
      if (ctx->h_out) cudaFreeHost(ctx->h_out);
      ctx->h_out = nullptr;
      ctx->c_hout = 0;
      CK(cudaMallocHost(&ctx->h_out, need * sizeof(float)));
      ctx->c_hout = need;
    }
  }
  auto post_chain = [&]() -> cudaError_t {
    cudaError_t e;
    GK(launch_minmax(b.patches, (int)np, b.evec, L.lvec, b.dis, ctx->prm.nvec, b.mm, s));
    GK(launch_spb(b.patches, b.work16, (int)L.work16.size(), b.evec, L.lvec, b.dis, b.evals, b.mm, ctx->prm.nvec,
                  b.go, b.mpb, ctx->prm.compat, ctx->prm.keep_intermediates ? b.spb : nullptr,
                  ctx->prm.keep_intermediates ? b.gpbo : nullptr, o_nmax, o_orient, s));
    ctx->launches += 2;
    GK(stage_mark(ctx->ev[7], s));
    if (host_out) {
      GK(cudaMemcpyAsync(ctx->h_out, o_nmax, L.total_pix * sizeof(float), cudaMemcpyDeviceToHost, s));
      GK(cudaMemcpyAsync(ctx->h_out + L.total_pix, o_orient, 8 * L.total_pix * sizeof(float),
                         cudaMemcpyDeviceToHost, s));
    }
    GK(stage_mark(ctx->ev[8], s));
    return cudaSuccess;
#undef GK
  };
  CK(graph_run(ctx,
               gkey("post", L.total_pix, L.lvec, np, L.work16.size(), ctx->prm.nvec, ctx->prm.compat,
                    ctx->prm.keep_intermediates, host_out != nullptr) +
                   gkey("", b.patches, b.evec, b.dis, b.mm, b.work16, b.evals, b.go, b.mpb, b.spb, b.gpbo, o_nmax,
                        o_orient, ctx->h_out),
               post_chain));
  CK(cudaStreamSynchronize(s));
  ctx->tuner.collect();
  if (host_out) {  // staging to the caller's buffers, on the host pool
    std::vector<CopyJob> jobs;
    for (size_t i = 0; i < n; i++) {
      const PatchDev& P = L.patches[i];
      gpb_result& r = host_out[i];
      if (!r.nmax) r.nmax = (float*)malloc((size_t)P.N * sizeof(float));
      if (!r.orient) r.orient = (float*)malloc(8 * (size_t)P.N * sizeof(float));
      if (!r.nmax || !r.orient) return GPB_ERR_NOMEM;
      jobs.push_back({r.nmax, ctx->h_out + P.pix, (size_t)P.N * sizeof(float)});
      jobs.push_back({r.orient, ctx->h_out + L.total_pix + 8 * P.pix, 8 * (size_t)P.N * sizeof(float)});
    }
    parallel_copy(ctx->host_pool(), jobs);
  }
  float ms[9];
  for (int i = 1; i <= 8; i++) cudaEventElapsedTime(&ms[i], ctx->ev[i - 1], ctx->ev[i]);
  ctx->stats.ms_h2d = ms[1];
  ctx->stats.ms_texton = ms[2];
  ctx->stats.ms_cues = ms[3];
  ctx->stats.ms_nms = ms[4];
  ctx->stats.ms_buildw = ms[5];
  ctx->stats.ms_eig = ms[6];
  ctx->stats.ms_spb = ms[7];
  ctx->stats.ms_d2h = ms[8];
  cudaEventElapsedTime(&ms[0], ctx->ev[0], ctx->ev[8]);
  ctx->stats.ms_total = ms[0];
  ctx->stats.gpu_launches = ctx->launches;
  int rc = 0;
  cudaMemcpy(&rc, b.repair_count, sizeof(int), cudaMemcpyDeviceToHost);
  ctx->stats.texton_repaired = rc;
  ctx->patches = L.patches;
  ctx->total_pix = L.total_pix;
  ctx->lvec = L.lvec;
  if (cudaGetLastError() != cudaSuccess) return GPB_ERR_CUDA;
  return es;
}

extern "C" gpb_status gpb_compute_batch(gpb_ctx* ctx, const gpb_patch* patches, size_t n, gpb_result* out) {
  return guarded(ctx, [&]() -> gpb_status {
    if (!ctx || !patches || !out || n == 0) return GPB_ERR_ARG;
    std::vector<uint32_t> ws(n), hs(n);
    std::vector<const uint32_t*> in(n);
    std::vector<size_t> stride(n);
    for (size_t i = 0; i < n; i++) {
      if (!patches[i].packed_bgr) return GPB_ERR_ARG;
      ws[i] = patches[i].width;
      hs[i] = patches[i].height;
      in[i] = patches[i].packed_bgr;
      stride[i] = patches[i].stride ? patches[i].stride : patches[i].width;
    }
    return run_batch(ctx, n, ws.data(), hs.data(), in.data(), stride.data(), nullptr, nullptr, nullptr, nullptr,
                     out);
  });
}

extern "C" gpb_status gpb_compute(gpb_ctx* ctx, uint32_t width, uint32_t height, const uint32_t* packed,
                                  float** out_nmax, float** out_orient) {
  if (!ctx || !packed || !out_nmax || !out_orient) return GPB_ERR_ARG;
  gpb_patch p = {width, height, packed, width};
  gpb_result r = {nullptr, nullptr};
  gpb_status s = gpb_compute_batch(ctx, &p, 1, &r);
  if (s != GPB_OK && s != GPB_ERR_NOCONV) {
    free(r.nmax);
    free(r.orient);
    return s;
  }
  *out_nmax = r.nmax;
  *out_orient = r.orient;
  return s;
}

extern "C" gpb_status gpb_compute_batch_device(gpb_ctx* ctx, size_t n, const uint32_t* widths,
                                               const uint32_t* heights, const size_t* offsets,
                                               const uint32_t* d_packed, float* d_nmax, float* d_orient) {
  return guarded(ctx, [&]() -> gpb_status {
    if (!ctx || !widths || !heights || !offsets || !d_packed || !d_nmax || !d_orient || n == 0) return GPB_ERR_ARG;
    // outputs are written in the library's compact layout, then moved to the
    // caller's offsets when they differ
    gpb_status s = run_batch(ctx, n, widths, heights, nullptr, nullptr, d_packed, offsets, nullptr, nullptr, nullptr);
    if (s != GPB_OK && s != GPB_ERR_NOCONV) return s;
    for (size_t i = 0; i < n; i++) {
      const PatchDev& P = ctx->patches[i];
      CK(cudaMemcpyAsync(d_nmax + offsets[i], ctx->b.nmax + P.pix, (size_t)P.N * sizeof(float),
                         cudaMemcpyDeviceToDevice, ctx->st));
      CK(cudaMemcpyAsync(d_orient + 8 * offsets[i], ctx->b.orient + 8 * P.pix, 8 * (size_t)P.N * sizeof(float),
                         cudaMemcpyDeviceToDevice, ctx->st));
    }
    CK(cudaStreamSynchronize(ctx->st));
    return s;
  });
}

extern "C" gpb_status gpb_last_stats(gpb_ctx* ctx, gpb_stats* st) {
  if (!ctx || !st) return GPB_ERR_ARG;
  *st = ctx->stats;
  return GPB_OK;
}

extern "C" gpb_status gpb_fetch(gpb_ctx* ctx, int stage, size_t patch, void* dst, size_t bytes) {
  return guarded(ctx, [&]() -> gpb_status {
    if (!ctx || !dst || patch >= ctx->patches.size()) return GPB_ERR_ARG;
    cudaSetDevice(ctx->device);
    const PatchDev& P = ctx->patches[patch];
    const size_t N = P.N;
    Buf& b = ctx->b;
    const int nvec = ctx->prm.nvec;
    auto need = [&](size_t x) { return bytes >= x; };
    cudaError_t e = cudaSuccess;
    switch (stage) {
      case GPB_STAGE_TEXTON:
      case GPB_STAGE_LABBINS: {
        std::vector<uint32_t> v(N);
        e = cudaMemcpy(v.data(), b.lab4 + P.pix, N * 4, cudaMemcpyDeviceToHost);
        uint8_t* o = (uint8_t*)dst;
        if (stage == GPB_STAGE_TEXTON) {
          if (!need(N)) return GPB_ERR_ARG;
          for (size_t i = 0; i < N; i++) o[i] = (uint8_t)(v[i] >> 24);
        } else {
          if (!need(3 * N)) return GPB_ERR_ARG;
          for (int c = 0; c < 3; c++)
            for (size_t i = 0; i < N; i++) o[c * N + i] = (uint8_t)((v[i] >> (8 * c)) & 255);
        }
        break;
      }
      case GPB_STAGE_MPB_O:
        if (!need(8 * N * 4)) return GPB_ERR_ARG;
        e = cudaMemcpy(dst, b.mpbo + 8 * P.pix, 8 * N * 4, cudaMemcpyDeviceToHost);
        break;
      case GPB_STAGE_MPB:
        if (!need(N * 4)) return GPB_ERR_ARG;
        e = cudaMemcpy(dst, b.mpb + P.pix, N * 4, cudaMemcpyDeviceToHost);
        break;
      case GPB_STAGE_DEG:
        if (!need(N * 4)) return GPB_ERR_ARG;
        e = cudaMemcpy(dst, b.deg + P.vec, N * 4, cudaMemcpyDeviceToHost);
        break;
      case GPB_STAGE_W:
        if (!b.wfull || !need(81 * N * 4)) return GPB_ERR_ARG;
        e = cudaMemcpy(dst, b.wfull + 81 * P.pix, 81 * N * 4, cudaMemcpyDeviceToHost);
        break;
      case GPB_STAGE_EVALS:
        if (!need((size_t)nvec * 4) || ctx->evals_host.size() < (patch + 1) * nvec) return GPB_ERR_ARG;
        memcpy(dst, ctx->evals_host.data() + patch * nvec, (size_t)nvec * 4);
        break;
      case GPB_STAGE_EVECS:
        if (!need((size_t)nvec * N * 4)) return GPB_ERR_ARG;
        for (int i = 0; i < nvec && e == cudaSuccess; i++)
          e = cudaMemcpy((float*)dst + i * N, b.evec + (size_t)i * ctx->lvec + P.vec, N * 4, cudaMemcpyDeviceToHost);
        break;
      case GPB_STAGE_SPB:
        if (!b.spb || !need(8 * N * 4)) return GPB_ERR_ARG;
        e = cudaMemcpy(dst, b.spb + 8 * P.pix, 8 * N * 4, cudaMemcpyDeviceToHost);
        break;
      case GPB_STAGE_CUES:
        if (!b.raw || !need(96 * N * 4)) return GPB_ERR_ARG;
        e = cudaMemcpy(dst, b.raw + 96 * P.pix, 96 * N * 4, cudaMemcpyDeviceToHost);
        break;
      case GPB_STAGE_GPB_O:
        if (!b.gpbo || !need(8 * N * 4)) return GPB_ERR_ARG;
        e = cudaMemcpy(dst, b.gpbo + 8 * P.pix, 8 * N * 4, cudaMemcpyDeviceToHost);
        break;
      case GPB_STAGE_WARM0: {  // first 9 columns of the captured start block, pixel-major
        if (!ctx->d_wn_x0 || !need(N * kWnOut * 4)) return GPB_ERR_ARG;
        std::vector<float> blk(N * kBlk);
        e = cudaMemcpy(blk.data(), ctx->d_wn_x0 + (size_t)P.vec * kBlk, N * kBlk * 4, cudaMemcpyDeviceToHost);
        float* o = (float*)dst;
        for (size_t i = 0; i < N; i++)
          for (int c = 0; c < kWnOut; c++) o[i * kWnOut + c] = blk[i * kBlk + c];
        break;
      }
      case GPB_STAGE_COUNTS: {
        const size_t per = (size_t)kNannulus * 4 * 32 * 32;
        if (!b.counts || !need(per * N)) return GPB_ERR_ARG;
        e = cudaMemcpy(dst, b.counts + per * P.pix, per * N, cudaMemcpyDeviceToHost);
        break;
      }
      default:
        return GPB_ERR_ARG;
    }
    return e == cudaSuccess ? GPB_OK : GPB_ERR_CUDA;
  });
}

// Whole-image planes from the last batch's patches (Pieces2Gpb,
// src/utilities.cpp:180-213, on the device)
extern "C" gpb_status gpb_stitch_device(gpb_ctx* ctx, int mode, uint32_t width, uint32_t height,
                                        const gpb_place* places, size_t n, int ramp, float* d_nmax,
                                        float* d_orient) {
  return guarded(ctx, [&]() -> gpb_status {
    if (!ctx || !places || !d_nmax || !d_orient || width == 0 || height == 0) return GPB_ERR_ARG;
    if (mode < GPB_STITCH_LAST || mode > GPB_STITCH_BLEND) return GPB_ERR_ARG;
    if (n == 0 || n != ctx->patches.size()) {
      ctx->last_error = "place count differs from the last batch";
      return GPB_ERR_ARG;
    }
    for (size_t i = 0; i < n; i++) {
      const gpb_place& q = places[i];
      const PatchDev& P = ctx->patches[i];
      if (q.ix < 0 || q.iy < 0 || q.iw < 0 || q.ih < 0 || q.ix + q.iw > P.W || q.iy + q.ih > P.H) return GPB_ERR_ARG;
    }
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->st;
    Buf& b = ctx->b;
    const int colmajor = ctx->prm.compat == GPB_COMPAT_DAMASCENE;
    const long long plane = (long long)width * height;
    if (mode == GPB_STITCH_BLEND) {
      CK(grow(b.stitch, b.c_stitch, 10 * (size_t)plane));
      CK(cudaMemsetAsync(b.stitch, 0, 10 * (size_t)plane * sizeof(float), s));
    }
    const float rmp = (float)(ramp > 0 ? ramp : 10);
    for (size_t i = 0; i < n; i++) {
      const gpb_place& q = places[i];
      const PatchDev& P = ctx->patches[i];
      StitchBox bx;
      bx.ox = q.x0;
      bx.oy = q.y0;
      if (mode == GPB_STITCH_INTERIOR) {
        bx.x = q.ix;
        bx.y = q.iy;
        bx.w = q.iw;
        bx.h = q.ih;
      } else {
        bx.x = 0;
        bx.y = 0;
        bx.w = P.W;
        bx.h = P.H;
      }
      if (mode == GPB_STITCH_BLEND)
        CK(launch_stitch_acc(b.patches, (int)i, P.N, b.nmax, b.orient, colmajor, bx, (int)width, (int)height, rmp,
                             b.stitch, s));
      else
        CK(launch_stitch_copy(b.patches, (int)i, b.nmax, b.orient, colmajor, bx, (int)width, (int)height, d_nmax,
                              d_orient, s));
    }
    if (mode == GPB_STITCH_BLEND) CK(launch_stitch_norm(b.stitch, plane, d_nmax, d_orient, s));
    CK(cudaStreamSynchronize(s));
    return GPB_OK;
  });
}

// Superpixel descriptors of one patch of the last batch (SPFeatures,
// src/SPFeatures.cpp:101-114, 260-275, 380-391, on the device)
extern "C" gpb_status gpb_superpixel_features(gpb_ctx* ctx, size_t patch, const int32_t* d_labels, int32_t n_labels,
                                              int bin_step, int with_textons, double* d_out) {
  return guarded(ctx, [&]() -> gpb_status {
    if (!ctx || !d_labels || !d_out || n_labels <= 0 || bin_step < 1 || bin_step > 255) return GPB_ERR_ARG;
    if (patch >= ctx->patches.size()) return GPB_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->st;
    Buf& b = ctx->b;
    const int K = with_textons ? ctx->K : 0, nbins = 255 / bin_step + 1;
    CK(grow(b.spcount, b.c_spcount, (size_t)n_labels * (K + nbins + 1)));
    CK(grow(b.spcsum, b.c_spcsum, (size_t)n_labels * 3));
    CK(launch_sp_features(b.patches, (int)patch, ctx->patches[patch].N, d_labels, n_labels, b.lab4, b.grey, b.packed,
                          bin_step, K, nbins, b.spcount, b.spcsum, d_out, s));
    CK(cudaStreamSynchronize(s));
    return GPB_OK;
  });
}

// Texton labels of one device-resident image without allocating: the
// kernels of the batch pipeline's texton stage on the fixed scratch area of
// k_static.cu.  No counterpart in the reference.  Nothing here allocates,
// on the device or the host (no error strings either: the status says it).
extern "C" gpb_status gpb_texton_labels_static(gpb_ctx* ctx, uint32_t width, uint32_t height,
                                               const uint32_t* d_packed, uint32_t* d_labels, void* stream) {
  if (!ctx) return GPB_ERR_ARG;
  return guarded(ctx, [&]() -> gpb_status {
    if (!d_packed || !d_labels || (((uintptr_t)d_packed | (uintptr_t)d_labels) & 3u) || ctx->K == 0 ||
        width < (uint32_t)kMinSide || height < (uint32_t)kMinSide)
      return GPB_ERR_ARG;
    const long long N = (long long)width * height;
    const long long tiles = (long long)((width + 15) / 16) * ((height + 15) / 16);
    if (N > kStaticMaxPix || tiles > kStaticMaxTiles) return GPB_ERR_TOO_LARGE;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->st;
    ConstBank& bk = bank_of(ctx->device);
    std::lock_guard<std::mutex> lk(bk.mu);
    if (bk.owner != ctx->token) {  // this context's codebook into the constant bank first
      CK(load_tables(ctx));
      CK(cudaStreamSynchronize(ctx->st));
    }
    CK(launch_texton_static(d_packed, (int)width, (int)height, d_labels, ctx->d_k32_ring, ctx->d_ring_of,
                            ctx->tab.n_rings, s));
    if (bk.static_done) {  // a later reload of the tables waits for these kernels
      CK(cudaEventRecord(bk.static_done, s));
      bk.static_pending = true;
    }
    return GPB_OK;
  });
}

extern "C" size_t gpb_learned_nparams(void) { return ln_nparams(); }

static LearnedNet& net_of(gpb_ctx* ctx) {
  if (!ctx->net) ctx->net.reset(new LearnedNet());
  return *ctx->net;
}

extern "C" gpb_status gpb_learned_set(gpb_ctx* ctx, const float* params, size_t n) {
  if (!ctx) return GPB_ERR_ARG;
  return guarded(ctx, [&]() -> gpb_status {
    CK(cudaSetDevice(ctx->device));
    if (!params) {
      CK(cudaStreamSynchronize(ctx->st));
      ctx->net.reset();
      return GPB_OK;
    }
    if (n != ln_nparams()) return GPB_ERR_ARG;
    CK(net_of(ctx).set_params(params, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return GPB_OK;
  });
}

extern "C" gpb_status gpb_learned_get(gpb_ctx* ctx, float* params, size_t n) {
  if (!ctx || !params || n != ln_nparams()) return GPB_ERR_ARG;
  return guarded(ctx, [&]() -> gpb_status {
    if (!ctx->net || !ctx->net->has_params()) return GPB_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    CK(ctx->net->get_params(params, ctx->st));
    return GPB_OK;
  });
}

static gpb_status learned_layout(gpb_ctx* ctx, size_t n, const uint32_t* widths, const uint32_t* heights) {
  if (!ctx->net || !ctx->net->has_params() || n == 0 || !widths || !heights) return GPB_ERR_ARG;
  std::vector<int> H(n), W(n);
  for (size_t i = 0; i < n; i++) {
    if (widths[i] < 1 || heights[i] < 1 || widths[i] > 8192 || heights[i] > 8192) return GPB_ERR_ARG;
    H[i] = (int)heights[i];
    W[i] = (int)widths[i];
  }
  CK(cudaSetDevice(ctx->device));
  CK(ctx->net->layout(H, W, ctx->st));
  return GPB_OK;
}

extern "C" gpb_status gpb_learned_forward_device(gpb_ctx* ctx, size_t n, const uint32_t* widths,
                                                 const uint32_t* heights, const float* d_mpb, const float* d_deg,
                                                 float* d_y) {
  if (!ctx || !d_mpb || !d_deg || !d_y) return GPB_ERR_ARG;
  return guarded(ctx, [&]() -> gpb_status {
    gpb_status st = learned_layout(ctx, n, widths, heights);
    if (st != GPB_OK) return st;
    cudaStream_t s = ctx->st;
    CK(ctx->net->features(d_mpb, d_deg, s));
    CK(ctx->net->forward(s));
    CK(cudaMemcpyAsync(d_y, ctx->net->y(), (size_t)ctx->net->npix0() * kLnOut * sizeof(float),
                       cudaMemcpyDeviceToDevice, s));
    CK(cudaStreamSynchronize(s));
    return GPB_OK;
  });
}

extern "C" gpb_status gpb_learned_grad_device(gpb_ctx* ctx, size_t n, const uint32_t* widths, const uint32_t* heights,
                                              const float* d_mpb, const float* d_deg, const float* d_v, double* loss,
                                              float* grad) {
  if (!ctx || !d_mpb || !d_deg || !d_v || !loss || !grad) return GPB_ERR_ARG;
  return guarded(ctx, [&]() -> gpb_status {
    gpb_status st = learned_layout(ctx, n, widths, heights);
    if (st != GPB_OK) return st;
    cudaStream_t s = ctx->st;
    CK(ctx->net->features(d_mpb, d_deg, s));
    CK(ctx->net->forward(s));
    CK(ctx->net->loss_backward(d_v, loss, s));
    CK(cudaMemcpyAsync(grad, ctx->net->grad(), ln_nparams() * sizeof(float), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return GPB_OK;
  });
}

extern "C" gpb_status gpb_learned_train_device(gpb_ctx* ctx, size_t n, const uint32_t* widths,
                                               const uint32_t* heights, const float* d_mpb, const float* d_deg,
                                               const float* d_v, int batch, int epochs, float lr, uint64_t seed,
                                               double* loss_per_epoch) {
  if (!ctx || !d_mpb || !d_deg || !d_v || !widths || !heights || n == 0 || batch < 1 || epochs < 1 || !(lr > 0))
    return GPB_ERR_ARG;
  return guarded(ctx, [&]() -> gpb_status {
    if (!ctx->net || !ctx->net->has_params()) return GPB_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->st;
    std::vector<long long> off(n + 1, 0);
    for (size_t i = 0; i < n; i++) off[i + 1] = off[i] + (long long)widths[i] * heights[i];
    // staging of one minibatch: mPb, degree and targets, back to back
    long long most = 0;
    {
      std::vector<long long> sz(n);
      for (size_t i = 0; i < n; i++) sz[i] = off[i + 1] - off[i];
      std::sort(sz.begin(), sz.end(), std::greater<long long>());
      for (int i = 0; i < batch && i < (int)n; i++) most += sz[i];
    }
    CK(grow(ctx->d_tr, ctx->c_tr, (size_t)most * (2 + kLnTargets)));
    std::vector<int> order(n);
    for (size_t i = 0; i < n; i++) order[i] = (int)i;
    uint64_t rs = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    auto rnd = [&]() {
      rs = rs * 6364136223846793005ULL + 1442695040888963407ULL;
      return (uint32_t)(rs >> 33);
    };
    int t = 0;
    for (int ep = 0; ep < epochs; ep++) {
      for (size_t i = n - 1; i > 0; i--) std::swap(order[i], order[rnd() % (i + 1)]);
      double ep_loss = 0;
      for (size_t b0 = 0; b0 < n; b0 += batch) {
        const size_t nb = std::min(n - b0, (size_t)batch);
        std::vector<uint32_t> bw(nb), bh(nb);
        long long tot = 0;
        for (size_t k = 0; k < nb; k++) tot += off[order[b0 + k] + 1] - off[order[b0 + k]];
        float* m_mpb = ctx->d_tr;
        float* m_deg = m_mpb + tot;
        float* m_v = m_deg + tot;
        long long at = 0;
        for (size_t k = 0; k < nb; k++) {
          const int i = order[b0 + k];
          const long long N = off[i + 1] - off[i];
          bw[k] = widths[i];
          bh[k] = heights[i];
          CK(cudaMemcpyAsync(m_mpb + at, d_mpb + off[i], N * sizeof(float), cudaMemcpyDeviceToDevice, s));
          CK(cudaMemcpyAsync(m_deg + at, d_deg + off[i], N * sizeof(float), cudaMemcpyDeviceToDevice, s));
          CK(cudaMemcpyAsync(m_v + at * kLnTargets, d_v + off[i] * kLnTargets, N * kLnTargets * sizeof(float),
                             cudaMemcpyDeviceToDevice, s));
          at += N;
        }
        gpb_status st = learned_layout(ctx, nb, bw.data(), bh.data());
        if (st != GPB_OK) return st;
        double l = 0;
        CK(ctx->net->features(m_mpb, m_deg, s));
        CK(ctx->net->forward(s));
        CK(ctx->net->loss_backward(m_v, &l, s));
        CK(ctx->net->adam(lr, 0.9f, 0.999f, 1e-8f, ++t, s));
        ep_loss += l;
      }
      if (loss_per_epoch) loss_per_epoch[ep] = ep_loss / (double)n;
    }
    CK(cudaStreamSynchronize(s));
    return GPB_OK;
  });
}

extern "C" size_t gpb_tuning_report(gpb_ctx* ctx, char* buf, size_t n) {
  if (!ctx) return 0;
  try {
    const std::string r = ctx->tuner.report();
    if (buf && n) {
      const size_t m = std::min(n - 1, r.size());
      memcpy(buf, r.data(), m);
      buf[m] = 0;
    }
    return r.size();
  } catch (...) {
    return 0;
  }
}

// Accessors for the stages compiled in other translation units.
namespace gpb {
int ctx_device(gpb_ctx* c) { return c->device; }
cudaStream_t ctx_stream(gpb_ctx* c) { return c->st; }
void ctx_set_error(gpb_ctx* c, const char* m) {
  try {
    c->last_error = m;
  } catch (...) {  // the message is lost, the status still tells
  }
}
void ctx_parallel_for(gpb_ctx* c, int n, const std::function<void(int)>& f) { c->host_pool().run(n, f); }
void*& ctx_ucm_state(gpb_ctx* c, void (*release)(void*)) {
  c->ucm_free = release;
  return c->ucm_state;
}
}  // namespace gpb

extern "C" gpb_status gpb_warmnet_set(gpb_ctx* ctx, const float* weights, size_t n) {
  if (!ctx) return GPB_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  if (!weights) {
    cudaFree(ctx->d_wn);
    ctx->d_wn = nullptr;
    return GPB_OK;
  }
  if (n != (size_t)kWnParams) return GPB_ERR_ARG;
  if (!ctx->d_wn) CK(cudaMalloc(&ctx->d_wn, kWnParams * sizeof(float)));
  CK(cudaMemcpy(ctx->d_wn, weights, kWnParams * sizeof(float), cudaMemcpyHostToDevice));
  return GPB_OK;
}

extern "C" gpb_status gpb_warmnet_capture(gpb_ctx* ctx, int on) {
  if (!ctx) return GPB_ERR_ARG;
  ctx->wn_capture = on != 0;
  return GPB_OK;
}

extern "C" gpb_status gpb_warmnet_grad_device(gpb_ctx* ctx, size_t n, const uint32_t* widths, const uint32_t* heights,
                                              const float* d_xt, const float* d_mpb, const float* d_vt,
                                              const float* weights, double* loss, float* grad) {
  return guarded(ctx, [&]() -> gpb_status {
    if (!ctx || n == 0 || !widths || !heights || !d_xt || !d_mpb || !d_vt || !weights || !loss || !grad)
      return GPB_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->st;
    std::vector<int4> geo(n);
    long long tot = 0;
    int max_n = 0;
    for (size_t i = 0; i < n; i++) {
      if (widths[i] == 0 || heights[i] == 0) return GPB_ERR_ARG;
      geo[i] = make_int4((int)widths[i], (int)heights[i], (int)tot, 0);
      tot += (long long)widths[i] * heights[i];
      max_n = std::max(max_n, (int)(widths[i] * heights[i]));
    }
    if (tot >= (1ll << 31)) return GPB_ERR_ARG;
    void* buf = nullptr;
    const size_t bytes = n * sizeof(int4) + kWnParams * 2 * sizeof(float) + sizeof(double);
    CK(cudaMalloc(&buf, bytes));
    int4* d_geo = (int4*)buf;
    float* d_w = (float*)(d_geo + n);
    float* d_g = d_w + kWnParams;
    double* d_l = (double*)(((uintptr_t)(d_g + kWnParams) + 7) & ~(uintptr_t)7);
    cudaError_t e = cudaMemcpyAsync(d_geo, geo.data(), n * sizeof(int4), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_w, weights, kWnParams * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_g, 0, kWnParams * sizeof(float), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_l, 0, sizeof(double), s);
    if (e == cudaSuccess)
      e = wn_launch_grad(d_geo, (int)n, max_n, d_xt, d_mpb, d_vt, d_w, 1.0f / (float)(tot * kWnOut), d_g, d_l, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(grad, d_g, kWnParams * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(loss, d_l, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(buf);
    if (e != cudaSuccess) {
      ctx->last_error = cudaGetErrorString(e);
      return GPB_ERR_CUDA;
    }
    return GPB_OK;
  });
}
