// gpb_internal.h -- shared host/device definitions of libgpb.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <new>
#include <vector>

#include "../../include/gpb.h"

struct gpb_ctx;

namespace gpb {

constexpr int kNori = 8;
constexpr int kNcue = 12;
constexpr int kNschmid = 13;
constexpr int kSchmidHalf = 24;          // 49 x 49 S filters
constexpr int kSchmidGroups = 325;       // (a, b), 0 <= a <= b <= 24
constexpr int kMaxCodewords = 32;
constexpr int kStencilR = 5;
constexpr int kStencilN = 81;            // radius-5 disc
constexpr int kUpper = 40;               // strictly upper offsets (k = 41..80)
constexpr int kCueBorder = 30;           // mirror border of the local cues
constexpr int kMaxRadius = 20;           // largest half-disc radius
constexpr int kNannulus = 4;             // r <= 3, 5, 10, 20
constexpr int kMaxBins = 32;
constexpr int kMinSide = 32;
constexpr int kIcConfigs = 6 * 6 * 6 * 6;
constexpr int kIcMaxPath = 24;
constexpr int kMaxNvec = 16;

// one patch of a batch, as the kernels see it
struct PatchDev {
  int W, H, N;
  int nb[4];        // histogram lengths (max label + 1) of L, a, b, texton
  long long pix;    // offset into compact per-pixel arrays
  long long vec;    // offset of pixel 0 in padded vector arrays
};

// IC path table entry: the mPb pixels whose max is the intervening contour
// from the centre to one stencil offset (count < 0: the reference finds no
// path and uses icsim = 0, i.e. maxpb = 1)
struct IcPath {
  int8_t count;
  int8_t dy[kIcMaxPath];
  int8_t dx[kIcMaxPath];
};

struct HostTables {
  // stencil
  int sdy[kStencilN], sdx[kStencilN];
  // Schmid
  float k32_group[kNschmid][kSchmidGroups];
  int group_a[kSchmidGroups], group_b[kSchmidGroups];
  int group_ring[kSchmidGroups];
  int n_rings;
  std::vector<double> k32_ring;  // [13][n_rings]
  float err_bound[kNschmid];     // FP32 response error bound per filter
  // colour
  double gamma_lut[256];
  // local cues
  float kbg[17];
  int nkbg;
  float kcg[9];
  int nkcg;
  // annulus offset lists: for annulus a and lane l (half = l / 16, slice = l % 16)
  std::vector<int16_t> ann_dy, ann_dx;   // concatenated
  int ann_start[kNannulus][32];
  int ann_count[kNannulus][32];
  int slice_pixels[kNannulus][16];       // cumulative per radius
  // weights
  float w_mpb[kNcue], w_g[kNcue], w_spb;
  // NMS
  int nms_nb[kNori][4][2];    // (drow, dcol) of neighbours 0a, 0b, 1a, 1b
  float nms_d[kNori];
  float nms_cos[kNori][kNori];
  // IC
  std::vector<IcPath> ic;     // [config][81]
  // sPb filters
  float oe[kNori][49];
  int ch_per[kNori];
};

void build_tables(HostTables& t, int compat);
int slice_of(int drow, int dcol);
void oe_filter(double theta, double* out49);

// kernel launchers (defined in the .cu files); all return cudaError_t of the launch
struct DevTables;

// context accessors for stages in other translation units (gpb_api.cpp)
int ctx_device(gpb_ctx* c);
cudaStream_t ctx_stream(gpb_ctx* c);
void ctx_set_error(gpb_ctx* c, const char* m);
void*& ctx_ucm_state(gpb_ctx* c, void (*release)(void*));
void ctx_parallel_for(gpb_ctx* c, int n, const std::function<void(int)>& f);  // f(0..n-1) on the host pool

// Runs an entry point's body.  A host exception (an allocation that failed,
// a thread that could not start) ends the call with a status and a message
// on the context instead of leaving the C ABI.
template <class F>
gpb_status guarded(gpb_ctx* ctx, F&& body) noexcept {
  const char* what;
  gpb_status s;
  try {
    return body();
  } catch (const std::bad_alloc&) {
    what = "host allocation failed";
    s = GPB_ERR_NOMEM;
  } catch (...) {
    what = "host exception";
    s = GPB_ERR_INTERNAL;
  }
  if (ctx) ctx_set_error(ctx, what);
  return s;
}

}  // namespace gpb
