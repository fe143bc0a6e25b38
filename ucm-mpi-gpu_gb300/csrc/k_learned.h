// k_learned.h -- the learned warm start: a 4-level convolutional
// encoder-decoder, BF16 on the tensor cores with FP32 accumulation, that maps
// a patch's mPb and affinity degree to 32 fields starting the block
// eigensolver, with its own training kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <vector>

#include "gpb_internal.h"

namespace gpb {

constexpr int kLnIn = 16, kLnOut = 32, kLnConvs = 15, kLnLevels = 4, kLnTargets = 9;

// one patch at one level: its size and its first pixel in the level's tensors
struct LnPatch {
  int H, W;
  long long off;
};
// an 8 x 16 output tile of a patch at one level
struct LnTile {
  int patch, y0, x0, pad;
};

// (cin, cout, relu) of the 15 convolutions, in parameter order:
// e0a e0b e1a e1b e2a e2b e3a e3b d2a d2b d1a d1b d0a d0b head
struct LnConv {
  int cin, cout, relu;
};
extern const LnConv kLnNet[kLnConvs];
size_t ln_nparams();

class LearnedNet {
 public:
  LearnedNet();
  ~LearnedNet();
  // the FP32 master weights (BF16 and transposed BF16 copies are derived)
  cudaError_t set_params(const float* host_params, cudaStream_t s);
  cudaError_t get_params(float* host_params, cudaStream_t s);
  bool has_params() const;
  // the patches' full-resolution sizes; builds the four levels' layouts
  cudaError_t layout(const std::vector<int>& H, const std::vector<int>& W, cudaStream_t s);
  const std::vector<LnPatch>& patches0() const;
  const LnPatch* patches0_dev() const;
  long long npix0() const;
  // mPb and degree, each H*W per patch back to back at the level-0 offsets
  cudaError_t features(const float* d_mpb, const float* d_deg, cudaStream_t s);
  // the same from the pipeline's buffers: mPb at each patch's pixel offset,
  // degree at its vector offset
  cudaError_t features_from(const PatchDev* patches, const float* d_mpb, const float* d_deg, cudaStream_t s);
  // forward pass; the 32 fields land in y() (FP32, [pixel][32], level-0 offsets)
  cudaError_t forward(cudaStream_t s);
  float* y();
  // the subspace loss of y() against the 9 orthonormal target fields of each
  // patch (d_v: [pixel][9] FP32 at the level-0 offsets), and the gradient of
  // every parameter into grad() (FP32, parameter layout); *loss gets the sum
  // over the patches.  Synchronises the stream once.
  cudaError_t loss_backward(const float* d_v, double* loss, cudaStream_t s);
  float* grad();
  // one Adam step of the master weights with grad(); t counts from 1
  cudaError_t adam(float lr, float b1, float b2, float eps, int t, cudaStream_t s);
  int launches() const;

 private:
  struct Impl;
  std::unique_ptr<Impl> im_;
};

// The block solver's pixel-major [vec][32] start block X from the net's
// fields y (level-0 layout), with a small seeded perturbation per pixel
// relative to its own magnitude, so no column of the block is zero.
cudaError_t ln_launch_start(const LnPatch* lp, const PatchDev* patches, int npatch, int maxN, const float* y,
                            float* X, cudaStream_t s);

}  // namespace gpb
