// k_warmnet.h -- the learned correction of the warm-start block (k_warmnet.cu).
#pragma once
#include <cuda_runtime.h>

#include "gpb_internal.h"

namespace gpb {

constexpr int kWnIn = 10;   // 9 start columns + mPb
constexpr int kWnHid = 16;  // hidden channels
constexpr int kWnOut = 9;   // corrected columns
// W1 [16][10][9], b1 [16], W2 [9][16], b2 [9]
constexpr int kWnParams = kWnHid * kWnIn * 9 + kWnHid + kWnOut * kWnHid + kWnOut;

// block X (pixel-major, 32 columns) -> Y with its first 9 columns refined; scale: npatch x 9 scratch
cudaError_t wn_launch_apply(const PatchDev* patches, int npatch, int max_n, const float* X, const float* mpb,
                            const float* w, float* scale, float* Y, cudaStream_t s);
// geo: per patch (W, H, first pixel, 0); adds the gradient into grad and the loss into *loss
cudaError_t wn_launch_grad(const int4* geo, int npatch, int max_n, const float* xt, const float* mpb, const float* vt,
                           const float* w, float inv_n, float* grad, double* loss, cudaStream_t s);

}  // namespace gpb
