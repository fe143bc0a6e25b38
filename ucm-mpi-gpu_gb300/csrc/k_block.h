// k_block.h -- block (Chebyshev-filtered subspace iteration) kernels.
#pragma once

#include <cuda_runtime.h>

#include "gpb_internal.h"
#include "k_eig.h"

namespace gpb {

constexpr int kBlk = 32;          // block width
constexpr int kBlkThreads = 256;  // 64 pixels x 4 quarters per pass
constexpr int kMaxCheb = 128;     // largest filter degree

struct BlkArgs {
  const PatchDev* patches;
  const EigTile* tiles;
  const int* tile_begin;
  const int* tile_count;
  const float* a_up;
  const float* a_diag;
  long long lvec;
  const float3* coef;   // [npatch][max_steps] (alpha, beta, gamma)
  int max_steps;
  double* part;         // [ntiles][32*32]
  int* counter;         // [npatch]
  const int* active;    // [npatch]
  const int* done;      // [npatch]
  const double* mat;    // [npatch][32*32]
  const double* theta;  // [npatch][32]
  int coarse;           // 0: fine radius-5 disk, 1: coarse 7 x 7 square
  const float* afull;   // pixel-major stencil rows: 84 floats (fine) / 52 (coarse)
  int* err;             // set to 1 when a tile's staging wait gave up
  int* queue;           // [2]: the block step's next tile ticket and finished-CTA
                        // count; zero between launches (the last CTA resets them)
};

// coarse level (2 x 2 aggregation)
constexpr int kCR = 3, kCW = 2 * kCR + 1, kCN = kCW * kCW;
struct CoarseArgs {
  const PatchDev* fine;
  const PatchDev* coarse;
  const int4* work;      // coarse 16 x 16 tiles
  const int4* work_f;    // fine 16 x 16 tiles
  const float* wsym_up;  // fine symmetric affinities (upper offsets)
  const float* deg;      // fine degrees
  long long lvec_f, lvec_c;
  float* wc;             // [lvec_c][kCoarseNC] pixel-major: W_c, then A_c
  float* degc;
  float* disc;
};
cudaError_t cf_launch_coarsen(const CoarseArgs& c, int nwork_c, cudaStream_t s);
cudaError_t cf_launch_full(const PatchDev* patches, const int4* work16, int nwork, const float* a_up,
                           const float* a_diag, long long lvec, float* afull, cudaStream_t s);
cudaError_t cf_launch_prolong(const CoarseArgs& c, int nwork_f, const float* xc, float* xf, cudaStream_t s);

void upload_block(const HostTables& t, cudaStream_t s);
constexpr int kStepTileH = 8, kStepTileW = 16;  // cf_step tile (work list entries)
constexpr int kFullNC = 84, kCoarseNC = 52;      // floats per pixel-major stencil row
constexpr int kBlkSplit = 4;  // CTAs per eigensolver tile in cf_gram / cf_rotate / cf_resid
// variant (bit-identical results, chosen by the autotuner): bit 0 stages X
// through shared memory, bit 1 takes tiles from the device work queue
constexpr int kStepVariants = 4, kStepDefault = 1;  // default (untuned): X staged, static tiles
cudaError_t cf_launch_step(const BlkArgs& a, const int4* work, int nwork, const float* Y, const float* X, float* out,
                           int step, cudaStream_t s, bool comp = false, int variant = kStepDefault);
// out = U^T V per patch; with out2, out2 = U^T U in the same pass
cudaError_t cf_launch_gram(const BlkArgs& a, int ntiles, const float* U, const float* V, double* out,
                           cudaStream_t s, double* out2 = nullptr);
cudaError_t cf_launch_rotate(const BlkArgs& a, int ntiles, float* U, float* V, int ncols, cudaStream_t s,
                             bool comp = false);
cudaError_t cf_launch_resid(const BlkArgs& a, int ntiles, const float* X, const float* AX, double* out,
                            cudaStream_t s);
cudaError_t cf_launch_extract(const BlkArgs& a, int ntiles, const float* X, float* evec, int nvec,
                              cudaStream_t s);
cudaError_t cf_launch_init(const BlkArgs& a, int ntiles, float* X, cudaStream_t s);

}  // namespace gpb
