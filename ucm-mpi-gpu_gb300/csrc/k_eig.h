// k_eig.h -- shared definitions of the eigensolver kernels.
#pragma once

#include <cuda_runtime.h>

#include "gpb_internal.h"

namespace gpb {

constexpr int kEigThreads = 256;
constexpr int kEigWarps = kEigThreads / 32;
constexpr int kEigPix = 8;                          // pixels per thread
constexpr int kEigTile = kEigThreads * kEigPix;     // pixels per CTA
constexpr int kMaxKrylov = 64;

struct EigTile {
  int patch, p0, p1, pad;
};

// everything the eigensolver kernels read, passed by value
struct EigArgs {
  const PatchDev* patches;
  const EigTile* tiles;
  const int* tile_begin;
  const int* tile_count;
  const float* a_up;     // 40 x lvec
  const float* a_diag;   // lvec
  float* V;              // (m+1) x lvec, current basis
  double* part;          // [ntiles * warps][m+1]
  double* hbuf;          // [npatch][m+1]
  double* T;             // [npatch][m*m]
  double* Y;             // [npatch][m*m]
  double* beta2;         // [npatch]
  int* counter;          // [npatch]
  const int* active;     // [npatch]
  const int* decision;   // [npatch]
  const int* nkeep;      // [npatch]
  long long lvec;
  int m, mp1;
};

void upload_eig(const HostTables& t, cudaStream_t s);
cudaError_t ks_launch_init(const EigArgs& a, int ntiles, float* w, cudaStream_t s);
cudaError_t ks_launch_spmv(const EigArgs& a, int ntiles, int j, const float* src, int use_beta,
                           float* dst, cudaStream_t s);
cudaError_t ks_launch_orth(const EigArgs& a, int ntiles, int j, int mode, float* w, cudaStream_t s);
// the restart of the patches whose decision is 1 and the final Ritz vectors
// of those whose decision is 2 (each launched only when some patch needs it)
cudaError_t ks_launch_restart(const EigArgs& a, int ntiles, const float* w, float* vout, float* evec,
                              cudaStream_t s, bool any_restart, bool any_final);

}  // namespace gpb
