// k_dense.cu -- the 32 x 32 dense steps of the block eigensolver on the
// device, so that an outer iteration needs one host round trip (for the
// convergence decisions) instead of four.
//
//   cf_dense<<<npatch, 256>>>  per active patch, the symmetric part of a
//   32 x 32 FP64 Gram / projected matrix is diagonalised by parallel cyclic
//   Jacobi (16 disjoint rotations per round, round-robin pairing, 31 rounds
//   per sweep, at most 20 sweeps), then
//     mode 0 (symmetric orthonormalisation): M = V diag(max(w, w_max 1e-15))^-1/2 V^T
//     mode 1 (Rayleigh-Ritz): theta = w ascending, M = the matching eigenvectors
//   The host versions (Householder tridiagonalisation + implicit QR, eig_host.cpp)
//   give the same matrices to FP64 rounding.
#include <stdint.h>

#include "k_block.h"

namespace gpb {

namespace {

constexpr int N = kBlk;     // 32
constexpr int LD = N + 1;   // padded row

__device__ __forceinline__ void pair_of(int round, int k, int& p, int& q) {
  // round-robin tournament over 32 players: 0 fixed, 1..31 rotate
  if (k == 0) {
    p = 0;
    q = 1 + round;
  } else {
    p = 1 + (round + k) % 31;
    q = 1 + (round - k + 31) % 31;
  }
  if (p > q) {
    const int t = p;
    p = q;
    q = t;
  }
}

}  // namespace

__global__ void __launch_bounds__(256) cf_dense(const double* __restrict__ G, const int* __restrict__ active, int mode,
                                                double* __restrict__ M, double* __restrict__ theta) {
  __shared__ double A[N * LD], V[N * LD];
  __shared__ double rc[16], rs[16], w[N];
  __shared__ int rp[16], rq[16], perm[N];
  __shared__ double red[2][8];
  __shared__ int stop;
  const int pi = blockIdx.x, t = threadIdx.x;
  if (!active[pi]) return;
  const double* g = G + (size_t)pi * N * N;
  for (int e = t; e < N * N; e += blockDim.x) {
    const int i = e / N, j = e % N;
    A[i * LD + j] = 0.5 * (g[i * N + j] + g[j * N + i]);
    V[i * LD + j] = (i == j) ? 1.0 : 0.0;
  }
  __syncthreads();
  for (int sweep = 0; sweep < 20; sweep++) {
    for (int round = 0; round < 31; round++) {
      if (t < 16) {
        int p, q;
        pair_of(round, t, p, q);
        const double app = A[p * LD + p], aqq = A[q * LD + q], apq = A[p * LD + q];
        double c = 1.0, s = 0.0;
        if (apq != 0.0) {
          const double th = (aqq - app) / (2.0 * apq);
          const double tt = fabs(th) > 1e150 ? 0.5 / th : (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
          c = 1.0 / sqrt(tt * tt + 1.0);
          s = tt * c;
        }
        rp[t] = p;
        rq[t] = q;
        rc[t] = c;
        rs[t] = s;
      }
      __syncthreads();
      for (int e = t; e < 16 * N; e += blockDim.x) {  // columns: A <- A J, V <- V J
        const int k = e / N, i = e % N, p = rp[k], q = rq[k];
        const double c = rc[k], s = rs[k];
        const double aip = A[i * LD + p], aiq = A[i * LD + q];
        A[i * LD + p] = c * aip - s * aiq;
        A[i * LD + q] = s * aip + c * aiq;
        const double vip = V[i * LD + p], viq = V[i * LD + q];
        V[i * LD + p] = c * vip - s * viq;
        V[i * LD + q] = s * vip + c * viq;
      }
      __syncthreads();
      for (int e = t; e < 16 * N; e += blockDim.x) {  // rows: A <- J^T A
        const int k = e / N, j = e % N, p = rp[k], q = rq[k];
        const double c = rc[k], s = rs[k];
        const double apj = A[p * LD + j], aqj = A[q * LD + j];
        A[p * LD + j] = c * apj - s * aqj;
        A[q * LD + j] = s * apj + c * aqj;
      }
      __syncthreads();
      if (t < 16 && rs[t] != 0.0) {  // the rotated pair is zero by construction
        A[rp[t] * LD + rq[t]] = 0.0;
        A[rq[t] * LD + rp[t]] = 0.0;
      }
      __syncthreads();
    }
    // stop once every off-diagonal entry is below 1e-15 of the largest diagonal one
    double off = 0.0, dia = 0.0;
    for (int e = t; e < N * N; e += blockDim.x) {
      const int i = e / N, j = e % N;
      const double v = fabs(A[i * LD + j]);
      if (i == j) dia = fmax(dia, v);
      else off = fmax(off, v);
    }
    for (int d = 16; d; d >>= 1) {
      off = fmax(off, __shfl_xor_sync(0xffffffffu, off, d));
      dia = fmax(dia, __shfl_xor_sync(0xffffffffu, dia, d));
    }
    if ((t & 31) == 0) {
      red[0][t >> 5] = off;
      red[1][t >> 5] = dia;
    }
    __syncthreads();
    if (t == 0) {
      double o = 0, m = 0;
      for (int k = 0; k < 8; k++) o = fmax(o, red[0][k]), m = fmax(m, red[1][k]);
      stop = (o <= 1e-15 * m);
    }
    __syncthreads();
    if (stop) break;
  }
  if (t < N) w[t] = A[t * LD + t];
  __syncthreads();
  if (t < N) {  // ascending order, ties by index
    int r = 0;
    for (int k = 0; k < N; k++) r += (w[k] < w[t]) || (w[k] == w[t] && k < t);
    perm[r] = t;
  }
  __syncthreads();
  double* m = M + (size_t)pi * N * N;
  if (mode == 0) {
    double wmax = w[perm[N - 1]];
    const double floor_ = fmax(wmax, 1e-300) * 1e-15;
    __shared__ double inv[N];
    if (t < N) inv[t] = 1.0 / sqrt(fmax(w[perm[t]], floor_));
    __syncthreads();
    for (int e = t; e < N * N; e += blockDim.x) {
      const int i = e / N, j = e % N;
      double v = 0.0;
      for (int k = 0; k < N; k++) v += V[i * LD + perm[k]] * V[j * LD + perm[k]] * inv[k];
      m[i * N + j] = v;
    }
  } else {
    if (t < N) theta[(size_t)pi * N + t] = w[perm[t]];
    for (int e = t; e < N * N; e += blockDim.x) {
      const int r = e / N, c = e % N;
      m[r * N + c] = V[r * LD + perm[c]];
    }
  }
}

cudaError_t cf_launch_dense(int npatch, const int* active, const double* G, int mode, double* M, double* theta,
                            cudaStream_t s) {
  if (npatch <= 0) return cudaSuccess;
  cf_dense<<<npatch, 256, 0, s>>>(G, active, mode, M, theta);
  return cudaGetLastError();
}

}  // namespace gpb
