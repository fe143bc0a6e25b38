// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A thin extern "C" shim, written for this project, around the reference's
// own CPU cores compiled from their sources in place (see Makefile.ref):
// Berkeley lib_image (globalPb/src), buildW (buildW/src) and the vendored
// Spectra + Eigen.  The OpenCV glue of src/*.cpp is not compilable here
// (OpenCV is absent); the few lines of glue this shim needs restate
// src/buildW.cpp:55-116 and src/spectralPb.cpp:197-245.  Used only to pin the
// oracle restatement (gpb_oracle.c); never part of the product.
#include <stdint.h>
#include <string.h>

#include <vector>

#include "collections/array_list.hh"
#include "collections/pointers/auto_collection.hh"
#include "math/libraries/lib_image.hh"
#include "math/matrices/matrix.hh"

#include "affinity.hh"
#include "ic.hh"
#include "smatrix.hh"

#include <Eigen/Dense>
#include <Eigen/Sparse>
#include <MatOp/SparseCholesky.h>
#include <MatOp/SparseGenMatProd.h>
#include <SymGEigsSolver.h>

using collections::array_list;
using collections::pointers::auto_collection;
using math::libraries::lib_image;
using math::matrices::matrix;

extern "C" {

// lib_image::gaussian(sigma) -> k; returns length
int ref_gaussian(double sigma, double* k) {
  matrix<> g = lib_image::gaussian(sigma);
  for (unsigned long i = 0; i < g.size(); i++) k[i] = g[i];
  return (int)g.size();
}

// lib_image::hist_gradient_2D over a full (padded) label image; out = 8 x Hp x Wp
int ref_hist_gradient(const uint8_t* lab, int Hp, int Wp, int r, const double* kern, int klen,
                      double* out) {
  matrix<unsigned long> labels(Hp, Wp);
  for (long n = 0; n < (long)Hp * Wp; n++) labels[n] = lab[n];
  matrix<> k;
  if (klen > 0) {
    k = matrix<>(klen, 1);
    for (int i = 0; i < klen; i++) k[i] = kern[i];
  }
  auto_collection<matrix<>, array_list<matrix<> > > g =
      lib_image::hist_gradient_2D(labels, (unsigned long)r, 8, k);
  for (int o = 0; o < 8; o++)
    for (long n = 0; n < (long)Hp * Wp; n++) out[(size_t)o * Hp * Wp + n] = (*g)[o][n];
  return 0;
}

// colour chain of mex_pb_parts_final_selected.cpp:97-134 on n pixels given as
// doubles in [0,1] (r,g,b already in the order lib_image receives them)
void ref_lab_bins(const double* r, const double* g, const double* b, long n, int nbins,
                  uint8_t* Lq, uint8_t* aq, uint8_t* bq) {
  matrix<> R(n, 1), G(n, 1), B(n, 1);
  for (long i = 0; i < n; i++) {
    R[i] = r[i];
    G[i] = g[i];
    B[i] = b[i];
  }
  lib_image::rgb_gamma_correct(R, G, B, 2.5);
  lib_image::rgb_to_lab(R, G, B);
  lib_image::lab_normalize(R, G, B);
  matrix<unsigned long> q0 = lib_image::quantize_values(R, nbins);
  matrix<unsigned long> q1 = lib_image::quantize_values(G, nbins);
  matrix<unsigned long> q2 = lib_image::quantize_values(B, nbins);
  for (long i = 0; i < n; i++) {
    Lq[i] = (uint8_t)q0[i];
    aq[i] = (uint8_t)q1[i];
    bq[i] = (uint8_t)q2[i];
  }
}

// lib_image::nonmax_oriented_2D(pb, ori, tol) on an H x W image
void ref_nonmax_oriented(const double* a, const double* ind, int H, int W, double tol, double* out) {
  matrix<> pb(H, W), po(H, W);
  for (long n = 0; n < (long)H * W; n++) {
    pb[n] = a[n];
    po[n] = ind[n];
  }
  matrix<> nm = lib_image::nonmax_oriented_2D(pb, po, tol);
  for (long n = 0; n < (long)H * W; n++) out[n] = nm[n];
}

// buildW (computeSupport + computeAffinities2 + symmetrize) on an H x W mPb,
// with the DualLattice layout of src/buildW.cpp:55-116 and src/spectralPb.cpp:
// 51-57.  Output: full symmetric W as CSR (rowptr N+1, cols/vals nnz).
// Returns nnz; call first with cols == NULL to size.
long ref_buildW(const double* mpb, int H, int W, long* rowptr, int* cols, double* vals) {
  Group::DualLattice L;
  // l1 = (H+1) x W with mPb in rows 1..H; l2 = H x (W+1) with mPb in cols 1..W
  L.H.resize(W, H + 1);
  L.V.resize(W + 1, H);
  for (int i = 0; i < W; i++)
    for (int j = 0; j < H + 1; j++) L.H(i, j) = (j > 0) ? (float)mpb[(size_t)(j - 1) * W + i] : 0.0f;
  for (int i = 0; i < W + 1; i++)
    for (int j = 0; j < H; j++) L.V(i, j) = (i > 0) ? (float)mpb[(size_t)j * W + (i - 1)] : 0.0f;
  L.width = L.H.size(0);
  L.height = L.V.size(1);
  Group::SupportMap ic;
  Group::computeSupport(L, 5, 1.0f, ic);
  SMatrix* Wm = NULL;
  Group::computeAffinities2(ic, 0.1f, 5, &Wm);
  long nnz = 0;
  for (int i = 0; i < Wm->n; i++) nnz += Wm->nz[i];
  if (cols) {
    long c = 0;
    for (int i = 0; i < Wm->n; i++) {
      rowptr[i] = c;
      for (int j = 0; j < Wm->nz[i]; j++) {
        cols[c] = Wm->col[i][j];
        vals[c] = Wm->values[i][j];
        c++;
      }
    }
    rowptr[Wm->n] = c;
  }
  delete Wm;
  return nnz;
}

// Spectra SymGEigsSolver<SMALLEST_MAGN, SparseGenMatProd, SparseCholesky,
// GEIGS_CHOLESKY> on the full symmetric D-W (D2 fixed), as in
// src/spectralPb.cpp:197-245.  Eigenvalues come back in Spectra's default
// (descending) order.  Returns the number converged.
int ref_spectra_geigs(int n, const long* rowptr, const int* cols, const double* vals, int nev,
                      int ncv, double* evals, double* evecs /* nev x n */) {
  typedef Eigen::Triplet<double> T;
  std::vector<T> tl, td;
  std::vector<double> d(n, 0.0);
  for (int i = 0; i < n; i++)
    for (long k = rowptr[i]; k < rowptr[i + 1]; k++) d[i] += vals[k];
  for (int i = 0; i < n; i++)
    for (long k = rowptr[i]; k < rowptr[i + 1]; k++) {
      const int j = cols[k];
      tl.push_back(T(i, j, (i == j) ? d[i] - vals[k] : -vals[k]));
    }
  for (int i = 0; i < n; i++) td.push_back(T(i, i, d[i]));
  Eigen::SparseMatrix<double> A(n, n), B(n, n);
  A.setFromTriplets(tl.begin(), tl.end());
  B.setFromTriplets(td.begin(), td.end());
  A.makeCompressed();
  B.makeCompressed();
  Spectra::SparseGenMatProd<double> opA(A);
  Spectra::SparseCholesky<double> opB(B);
  Spectra::SymGEigsSolver<double, Spectra::SMALLEST_MAGN, Spectra::SparseGenMatProd<double>,
                          Spectra::SparseCholesky<double>, Spectra::GEIGS_CHOLESKY>
      geigs(&opA, &opB, nev, ncv);
  geigs.init();
  int nconv = geigs.compute();
  if (geigs.info() != Spectra::SUCCESSFUL) return -1;
  Eigen::VectorXd ev = geigs.eigenvalues();
  Eigen::MatrixXd V = geigs.eigenvectors();
  for (int i = 0; i < nev; i++) {
    evals[i] = ev(i);
    for (int j = 0; j < n; j++) evecs[(size_t)i * n + j] = V(j, i);
  }
  return nconv;
}

}  // extern "C"
