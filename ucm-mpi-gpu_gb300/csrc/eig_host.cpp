// eig_host.cpp -- dense symmetric eigensolver for the small projected
// matrices of the Krylov methods (n <= 128), FP64 on the host.
//
// Householder reduction to tridiagonal form followed by the implicit
// symmetric QR iteration with Wilkinson shifts (Golub & Van Loan, Matrix
// Computations, 4th ed., Algorithms 8.3.1 and 8.3.3), accumulating the
// orthogonal transformations.  It replaces the ACML dstebz/dstein calls of
// damascene/src/noReorthog/lanczos.cu:284-391.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

namespace gpb {

// A (n x n, row-major, symmetric) -> eigenvalues w ascending, eigenvectors as
// the columns of Z (row-major n x n).  A is destroyed.
void sym_eig(double* A, int n, double* w, double* Z) {
  std::vector<double> d(n), e(n, 0.0), v(n), p(n), q(n);
  // Q accumulates the Householder reflections; start from I
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) Z[i * n + j] = (i == j) ? 1.0 : 0.0;
  // Householder tridiagonalisation: for column k, reflect rows k+1..n-1
  for (int k = 0; k < n - 2; k++) {
    double alpha = 0;
    for (int i = k + 1; i < n; i++) alpha += A[i * n + k] * A[i * n + k];
    alpha = sqrt(alpha);
    if (alpha == 0) continue;
    if (A[(k + 1) * n + k] > 0) alpha = -alpha;
    // v = x - alpha e1, normalised
    for (int i = 0; i < n; i++) v[i] = 0;
    v[k + 1] = A[(k + 1) * n + k] - alpha;
    for (int i = k + 2; i < n; i++) v[i] = A[i * n + k];
    double vn = 0;
    for (int i = k + 1; i < n; i++) vn += v[i] * v[i];
    if (vn == 0) continue;
    const double beta = 2.0 / vn;
    // A <- H A H with H = I - beta v v^T:  p = beta A v, K = beta/2 v^T p,
    // q = p - K v, A <- A - v q^T - q v^T
    for (int i = 0; i < n; i++) {
      double s = 0;
      for (int j = k + 1; j < n; j++) s += A[i * n + j] * v[j];
      p[i] = beta * s;
    }
    double K = 0;
    for (int i = k + 1; i < n; i++) K += v[i] * p[i];
    K *= beta / 2;
    for (int i = 0; i < n; i++) q[i] = p[i] - K * v[i];
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) A[i * n + j] -= v[i] * q[j] + q[i] * v[j];
    // Z <- Z H
    for (int i = 0; i < n; i++) {
      double s = 0;
      for (int j = k + 1; j < n; j++) s += Z[i * n + j] * v[j];
      s *= beta;
      for (int j = k + 1; j < n; j++) Z[i * n + j] -= s * v[j];
    }
  }
  // the reduced matrix is tridiagonal; clean the rounding outside the band
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (abs(i - j) > 1) A[i * n + j] = 0;
  // implicit symmetric QR with Wilkinson shift, rotations applied to the
  // rows and columns of A (dense, n is small) and accumulated into Z
  auto T = [&](int i, int j) -> double& { return A[i * n + j]; };
  int hi = n - 1;
  for (int iter = 0; iter < 100 * n && hi > 0; iter++) {
    while (hi > 0 && fabs(T(hi, hi - 1)) <= 1e-15 * (fabs(T(hi - 1, hi - 1)) + fabs(T(hi, hi)))) {
      T(hi, hi - 1) = T(hi - 1, hi) = 0;
      hi--;
    }
    if (hi == 0) break;
    int lo = hi - 1;
    while (lo > 0 && fabs(T(lo, lo - 1)) > 1e-15 * (fabs(T(lo - 1, lo - 1)) + fabs(T(lo, lo)))) lo--;
    const double dd = (T(hi - 1, hi - 1) - T(hi, hi)) / 2;
    const double ee = T(hi, hi - 1);
    const double den = dd + (dd >= 0 ? 1.0 : -1.0) * sqrt(dd * dd + ee * ee);
    const double mu = den != 0 ? T(hi, hi) - ee * ee / den : T(hi, hi);
    double x = T(lo, lo) - mu, z = T(lo + 1, lo);
    for (int k = lo; k < hi; k++) {
      double c, s;
      if (z == 0) {
        c = 1;
        s = 0;
      } else if (fabs(z) > fabs(x)) {
        const double t = -x / z;
        s = 1 / sqrt(1 + t * t);
        c = s * t;
      } else {
        const double t = -z / x;
        c = 1 / sqrt(1 + t * t);
        s = c * t;
      }
      const int j0 = std::max(lo, k - 1), j1 = std::min(hi, k + 2);
      for (int j = j0; j <= j1; j++) {  // rows: A <- G^T A
        const double a = T(k, j), b = T(k + 1, j);
        T(k, j) = c * a - s * b;
        T(k + 1, j) = s * a + c * b;
      }
      for (int i = j0; i <= j1; i++) {  // columns: A <- A G
        const double a = T(i, k), b = T(i, k + 1);
        T(i, k) = c * a - s * b;
        T(i, k + 1) = s * a + c * b;
      }
      for (int i = 0; i < n; i++) {
        const double a = Z[i * n + k], b = Z[i * n + k + 1];
        Z[i * n + k] = c * a - s * b;
        Z[i * n + k + 1] = s * a + c * b;
      }
      if (k < hi - 1) {
        x = T(k + 1, k);
        z = T(k + 2, k);
      }
    }
  }
  for (int i = 0; i < n; i++) d[i] = T(i, i);
  // sort ascending
  std::vector<int> idx(n);
  for (int i = 0; i < n; i++) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int a, int b) { return d[a] < d[b]; });
  std::vector<double> Zc(Z, Z + (size_t)n * n);
  for (int j = 0; j < n; j++) {
    w[j] = d[idx[j]];
    for (int i = 0; i < n; i++) Z[i * n + j] = Zc[i * n + idx[j]];
  }
}

}  // namespace gpb
