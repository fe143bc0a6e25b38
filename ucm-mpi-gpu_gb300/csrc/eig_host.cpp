// eig_host.cpp -- dense symmetric eigensolver for the small projected
// matrices of the Krylov methods (n <= 128), FP64 on the host, and the
// 32 x 32 products and Loewdin orthonormalisation of the block solver's
// Rayleigh-Ritz steps.
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
//
// The eigenvector matrix is kept transposed while it is built (row k of Zt
// is column k of Z), so each reflection and each rotation runs over
// contiguous rows, and the reflections update only the block that is not
// yet reduced: rows and columns before column k hold nothing but the band
// and rounding residue there, which the band clean-up zeroes anyway.  Every
// entry of the band and of the eigenvectors goes through the same
// operations in the same order as in the textbook loop over the whole
// matrix, so the results are the same to the bit.
void sym_eig(double* A, int n, double* w, double* Z) {
  std::vector<double> d(n), v(n), p(n), q(n), s(n), Zt((size_t)n * n);
  // Q accumulates the Householder reflections; start from I
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) Zt[i * n + j] = (i == j) ? 1.0 : 0.0;
  // Householder tridiagonalisation: for column k, reflect rows k+1..n-1
  for (int k = 0; k < n - 2; k++) {
    double alpha = 0;
    for (int i = k + 1; i < n; i++) alpha += A[i * n + k] * A[i * n + k];
    alpha = sqrt(alpha);
    if (alpha == 0) continue;
    if (A[(k + 1) * n + k] > 0) alpha = -alpha;
    // v = x - alpha e1 (v_i = 0 for i <= k)
    for (int i = 0; i < n; i++) v[i] = 0;
    v[k + 1] = A[(k + 1) * n + k] - alpha;
    for (int i = k + 2; i < n; i++) v[i] = A[i * n + k];
    double vn = 0;
    for (int i = k + 1; i < n; i++) vn += v[i] * v[i];
    if (vn == 0) continue;
    const double beta = 2.0 / vn;
    // A <- H A H with H = I - beta v v^T:  p = beta A v, K = beta/2 v^T p,
    // q = p - K v, A <- A - v q^T - q v^T, on rows and columns k..n-1.  A
    // stays exactly symmetric (each update adds the same two products to
    // (i, j) and (j, i)), so A(i, j) v_j is summed over j from row j, which
    // is contiguous in i
    for (int i = k; i < n; i++) p[i] = 0;
    for (int j = k + 1; j < n; j++) {
      const double vj = v[j];
      const double* row = A + (size_t)j * n;
      for (int i = k; i < n; i++) p[i] += row[i] * vj;
    }
    for (int i = k; i < n; i++) p[i] *= beta;
    double K = 0;
    for (int i = k + 1; i < n; i++) K += v[i] * p[i];
    K *= beta / 2;
    for (int i = k; i < n; i++) q[i] = p[i] - K * v[i];
    for (int i = k; i < n; i++) {
      const double vi = v[i], qi = q[i];
      double* row = A + (size_t)i * n;
      for (int j = k; j < n; j++) row[j] -= vi * q[j] + qi * v[j];
    }
    // Z <- Z H, on the transposed rows: s_i = beta sum_j Z(i, j) v_j
    for (int i = 0; i < n; i++) s[i] = 0;
    for (int j = k + 1; j < n; j++) {
      const double vj = v[j];
      const double* zr = Zt.data() + (size_t)j * n;
      for (int i = 0; i < n; i++) s[i] += zr[i] * vj;
    }
    for (int i = 0; i < n; i++) s[i] *= beta;
    for (int j = k + 1; j < n; j++) {
      const double vj = v[j];
      double* zr = Zt.data() + (size_t)j * n;
      for (int i = 0; i < n; i++) zr[i] -= s[i] * vj;
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
      double c, sn;
      if (z == 0) {
        c = 1;
        sn = 0;
      } else if (fabs(z) > fabs(x)) {
        const double t = -x / z;
        sn = 1 / sqrt(1 + t * t);
        c = sn * t;
      } else {
        const double t = -z / x;
        c = 1 / sqrt(1 + t * t);
        sn = c * t;
      }
      const int j0 = std::max(lo, k - 1), j1 = std::min(hi, k + 2);
      for (int j = j0; j <= j1; j++) {  // rows: A <- G^T A
        const double a = T(k, j), b = T(k + 1, j);
        T(k, j) = c * a - sn * b;
        T(k + 1, j) = sn * a + c * b;
      }
      for (int i = j0; i <= j1; i++) {  // columns: A <- A G
        const double a = T(i, k), b = T(i, k + 1);
        T(i, k) = c * a - sn * b;
        T(i, k + 1) = sn * a + c * b;
      }
      double* z0 = Zt.data() + (size_t)k * n;
      double* z1 = z0 + n;
      for (int i = 0; i < n; i++) {
        const double a = z0[i], b = z1[i];
        z0[i] = c * a - sn * b;
        z1[i] = sn * a + c * b;
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
  for (int j = 0; j < n; j++) {
    w[j] = d[idx[j]];
    const double* zr = Zt.data() + (size_t)idx[j] * n;
    for (int i = 0; i < n; i++) Z[i * n + j] = zr[i];
  }
}

// C = A B (A^T B when at), n x n row-major; C must not alias A or B.  Each
// C(r, c) is the sum over k in ascending order, as a dot product loop would
// form it; the loops run over c innermost so the compiler can vectorise.
void mat_mul(const double* A, const double* B, double* C, int n, bool at) {
  for (int r = 0; r < n; r++) {
    double* cr = C + (size_t)r * n;
    for (int c = 0; c < n; c++) cr[c] = 0;
    for (int k = 0; k < n; k++) {
      const double a = at ? A[(size_t)k * n + r] : A[(size_t)r * n + k];
      const double* bk = B + (size_t)k * n;
      for (int c = 0; c < n; c++) cr[c] += a * bk[c];
    }
  }
}

// M = G^-1/2 (Loewdin; eigenvalues clamped at 1e-15 of the largest), so that
// U M has orthonormal columns.  M(i, j) = sum_k Z(i, k) Z(j, k) / sqrt(w_k),
// k ascending.
void lowdin(const double* G, int n, double* M) {
  std::vector<double> A((size_t)n * n), w(n), Z((size_t)n * n), Zt((size_t)n * n), sq(n);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) A[i * n + j] = 0.5 * (G[i * n + j] + G[j * n + i]);
  sym_eig(A.data(), n, w.data(), Z.data());
  const double floor_ = std::max(w[n - 1], 1e-300) * 1e-15;
  for (int k = 0; k < n; k++) sq[k] = sqrt(std::max(w[k], floor_));
  for (int i = 0; i < n; i++)
    for (int k = 0; k < n; k++) Zt[k * n + i] = Z[i * n + k];
  for (int i = 0; i < n; i++) {
    double* mi = M + (size_t)i * n;
    for (int j = 0; j < n; j++) mi[j] = 0;
    for (int k = 0; k < n; k++) {
      const double zik = Z[i * n + k], sk = sq[k];
      const double* zk = Zt.data() + (size_t)k * n;
      for (int j = 0; j < n; j++) mi[j] += zik * zk[j] / sk;
    }
  }
}

}  // namespace gpb
