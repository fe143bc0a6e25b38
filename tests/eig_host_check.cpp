// Host-only checks of the dense linear algebra of eig_host.cpp: for random
// symmetric and Gram matrices (n = 9 .. 64), the decomposition reproduces A
// (|A Z - Z diag(w)| small, Z orthonormal, w ascending); the product helper
// agrees with the plain triple loop to the bit; U G^-1/2 is orthonormal for
// the Gram matrix G = U^T U of a well-conditioned block.  Prints "ok".
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

namespace gpb {
void sym_eig(double* A, int n, double* w, double* Z);
void lowdin(const double* G, int n, double* M);
void mat_mul(const double* A, const double* B, double* C, int n, bool at);
}

static int fail(const char* what, int n, double v) {
  printf("FAIL %s n=%d value=%g\n", what, n, v);
  return 1;
}

int main() {
  std::mt19937 rng(11);
  std::normal_distribution<double> nd;
  for (int n : {9, 26, 32, 40, 64}) {
    for (int t = 0; t < 20; t++) {
      std::vector<double> A((size_t)n * n), A0, w(n), Z((size_t)n * n);
      const int m = 2 * n;
      std::vector<double> U((size_t)m * n);
      for (auto& x : U) x = nd(rng);
      if (t % 2) {
        for (int i = 0; i < n; i++)
          for (int j = 0; j < n; j++) {
            double s = 0;
            for (int k = 0; k < m; k++) s += U[k * n + i] * U[k * n + j];
            A[i * n + j] = s;
          }
      } else {
        for (int i = 0; i < n; i++)
          for (int j = 0; j <= i; j++) A[i * n + j] = A[j * n + i] = nd(rng);
      }
      A0 = A;
      double anorm = 0;
      for (double x : A0) anorm = std::max(anorm, fabs(x));
      gpb::sym_eig(A.data(), n, w.data(), Z.data());
      for (int j = 1; j < n; j++)
        if (w[j] < w[j - 1]) return fail("eigenvalues not ascending", n, w[j] - w[j - 1]);
      double res = 0, orth = 0;
      for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
          double az = 0, zz = 0;
          for (int k = 0; k < n; k++) {
            az += A0[i * n + k] * Z[k * n + j];
            zz += Z[k * n + i] * Z[k * n + j];
          }
          res = std::max(res, fabs(az - Z[i * n + j] * w[j]));
          orth = std::max(orth, fabs(zz - (i == j ? 1.0 : 0.0)));
        }
      if (res > 1e-11 * anorm * n) return fail("residual |A Z - Z diag(w)|", n, res);
      if (orth > 1e-12 * n) return fail("orthonormality of Z", n, orth);
      // the product helper against the plain loops, bit for bit
      std::vector<double> B((size_t)n * n), C1((size_t)n * n), C2((size_t)n * n);
      for (auto& x : B) x = nd(rng);
      for (int at = 0; at < 2; at++) {
        gpb::mat_mul(A0.data(), B.data(), C1.data(), n, at);
        for (int r = 0; r < n; r++)
          for (int c = 0; c < n; c++) {
            double v = 0;
            for (int k = 0; k < n; k++) v += (at ? A0[k * n + r] : A0[r * n + k]) * B[k * n + c];
            C2[r * n + c] = v;
          }
        for (size_t e = 0; e < C1.size(); e++)
          if (C1[e] != C2[e]) return fail("mat_mul differs from the plain loop", n, C1[e] - C2[e]);
      }
      // Loewdin: U G^-1/2 has orthonormal columns
      if (t % 2) {
        std::vector<double> M((size_t)n * n), Q((size_t)m * n);
        gpb::lowdin(A0.data(), n, M.data());
        double e = 0;
        for (int k = 0; k < m; k++)
          for (int j = 0; j < n; j++) {
            double s = 0;
            for (int l = 0; l < n; l++) s += U[k * n + l] * M[l * n + j];
            Q[k * n + j] = s;
          }
        for (int i = 0; i < n; i++)
          for (int j = 0; j < n; j++) {
            double s = 0;
            for (int k = 0; k < m; k++) s += Q[k * n + i] * Q[k * n + j];
            e = std::max(e, fabs(s - (i == j ? 1.0 : 0.0)));
          }
        if (e > 1e-10) return fail("Loewdin orthonormality", n, e);
      }
    }
  }
  printf("ok\n");
  return 0;
}
