// Register-blocked FP64 GEMMs for the CPU oracle -- TEST INFRASTRUCTURE.
// The reference forms its per-leaf contractions with Eigen GEMMs
// (src/gto/density.cpp:33-43 Phi * D; src/dft/xc_potential_matrix.cpp:9-41
// Phi^T * X); these two kernels play that part so that the timed CPU
// baseline runs the contractions at GEMM speed rather than as axpy or dot
// loops.  Plain C++ with GCC's generic vector extension (two doubles per
// vector: NEON on Arm, SSE2 on x86; no intrinsics, no target flags),
// column-major operands:
//
//   gemm_nn: C (n x q) += A (n x k) * B (k x q)     A, C: points contiguous
//   gemm_tn: C (p x q) += A (n x p)^T * B (n x q)   reduction over points
#pragma once
#include <cstddef>
#include <cstring>

namespace oracle_gemm {

typedef double v2d __attribute__((vector_size(16)));

inline v2d load2(const double *p) {
  v2d v;
  std::memcpy(&v, p, sizeof(v));
  return v;
}
inline void store2(double *p, v2d v) { std::memcpy(p, &v, sizeof(v)); }

// C += A B.  Tiles of 8 rows x 4 columns of C in 16 vector registers; each
// step of k loads one 8-row slice of A's column (4 vectors) and four entries
// of B (broadcast).
inline void gemm_nn(long n, long q, long k, const double *A, long lda, const double *B, long ldb,
                    double *C, long ldc) {
  long j = 0;
  for (; j + 4 <= q; j += 4) {
    const double *b0 = B + (j + 0) * ldb, *b1 = B + (j + 1) * ldb, *b2 = B + (j + 2) * ldb,
                 *b3 = B + (j + 3) * ldb;
    long i = 0;
    for (; i + 8 <= n; i += 8) {
      v2d c[4][4];
      for (int r = 0; r < 4; r++)
        for (int s = 0; s < 4; s++)
          c[r][s] = v2d{0.0, 0.0};
      for (long l = 0; l < k; l++) {
        const double *a = A + l * lda + i;
        const v2d a0 = load2(a), a1 = load2(a + 2), a2 = load2(a + 4), a3 = load2(a + 6);
        const v2d x[4] = {v2d{b0[l], b0[l]}, v2d{b1[l], b1[l]}, v2d{b2[l], b2[l]},
                          v2d{b3[l], b3[l]}};
        for (int s = 0; s < 4; s++) {
          c[0][s] += a0 * x[s];
          c[1][s] += a1 * x[s];
          c[2][s] += a2 * x[s];
          c[3][s] += a3 * x[s];
        }
      }
      for (int s = 0; s < 4; s++) {
        double *cc = C + (j + s) * ldc + i;
        for (int r = 0; r < 4; r++)
          store2(cc + 2 * r, load2(cc + 2 * r) + c[r][s]);
      }
    }
    for (; i < n; i++)
      for (long l = 0; l < k; l++) {
        const double a = A[l * lda + i];
        C[(j + 0) * ldc + i] += a * b0[l];
        C[(j + 1) * ldc + i] += a * b1[l];
        C[(j + 2) * ldc + i] += a * b2[l];
        C[(j + 3) * ldc + i] += a * b3[l];
      }
  }
  for (; j < q; j++)
    for (long l = 0; l < k; l++) {
      const double x = B[j * ldb + l];
      const double *a = A + l * lda;
      double *c = C + j * ldc;
      for (long i = 0; i < n; i++)
        c[i] += a[i] * x;
    }
}

// C += A^T B.  Tiles of 4 x 4 entries of C; the reduction over points runs
// in two lanes per entry (one vector register each, 16 in all), summed at
// the end.
inline void gemm_tn(long p, long q, long n, const double *A, long lda, const double *B, long ldb,
                    double *C, long ldc) {
  const long n2 = n & ~1L;
  long j = 0;
  for (; j + 4 <= q; j += 4) {
    long i = 0;
    for (; i + 4 <= p; i += 4) {
      v2d s[4][4];
      for (int u = 0; u < 4; u++)
        for (int v = 0; v < 4; v++)
          s[u][v] = v2d{0.0, 0.0};
      const double *a[4] = {A + (i + 0) * lda, A + (i + 1) * lda, A + (i + 2) * lda,
                            A + (i + 3) * lda};
      const double *b[4] = {B + (j + 0) * ldb, B + (j + 1) * ldb, B + (j + 2) * ldb,
                            B + (j + 3) * ldb};
      for (long t = 0; t < n2; t += 2) {
        const v2d av[4] = {load2(a[0] + t), load2(a[1] + t), load2(a[2] + t), load2(a[3] + t)};
        const v2d bv[4] = {load2(b[0] + t), load2(b[1] + t), load2(b[2] + t), load2(b[3] + t)};
        for (int u = 0; u < 4; u++)
          for (int v = 0; v < 4; v++)
            s[u][v] += av[u] * bv[v];
      }
      for (int u = 0; u < 4; u++)
        for (int v = 0; v < 4; v++) {
          double acc = s[u][v][0] + s[u][v][1];
          for (long t = n2; t < n; t++)
            acc += a[u][t] * b[v][t];
          C[(j + v) * ldc + i + u] += acc;
        }
    }
    for (; i < p; i++)
      for (int v = 0; v < 4; v++) {
        const double *aa = A + i * lda, *bb = B + (j + v) * ldb;
        double acc = 0.0;
        for (long t = 0; t < n; t++)
          acc += aa[t] * bb[t];
        C[(j + v) * ldc + i] += acc;
      }
  }
  for (; j < q; j++)
    for (long i = 0; i < p; i++) {
      const double *aa = A + i * lda, *bb = B + j * ldb;
      double acc = 0.0;
      for (long t = 0; t < n; t++)
        acc += aa[t] * bb[t];
      C[j * ldc + i] += acc;
    }
}

} // namespace oracle_gemm
