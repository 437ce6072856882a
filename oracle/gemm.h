// Register-blocked FP64 GEMMs for the CPU oracle -- TEST INFRASTRUCTURE.
// The reference forms its per-leaf contractions with Eigen GEMMs
// (src/gto/density.cpp:33-43 Phi * D; src/dft/xc_potential_matrix.cpp:9-41
// Phi^T * X); these two kernels play that part so that the timed CPU
// baseline runs the contractions at GEMM speed rather than as axpy or dot
// loops.  Plain C++ that the compiler vectorises for the host's baseline
// vector unit (no intrinsics, no target flags), column-major operands:
//
//   gemm_nn: C (n x q) += A (n x k) * B (k x q)     A, C: points contiguous
//   gemm_tn: C (p x q) += A (n x p)^T * B (n x q)   reduction over points
#pragma once
#include <cstddef>

namespace oracle_gemm {

// C += A B.  Tiles of 8 rows x 4 columns of C in registers; each step of k
// loads one 8-row slice of A's column and four entries of B.
inline void gemm_nn(long n, long q, long k, const double *A, long lda, const double *B, long ldb,
                    double *C, long ldc) {
  long j = 0;
  for (; j + 4 <= q; j += 4) {
    const double *b0 = B + (j + 0) * ldb, *b1 = B + (j + 1) * ldb, *b2 = B + (j + 2) * ldb,
                 *b3 = B + (j + 3) * ldb;
    long i = 0;
    for (; i + 8 <= n; i += 8) {
      double c0[8] = {0}, c1[8] = {0}, c2[8] = {0}, c3[8] = {0};
      for (long l = 0; l < k; l++) {
        const double *a = A + l * lda + i;
        const double x0 = b0[l], x1 = b1[l], x2 = b2[l], x3 = b3[l];
        for (int r = 0; r < 8; r++) {
          c0[r] += a[r] * x0;
          c1[r] += a[r] * x1;
          c2[r] += a[r] * x2;
          c3[r] += a[r] * x3;
        }
      }
      for (int r = 0; r < 8; r++) {
        C[(j + 0) * ldc + i + r] += c0[r];
        C[(j + 1) * ldc + i + r] += c1[r];
        C[(j + 2) * ldc + i + r] += c2[r];
        C[(j + 3) * ldc + i + r] += c3[r];
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
  const long n8 = n & ~1L;
  long j = 0;
  for (; j + 4 <= q; j += 4) {
    long i = 0;
    for (; i + 4 <= p; i += 4) {
      double s[4][4][2] = {};
      const double *a[4] = {A + (i + 0) * lda, A + (i + 1) * lda, A + (i + 2) * lda,
                            A + (i + 3) * lda};
      const double *b[4] = {B + (j + 0) * ldb, B + (j + 1) * ldb, B + (j + 2) * ldb,
                            B + (j + 3) * ldb};
      for (long t = 0; t < n8; t += 2)
        for (int u = 0; u < 4; u++)
          for (int v = 0; v < 4; v++)
            for (int r = 0; r < 2; r++)
              s[u][v][r] += a[u][t + r] * b[v][t + r];
      for (int u = 0; u < 4; u++)
        for (int v = 0; v < 4; v++) {
          double acc = s[u][v][0] + s[u][v][1];
          for (long t = n8; t < n; t++)
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
