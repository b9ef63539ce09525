/* A C99 caller written the way the reference's sgemm_test.c selects its GPU
 * backend (sgemm_test.c:25-33): the sgemm_init / sgemm_rnn / sgemm_rnt /
 * sgemm_rtn / sgemm_finish macros point at this library's compat entry
 * points, and the arena is sized by the reference's own rule, ten times the
 * three matrices of the product (sgemm_test.c:29, :208).  Built and linked by
 * tests/test_gpu_zdropin.py; with a GPU (argument "run") it multiplies the
 * known-answer matrices of sgemm_test.c:186-200 and a small product in each
 * transpose form against a double-precision loop; without one it only checks
 * the calls a host without a device can make. */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "sgemm_cuda.h"

#define sgemm_init(s1, s2, s3) sgemm_cuda_init(0, 0, (s1 + s2 + s3) * 10 * sizeof(float))
#define sgemm_finish() sgemm_cuda_finish()
#define sgemm_rnn(M, N, K, ALPHA, A, B, BETA, C) sgemm_cuda('N', 'N', M, N, K, ALPHA, A, B, BETA, C)
#define sgemm_rnt(M, N, K, ALPHA, A, B, BETA, C) sgemm_cuda('N', 'T', M, N, K, ALPHA, A, B, BETA, C)
#define sgemm_rtn(M, N, K, ALPHA, A, B, BETA, C) sgemm_cuda('T', 'N', M, N, K, ALPHA, A, B, BETA, C)

#define PM 61
#define PN 47
#define PK 39

/* C = alpha*op(A)*op(B) + beta*C in double, sgemm_test.c's loops (:40-105):
 * ta: A stored K x M; tb: B stored N x K */
static void ref_gemm(int ta, int tb, int M, int N, int K, double alpha, const float *A,
                     const float *B, double beta, const float *C0, double *R) {
  int i, j, k;
  for (i = 0; i < M; ++i)
    for (j = 0; j < N; ++j) {
      double s = 0;
      for (k = 0; k < K; ++k)
        s += (double)(ta ? A[k * M + i] : A[i * K + k]) * (tb ? B[j * K + k] : B[k * N + j]);
      R[i * N + j] = alpha * s + beta * C0[i * N + j];
    }
}

int main(int argc, char **argv) {
  /* without init the compat call fails cleanly, no device needed */
  if (sgemm_cuda_status('N', 'N', 2, 2, 2, 1.f, 0, 0, 0.f, 0) != UGEMM_ERR_NOT_INIT) return 1;
  if (strcmp(ugemm_status_string(UGEMM_OK), "ok") != 0) return 2;
  if (argc > 1 && strcmp(argv[1], "run") == 0) {
    /* 3 x 2 times 2 x 3, row-major: the known answer of sgemm_test.c */
    static float a[6] = {1, 2, 3, 4, 5, 6}, b[6] = {1, 2, 3, 4, 5, 6}, c[9];
    const float want[9] = {9, 12, 15, 19, 26, 33, 29, 40, 51};
    static float A[PM * PK], B[PK * PN], C[PM * PN], C0[PM * PN];
    static double R[PM * PN];
    int i, form;
    const int M = 3, N = 3, K = 2;
    for (i = 0; i < 9; ++i) c[i] = 1.f; /* sgemm_test.c:224; beta = 0 ignores it */
    sgemm_init(M * K, K * N, M * N);   /* 840 bytes, as the reference's test passes */
    if (ugemm_last_error() != UGEMM_OK) {
      fprintf(stderr, "init: %s\n", ugemm_last_error_message());
      return 3;
    }
    sgemm_rnn(M, N, K, 1.f, a, b, 0.f, c);
    if (ugemm_last_error() != UGEMM_OK) {
      fprintf(stderr, "rnn: %s\n", ugemm_last_error_message());
      return 4;
    }
    sgemm_finish();
    for (i = 0; i < 9; ++i)
      if (c[i] != want[i]) return 5;
    /* a ragged product in the three forms of sgemm_test.c, alpha and beta set */
    for (i = 0; i < PM * PK; ++i) A[i] = (float)((i * 37 % 101) - 50) / 64.f;
    for (i = 0; i < PK * PN; ++i) B[i] = (float)((i * 53 % 89) - 44) / 32.f;
    for (i = 0; i < PM * PN; ++i) C0[i] = (float)((i * 29 % 71) - 35) / 16.f;
    sgemm_init(PM * PK, PK * PN, PM * PN);
    for (form = 0; form < 3; ++form) {
      const int ta = form == 2, tb = form == 1;
      double err = 0, ref = 0;
      memcpy(C, C0, sizeof C);
      if (form == 0) sgemm_rnn(PM, PN, PK, 1.5f, A, B, 0.5f, C);
      if (form == 1) sgemm_rnt(PM, PN, PK, 1.5f, A, B, 0.5f, C);
      if (form == 2) sgemm_rtn(PM, PN, PK, 1.5f, A, B, 0.5f, C);
      if (ugemm_last_error() != UGEMM_OK) {
        fprintf(stderr, "form %d: %s\n", form, ugemm_last_error_message());
        return 6;
      }
      ref_gemm(ta, tb, PM, PN, PK, 1.5, A, B, 0.5, C0, R);
      for (i = 0; i < PM * PN; ++i) {
        err += (C[i] - R[i]) * (C[i] - R[i]);
        ref += R[i] * R[i];
      }
      if (!(sqrt(err / ref) < 2e-6)) {
        fprintf(stderr, "form %d: normwise error %.3e\n", form, sqrt(err / ref));
        return 7;
      }
    }
    sgemm_finish();
  }
  puts("dropin ok");
  return 0;
}
