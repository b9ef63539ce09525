/* A C99 caller written the way the reference's sgemm_test.c selects its GPU
 * backend (sgemm_test.c:25-33): the sgemm_init / sgemm_rnn / sgemm_finish
 * macros point at this library's compat entry points.  Built and linked by
 * tests/test_gpu_zdropin.py; with a GPU (argument "run") it multiplies the
 * known-answer matrices of sgemm_test.c:186-200, without one it only checks
 * the calls a host without a device can make. */
#include <stdio.h>
#include <string.h>

#include "sgemm_cuda.h"

#define sgemm_init(s1, s2, s3) sgemm_cuda_init(0, 0, (s1 + s2 + s3) * 10 * sizeof(float))
#define sgemm_finish() sgemm_cuda_finish()
#define sgemm_rnn(M, N, K, ALPHA, A, B, BETA, C) sgemm_cuda('N', 'N', M, N, K, ALPHA, A, B, BETA, C)

int main(int argc, char **argv) {
  /* without init the compat call fails cleanly, no device needed */
  if (sgemm_cuda_status('N', 'N', 2, 2, 2, 1.f, 0, 0, 0.f, 0) != UGEMM_ERR_NOT_INIT) return 1;
  if (strcmp(ugemm_status_string(UGEMM_OK), "ok") != 0) return 2;
  if (argc > 1 && strcmp(argv[1], "run") == 0) {
    /* 3 x 2 times 2 x 3, row-major: the known answer of sgemm_test.c */
    float a[6] = {1, 2, 3, 4, 5, 6}, b[6] = {1, 2, 3, 4, 5, 6}, c[9] = {0};
    const float want[9] = {9, 12, 15, 19, 26, 33, 29, 40, 51};
    int i;
    /* the arena as sgemm_test.c sizes it, for its own 1023 x 1000 x 1023
     * test (the 3 x 3 x 2 product alone is too small to hold the arena's
     * 256-byte-aligned regions) */
    sgemm_init(1023 * 1023, 1023 * 1000, 1023 * 1000);
    sgemm_rnn(3, 3, 2, 1.f, a, b, 0.f, c);
    if (ugemm_last_error() != UGEMM_OK) {
      fprintf(stderr, "%s\n", ugemm_last_error_message());
      return 3;
    }
    sgemm_finish();
    for (i = 0; i < 9; ++i)
      if (c[i] != want[i]) return 4;
  }
  puts("dropin ok");
  return 0;
}
