/*
 * ref_shim.c -- compiles the reference ugemm's own CPU GEMMs, from their
 * sources where they lie, into oracle/_ref/*.so so that the tests' golden
 * fixtures come from the reference itself.  x86-64 only (the reference uses
 * AVX intrinsics and x86 inline assembly); built by oracle/Makefile when the
 * reference tree is present.  TEST INFRASTRUCTURE ONLY.
 *
 * check_sgemm.c is included for its static cmp_results (check_sgemm.c:56-85);
 * its main() is renamed out of the way.
 */
#define main ugemm_ref_check_sgemm_main
#include "check_sgemm.c"
#undef main

void ref_cmp_results(int M, int N, const float *ref, const float *res, int ld)
{
	cmp_results(M, N, ref, res, ld);
	fflush(stdout);
}

void ref_sgemm_sse(char major, char ta, char tb, int M, int N, int K, float alpha,
                   const float *A, int lda, const float *B, int ldb, float beta, float *C, int ldc)
{
	sgemm_sse(major, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
}
