/*
 * ugemm_oracle.h -- CPU oracle for the ugemm SGEMM path (test infrastructure
 * only: used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg; never linked into the product library).
 */
#ifndef UGEMM_ORACLE_H
#define UGEMM_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

int oracle_sgemm_cpu(char major, char ta, char tb, int M, int N, int K, float alpha,
                     const float *A, int lda, const float *B, int ldb, float beta,
                     float *C, int ldc);
int oracle_dgemm_cpu(char major, char ta, char tb, int M, int N, int K, double alpha,
                     const double *A, int lda, const double *B, int ldb, double beta,
                     double *C, int ldc);
int oracle_sgemm_c(char major, char ta, char tb, int M, int N, int K, float alpha,
                   const float *A, int lda, const float *B, int ldb, float beta,
                   float *C, int ldc);
int oracle_dgemm_c(char major, char ta, char tb, int M, int N, int K, double alpha,
                   const double *A, int lda, const double *B, int ldb, double beta,
                   double *C, int ldc);
void oracle_sgemm_avx256(int M, int N, int K, float alpha, const float *A, int lda,
                         const float *B, int ldb, float beta, float *C, int ldc);
int oracle_sgemm_avx256_mt(int nthreads, char ta, char tb, int M, int N, int K, float alpha,
                           const float *A, int lda, const float *B, int ldb, float beta,
                           float *C, int ldc);
void oracle_sgemm_sse(char major, char ta, char tb, int m, int n, int k, float alpha,
                      const float *A, int lda, const float *B, int ldb, float beta, float *C,
                      int ldc);
void oracle_gemm_rnn(int M, int N, int K, float alpha, const float *A, const float *B, float beta,
                     float *C);
void oracle_gemm_rnt(int M, int N, int K, float alpha, const float *A, const float *B, float beta,
                     float *C);
void oracle_gemm_rtn(int M, int N, int K, float alpha, const float *A, const float *B, float beta,
                     float *C);
int oracle_cmp_results(int M, int N, const float *ref, const float *res, int ld, double out[4]);
void oracle_im2col(const float *im, int channels, int height, int width, int ksize, int pad,
                   int stride, float *col);
void oracle_bias_leaky(float *out, int channels, int pixels, const float *bias);
void oracle_saxpy_cpu(int N, float alpha, const float *x, int incx, float *y, int incy);
void oracle_sgemv_cpu(char trans, int M, int N, float alpha, const float *A, int lda,
                      const float *x, int incx, float beta, float *y, int incy);

#ifdef __cplusplus
}
#endif
#endif
