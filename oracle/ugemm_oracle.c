/*
 * ugemm_oracle.c -- CPU restatement of the reference ugemm SGEMM path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (ugemm_gb300/, the
 * libugemm_cuda.so C ABI) links or calls this file.  It is used by tests/ as
 * the checker, by __graft_entry__.smoke() as the checker, and by bench.py as
 * the timed CPU baseline ("port" of the reference's AVX256 SGEMM).
 *
 * Every function restates, in portable C, the arithmetic of one reference
 * function (cited file:line, paths relative to the ugemm project root), in the
 * same per-element order of operations, so that results are bit-identical to
 * the reference built with the same floating-point contraction setting:
 *
 *   oracle_sgemm_cpu      ugemm.h:287-411   naive FP32 triple loop, 'R'/'C', N/T
 *   oracle_dgemm_cpu      ugemm.h:162-286   the same in FP64
 *   oracle_sgemm_c        gemm_cpu.h:238-363 (via ugemm.h:35-39) KC-blocked GEMM
 *   oracle_dgemm_c        gemm_cpu.h:238-363 (via ugemm.h:29-33) FP64 of the above
 *   oracle_sgemm_avx256   sgemm_avx256.h:308-390 35x96 B-block, 2x24 core (NN)
 *   oracle_sgemm_avx256_mt  band-parallel harness around the above (all trans)
 *   oracle_sgemm_sse      sgemm_sse.h:20-451   Goto-style blocks, 8x8 AVX tiles (all trans)
 *   oracle_gemm_rnn/rnt/rtn  sgemm_test.c:40-105  the GPU test's CPU loops (tight ld)
 *   oracle_cmp_results    check_sgemm.c:56-85  stdErr/stdRef/maxErr metric
 *   oracle_im2col         sgemm_ocl1.h:81-119  im2col (one image, square kernel)
 *   oracle_saxpy_cpu      ugemm.h:86-97        y += alpha*x with strides
 *   oracle_sgemv_cpu      ugemm.h:129-160      column-major GEMV (x read with incy)
 *   oracle_bias_leaky     sgemm_gl1.h:210-217  bias + LeakyReLU(0.1) after a conv GEMM
 *
 * Build flags matter and are fixed by oracle/Makefile: the naive and blocked
 * restatements are compiled with -ffp-contract=off (no fused multiply-add, no
 * fast-math), the AVX256 port with -ffp-contract=fast, exactly as the reference
 * builds are made for the golden fixtures in tests/golden/.
 */
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "ugemm_oracle.h"

/* ------------------------------------------------------------------------ */
/* Operand addressing shared by the naive and blocked restatements.         */
/* Row-major ('R'):  op(A)[m][k] = A[k + m*lda] ('N') or A[m + k*lda] ('T'). */
/* Column-major ('C'): op(A)[m][k] = A[m + k*lda] ('N') or A[k + m*lda] ('T')*/
/* (ugemm.h:178-285 for 'R', :226-284 for 'C').                               */
/* ------------------------------------------------------------------------ */
typedef struct {
    ptrdiff_t a_m, a_k; /* strides of op(A) along m and k */
    ptrdiff_t b_k, b_n; /* strides of op(B) along k and n */
    ptrdiff_t c_m, c_n; /* strides of C along m and n     */
} strides_t;

static int make_strides(char major, char ta, char tb, int lda, int ldb, int ldc, strides_t *s)
{
    if ((ta != 'N' && ta != 'T') || (tb != 'N' && tb != 'T')) return -1;
    if (major == 'R') {
        if (ta == 'N') { s->a_m = lda; s->a_k = 1; } else { s->a_m = 1; s->a_k = lda; }
        if (tb == 'N') { s->b_k = ldb; s->b_n = 1; } else { s->b_k = 1; s->b_n = ldb; }
        s->c_m = ldc; s->c_n = 1;
    } else {
        if (ta == 'N') { s->a_m = 1; s->a_k = lda; } else { s->a_m = lda; s->a_k = 1; }
        if (tb == 'N') { s->b_k = 1; s->b_n = ldb; } else { s->b_k = ldb; s->b_n = 1; }
        s->c_m = 1; s->c_n = ldc;
    }
    return 0;
}

/*
 * ugemm.h:287-411 (sgemm_cpu).  Per element: sum = 0.0f; for k ascending:
 * tmp = a*b; sum += tmp; then C = alpha*sum + beta*C (C is always read, so a
 * NaN in C survives beta == 0 -- unlike the GPU kernels, sgemm_ocl2.h:86-87).
 * The loop nest is reordered (k outside n) so the compiler can vectorise over
 * n; the per-element operation sequence is unchanged.
 */
int oracle_sgemm_cpu(char major, char ta, char tb, int M, int N, int K, float alpha,
                     const float *A, int lda, const float *B, int ldb, float beta,
                     float *C, int ldc)
{
    strides_t s;
    if (make_strides(major, ta, tb, lda, ldb, ldc, &s)) return -1;
    if (M <= 0 || N <= 0) return 0;
    float *sum = (float *)malloc(sizeof(float) * (size_t)N);
    if (!sum) return -2;
    for (int m = 0; m < M; m++) {
        for (int n = 0; n < N; n++) sum[n] = 0.0f;
        for (int k = 0; k < K; k++) {
            const float a = A[m * s.a_m + k * s.a_k];
            const float *brow = B + k * s.b_k;
            for (int n = 0; n < N; n++) {
                float tmp = a * brow[n * s.b_n];
                sum[n] += tmp;
            }
        }
        for (int n = 0; n < N; n++) {
            float *c = &C[m * s.c_m + n * s.c_n];
            *c = alpha * sum[n] + beta * *c;
        }
    }
    free(sum);
    return 0;
}

/* ugemm.h:162-286 (dgemm_cpu): the FP64 twin of oracle_sgemm_cpu. */
int oracle_dgemm_cpu(char major, char ta, char tb, int M, int N, int K, double alpha,
                     const double *A, int lda, const double *B, int ldb, double beta,
                     double *C, int ldc)
{
    strides_t s;
    if (make_strides(major, ta, tb, lda, ldb, ldc, &s)) return -1;
    if (M <= 0 || N <= 0) return 0;
    double *sum = (double *)malloc(sizeof(double) * (size_t)N);
    if (!sum) return -2;
    for (int m = 0; m < M; m++) {
        for (int n = 0; n < N; n++) sum[n] = 0.0;
        for (int k = 0; k < K; k++) {
            const double a = A[m * s.a_m + k * s.a_k];
            const double *brow = B + k * s.b_k;
            for (int n = 0; n < N; n++) {
                double tmp = a * brow[n * s.b_n];
                sum[n] += tmp;
            }
        }
        for (int n = 0; n < N; n++) {
            double *c = &C[m * s.c_m + n * s.c_n];
            *c = alpha * sum[n] + beta * *c;
        }
    }
    free(sum);
    return 0;
}

/*
 * gemm_cpu.h:238-363 (GEMM(_c) -> GEMM(_nn_cpu) -> macro/micro kernel).
 * Blocking constant KC = 384 (gemm_cpu.h:2).  Per element and per K block l:
 *   AB = 0; AB += a*b over the block's k in ascending order  (micro kernel :108)
 *   first block:  C = beta*C (beta==0 -> 0, beta==1 -> unchanged)  (:118-130)
 *   every block:  C = C + alpha*AB   (alpha==1 -> C + AB)          (:133-145)
 * Edge tiles (gemm_cpu.h:229-231) give the same values: 0 + alpha*AB is
 * alpha*AB exactly, then gescal(beta) and geaxpy(1.0).  MC/NC/MR/NR only
 * change the traversal, not the arithmetic, so they are not restated.
 * Quick returns and the alpha==0 path follow gemm_cpu.h:303-323.
 */
#define ORACLE_KC 384

#define DEFINE_BLOCKED(NAME, real)                                                          \
int NAME(char major, char ta, char tb, int M, int N, int K, real alpha,                     \
         const real *A, int lda, const real *B, int ldb, real beta, real *C, int ldc)       \
{                                                                                           \
    strides_t s;                                                                            \
    if (make_strides(major, ta, tb, lda, ldb, ldc, &s)) return -1;                          \
    if (M <= 0 || N <= 0 || ((alpha == 0 || K == 0) && beta == 1)) return 0;                \
    if (alpha == 0 || K == 0) {                                                             \
        for (int m = 0; m < M; m++)                                                         \
            for (int n = 0; n < N; n++) {                                                   \
                real *c = &C[m * s.c_m + n * s.c_n];                                        \
                *c = (beta == 0) ? (real)0 : *c * beta;                                     \
            }                                                                               \
        return 0;                                                                           \
    }                                                                                       \
    real *ab = (real *)malloc(sizeof(real) * (size_t)N);                                    \
    if (!ab) return -2;                                                                     \
    for (int m = 0; m < M; m++) {                                                           \
        for (int l0 = 0; l0 < K; l0 += ORACLE_KC) {                                         \
            const int l1 = (l0 + ORACLE_KC < K) ? l0 + ORACLE_KC : K;                       \
            for (int n = 0; n < N; n++) ab[n] = 0;                                          \
            for (int k = l0; k < l1; k++) {                                                 \
                const real a = A[m * s.a_m + k * s.a_k];                                    \
                const real *brow = B + k * s.b_k;                                           \
                for (int n = 0; n < N; n++) ab[n] += a * brow[n * s.b_n];                   \
            }                                                                               \
            for (int n = 0; n < N; n++) {                                                   \
                real *c = &C[m * s.c_m + n * s.c_n];                                        \
                real cv = *c;                                                               \
                if (l0 == 0) {                                                              \
                    if (beta == 0) cv = 0;                                                  \
                    else if (beta != 1) cv *= beta;                                         \
                }                                                                           \
                *c = (alpha == 1) ? cv + ab[n] : cv + alpha * ab[n];                        \
            }                                                                               \
        }                                                                                   \
    }                                                                                       \
    free(ab);                                                                               \
    return 0;                                                                               \
}

DEFINE_BLOCKED(oracle_sgemm_c, float)
DEFINE_BLOCKED(oracle_dgemm_c, double)

/*
 * check_sgemm.c:56-85 (cmp_results).  Returns stdErr, stdRef, maxErr and the
 * flat index of maxErr; the label is 2 ("FAIL !!!") if maxErr > 1e-5*stdRef,
 * 1 ("Sucks !") if maxErr > 3e-5*stdRef or stdErr > 1e-6*stdRef, else 0.
 */
int oracle_cmp_results(int M, int N, const float *ref, const float *res, int ld, double out[4])
{
    double max_err = 0, s2_err = 0, s1_ref = 0, s2_ref = 0;
    int max_i = 0;
    for (int m = 0; m < M; ++m) {
        for (int n = 0; n < N; ++n) {
            double r = ref[m * ld + n], v = res[m * ld + n], e = v - r;
            if (max_err < fabs(e)) { max_err = fabs(e); max_i = m * ld + n; }
            s2_err += e * e;
            s1_ref += r;
            s2_ref += r * r;
        }
    }
    double cnt = (double)M * (double)N;
    double std_err = sqrt(s2_err / cnt);
    double std_ref = sqrt(s2_ref * cnt - s1_ref * s1_ref) / cnt;
    out[0] = std_err; out[1] = std_ref; out[2] = max_err; out[3] = (double)max_i;
    if (max_err > std_ref * 1e-5) return 2;
    if (max_err > std_ref * 3e-5 || std_err > std_ref * 1e-6) return 1;
    return 0;
}

/*
 * sgemm_sse.h:20-451 (sgemm_sse): a Goto-style SGEMM.  C is updated in blocks
 * of 4096 columns x 384 k x 384 rows, each block in 8 x 8 tiles; a tile's
 * product over one k block is, per element, a chain of multiply-adds from
 * zero over k, fused as the reference's AVX kernel (sgemm_sse.h:106-170) is
 * when built with FMA contraction (its Makefile).  Then per tile, with
 * beta' = beta for the first k block and 1 for the others:
 *   full 8 x 8 tile (sgemm_sse.h:204-232):  C = 0 (beta' == 0) or C *= beta'
 *     (beta' != 1); C += AB (alpha == 1) or C = fma(alpha, AB, C);
 *   edge tile (sgemm_sse.h:329-333):        T = alpha * AB; C *= beta' (or 0
 *     when beta' == 0); C += T.
 * The alpha == 0 shortcut (sgemm_sse.h:383-397) indexes C column-major
 * whatever the major, as the reference does.
 */
#define SSE_MC 384
#define SSE_KC 384
#define SSE_NC 4096

static void sse_scale(int m, int n, float beta, float *C, long cr, long cc)
{
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < m; ++i)
            C[i * cr + j * cc] = beta != 0.0f ? C[i * cr + j * cc] * beta : 0.0f;
}

static void sse_nn(int m, int n, int k, float alpha, const float *A, long ar, long ac,
                   const float *B, long br, long bc, float beta, float *C, long cr, long cc)
{
    if (alpha == 0.0f || k == 0) {
        sse_scale(m, n, beta, C, cr, cc);
        return;
    }
    float ab[64];
    for (int j0 = 0; j0 < n; j0 += SSE_NC) {
        const int nc = n - j0 < SSE_NC ? n - j0 : SSE_NC;
        for (int l0 = 0; l0 < k; l0 += SSE_KC) {
            const int kc = k - l0 < SSE_KC ? k - l0 : SSE_KC;
            const float bp = l0 == 0 ? beta : 1.0f;
            for (int i0 = 0; i0 < m; i0 += SSE_MC) {
                const int mc = m - i0 < SSE_MC ? m - i0 : SSE_MC;
                for (int tj = 0; tj < nc; tj += 8) {
                    for (int ti = 0; ti < mc; ti += 8) {
                        const int mr = mc - ti < 8 ? mc - ti : 8, nr = nc - tj < 8 ? nc - tj : 8;
                        const float *a = A + (long)(i0 + ti) * ar + (long)l0 * ac;
                        const float *b = B + (long)l0 * br + (long)(j0 + tj) * bc;
                        float *c = C + (long)(i0 + ti) * cr + (long)(j0 + tj) * cc;
                        for (int j = 0; j < nr; ++j)
                            for (int i = 0; i < mr; ++i) {
                                float s = 0.0f;
                                for (int l = 0; l < kc; ++l)
                                    s = fmaf(a[i * ar + l * ac], b[l * br + j * bc], s);
                                ab[i + 8 * j] = s;
                            }
                        for (int j = 0; j < nr; ++j)
                            for (int i = 0; i < mr; ++i) {
                                float *e = &c[i * cr + j * cc];
                                const float p = ab[i + 8 * j];
                                if (mr == 8 && nr == 8) {
                                    float v = *e;
                                    if (bp == 0.0f) v = 0.0f;
                                    else if (bp != 1.0f) v = v * bp;
                                    *e = alpha == 1.0f ? v + p : fmaf(alpha, p, v);
                                } else {
                                    const float t = alpha == 1.0f ? p : alpha * p;
                                    const float v = bp != 0.0f ? *e * bp : 0.0f;
                                    *e = v + t;
                                }
                            }
                    }
                }
            }
        }
    }
}

void oracle_sgemm_sse(char major, char ta, char tb, int m, int n, int k, float alpha,
                      const float *A, int lda, const float *B, int ldb, float beta, float *C,
                      int ldc)
{
    if (m == 0 || n == 0 || ((alpha == 0.0f || k == 0) && beta == 1.0f)) return;
    if (alpha == 0.0f) {
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < m; ++i)
                C[i + (long)j * ldc] = beta == 0.0f ? 0.0f : C[i + (long)j * ldc] * beta;
        return;
    }
    const int tA = ta == 'T', tB = tb == 'T';
    if (major == 'C') {
        /* column-major: A(i, l) at A[i + l*lda] ('N') or A[l + i*lda] ('T') */
        sse_nn(m, n, k, alpha, A, tA ? lda : 1, tA ? 1 : lda, B, tB ? ldb : 1, tB ? 1 : ldb, beta,
               C, 1, ldc);
    } else {
        /* row-major: A(i, l) at A[i*lda + l] ('N') or A[l*lda + i] ('T') */
        sse_nn(m, n, k, alpha, A, tA ? 1 : lda, tA ? lda : 1, B, tB ? 1 : ldb, tB ? ldb : 1, beta,
               C, ldc, 1);
    }
}

/*
 * sgemm_test.c:40-105: the CPU loops the reference's GPU test checks its
 * kernels against, row-major with tight leading dimensions.  C is first
 * zeroed (beta == 0) or scaled (beta != 1); then
 *   rnn (A M x K, B K x N) and rtn (A stored K x M): for each row m and each
 *     k in order, a = alpha * A(m, k) rounded, then C(m, n) += a * B(k, n);
 *   rnt (B stored N x K): C(m, n) += alpha * (sum over k in order of A(m, k)
 *     * B(n, k), accumulated in float).
 * sgemm_test.c itself needs the OpenCL headers and cannot be compiled here;
 * these restatements are pinned by the tests (exact integer inputs against
 * oracle_sgemm_cpu, and the known-answer test).
 */
static void gemm_beta(int M, int N, float beta, float *C)
{
    if (beta == 0.0f) memset(C, 0, sizeof(float) * (size_t)M * N);
    else if (beta != 1.0f)
        for (long i = 0; i < (long)M * N; ++i) C[i] *= beta;
}

void oracle_gemm_rnn(int M, int N, int K, float alpha, const float *A, const float *B, float beta,
                     float *C)
{
    gemm_beta(M, N, beta, C);
    for (int m = 0; m < M; ++m)
        for (int k = 0; k < K; ++k) {
            const float a = alpha * A[(long)m * K + k];
            for (int n = 0; n < N; ++n) C[(long)m * N + n] += a * B[(long)k * N + n];
        }
}

void oracle_gemm_rtn(int M, int N, int K, float alpha, const float *A, const float *B, float beta,
                     float *C)
{
    gemm_beta(M, N, beta, C);
    for (int m = 0; m < M; ++m)
        for (int k = 0; k < K; ++k) {
            const float a = alpha * A[m + (long)M * k];
            for (int n = 0; n < N; ++n) C[(long)m * N + n] += a * B[(long)k * N + n];
        }
}

void oracle_gemm_rnt(int M, int N, int K, float alpha, const float *A, const float *B, float beta,
                     float *C)
{
    gemm_beta(M, N, beta, C);
    for (int m = 0; m < M; ++m)
        for (int n = 0; n < N; ++n) {
            float sum = 0.0f;
            for (int k = 0; k < K; ++k) sum += A[(long)m * K + k] * B[k + (long)K * n];
            C[(long)m * N + n] += alpha * sum;
        }
}

/*
 * sgemm_ocl1.h:81-119 (im2col): one CHW image -> (C*k*k) x (Ho*Wo) columns,
 * square kernel, equal padding and stride in both directions; out-of-image
 * taps read 0.  Row (c*k*k + ki*k + kj), column (i*Wo + j).
 */
void oracle_im2col(const float *im, int channels, int height, int width, int ksize, int pad,
                   int stride, float *col)
{
    const int ho = (height + 2 * pad - ksize) / stride + 1;
    const int wo = (width + 2 * pad - ksize) / stride + 1;
    for (int c = 0; c < channels; c++)
        for (int ki = 0; ki < ksize; ki++)
            for (int kj = 0; kj < ksize; kj++) {
                float *dst = col + ((size_t)(c * ksize + ki) * ksize + kj) * ho * wo;
                for (int i = 0; i < ho; i++)
                    for (int j = 0; j < wo; j++) {
                        const int y = i * stride - pad + ki, x = j * stride - pad + kj;
                        dst[i * wo + j] = (y >= 0 && x >= 0 && y < height && x < width)
                                              ? im[((size_t)c * height + y) * width + x]
                                              : 0.f;
                    }
            }
}

/* ugemm.h:86-97 (saxpy_cpu): y[n*incy] += alpha * x[n*incx]. */
void oracle_saxpy_cpu(int N, float alpha, const float *x, int incx, float *y, int incy)
{
    for (int n = 0; n < N; n++) y[n * incy] += alpha * x[n * incx];
}

/* ugemm.h:129-160 (sgemv_cpu).  Column-major A; 'N': sum over n of
 * A[m + n*lda] * x[n*incy]; otherwise A[n + m*lda] * x[n*incy] (the
 * reference indexes x with incy); y[m*incy] = alpha*sum + beta*y[m*incy]. */
void oracle_sgemv_cpu(char trans, int M, int N, float alpha, const float *A, int lda,
                      const float *x, int incx, float beta, float *y, int incy)
{
    (void)incx;
    for (int m = 0; m < M; m++) {
        float sum = 0.0f;
        for (int n = 0; n < N; n++)
            sum += (trans == 'N' ? A[m + n * lda] : A[n + m * lda]) * x[n * incy];
        y[m * incy] = alpha * sum + beta * y[m * incy];
    }
}

/* sgemm_gl1.h:210-217 (the loop after the GEMM in gl_convolution_LReLU):
 * out[c][p] += bias[c]; out = out > 0 ? out : out * 0.1, with the multiply
 * done in double (the literal 0.1 is a double) and rounded back to float. */
void oracle_bias_leaky(float *out, int channels, int pixels, const float *bias)
{
    float *p = out;
    for (int i = 0; i < channels; i++)
        for (int n = 0; n < pixels; n++, p++) {
            *p += bias[i];
            *p = *p > 0 ? (*p) : (float)((double)(*p) * 0.1);
        }
}
