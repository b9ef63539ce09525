/*
 * ugemm_oracle_port.c -- portable restatement of the reference's AVX256 SGEMM
 * (sgemm_avx256.h:1-390) and the band-parallel harness used as the timed CPU
 * baseline.
 *
 * TEST INFRASTRUCTURE ONLY (see ugemm_oracle.c).  Compiled with
 * -ffp-contract=fast, like the reference (Makefile:12), so that acc + a*b and
 * acc*alpha + C become fused multiply-adds as the reference's intrinsics do.
 */
#include <pthread.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

#include "ugemm_oracle.h"

/* ------------------------------------------------------------------------ */
/* AVX256 SGEMM port (sgemm_avx256.h:1-390), NN, row-major.                   */
/* Blocking table kept identical to the reference (sgemm_avx256.h:1-9):       */
/*   8-wide vectors, 3 vectors per column step, 4 steps -> 96-column B block,  */
/*   35-row B block, 32-row partial-result buffer for the rightmost columns.  */
/* The 8-wide vector is a GCC vector extension, so the same code compiles to */
/* AVX on x86-64 and to NEON on aarch64.  With -ffp-contract=fast, acc+a*b    */
/* and acc*alpha+C contract to FMAs as the reference's intrinsics do.         */
/* ------------------------------------------------------------------------ */
typedef float v8f __attribute__((vector_size(32), aligned(32)));

enum {
    P_SIMD = 8,
    P_COLS_PER_LOOP = 3,
    P_COL_STEPS = 4,
    P_VEC_PER_ROW = P_COLS_PER_LOOP * P_COL_STEPS, /* 12 vectors = 96 floats */
    P_BB_COLS = P_VEC_PER_ROW * P_SIMD,            /* 96 */
    P_BB_ROWS = 35,
    P_CC_ROWS = 32,
};

typedef struct {
    v8f bb[P_VEC_PER_ROW * P_BB_ROWS];
    v8f cc[P_CC_ROWS * P_VEC_PER_ROW];
    int M, lda, ldc;
    float alpha;
} port_prm_t;

static inline v8f splat(float x) { v8f v = {x, x, x, x, x, x, x, x}; return v; }
static inline v8f loadu(const float *p) { v8f v; memcpy(&v, p, sizeof v); return v; }
static inline void storeu(float *p, v8f v) { memcpy(p, &v, sizeof v); }

/* sgemm_avx256.h:20-125: full 35-row x 96-column block, two rows at a time;
 * the first k is a plain product, later k accumulate; C += alpha*acc. */
static void port_core(const port_prm_t *p, const float *A, float *C)
{
    const int lda = p->lda, ldc = p->ldc;
    const v8f va = splat(p->alpha);
    int m;
    for (m = 0; m < p->M - 1; A += 2 * lda, C += 2 * ldc, m += 2) {
        float *c0 = C, *c1 = C + ldc;
        for (int n = 0; n < P_VEC_PER_ROW; n += P_COLS_PER_LOOP) {
            const v8f *bc = &p->bb[n];
            v8f a0 = splat(A[0]), a1 = splat(A[lda]);
            v8f x00 = a0 * bc[0], x01 = a1 * bc[0];
            v8f x10 = a0 * bc[1], x11 = a1 * bc[1];
            v8f x20 = a0 * bc[2], x21 = a1 * bc[2];
            for (int k = 1; k < P_BB_ROWS; k++) {
                bc += P_VEC_PER_ROW;
                a0 = splat(A[k]);
                a1 = splat(A[k + lda]);
                x00 = x00 + a0 * bc[0]; x01 = x01 + a1 * bc[0];
                x10 = x10 + a0 * bc[1]; x11 = x11 + a1 * bc[1];
                x20 = x20 + a0 * bc[2]; x21 = x21 + a1 * bc[2];
            }
            storeu(c0 + 0, x00 * va + loadu(c0 + 0));
            storeu(c0 + 8, x10 * va + loadu(c0 + 8));
            storeu(c0 + 16, x20 * va + loadu(c0 + 16));
            storeu(c1 + 0, x01 * va + loadu(c1 + 0));
            storeu(c1 + 8, x11 * va + loadu(c1 + 8));
            storeu(c1 + 16, x21 * va + loadu(c1 + 16));
            c0 += P_COLS_PER_LOOP * P_SIMD;
            c1 += P_COLS_PER_LOOP * P_SIMD;
        }
    }
    if (m < p->M) { /* odd last row */
        float *c0 = C;
        for (int n = 0; n < P_VEC_PER_ROW; n += P_COLS_PER_LOOP) {
            const v8f *bc = &p->bb[n];
            v8f x00 = splat(0.f), x10 = splat(0.f), x20 = splat(0.f);
            for (int k = 0; k < P_BB_ROWS; k++) {
                v8f a0 = splat(A[k]);
                x00 = x00 + a0 * bc[0];
                x10 = x10 + a0 * bc[1];
                x20 = x20 + a0 * bc[2];
                bc += P_VEC_PER_ROW;
            }
            storeu(c0 + 0, x00 * va + loadu(c0 + 0));
            storeu(c0 + 8, x10 * va + loadu(c0 + 8));
            storeu(c0 + 16, x20 * va + loadu(c0 + 16));
            c0 += P_COLS_PER_LOOP * P_SIMD;
        }
    }
}

/* sgemm_avx256.h:127-209: full-width columns, fewer than 35 k rows. */
static void port_bottom(const port_prm_t *p, const float *A, float *C, int nrows)
{
    const int lda = p->lda, ldc = p->ldc;
    const v8f va = splat(p->alpha);
    int m;
    for (m = 0; m < p->M - 1; A += 2 * lda, C += 2 * ldc, m += 2) {
        float *c0 = C, *c1 = C + ldc;
        for (int n = 0; n < P_VEC_PER_ROW; n += P_COLS_PER_LOOP) {
            const v8f *bc = &p->bb[n];
            v8f x00 = splat(0.f), x01 = splat(0.f), x10 = splat(0.f);
            v8f x11 = splat(0.f), x20 = splat(0.f), x21 = splat(0.f);
            for (int k = 0; k < nrows; k++) {
                v8f a0 = splat(A[k]), a1 = splat(A[k + lda]);
                x00 = x00 + a0 * bc[0]; x01 = x01 + a1 * bc[0];
                x10 = x10 + a0 * bc[1]; x11 = x11 + a1 * bc[1];
                x20 = x20 + a0 * bc[2]; x21 = x21 + a1 * bc[2];
                bc += P_VEC_PER_ROW;
            }
            storeu(c0 + 0, x00 * va + loadu(c0 + 0));
            storeu(c0 + 8, x10 * va + loadu(c0 + 8));
            storeu(c0 + 16, x20 * va + loadu(c0 + 16));
            storeu(c1 + 0, x01 * va + loadu(c1 + 0));
            storeu(c1 + 8, x11 * va + loadu(c1 + 8));
            storeu(c1 + 16, x21 * va + loadu(c1 + 16));
            c0 += P_COLS_PER_LOOP * P_SIMD;
            c1 += P_COLS_PER_LOOP * P_SIMD;
        }
    }
    if (m < p->M) {
        float *c0 = C;
        for (int n = 0; n < P_VEC_PER_ROW; n += P_COLS_PER_LOOP) {
            const v8f *bc = &p->bb[n];
            v8f x00 = splat(0.f), x10 = splat(0.f), x20 = splat(0.f);
            for (int k = 0; k < nrows; k++) {
                v8f a0 = splat(A[k]);
                x00 = x00 + a0 * bc[0];
                x10 = x10 + a0 * bc[1];
                x20 = x20 + a0 * bc[2];
                bc += P_VEC_PER_ROW;
            }
            storeu(c0 + 0, x00 * va + loadu(c0 + 0));
            storeu(c0 + 8, x10 * va + loadu(c0 + 8));
            storeu(c0 + 16, x20 * va + loadu(c0 + 16));
            c0 += P_COLS_PER_LOOP * P_SIMD;
        }
    }
}

/* sgemm_avx256.h:211-306: the rightmost (narrower than 96) columns.  Partial
 * products alpha*acc go to the cc buffer in 32-row slabs, then C[n] += cc[n]
 * (a separate add, never fused with the multiply). */
static void port_rightmost(port_prm_t *p, const float *A, float *C, int ncols, int nrows)
{
    const int lda = p->lda, ldc = p->ldc;
    const int ldcc = ((ncols - 1) / (P_COLS_PER_LOOP * P_SIMD) + 1) * P_COLS_PER_LOOP;
    const v8f va = splat(p->alpha);
    for (int m0 = 0; m0 < p->M; m0 += P_CC_ROWS) {
        const int mlast = (m0 + P_CC_ROWS <= p->M) ? m0 + P_CC_ROWS : p->M;
        v8f *pc = p->cc;
        const int mlast_even = mlast & ~1;
        for (int m = m0; m < mlast_even; A += 2 * lda, m += 2) {
            for (int n = 0; n < ldcc; n += P_COLS_PER_LOOP) {
                const v8f *bc = &p->bb[n];
                v8f x00 = splat(0.f), x01 = splat(0.f), x10 = splat(0.f);
                v8f x11 = splat(0.f), x20 = splat(0.f), x21 = splat(0.f);
                for (int k = 0; k < nrows; k++) {
                    v8f a0 = splat(A[k]), a1 = splat(A[k + lda]);
                    x00 = x00 + a0 * bc[0]; x01 = x01 + a1 * bc[0];
                    x10 = x10 + a0 * bc[1]; x11 = x11 + a1 * bc[1];
                    x20 = x20 + a0 * bc[2]; x21 = x21 + a1 * bc[2];
                    bc += P_VEC_PER_ROW;
                }
                pc[0] = x00 * va; pc[1] = x10 * va; pc[2] = x20 * va;
                pc[ldcc + 0] = x01 * va; pc[ldcc + 1] = x11 * va; pc[ldcc + 2] = x21 * va;
                pc += P_COLS_PER_LOOP;
            }
            pc += ldcc;
        }
        if (mlast & 1) {
            for (int n = 0; n < ldcc; n += P_COLS_PER_LOOP) {
                const v8f *bc = &p->bb[n];
                v8f x00 = splat(0.f), x10 = splat(0.f), x20 = splat(0.f);
                for (int k = 0; k < nrows; k++) {
                    v8f a0 = splat(A[k]);
                    x00 = x00 + a0 * bc[0];
                    x10 = x10 + a0 * bc[1];
                    x20 = x20 + a0 * bc[2];
                    bc += P_VEC_PER_ROW;
                }
                pc[0] = x00 * va; pc[1] = x10 * va; pc[2] = x20 * va;
                pc += P_COLS_PER_LOOP;
            }
        }
        pc = p->cc;
        for (int m = 0; m < mlast - m0; C += ldc, pc += ldcc, m++) {
            const float *res = (const float *)pc;
            for (int n = 0; n < ncols; n++) C[n] += res[n];
        }
    }
}

/* sgemm_avx256.h:308-390 (avx256_noncblas_sgemm): row-major NN,
 * C = beta*C (or 0), then accumulate alpha*A*B block by block. */
void oracle_sgemm_avx256(int M, int N, int K, float alpha, const float *A, int lda,
                         const float *B, int ldb, float beta, float *C, int ldc)
{
    float *c = C;
    for (int m = 0; m < M; m++, c += ldc)
        for (int n = 0; n < N; n++) c[n] = (beta != 0) ? c[n] * beta : 0.f;

    port_prm_t *p = (port_prm_t *)aligned_alloc(64, sizeof(port_prm_t));
    if (!p) return;
    p->M = M; p->lda = lda; p->ldc = ldc; p->alpha = alpha;
    const int rsteps = K / P_BB_ROWS, csteps = N / P_BB_COLS;
    int row = 0;
    for (int ri = 0; ri < rsteps; ri++, row += P_BB_ROWS) {
        int col = 0;
        for (int ci = 0; ci < csteps; ci++, col += P_BB_COLS) {
            for (int i = 0; i < P_BB_ROWS; i++)
                memcpy(&p->bb[P_VEC_PER_ROW * i], &B[(size_t)(row + i) * ldb + col],
                       P_BB_COLS * sizeof(float));
            port_core(p, &A[row], &C[col]);
        }
        if (col < N) {
            for (int i = 0; i < P_BB_ROWS; i++)
                memcpy(&p->bb[P_VEC_PER_ROW * i], &B[(size_t)(row + i) * ldb + col],
                       (size_t)(N - col) * sizeof(float));
            port_rightmost(p, &A[row], &C[col], N - col, P_BB_ROWS);
        }
    }
    if (row < K) {
        int col = 0;
        for (int ci = 0; ci < csteps; ci++, col += P_BB_COLS) {
            for (int i = 0; i < K - row; i++)
                memcpy(&p->bb[P_VEC_PER_ROW * i], &B[(size_t)(row + i) * ldb + col],
                       P_BB_COLS * sizeof(float));
            port_bottom(p, &A[row], &C[col], K - row);
        }
        if (col < N) {
            for (int i = 0; i < K - row; i++)
                memcpy(&p->bb[P_VEC_PER_ROW * i], &B[(size_t)(row + i) * ldb + col],
                       (size_t)(N - col) * sizeof(float));
            port_rightmost(p, &A[row], &C[col], N - col, K - row);
        }
    }
    free(p);
}

/* ------------------------------------------------------------------------ */
/* Band-parallel harness for the CPU baseline.  The AVX256 kernel keeps all   */
/* state in its parameter block, so row bands of C can run concurrently.      */
/* Transposed operands are first transposed into scratch (part of the timed  */
/* work), because the reference kernel is NN only (sgemm_avx256.h:433-453).  */
/* ------------------------------------------------------------------------ */
typedef struct {
    int m0, m1, N, K;
    float alpha, beta;
    const float *A; int lda;
    const float *B; int ldb;
    float *C; int ldc;
} band_t;

static void *band_worker(void *arg)
{
    band_t *b = (band_t *)arg;
    if (b->m1 > b->m0)
        oracle_sgemm_avx256(b->m1 - b->m0, b->N, b->K, b->alpha, b->A + (size_t)b->m0 * b->lda,
                            b->lda, b->B, b->ldb, b->beta, b->C + (size_t)b->m0 * b->ldc, b->ldc);
    return NULL;
}

typedef struct { const float *src; float *dst; int rows, cols, lds, r0, r1; } tr_t;

static void *transpose_worker(void *arg)
{
    tr_t *t = (tr_t *)arg; /* dst[c][r] = src[r][c] for rows r in [r0, r1) */
    for (int r = t->r0; r < t->r1; r++)
        for (int c = 0; c < t->cols; c++) t->dst[(size_t)c * t->rows + r] = t->src[(size_t)r * t->lds + c];
    return NULL;
}

static int run_parallel(int nthreads, void *(*fn)(void *), void *args, size_t argsz)
{
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    if (!th) return -2;
    int started = 0;
    for (int i = 1; i < nthreads; i++) {
        if (pthread_create(&th[i], NULL, fn, (char *)args + argsz * i) != 0) break;
        started = i;
    }
    fn(args);
    for (int i = 1; i <= started; i++) pthread_join(th[i], NULL);
    for (int i = started + 1; i < nthreads; i++) fn((char *)args + argsz * i);
    free(th);
    return 0;
}

static float *transpose_mt(int nthreads, const float *src, int rows, int cols, int lds)
{
    float *dst = (float *)malloc(sizeof(float) * (size_t)rows * cols);
    if (!dst) return NULL;
    tr_t *t = (tr_t *)malloc(sizeof(tr_t) * (size_t)nthreads);
    if (!t) { free(dst); return NULL; }
    for (int i = 0; i < nthreads; i++) {
        t[i].src = src; t[i].dst = dst; t[i].rows = rows; t[i].cols = cols; t[i].lds = lds;
        t[i].r0 = (int)((long long)rows * i / nthreads);
        t[i].r1 = (int)((long long)rows * (i + 1) / nthreads);
    }
    run_parallel(nthreads, transpose_worker, t, sizeof(tr_t));
    free(t);
    return dst;
}

/* Row-major C(MxN) = alpha*op(A)*op(B) + beta*C on `nthreads` threads. */
int oracle_sgemm_avx256_mt(int nthreads, char ta, char tb, int M, int N, int K, float alpha,
                           const float *A, int lda, const float *B, int ldb, float beta,
                           float *C, int ldc)
{
    if ((ta != 'N' && ta != 'T') || (tb != 'N' && tb != 'T') || nthreads < 1) return -1;
    float *at = NULL, *bt = NULL;
    if (ta == 'T') { at = transpose_mt(nthreads, A, K, M, lda); if (!at) return -2; A = at; lda = K; }
    if (tb == 'T') { bt = transpose_mt(nthreads, B, N, K, ldb); if (!bt) { free(at); return -2; } B = bt; ldb = N; }
    band_t *b = (band_t *)malloc(sizeof(band_t) * (size_t)nthreads);
    if (!b) { free(at); free(bt); return -2; }
    for (int i = 0; i < nthreads; i++) {
        b[i].m0 = (int)((long long)M * i / nthreads);
        b[i].m1 = (int)((long long)M * (i + 1) / nthreads);
        b[i].N = N; b[i].K = K; b[i].alpha = alpha; b[i].beta = beta;
        b[i].A = A; b[i].lda = lda; b[i].B = B; b[i].ldb = ldb; b[i].C = C; b[i].ldc = ldc;
    }
    run_parallel(nthreads, band_worker, b, sizeof(band_t));
    free(b); free(at); free(bt);
    return 0;
}

