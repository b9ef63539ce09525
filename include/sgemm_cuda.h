/*
 * sgemm_cuda.h -- GB300 (sm_103a) SGEMM backend for ugemm: C ABI of
 * libugemm_cuda.so.
 *
 * Drop-in for the reference's GPU entry point (sgemm_ocl2.h:158-224, same
 * API in sgemm_ocl.h:606-665 and sgemm_ocl1.h:159-252) and for its CPU GEMM
 * signature (ugemm.h:287-301, the `uut` pointer of check_sgemm.c:96-103).
 * All matrices are FP32.  Row-major unless a `major` argument says 'C'.
 *
 * Semantics kept from the reference:
 *   - C = alpha * op(A) * op(B) + beta * C, op(X) = X ('N') or X^T ('T');
 *   - sgemm_cuda: tight leading dimensions; ta == 'T' means A is stored K x M,
 *     tb == 'T' means B is stored N x K (sgemm_ocl2.h:180-199);
 *   - beta == 0 means C is not read, so NaNs in C do not propagate
 *     (sgemm_ocl2.h:86-88, :177);
 *   - one process-wide context for the compat API, set up by *_init and torn
 *     down by *_finish (sgemm_ocl2.h:133-165, :220-224).
 * Added: status codes instead of silent failure, device-pointer and stream
 * entry points, split-precision tensor-core forms, the adjoint, grouped GEMM.
 */
#ifndef UGEMM_SGEMM_CUDA_H
#define UGEMM_SGEMM_CUDA_H

#include <stddef.h>

#if defined(__GNUC__)
#define UGEMM_API __attribute__((visibility("default")))
#else
#define UGEMM_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  UGEMM_OK = 0,
  UGEMM_ERR_ARG = 1,              /* bad transpose flag, size, leading dimension or pointer */
  UGEMM_ERR_ALLOC = 2,            /* device or host allocation failed */
  UGEMM_ERR_ARENA_TOO_SMALL = 3,  /* the init-time arena cannot hold this call */
  UGEMM_ERR_CUDA = 4,             /* a CUDA runtime/driver call failed */
  UGEMM_ERR_TIMEOUT = 5,          /* a kernel's bounded wait gave up (pipeline fault) */
  UGEMM_ERR_NOT_INIT = 6,         /* compat call before sgemm_cuda_init */
  UGEMM_ERR_UNSUPPORTED = 7,      /* no sm_103a device, or a form not available */
} ugemm_status;

/* Arithmetic form of a GEMM. */
typedef enum {
  UGEMM_PREC_AUTO = 0,   /* split-precision tensor cores when the problem is large enough */
  UGEMM_PREC_SIMT = 1,   /* plain FP32 FMA on the CUDA cores */
  UGEMM_PREC_BF16X6 = 2, /* 3 bf16 pieces per operand, 6 piece products (tcgen05) */
  UGEMM_PREC_BF16X9 = 3, /* 3 bf16 pieces per operand, all 9 piece products (tcgen05) */
  UGEMM_PREC_BF16X3 = 4, /* 2 bf16 pieces, 3 products: ~16-bit accuracy, for error studies */
  UGEMM_PREC_FP16X3 = 5, /* 2 fp16 pieces per element, every row of op(A) and column of op(B)
                            scaled by its own power of two; 3 products (tcgen05): 22-bit
                            operands, half the MMAs of BF16X6 */
  UGEMM_PREC_TF32X3 = 6, /* 2 tf32 pieces per element (FP32's exponent range, no scaling),
                            3 products on the tf32 tensor path (tcgen05 kind::tf32, half the
                            16-bit rate): 22-bit operands */
} ugemm_precision;

/* ------------------------------------------------------------------ */
/* Compat API: mirrors sgemm_ocl_init / sgemm_ocl / sgemm_ocl_finish.   */
/* ------------------------------------------------------------------ */

/* sgemm_ocl2.h:158 (sgemm_ocl_init).  `platform` is ignored (there is one
 * CUDA platform); `device` selects the CUDA device; `size` is the byte size of
 * the device arena that holds A, B, C and the call's scratch, as the
 * reference's single OpenCL buffer does (sgemm_test.c:29 passes
 * (M*K + K*N + M*N) * 10 * sizeof(float)).  Errors are kept in the last-error
 * slot (ugemm_last_error). */
UGEMM_API void sgemm_cuda_init(int platform, int device, size_t size);

/* sgemm_ocl2.h:166 (sgemm_ocl).  Host pointers; synchronous; copies A, B
 * (and C when beta != 0) to the device, runs the GEMM in the form chosen by
 * sgemm_cuda_set_precision (default UGEMM_PREC_AUTO) and copies C back. */
UGEMM_API void sgemm_cuda(char ta, char tb, int m, int n, int k, float alpha, float *a, float *b,
                float beta, float *c);

/* sgemm_ocl2.h:220 (sgemm_ocl_finish): frees the arena and the context. */
UGEMM_API void sgemm_cuda_finish(void);

/* Status-returning variant of sgemm_cuda (the compat call stores the same
 * status in the last-error slot). */
UGEMM_API int sgemm_cuda_status(char ta, char tb, int m, int n, int k, float alpha, const float *a,
                      const float *b, float beta, float *c);

/* Form used by sgemm_cuda / ugemm_sgemm (a ugemm_precision value). */
UGEMM_API int sgemm_cuda_set_precision(int precision);

/* Last status of a void entry point on this thread, and its message. */
UGEMM_API int ugemm_last_error(void);
UGEMM_API const char *ugemm_last_error_message(void);
UGEMM_API const char *ugemm_status_string(int status);

/* ------------------------------------------------------------------ */
/* BLAS-style host API: the signature of ugemm.h:287 (sgemm_cpu) and of */
/* the uut pointer in check_sgemm.c:96-103; works with or without init. */
/* ------------------------------------------------------------------ */
UGEMM_API void ugemm_sgemm(char major, char transa, char transb, int M, int N, int K, float alpha,
                 const float *A, int lda, const float *B, int ldb, float beta, float *C,
                 int ldc);
UGEMM_API int ugemm_sgemm_host(char major, char transa, char transb, int M, int N, int K, float alpha,
                     const float *A, int lda, const float *B, int ldb, float beta, float *C,
                     int ldc, int precision);

/* ------------------------------------------------------------------ */
/* Device-pointer, stream-ordered API (no reference counterpart: the     */
/* reference only has host pointers).  `stream` is a cudaStream_t (NULL */
/* = legacy default stream).  Scratch comes from a library-owned device */
/* workspace that grows on demand; reserve it with                      */
/* ugemm_reserve_workspace before capturing these calls in a CUDA graph. */
/* ------------------------------------------------------------------ */
UGEMM_API int ugemm_sgemm_dev(char major, char transa, char transb, int M, int N, int K, float alpha,
                    const float *A, int lda, const float *B, int ldb, float beta, float *C,
                    int ldc, int precision, void *stream);

/* Allocation-free variant of ugemm_sgemm_dev for the split-precision forms
 * (UGEMM_PREC_AUTO, BF16X6, BF16X9, BF16X3).  It has no counterpart in the
 * reference.  It is for callers that must not allocate device memory while
 * they run -- a process whose device-memory budget is fixed at start-up, a
 * framework whose own allocator owns all device memory, a latency-critical
 * loop where an allocation could stall or fail -- and it calls no
 * cudaMalloc, cudaFree or allocating routine.  The split pieces of A and B
 * live in a fixed 64 MiB array in the library's device memory, held by every
 * GPU that loads the library until the process exits; calls whose scratch
 * exceeds it return UGEMM_ERR_ARENA_TOO_SMALL.  The scratch of a call is
 * exactly ugemm_workspace_bytes with the same arguments: about
 * 6 * (M + N) * roundup(K, 32) bytes of pieces for the three-piece forms,
 * plus, when the last wave of output tiles runs as the wave-tail launch, its
 * partial tiles.  The first call on a device looks up the array's device
 * address (with that device current); make that first call before any stream
 * capture.  All calls share the array: calls that overlap on the GPU (other
 * streams or host threads) race on it.  A kernel wait that gives up is
 * reported by ugemm_check.  Device pointers, stream-ordered, same arguments
 * as ugemm_sgemm_dev. */
UGEMM_API int ugemm_sgemm_dev_noalloc(char major, char transa, char transb, int M, int N, int K,
                                      float alpha, const float *A, int lda, const float *B,
                                      int ldb, float beta, float *C, int ldc, int precision,
                                      void *stream);

/* ugemm_sgemm_dev with a fused epilogue (row-major only):
 *   C = act(alpha*op(A)*op(B) + beta*C + bias[row]),
 * bias: M floats on the device or NULL; act: 0 none, 1 LeakyReLU with
 * `slope` (0.1 is the reference's; 0 gives ReLU).  This moves the
 * reference's post-GEMM loop of gl_convolution_LReLU (sgemm_gl1.h:210-217:
 * add the channel bias, then x > 0 ? x : 0.1*x) into the GEMM epilogue; the
 * leak is applied in FP32 (the reference multiplies by the double 0.1). */
UGEMM_API int ugemm_sgemm_dev_ex(char major, char transa, char transb, int M, int N, int K,
                                 float alpha, const float *A, int lda, const float *B, int ldb,
                                 float beta, float *C, int ldc, const float *bias, int act,
                                 float slope, int precision, void *stream);

/* Scratch bytes ugemm_sgemm_dev needs for this call (0 for most SIMT calls). */
UGEMM_API size_t ugemm_workspace_bytes(char major, char transa, char transb, int M, int N, int K,
                             int lda, int ldb, int precision);
/* Grow the current device's workspace to at least `bytes`. */
UGEMM_API int ugemm_reserve_workspace(size_t bytes);

/* Adjoint of C = alpha*op(A)*op(B) + beta*C (spec differentiation form;
 * no reference counterpart).  Given dC (M x N, row-major, lddc), writes
 *   dA = alpha * dC * op(B)^T  (stored like A: M x K if transa=='N', else K x M)
 *   dB = alpha * op(A)^T * dC  (stored like B: K x N if transb=='N', else N x K)
 * as dX = grad + beta_x * dX (beta_x == 0: dX is not read).  dA or dB may be
 * NULL to skip it.  Device pointers, row-major. */
UGEMM_API int ugemm_sgemm_backward(char transa, char transb, int M, int N, int K, float alpha,
                         const float *A, int lda, const float *B, int ldb, const float *dC,
                         int lddc, float beta_a, float *dA, int ldda, float beta_b, float *dB,
                         int lddb, int precision, void *stream);

/* Report a kernel wait timeout of the device-pointer calls (no reference
 * counterpart: the reference reports no device errors).  The calls above are
 * stream-ordered and return before their kernels run, so a bounded wait that
 * gives up (UGEMM_ERR_TIMEOUT on the host-pointer calls) cannot be returned
 * by them; it is recorded in a per-device error word instead.  This call
 * synchronises `stream`, reads the word of ugemm_sgemm_dev, _dev_ex,
 * ugemm_sgemm_backward and ugemm_sgemm_dev_noalloc on the current device,
 * clears it and returns UGEMM_ERR_TIMEOUT (with the code in the last-error
 * message) if any of their kernels gave up since the last check, else
 * UGEMM_OK.  A stale code never disturbs a later call: each call moves it
 * aside before its own kernels run.  The word is per device, shared by all
 * streams.  (Grouped plans have their own word: ugemm_grouped_check.) */
UGEMM_API int ugemm_check(void *stream);

/* Test hook for the error reporting above (no reference counterpart): writes
 * `code` into an error word of the current device with a synchronous host
 * copy, as a timed-out kernel wait would -- which 0: the device-pointer
 * calls' word, 1: the allocation-free entry point's (after its first call
 * on the device).  Launches nothing; for tests of ugemm_check only. */
UGEMM_API int ugemm_debug_set_error_word(int which, int code);

/* FP64 GEMM on the GPU, C = alpha*op(A)*op(B) + beta*C on device pointers
 * (same argument meaning as ugemm_sgemm_dev, double precision, no precision
 * argument).  The accuracy oracle of the FP32 forms at sizes the reference's
 * FP64 CPU GEMMs (dgemm_cpu, ugemm.h:162; _dgemm_c, gemm_cpu.h:284;
 * dgemm_avx, dgemm_avx.h:844) cannot reach in test time: one FP64 fused
 * multiply-add chain over k per element, no emulation.  Not on the FP32
 * product path. */
UGEMM_API int ugemm_dgemm_oracle_dev(char major, char transa, char transb, int M, int N, int K,
                                     double alpha, const double *A, int lda, const double *B,
                                     int ldb, double beta, double *C, int ldc, void *stream);

/* Device information: SM count and compute capability of the current device. */
UGEMM_API int ugemm_device_info(int *sm_count, int *cc_major, int *cc_minor);

/* ------------------------------------------------------------------ */
/* Grouped GEMM (spec batching form; no reference counterpart).  */
/* Many independent row-major problems, one batched pre-pass launch and */
/* one persistent GEMM launch; the plan can hold a CUDA graph of both.  */
/* ------------------------------------------------------------------ */
typedef struct {
  char transa, transb; /* 'N' or 'T', as in sgemm_cuda */
  int M, N, K;
  float alpha, beta;
  const float *A; /* device pointers */
  int lda;
  const float *B;
  int ldb;
  float *C;
  int ldc;
  const float *bias; /* optional fused epilogue, as in ugemm_sgemm_dev_ex (NULL: none) */
  int act;           /* 0 none, 1 LeakyReLU(slope) */
  float slope;
} ugemm_problem;

/* Tile configuration and schedule of a grouped launch (chosen by
 * ugemm_tune_grouped; all zero = the library's defaults). */
typedef struct {
  int block_n;   /* split form: CTA tile width 128 or 256; SIMT form: square tile 64 or 128 */
  int chunk_k;   /* split form: k depth between main-accumulator drains (multiple of 32) */
  int max_ctas;  /* persistent CTAs; 0 = one per SM */
  int split_k;   /* split-K threshold: a problem whose tiles are longer than the launch's
                    k-work / (split_k * CTAs) is cut into k slices of about that length;
                    0 = 2, negative = never split */
  int deal;      /* split form: tiles dealt to the persistent CTAs 0 = longest first to the
                    least-loaded CTA, 1 = round robin */
  int transpose; /* split form: 0 = compute C^T = op(B)^T op(A)^T where that wastes less of
                    the 128-row tiles, 1 = never */
  int fused;     /* BF16X6 / BF16X9: 1 = the GEMM kernel copies the FP32 operands with TMA
                    and splits them itself (no pre-pass, no pieces in memory), 0 = a
                    pre-pass launch writes the pieces first.  Taken only when
                    every problem has k > 0, unit-stride operands and 16-byte aligned bases
                    and leading dimensions (implicit im2col operands take the pre-pass);
                    the plan's config reports whether it was */
} ugemm_tile_config;

typedef struct ugemm_grouped_plan_s ugemm_grouped_plan;

#define UGEMM_PLAN_GRAPH 1 /* capture the plan's launches once into a CUDA graph */

/* Build a plan (allocates its scratch and device tables; do this outside
 * stream capture).  `config` NULL: the tuned configuration cached for this
 * problem set (UGEMM_TUNE_CACHE file), else a default.  Problems keep their
 * device pointers: a plan replays on the same buffers. */
UGEMM_API int ugemm_grouped_plan_create(int count, const ugemm_problem *problems, int precision,
                                        const ugemm_tile_config *config, int flags,
                                        ugemm_grouped_plan **plan);
/* Enqueue the plan on `stream` (graph launch when built with UGEMM_PLAN_GRAPH). */
UGEMM_API int ugemm_grouped_run(ugemm_grouped_plan *plan, void *stream);
/* Synchronise `stream` and report a kernel wait timeout of this plan. */
UGEMM_API int ugemm_grouped_check(ugemm_grouped_plan *plan, void *stream);
UGEMM_API int ugemm_grouped_plan_destroy(ugemm_grouped_plan *plan);
UGEMM_API double ugemm_grouped_flops(const ugemm_grouped_plan *plan);
UGEMM_API int ugemm_grouped_config(const ugemm_grouped_plan *plan, ugemm_tile_config *config);
/* One-shot: plan, run, check, destroy (synchronous). */
UGEMM_API int ugemm_sgemm_grouped(int count, const ugemm_problem *problems, int precision,
                                  void *stream);

/* Autotuner: time candidate configurations of this problem set and form on
 * the current device (CUDA events, after warm-up; the best of three timed
 * batches each) -- first the tile shape (block_n x chunk_k), then, one knob
 * at a time from the best so far, the split-K threshold, the tile deal, the
 * transposed tiles and the persistent grid size -- return the fastest and
 * remember it in the tuning cache (JSON lines at $UGEMM_TUNE_CACHE, default
 * ./ugemm_tune_cache.jsonl; each line also lists every candidate with its
 * time).  A cached entry is returned without timing unless `force` is
 * non-zero.  The problems' C buffers are overwritten while timing. */
UGEMM_API int ugemm_tune_grouped(int count, const ugemm_problem *problems, int precision,
                                 int force, ugemm_tile_config *best, double *best_ms);

/* ------------------------------------------------------------------ */
/* im2col convolution (sgemm_ocl1.h:81-119 im2col, :271-300              */
/* ocl_convolution).  Activations are C x (B*H*W) ("CNHW"); with B = 1    */
/* this is the reference's CHW image and its im2col matrix               */
/* (C*k*k) x (Ho*Wo), row (c*k*k + ki*k + kj), column (i*Wo + j).        */
/* ------------------------------------------------------------------ */
UGEMM_API int ugemm_im2col(const float *x, int channels, int batch, int height, int width,
                           int ksize, int pad, int stride, float *col, void *stream);
/* Adjoint of ugemm_im2col: x = sum of the col entries that read it (overwrites x). */
UGEMM_API int ugemm_col2im(const float *col, int channels, int batch, int height, int width,
                           int ksize, int pad, int stride, float *x, void *stream);

/* A stack of convolutions run as GEMMs: layer l computes
 *   forward  Y_l = W_l * im2col(X_l)                 (M = cout, N = B*Ho*Wo, K = cin*k*k)
 *   backward dW_l = dY_l * col_l^T, dcol_l = W_l^T * dY_l (one grouped launch),
 *            dX_l = col2im(dcol_l) = dY_{l-1}
 * with X_{l+1} = Y_l.  By default the GEMMs read col_l = im2col(X_l)
 * implicitly: the operand pass of the forward and dW GEMMs gathers it from
 * X_l, and no col buffer exists; in the split forms a stride-1 layer's dX is
 * then one GEMM, dX_l = Wt_l * im2col(dY_l, pad k-1-p) with Wt_l the weights
 * transposed in the channels and flipped in the taps, and has no dcol
 * buffer.  UGEMM_CONV_IM2COL materialises col_l with an im2col pass first
 * and keeps dcol + col2im for every layer (the reference's formulation).  The gradient entering the last layer is its own
 * output (loss 0.5 * ||Y_last||^2).  With act == 1 a layer computes
 * Y_l = LeakyReLU(W_l * col_l + bias_l) in the GEMM epilogue
 * (gl_convolution_LReLU, sgemm_gl1.h:192-218), and its backward first scales
 * dY_l by the activation's slope where Y_l <= 0 and sums it into dbias_l.  No
 * reference counterpart beyond the single-layer forward ocl_convolution. */
typedef struct {
  int cin, cout, height, width; /* input channels/size of the layer */
  int ksize, pad, stride;       /* square kernel, equal padding and stride */
  int act;                      /* 0: Y = W*col; 1: Y = LeakyReLU(W*col + bias, slope) */
  float slope;                  /* leak of the activation (the reference uses 0.1) */
} ugemm_conv_layer;

typedef struct ugemm_conv_stack_s ugemm_conv_stack;

#define UGEMM_CONV_FORWARD 1
#define UGEMM_CONV_BACKWARD 2
#define UGEMM_CONV_IM2COL 2 /* create flag (with UGEMM_PLAN_GRAPH = 1): explicit im2col */
enum {
  UGEMM_CONV_X = 0, /* layer input (fill layer 0's before a forward run) */
  UGEMM_CONV_W = 1, /* weights, cout x cin*k*k (fill before running) */
  UGEMM_CONV_Y = 2,
  UGEMM_CONV_COL = 3, /* UGEMM_CONV_IM2COL stacks only */
  UGEMM_CONV_DW = 4,
  UGEMM_CONV_DCOL = 5, /* not for the direct-dX layers of implicit stacks */
  UGEMM_CONV_DX = 6,
  UGEMM_CONV_DY = 7,
  UGEMM_CONV_BIAS = 8, /* cout floats, used when act == 1 (fill before running) */
  UGEMM_CONV_DBIAS = 9 /* cout floats, written by the backward run when act == 1 */
};

/* Allocates every buffer and one grouped plan per layer and direction; with
 * UGEMM_PLAN_GRAPH the forward, backward and combined sequences are
 * captured into CUDA graphs. */
UGEMM_API int ugemm_conv_stack_create(int nlayers, const ugemm_conv_layer *layers, int batch,
                                      int precision, int flags, ugemm_conv_stack **stack);
/* Device pointer and element count of one buffer of one layer. */
UGEMM_API int ugemm_conv_stack_buffer(ugemm_conv_stack *stack, int layer, int which, float **ptr,
                                      size_t *count);
/* Run forward (1), backward (2) or both (3) on `stream`. */
UGEMM_API int ugemm_conv_stack_run(ugemm_conv_stack *stack, int what, void *stream);
UGEMM_API double ugemm_conv_stack_flops(const ugemm_conv_stack *stack, int what);
UGEMM_API int ugemm_conv_stack_destroy(ugemm_conv_stack *stack);

/* ------------------------------------------------------------------ */
/* Level-1/2 helpers of ugemm.h, on device pointers (stream-ordered).  */
/* ------------------------------------------------------------------ */
/* saxpy_cpu (ugemm.h:86-97): y[i*incy] += alpha * x[i*incx], i < N. */
UGEMM_API int ugemm_saxpy(int N, float alpha, const float *x, int incx, float *y, int incy,
                          void *stream);
/* sgemv_cpu (ugemm.h:129-160), column-major A: trans 'N': A is M x N,
 * y = alpha*A*x + beta*y; trans 'T': A is N x M, y = alpha*A^T*x + beta*y
 * (y has M entries, x has N in both cases, as in the reference).  x is read
 * with stride incx (the reference reads x with incy; the two agree whenever
 * incx == incy); beta == 0 means y is not read. */
UGEMM_API int ugemm_sgemv(char trans, int M, int N, float alpha, const float *A, int lda,
                          const float *x, int incx, float beta, float *y, int incy,
                          void *stream);

/* Per-kernel timing for benchmarks (no reference counterpart; the reference's
 * oclTime at ocl.h:344-352 is never enabled).  While enabled, each library
 * kernel launch is bracketed by CUDA events on its own stream.  collect()
 * synchronises, returns the summed milliseconds and launch counts per kind
 * (0 SIMT GEMM, 1 split pre-pass, 2 split tcgen05 GEMM, 3 auxiliary, 4 grouped
 * GEMM, 5 control: the one-thread error-word fold that starts each
 * device-pointer call, 6 copy: the copy kernels that read pageable host
 * buffers) and clears the record. */
UGEMM_API int ugemm_profile_enable(int on);
UGEMM_API int ugemm_profile_collect(double *ms_per_kind, int *launches_per_kind, int nkinds);

/* Measured FP32 FMA peak of the current device in TFLOP/s (no reference
 * counterpart; measurement infrastructure: the roofline of the plain SIMT
 * form).  Runs eight independent FMA chains per thread, 32 warps per SM, for
 * about `ms` milliseconds after a warm-up launch, timed with CUDA events. */
UGEMM_API int ugemm_fp32_peak(double ms, double *tflops);

/* Failure-detection self-test (no reference counterpart; the reference's
 * OpenCL calls have no device-side failure detection).  Runs one small
 * kernel whose threads wait, through the library's bounded mbarrier wait with
 * a 100 ms limit, on a barrier nothing arrives on.  Returns
 * UGEMM_ERR_TIMEOUT with the recorded device error code (1: a pipeline stage
 * never filled), the number of threads that gave up and returned, and the
 * wall time; the CUDA context stays usable.  Faults, traps and hangs nothing. */
UGEMM_API int ugemm_selftest_wait_timeout(int *code, int *threads_returned, double *seconds);

#ifdef __cplusplus
}
#endif
#endif /* UGEMM_SGEMM_CUDA_H */
