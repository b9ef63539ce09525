// conv.cu -- im2col / col2im kernels and the im2col convolution stack
// (forward, dX and dW of every layer as split-precision or SIMT grouped
// GEMMs, optionally captured in one CUDA graph).
//
// The reference convolves one image at a time: its OpenCL im2col
// (sgemm_ocl1.h:81-119) turns a CHW image into a (C*k*k) x (Ho*Wo) matrix and
// ocl_convolution (sgemm_ocl1.h:271-300) multiplies the weights
// (Cout x C*k*k) by it.  Here activations are stored C x (B*H*W) ("CNHW"),
// so a whole batch is one im2col matrix (C*k*k) x (B*Ho*Wo) and one GEMM per
// layer; with B = 1 the layout and the im2col result are the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "internal.h"

namespace ugemm {
namespace {

// col[(c*k*k + ki*k + kj)][(b*Ho + i)*Wo + j] = x[c][b][i*s - p + ki][j*s - p + kj]
// (0 outside the image).  One thread per output pixel (c, b, i, j) writing
// its k*k column entries, as the reference's work-item per (c, i, j)
// (sgemm_ocl1.h:97-118).  Grid: y walks the image planes (c, b), x the
// pixels of a plane, so the index arithmetic is 32-bit and per plane; the
// common kernel sizes and strides are compile-time constants (0: runtime).
template <int KS, int ST>
__global__ void __launch_bounds__(256) im2col_kernel(const float* __restrict__ x, int C, int B,
                                                     int H, int W, int k_rt, int pad, int st_rt,
                                                     int Ho, int Wo, float* __restrict__ col) {
  const int k = KS ? KS : k_rt, stride = ST ? ST : st_rt;
  const int plane_px = Ho * Wo;
  const long long n_pix = static_cast<long long>(B) * plane_px;
  for (int plane = blockIdx.y; plane < C * B; plane += gridDim.y) {
    const int c = plane / B, b = plane - c * B;
    const float* src = x + static_cast<long long>(plane) * H * W;
    float* dst0 = col + static_cast<long long>(c) * k * k * n_pix + static_cast<long long>(b) * plane_px;
    for (int pix = blockIdx.x * 256 + threadIdx.x; pix < plane_px; pix += 256 * gridDim.x) {
      const int i = pix / Wo, j = pix - i * Wo;
      const int y0 = i * stride - pad, x0 = j * stride - pad;
      float* dst = dst0 + pix;
#pragma unroll
      for (int ki = 0; ki < k; ++ki) {
        const int yy = y0 + ki;
        const bool row_in = yy >= 0 && yy < H;
#pragma unroll
        for (int kj = 0; kj < k; ++kj) {
          const int xx = x0 + kj;
          *dst = (row_in && xx >= 0 && xx < W) ? src[yy * W + xx] : 0.f;
          dst += n_pix;
        }
      }
    }
  }
}

// Adjoint of im2col: dx[c][b][y][x] = sum of the col entries that read it,
// taps in (ki, kj) order (gather form: no atomics, deterministic).  Same
// plane-by-plane grid as im2col_kernel.
template <int KS, int ST>
__global__ void __launch_bounds__(256) col2im_kernel(const float* __restrict__ col, int C, int B,
                                                     int H, int W, int k_rt, int pad, int st_rt,
                                                     int Ho, int Wo, float* __restrict__ dx) {
  const int k = KS ? KS : k_rt, stride = ST ? ST : st_rt;
  const int plane_px = Ho * Wo, plane_in = H * W;
  const long long n_pix = static_cast<long long>(B) * plane_px;
  for (int plane = blockIdx.y; plane < C * B; plane += gridDim.y) {
    const int c = plane / B, b = plane - c * B;
    const float* src0 = col + static_cast<long long>(c) * k * k * n_pix + static_cast<long long>(b) * plane_px;
    float* dst = dx + static_cast<long long>(plane) * plane_in;
    for (int p = blockIdx.x * 256 + threadIdx.x; p < plane_in; p += 256 * gridDim.x) {
      const int yy = p / W, xx = p - yy * W;
      float acc = 0.f;
#pragma unroll
      for (int ki = 0; ki < k; ++ki) {
        const int ty = yy + pad - ki;
        if (ty < 0 || ty % stride) continue;
        const int i = ty / stride;
        if (i >= Ho) continue;
#pragma unroll
        for (int kj = 0; kj < k; ++kj) {
          const int tx = xx + pad - kj;
          if (tx < 0 || tx % stride) continue;
          const int j = tx / stride;
          if (j >= Wo) continue;
          acc += src0[(ki * k + kj) * n_pix + i * Wo + j];
        }
      }
      dst[p] = acc;
    }
  }
}

dim3 plane_grid(int planes, int plane_px) {
  return dim3(static_cast<unsigned>(std::min(cdiv(plane_px, 256), 64)),
              static_cast<unsigned>(std::min(planes, 65535)));
}

int out_dim(int in, int k, int pad, int stride) { return (in + 2 * pad - k) / stride + 1; }

// wt[c][(co*k + k-1-ki)*k + k-1-kj] = w[co][(c*k + ki)*k + kj]: the weights of
// the adjoint (transposed) convolution of a stride-1 layer.
__global__ void flip_weights_kernel(const float* __restrict__ w, int cout, int cin, int k,
                                    float* __restrict__ wt) {
  const int kk = k * k;
  const int total = cout * cin * kk;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += gridDim.x * blockDim.x) {
    const int co = idx / (cin * kk), rem = idx - co * cin * kk;
    const int c = rem / kk, t = rem - c * kk, ki = t / k, kj = t - ki * k;
    wt[(static_cast<long long>(c) * cout + co) * kk + (k - 1 - ki) * k + (k - 1 - kj)] = w[idx];
  }
}

// Backward of the fused epilogue Y = LeakyReLU(W*col + bias): the incoming
// gradient dY (C x n, in place) is multiplied by the activation's slope
// where Y <= 0, and dbias[c] = sum over the row of the masked gradient.  One
// block per channel; fixed-order tree reduction (deterministic).
__global__ void __launch_bounds__(256) leaky_backward_kernel(float* __restrict__ dy,
                                                             const float* __restrict__ y,
                                                             long long n, float slope,
                                                             float* __restrict__ dbias) {
  __shared__ float part[256];
  const long long base = static_cast<long long>(blockIdx.x) * n;
  float s = 0.f;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const float g = dy[base + i];
    const float m = y[base + i] > 0.f ? g : g * slope;
    dy[base + i] = m;
    s += m;
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) dbias[blockIdx.x] = part[0];
}

}  // namespace

ugemm_status im2col_launch(const float* x, int C, int B, int H, int W, int k, int pad, int stride,
                           float* col, cudaStream_t st) {
  const int Ho = out_dim(H, k, pad, stride), Wo = out_dim(W, k, pad, stride);
  if (Ho <= 0 || Wo <= 0) return UGEMM_ERR_ARG;
  const dim3 grid = plane_grid(C * B, Ho * Wo);
  prof_begin(st);
  if (k == 3 && stride == 1)
    im2col_kernel<3, 1><<<grid, 256, 0, st>>>(x, C, B, H, W, k, pad, stride, Ho, Wo, col);
  else if (k == 3 && stride == 2)
    im2col_kernel<3, 2><<<grid, 256, 0, st>>>(x, C, B, H, W, k, pad, stride, Ho, Wo, col);
  else
    im2col_kernel<0, 0><<<grid, 256, 0, st>>>(x, C, B, H, W, k, pad, stride, Ho, Wo, col);
  prof_end(st, kProfAux);
  return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

ugemm_status flip_weights_launch(const float* w, int cout, int cin, int k, float* wt,
                                cudaStream_t st) {
  const int total = cout * cin * k * k;
  prof_begin(st);
  flip_weights_kernel<<<std::min(cdiv(total, 256), 1024), 256, 0, st>>>(w, cout, cin, k, wt);
  prof_end(st, kProfAux);
  return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

ugemm_status col2im_launch(const float* col, int C, int B, int H, int W, int k, int pad,
                           int stride, float* dx, cudaStream_t st) {
  const int Ho = out_dim(H, k, pad, stride), Wo = out_dim(W, k, pad, stride);
  if (Ho <= 0 || Wo <= 0) return UGEMM_ERR_ARG;
  const dim3 grid = plane_grid(C * B, H * W);
  prof_begin(st);
  if (k == 3 && stride == 1)
    col2im_kernel<3, 1><<<grid, 256, 0, st>>>(col, C, B, H, W, k, pad, stride, Ho, Wo, dx);
  else if (k == 3 && stride == 2)
    col2im_kernel<3, 2><<<grid, 256, 0, st>>>(col, C, B, H, W, k, pad, stride, Ho, Wo, dx);
  else
    col2im_kernel<0, 0><<<grid, 256, 0, st>>>(col, C, B, H, W, k, pad, stride, Ho, Wo, dx);
  prof_end(st, kProfAux);
  return cudaPeekAtLastError() == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
}

}  // namespace ugemm

// ---------------------------------------------------------------- the stack
struct ugemm_conv_stack_s {
  struct Layer {
    ugemm_conv_layer d;
    int Ho, Wo;
    long long n;          // batch * Ho * Wo (GEMM N)
    int kdim;             // cin * k * k (GEMM K)
    float *x, *col, *w, *y, *dw, *dcol, *dx;  // dy of layer l is dx of layer l+1
    float *bias = nullptr, *dbias = nullptr;  // act == 1 only
    ugemm::Im2col im;     // im2col geometry of x (the implicit operand)
    // implicit stacks, stride 1: dX as one GEMM, the convolution of dY with
    // the flipped, transposed weights wt (no dcol, no col2im)
    bool direct_dx = false;
    float* wt = nullptr;  // cin x cout*k*k
    ugemm::Im2col dy_im;  // im2col geometry of dY for that GEMM
    ugemm_grouped_plan* fwd = nullptr;
    ugemm_grouped_plan* bwd = nullptr;
  };
  std::vector<Layer> layers;
  int batch = 0, form = UGEMM_PREC_BF16X6;
  bool explicit_col = false;  // UGEMM_CONV_IM2COL: materialise col per layer
  float* dy_last = nullptr;
  void* arena = nullptr;
  double flops_fwd = 0, flops_bwd = 0;
  cudaGraphExec_t exec[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaGraph_t graph[4] = {nullptr, nullptr, nullptr, nullptr};
};

namespace {
using Stack = ugemm_conv_stack_s;

int run_stack(Stack* s, int what, cudaStream_t st) {
  using namespace ugemm;
  if (what & UGEMM_CONV_FORWARD) {
    for (auto& L : s->layers) {
      if (s->explicit_col) {
        ugemm_status r = im2col_launch(L.x, L.d.cin, s->batch, L.d.height, L.d.width, L.d.ksize,
                                       L.d.pad, L.d.stride, L.col, st);
        if (r != UGEMM_OK) return r;
      }
      int rc = ugemm_grouped_run(L.fwd, st);
      if (rc != UGEMM_OK) return rc;
    }
  }
  if (what & UGEMM_CONV_BACKWARD) {
    for (int l = static_cast<int>(s->layers.size()) - 1; l >= 0; --l) {
      auto& L = s->layers[l];
      if (L.d.act) {  // dY *= LeakyReLU'(Y); dbias = row sums
        prof_begin(st);
        leaky_backward_kernel<<<L.d.cout, 256, 0, st>>>(
            (l + 1 < static_cast<int>(s->layers.size())) ? s->layers[l + 1].dx : L.y, L.y, L.n,
            L.d.slope, L.dbias);
        prof_end(st, kProfAux);
        if (cudaPeekAtLastError() != cudaSuccess) return UGEMM_ERR_CUDA;
      }
      if (L.direct_dx) {
        ugemm_status r = flip_weights_launch(L.w, L.d.cout, L.d.cin, L.d.ksize, L.wt, st);
        if (r != UGEMM_OK) return r;
      }
      int rc = ugemm_grouped_run(L.bwd, st);
      if (rc != UGEMM_OK) return rc;
      if (!L.direct_dx) {
        ugemm_status r = col2im_launch(L.dcol, L.d.cin, s->batch, L.d.height, L.d.width,
                                       L.d.ksize, L.d.pad, L.d.stride, L.dx, st);
        if (r != UGEMM_OK) return r;
      }
    }
  }
  return UGEMM_OK;
}

void destroy_stack(Stack* s) {
  if (!s) return;
  for (int i = 0; i < 4; ++i) {
    if (s->exec[i]) cudaGraphExecDestroy(s->exec[i]);
    if (s->graph[i]) cudaGraphDestroy(s->graph[i]);
  }
  for (auto& L : s->layers) {
    if (L.fwd) ugemm_grouped_plan_destroy(L.fwd);
    if (L.bwd) ugemm_grouped_plan_destroy(L.bwd);
  }
  if (s->arena) cudaFree(s->arena);
  delete s;
}
}  // namespace

using namespace ugemm;

extern "C" {

UGEMM_API int ugemm_im2col(const float* x, int channels, int batch, int height, int width,
                           int ksize, int pad, int stride, float* col, void* stream) {
  if (!x || !col || channels <= 0 || batch <= 0 || height <= 0 || width <= 0 || ksize <= 0 ||
      pad < 0 || stride <= 0)
    return UGEMM_ERR_ARG;
  return im2col_launch(x, channels, batch, height, width, ksize, pad, stride, col,
                       static_cast<cudaStream_t>(stream));
}

UGEMM_API int ugemm_col2im(const float* col, int channels, int batch, int height, int width,
                           int ksize, int pad, int stride, float* x, void* stream) {
  if (!x || !col || channels <= 0 || batch <= 0 || height <= 0 || width <= 0 || ksize <= 0 ||
      pad < 0 || stride <= 0)
    return UGEMM_ERR_ARG;
  return col2im_launch(col, channels, batch, height, width, ksize, pad, stride, x,
                       static_cast<cudaStream_t>(stream));
}

UGEMM_API int ugemm_conv_stack_create(int nlayers, const ugemm_conv_layer* layers, int batch,
                                      int precision, int flags, ugemm_conv_stack** out) {
  if (!out || nlayers <= 0 || !layers || batch <= 0) return UGEMM_ERR_ARG;
  *out = nullptr;
  auto* s = new Stack;
  s->batch = batch;
  s->form = precision == UGEMM_PREC_AUTO ? UGEMM_PREC_BF16X6 : precision;
  s->explicit_col = (flags & UGEMM_CONV_IM2COL) != 0;
  if (s->form < UGEMM_PREC_SIMT || s->form > UGEMM_PREC_TF32X3) {
    destroy_stack(s);
    return UGEMM_ERR_ARG;
  }
  // shapes and arena layout
  size_t bytes = 0;
  auto take = [&](size_t n) { size_t o = bytes; bytes += align_up(n * sizeof(float), 256); return o; };
  std::vector<size_t> off;
  for (int l = 0; l < nlayers; ++l) {
    const ugemm_conv_layer& d = layers[l];
    if (d.cin <= 0 || d.cout <= 0 || d.height <= 0 || d.width <= 0 || d.ksize <= 0 || d.pad < 0 ||
        d.stride <= 0 || (d.act != 0 && d.act != 1)) {
      destroy_stack(s);
      return UGEMM_ERR_ARG;
    }
    Stack::Layer L{};
    L.d = d;
    L.Ho = out_dim(d.height, d.ksize, d.pad, d.stride);
    L.Wo = out_dim(d.width, d.ksize, d.pad, d.stride);
    if (L.Ho <= 0 || L.Wo <= 0) { destroy_stack(s); return UGEMM_ERR_ARG; }
    if (l > 0) {
      const auto& P = s->layers.back();
      if (P.d.cout != d.cin || P.Ho != d.height || P.Wo != d.width) {
        destroy_stack(s);
        return UGEMM_ERR_ARG;  // layer l must consume layer l-1's output
      }
    }
    L.n = static_cast<long long>(batch) * L.Ho * L.Wo;
    L.kdim = d.cin * d.ksize * d.ksize;
    // (split forms only: the SIMT form's K-major pack of the 9x wider
    // gathered dY costs more than dcol + col2im, measured)
    L.direct_dx = !s->explicit_col && s->form != UGEMM_PREC_SIMT && d.stride == 1 &&
                  d.pad <= d.ksize - 1;
    if (L.n > 0x7fffffffLL) { destroy_stack(s); return UGEMM_ERR_ARG; }
    s->layers.push_back(L);
  }
  // arena: x0 | per layer {col, w, y, dw, dcol, dx} | dy_last
  const size_t x0 = take(size_t(layers[0].cin) * batch * layers[0].height * layers[0].width);
  for (auto& L : s->layers) {
    off.push_back(s->explicit_col ? take(size_t(L.kdim) * L.n) : 0);  // col
    off.push_back(take(size_t(L.d.cout) * L.kdim));            // w
    off.push_back(take(size_t(L.d.cout) * L.n));               // y
    off.push_back(take(size_t(L.d.cout) * L.kdim));            // dw
    off.push_back(L.direct_dx ? take(size_t(L.d.cout) * L.kdim)   // wt
                              : take(size_t(L.kdim) * L.n));      // dcol
    off.push_back(take(size_t(L.d.cin) * batch * L.d.height * L.d.width));  // dx
    off.push_back(take(size_t(L.d.cout)));                     // bias
    off.push_back(take(size_t(L.d.cout)));                     // dbias
  }
  if (cudaMalloc(&s->arena, bytes) != cudaSuccess) { s->arena = nullptr; destroy_stack(s); return UGEMM_ERR_ALLOC; }
  cudaMemset(s->arena, 0, bytes);
  uint8_t* base = static_cast<uint8_t*>(s->arena);
  auto at = [&](size_t o) { return reinterpret_cast<float*>(base + o); };
  for (size_t l = 0; l < s->layers.size(); ++l) {
    auto& L = s->layers[l];
    L.x = l == 0 ? at(x0) : s->layers[l - 1].y;
    L.col = s->explicit_col ? at(off[8 * l]) : nullptr;
    L.w = at(off[8 * l + 1]);
    L.y = at(off[8 * l + 2]);
    L.dw = at(off[8 * l + 3]);
    L.dcol = L.direct_dx ? nullptr : at(off[8 * l + 4]);
    L.wt = L.direct_dx ? at(off[8 * l + 4]) : nullptr;
    L.dx = at(off[8 * l + 5]);
    L.bias = at(off[8 * l + 6]);
    L.dbias = at(off[8 * l + 7]);
  }
  for (size_t l = 0; l < s->layers.size(); ++l) {
    auto& L = s->layers[l];
    const float* dy = (l + 1 < s->layers.size()) ? s->layers[l + 1].dx : nullptr;
    if (!dy) {
      s->dy_last = L.y;  // the last layer's output buffer doubles as its incoming gradient slot
      dy = nullptr;
    }
    const int M = L.d.cout, N = static_cast<int>(L.n), K = L.kdim;
    // forward: y = w * col
    L.im = make_im2col(L.x, L.d.cin, batch, L.d.height, L.d.width, L.d.ksize, L.d.pad,
                       L.d.stride, L.Ho, L.Wo);
    // col = im2col(x): the materialised buffer, or read from x by the
    // GEMMs' operand pass
    const Im2col* im = s->explicit_col ? nullptr : &L.im;
    // forward: y = w * col
    Gemm f{'N', 'N', M, N, K, 1.f, 0.f, L.w, K, L.col, N, L.y, N};
    f.epi = Epilogue{L.d.act ? L.bias : nullptr, L.d.act, L.d.slope};
    f.b_im2col = im;
    // backward: dw = dy * col^T, and dcol = w^T * dy (dX = col2im(dcol)) or,
    // for a direct layer, dX = wt * im2col(dY; pad k-1-p): the adjoint of a
    // stride-1 convolution is the convolution of dY with the weights
    // transposed in the channels and flipped in the taps
    const float* g = dy ? dy : L.y;
    Gemm b[2] = {Gemm{'N', 'T', M, K, N, 1.f, 0.f, g, N, L.col, N, L.dw, K},
                 Gemm{'T', 'N', K, N, M, 1.f, 0.f, L.w, K, g, N, L.dcol, N}};
    b[0].b_im2col = im;
    if (L.direct_dx) {
      const int kk = L.d.ksize * L.d.ksize;
      const int npix = batch * L.d.height * L.d.width;
      L.dy_im = make_im2col(g, L.d.cout, batch, L.Ho, L.Wo, L.d.ksize, L.d.ksize - 1 - L.d.pad, 1,
                            L.d.height, L.d.width);
      b[1] = Gemm{'N', 'N', L.d.cin, npix, L.d.cout * kk, 1.f, 0.f, L.wt, L.d.cout * kk, nullptr,
                  npix, L.dx, npix};
      b[1].b_im2col = &L.dy_im;
    }
    ugemm_status rc = grouped_plan_build(&f, 1, s->form, nullptr, 0, &L.fwd);
    if (rc == UGEMM_OK) rc = grouped_plan_build(b, 2, s->form, nullptr, 0, &L.bwd);
    if (rc != UGEMM_OK) { destroy_stack(s); return rc; }
    s->flops_fwd += 2.0 * M * double(N) * K;
    s->flops_bwd += 4.0 * M * double(N) * K;
  }
  if (flags & UGEMM_PLAN_GRAPH) {
    for (int what = 1; what <= 3; ++what) {
      cudaStream_t cs;
      if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) {
        destroy_stack(s);
        return UGEMM_ERR_CUDA;
      }
      cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
      int rc = UGEMM_OK;
      if (e == cudaSuccess) {
        rc = run_stack(s, what, cs);
        e = cudaStreamEndCapture(cs, &s->graph[what]);
      }
      if (e == cudaSuccess && rc == UGEMM_OK) e = cudaGraphInstantiate(&s->exec[what], s->graph[what], 0);
      cudaStreamDestroy(cs);
      if (e != cudaSuccess || rc != UGEMM_OK) { destroy_stack(s); return UGEMM_ERR_CUDA; }
    }
  }
  *out = s;
  return UGEMM_OK;
}

UGEMM_API int ugemm_conv_stack_buffer(ugemm_conv_stack* s, int layer, int which, float** ptr,
                                      size_t* count) {
  if (!s || !ptr || layer < 0 || layer >= static_cast<int>(s->layers.size())) return UGEMM_ERR_ARG;
  const auto& L = s->layers[layer];
  const size_t x_n = size_t(L.d.cin) * s->batch * L.d.height * L.d.width;
  size_t n = 0;
  switch (which) {
    case UGEMM_CONV_X: *ptr = L.x; n = x_n; break;
    case UGEMM_CONV_W: *ptr = L.w; n = size_t(L.d.cout) * L.kdim; break;
    case UGEMM_CONV_Y: *ptr = L.y; n = size_t(L.d.cout) * L.n; break;
    case UGEMM_CONV_COL:
      if (!s->explicit_col) return UGEMM_ERR_UNSUPPORTED;  // read implicitly, never stored
      *ptr = L.col;
      n = size_t(L.kdim) * L.n;
      break;
    case UGEMM_CONV_DW: *ptr = L.dw; n = size_t(L.d.cout) * L.kdim; break;
    case UGEMM_CONV_DCOL:
      if (L.direct_dx) return UGEMM_ERR_UNSUPPORTED;  // dX computed without dcol
      *ptr = L.dcol;
      n = size_t(L.kdim) * L.n;
      break;
    case UGEMM_CONV_DX: *ptr = L.dx; n = x_n; break;
    case UGEMM_CONV_BIAS: *ptr = L.bias; n = L.d.cout; break;
    case UGEMM_CONV_DBIAS: *ptr = L.dbias; n = L.d.cout; break;
    case UGEMM_CONV_DY:
      *ptr = (layer + 1 < static_cast<int>(s->layers.size())) ? s->layers[layer + 1].dx : L.y;
      n = size_t(L.d.cout) * L.n;
      break;
    default: return UGEMM_ERR_ARG;
  }
  if (count) *count = n;
  return UGEMM_OK;
}

UGEMM_API int ugemm_conv_stack_run(ugemm_conv_stack* s, int what, void* stream) {
  if (!s || what < 1 || what > 3) return UGEMM_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (s->exec[what]) {
    return cudaGraphLaunch(s->exec[what], st) == cudaSuccess ? UGEMM_OK : UGEMM_ERR_CUDA;
  }
  return run_stack(s, what, st);
}

UGEMM_API double ugemm_conv_stack_flops(const ugemm_conv_stack* s, int what) {
  if (!s) return 0;
  return ((what & UGEMM_CONV_FORWARD) ? s->flops_fwd : 0) +
         ((what & UGEMM_CONV_BACKWARD) ? s->flops_bwd : 0);
}

UGEMM_API int ugemm_conv_stack_destroy(ugemm_conv_stack* s) {
  if (!s) return UGEMM_OK;
  cudaDeviceSynchronize();
  destroy_stack(s);
  return UGEMM_OK;
}

}  // extern "C"
