"""ugemm_gb300 -- Python host mirror of the GB300 SGEMM backend for ugemm.

The product is ``libugemm_cuda.so`` (C ABI in ``include/sgemm_cuda.h``); this
module loads it with ctypes and mirrors the reference's entry points with the
same names and argument meaning:

* ``sgemm_cuda_init(platform, device, size)`` / ``sgemm_cuda(ta, tb, m, n, k,
  alpha, a, b, beta, c)`` / ``sgemm_cuda_finish()`` -- the reference's
  ``sgemm_ocl_init`` / ``sgemm_ocl`` / ``sgemm_ocl_finish`` (sgemm_ocl2.h:158,
  166, 220) on numpy float32 host arrays;
* ``ugemm_sgemm(major, transa, transb, M, N, K, alpha, A, lda, B, ldb, beta,
  C, ldc)`` -- the signature of ``sgemm_cpu`` (ugemm.h:287);
* ``sgemm_dev`` / ``sgemm_backward`` -- device-pointer forms on torch CUDA
  tensors (torch is used only for device memory and streams).

There is no CPU fallback: if the CUDA library is missing or cannot run, every
call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libugemm_cuda.so")

OK = 0
ERR_ARG = 1
ERR_ALLOC = 2
ERR_ARENA_TOO_SMALL = 3
ERR_CUDA = 4
ERR_TIMEOUT = 5
ERR_NOT_INIT = 6
ERR_UNSUPPORTED = 7

PREC_AUTO = 0
PREC_SIMT = 1
PREC_BF16X6 = 2
PREC_BF16X9 = 3
PREC_BF16X3 = 4
PREC_FP16X3 = 5
PREC_TF32X3 = 6
PRECISIONS = {"auto": PREC_AUTO, "simt": PREC_SIMT, "bf16x6": PREC_BF16X6, "bf16x9": PREC_BF16X9,
              "bf16x3": PREC_BF16X3, "fp16x3": PREC_FP16X3, "tf32x3": PREC_TF32X3}

# Every symbol include/sgemm_cuda.h declares.
EXPORTS = (
    "sgemm_cuda_init", "sgemm_cuda", "sgemm_cuda_finish", "sgemm_cuda_status",
    "sgemm_cuda_set_precision", "ugemm_last_error", "ugemm_last_error_message",
    "ugemm_status_string", "ugemm_sgemm", "ugemm_sgemm_host", "ugemm_sgemm_dev",
    "ugemm_workspace_bytes", "ugemm_reserve_workspace", "ugemm_sgemm_backward",
    "ugemm_device_info", "ugemm_profile_enable", "ugemm_profile_collect",
    "ugemm_grouped_plan_create", "ugemm_grouped_run", "ugemm_grouped_check",
    "ugemm_grouped_plan_destroy", "ugemm_grouped_flops", "ugemm_grouped_config",
    "ugemm_sgemm_grouped", "ugemm_tune_grouped", "ugemm_check", "ugemm_dgemm_oracle_dev",
    "ugemm_sgemm_dev_noalloc", "ugemm_debug_set_error_word",
)
PROF_KINDS = ("simt", "split_prepass", "split_gemm", "aux", "grouped", "control", "copy")


class UgemmError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        super().__init__(f"ugemm status {status}: {msg}")


_lib = None
_c = ctypes.c_char
_i = ctypes.c_int
_f = ctypes.c_float
_p = ctypes.c_void_p
_sz = ctypes.c_size_t


def build(verbose: bool = False) -> str:
    from . import buildlib
    return buildlib.build(verbose=verbose)


def load() -> ctypes.CDLL:
    """Load libugemm_cuda.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise UgemmError(ERR_UNSUPPORTED, f"{LIB_PATH} is missing: run __graft_entry__.build()")
    lib = ctypes.CDLL(LIB_PATH)
    gemm = [_c, _c, _c, _i, _i, _i, _f, _p, _i, _p, _i, _f, _p, _i]
    lib.sgemm_cuda_init.argtypes = [_i, _i, _sz]
    lib.sgemm_cuda_init.restype = None
    lib.sgemm_cuda.argtypes = [_c, _c, _i, _i, _i, _f, _p, _p, _f, _p]
    lib.sgemm_cuda.restype = None
    lib.sgemm_cuda_status.argtypes = [_c, _c, _i, _i, _i, _f, _p, _p, _f, _p]
    lib.sgemm_cuda_status.restype = _i
    lib.sgemm_cuda_finish.argtypes = []
    lib.sgemm_cuda_finish.restype = None
    lib.sgemm_cuda_set_precision.argtypes = [_i]
    lib.sgemm_cuda_set_precision.restype = _i
    lib.ugemm_last_error.argtypes = []
    lib.ugemm_last_error.restype = _i
    lib.ugemm_last_error_message.argtypes = []
    lib.ugemm_last_error_message.restype = ctypes.c_char_p
    lib.ugemm_status_string.argtypes = [_i]
    lib.ugemm_status_string.restype = ctypes.c_char_p
    lib.ugemm_sgemm.argtypes = gemm
    lib.ugemm_sgemm.restype = None
    lib.ugemm_sgemm_host.argtypes = gemm + [_i]
    lib.ugemm_sgemm_host.restype = _i
    lib.ugemm_sgemm_dev.argtypes = gemm + [_i, _p]
    lib.ugemm_sgemm_dev.restype = _i
    lib.ugemm_workspace_bytes.argtypes = [_c, _c, _c, _i, _i, _i, _i, _i, _i]
    lib.ugemm_workspace_bytes.restype = _sz
    lib.ugemm_reserve_workspace.argtypes = [_sz]
    lib.ugemm_reserve_workspace.restype = _i
    lib.ugemm_sgemm_backward.argtypes = [_c, _c, _i, _i, _i, _f, _p, _i, _p, _i, _p, _i, _f, _p, _i,
                                         _f, _p, _i, _i, _p]
    lib.ugemm_sgemm_backward.restype = _i
    lib.ugemm_device_info.argtypes = [ctypes.POINTER(_i)] * 3
    lib.ugemm_device_info.restype = _i
    lib.ugemm_profile_enable.argtypes = [_i]
    lib.ugemm_profile_enable.restype = _i
    lib.ugemm_profile_collect.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_i), _i]
    lib.ugemm_profile_collect.restype = _i
    lib.ugemm_check.argtypes = [_p]
    lib.ugemm_check.restype = _i
    lib.ugemm_debug_set_error_word.argtypes = [_i, _i]
    lib.ugemm_debug_set_error_word.restype = _i
    lib.ugemm_sgemm_dev_noalloc.argtypes = gemm + [_i, _p]
    lib.ugemm_sgemm_dev_noalloc.restype = _i
    d = ctypes.c_double
    lib.ugemm_dgemm_oracle_dev.argtypes = [_c, _c, _c, _i, _i, _i, d, _p, _i, _p, _i, d, _p, _i, _p]
    lib.ugemm_dgemm_oracle_dev.restype = _i
    _lib = lib
    return lib


def _check(status: int) -> None:
    if status != OK:
        msg = load().ugemm_last_error_message().decode(errors="replace")
        raise UgemmError(status, msg)


def _prec(p) -> int:
    return PRECISIONS[p] if isinstance(p, str) else int(p)


def _host_ptr(a: np.ndarray, writable: bool = False) -> int:
    if a.dtype != np.float32 or not a.flags["C_CONTIGUOUS"]:
        raise UgemmError(ERR_ARG, "host arrays must be C-contiguous float32")
    if writable and not a.flags["WRITEABLE"]:
        raise UgemmError(ERR_ARG, "C must be writable")
    return a.ctypes.data


# --------------------------------------------------------------------------
# Reference-named compat API (sgemm_ocl2.h:158-224)
# --------------------------------------------------------------------------
def sgemm_cuda_init(platform: int = 0, device: int = 0, size: int = 0) -> None:
    lib = load()
    lib.sgemm_cuda_init(platform, device, size)
    _check(lib.ugemm_last_error())


def sgemm_cuda(ta: str, tb: str, m: int, n: int, k: int, alpha: float, a: np.ndarray,
               b: np.ndarray, beta: float, c: np.ndarray) -> None:
    """C = alpha*op(A)*op(B) + beta*C on host arrays (tight leading dims)."""
    lib = load()
    _check(lib.sgemm_cuda_status(ta.encode(), tb.encode(), m, n, k, alpha, _host_ptr(a),
                                 _host_ptr(b), beta, _host_ptr(c, True)))


def sgemm_cuda_finish() -> None:
    load().sgemm_cuda_finish()


def set_precision(precision) -> None:
    _check(load().sgemm_cuda_set_precision(_prec(precision)))


def ugemm_sgemm(major: str, transa: str, transb: str, M: int, N: int, K: int, alpha: float,
                A: np.ndarray, lda: int, B: np.ndarray, ldb: int, beta: float, C: np.ndarray,
                ldc: int, precision="auto") -> None:
    """BLAS-style host GEMM with the sgemm_cpu signature (ugemm.h:287)."""
    lib = load()
    _check(lib.ugemm_sgemm_host(major.encode(), transa.encode(), transb.encode(), M, N, K, alpha,
                                _host_ptr(A), lda, _host_ptr(B), ldb, beta, _host_ptr(C, True),
                                ldc, _prec(precision)))


# --------------------------------------------------------------------------
# Device-pointer API on torch tensors
# --------------------------------------------------------------------------
def _stream_ptr(stream) -> int:
    import torch
    if stream is None:
        stream = torch.cuda.current_stream()
    return stream.cuda_stream


def sgemm_dev(ta: str, tb: str, M: int, N: int, K: int, alpha: float, A, lda: int, B, ldb: int,
              beta: float, C, ldc: int, precision="auto", stream=None, major: str = "R") -> None:
    """Row-major (or 'C') GEMM on device memory (torch CUDA tensors or ints)."""
    lib = load()
    ptr = (lambda t: t if isinstance(t, int) else t.data_ptr())
    _check(lib.ugemm_sgemm_dev(major.encode(), ta.encode(), tb.encode(), M, N, K, alpha, ptr(A),
                               lda, ptr(B), ldb, beta, ptr(C), ldc, _prec(precision),
                               _stream_ptr(stream)))


def sgemm_dev_noalloc(ta: str, tb: str, M: int, N: int, K: int, alpha: float, A, lda: int, B,
                      ldb: int, beta: float, C, ldc: int, precision="bf16x6", stream=None,
                      major: str = "R") -> None:
    """ugemm_sgemm_dev_noalloc: the split forms with scratch in a fixed device array."""
    lib = load()
    ptr = (lambda t: t if isinstance(t, int) else t.data_ptr())
    _check(lib.ugemm_sgemm_dev_noalloc(major.encode(), ta.encode(), tb.encode(), M, N, K, alpha,
                                       ptr(A), lda, ptr(B), ldb, beta, ptr(C), ldc,
                                       _prec(precision), _stream_ptr(stream)))


def check(stream=None) -> None:
    """ugemm_check: synchronise `stream`; raise UgemmError(ERR_TIMEOUT) if a kernel wait of
    a device-pointer call gave up since the last check."""
    _check(load().ugemm_check(_stream_ptr(stream)))


def dgemm_oracle(ta: str, tb: str, M: int, N: int, K: int, alpha: float, A, lda: int, B,
                 ldb: int, beta: float, C, ldc: int, stream=None, major: str = "R") -> None:
    """ugemm_dgemm_oracle_dev: the FP64 GEMM the FP32 forms are checked against."""
    lib = load()
    ptr = (lambda t: t if isinstance(t, int) else t.data_ptr())
    _check(lib.ugemm_dgemm_oracle_dev(major.encode(), ta.encode(), tb.encode(), M, N, K, alpha,
                                      ptr(A), lda, ptr(B), ldb, beta, ptr(C), ldc,
                                      _stream_ptr(stream)))


def ref64(ta: str, tb: str, A, B, C0=None, alpha: float = 1.0, beta: float = 0.0):
    """alpha*op(A)*op(B) + beta*C0 in FP64 on the device (float64 result) through
    ugemm_dgemm_oracle_dev, from FP32 or FP64 row-major CUDA tensors."""
    import torch
    a, b = A.double().contiguous(), B.double().contiguous()
    M = a.shape[0] if ta == "N" else a.shape[1]
    K = a.shape[1] if ta == "N" else a.shape[0]
    N = b.shape[1] if tb == "N" else b.shape[0]
    if C0 is None or beta == 0.0:
        C = torch.zeros((M, N), dtype=torch.float64, device=a.device)
        beta = 0.0
    else:
        C = C0.double().contiguous().clone()
    dgemm_oracle(ta, tb, M, N, K, alpha, a, a.shape[1], b, b.shape[1], beta, C, N)
    return C


def gemm(A, B, C=None, *, ta: str = "N", tb: str = "N", alpha: float = 1.0, beta: float = 0.0,
         precision="auto", stream=None):
    """C = alpha*op(A)*op(B) + beta*C on 2-D row-major float32 CUDA tensors."""
    import torch
    M = A.shape[0] if ta == "N" else A.shape[1]
    K = A.shape[1] if ta == "N" else A.shape[0]
    N = B.shape[1] if tb == "N" else B.shape[0]
    if C is None:
        C = torch.empty((M, N), dtype=torch.float32, device=A.device)
    for t in (A, B, C):
        if t.dtype != torch.float32 or t.stride(1) != 1:
            raise UgemmError(ERR_ARG, "tensors must be float32 with unit column stride")
    sgemm_dev(ta, tb, M, N, K, alpha, A, A.stride(0), B, B.stride(0), beta, C, C.stride(0),
              precision, stream)
    return C


def sgemm_backward(ta: str, tb: str, M: int, N: int, K: int, alpha: float, A, lda: int, B,
                   ldb: int, dC, lddc: int, beta_a: float, dA, ldda: int, beta_b: float, dB,
                   lddb: int, precision="auto", stream=None) -> None:
    """dA = alpha*dC*op(B)^T (+beta_a*dA), dB = alpha*op(A)^T*dC (+beta_b*dB)."""
    lib = load()
    ptr = (lambda t: 0 if t is None else (t if isinstance(t, int) else t.data_ptr()))
    _check(lib.ugemm_sgemm_backward(ta.encode(), tb.encode(), M, N, K, alpha, ptr(A), lda, ptr(B),
                                    ldb, ptr(dC), lddc, beta_a, ptr(dA), ldda, beta_b, ptr(dB),
                                    lddb, _prec(precision), _stream_ptr(stream)))


def gemm_ex(A, B, C=None, *, bias=None, act=0, slope=0.1, ta="N", tb="N", alpha=1.0, beta=0.0,
            precision="auto", stream=None):
    """C = act(alpha*op(A)*op(B) + beta*C + bias[row]) on row-major CUDA tensors."""
    import torch
    lib = load()
    lib.ugemm_sgemm_dev_ex.argtypes = [_c, _c, _c, _i, _i, _i, _f, _p, _i, _p, _i, _f, _p, _i, _p,
                                       _i, _f, _i, _p]
    lib.ugemm_sgemm_dev_ex.restype = _i
    M = A.shape[0] if ta == "N" else A.shape[1]
    K = A.shape[1] if ta == "N" else A.shape[0]
    N = B.shape[1] if tb == "N" else B.shape[0]
    if C is None:
        C = torch.empty((M, N), dtype=torch.float32, device=A.device)
    _check(lib.ugemm_sgemm_dev_ex(b"R", ta.encode(), tb.encode(), M, N, K, alpha, A.data_ptr(),
                                  A.stride(0), B.data_ptr(), B.stride(0), beta, C.data_ptr(),
                                  C.stride(0), 0 if bias is None else bias.data_ptr(), act, slope,
                                  _prec(precision), _stream_ptr(stream)))
    return C


def workspace_bytes(ta: str, tb: str, M: int, N: int, K: int, lda: int, ldb: int,
                    precision="auto", major: str = "R") -> int:
    return int(load().ugemm_workspace_bytes(major.encode(), ta.encode(), tb.encode(), M, N, K, lda,
                                            ldb, _prec(precision)))


def reserve_workspace(nbytes: int) -> None:
    _check(load().ugemm_reserve_workspace(nbytes))


def device_info():
    lib = load()
    sm, ma, mi = _i(), _i(), _i()
    _check(lib.ugemm_device_info(ctypes.byref(sm), ctypes.byref(ma), ctypes.byref(mi)))
    return sm.value, ma.value, mi.value


def fp32_peak(ms: float = 200.0) -> float:
    """Measured FP32 FMA peak of the current device, TFLOP/s."""
    lib = load()
    lib.ugemm_fp32_peak.argtypes = [ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
    out = ctypes.c_double()
    _check(lib.ugemm_fp32_peak(ms, ctypes.byref(out)))
    return out.value


def profile_enable(on: bool = True) -> None:
    _check(load().ugemm_profile_enable(1 if on else 0))


def profile_collect() -> dict:
    """{kind: (milliseconds, launches)} since the last collect (synchronises)."""
    n = len(PROF_KINDS)
    ms = (ctypes.c_double * n)()
    cnt = (_i * n)()
    _check(load().ugemm_profile_collect(ms, cnt, n))
    return {k: (ms[i], cnt[i]) for i, k in enumerate(PROF_KINDS)}


def selftest_wait_timeout():
    """Run the bounded-wait self-test; returns (status, code, threads, seconds)."""
    lib = load()
    lib.ugemm_selftest_wait_timeout.argtypes = [ctypes.POINTER(_i), ctypes.POINTER(_i),
                                                ctypes.POINTER(ctypes.c_double)]
    code, threads, secs = _i(), _i(), ctypes.c_double()
    st = lib.ugemm_selftest_wait_timeout(ctypes.byref(code), ctypes.byref(threads),
                                         ctypes.byref(secs))
    return st, code.value, threads.value, secs.value


# --------------------------------------------------------------------------
# Grouped GEMM and autotuner
# --------------------------------------------------------------------------
PLAN_GRAPH = 1


class Problem(ctypes.Structure):
    """ugemm_problem: one row-major GEMM of a group (device pointers)."""
    _fields_ = [("transa", _c), ("transb", _c), ("M", _i), ("N", _i), ("K", _i),
                ("alpha", _f), ("beta", _f), ("A", _p), ("lda", _i), ("B", _p), ("ldb", _i),
                ("C", _p), ("ldc", _i), ("bias", _p), ("act", _i), ("slope", _f)]


class TileConfig(ctypes.Structure):
    """ugemm_tile_config: tile shape and schedule of a grouped launch."""
    _fields_ = [("block_n", _i), ("chunk_k", _i), ("max_ctas", _i), ("split_k", _i),
                ("deal", _i), ("transpose", _i), ("fused", _i)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


def _grouped_sigs(lib):
    if getattr(lib, "_grouped_ready", False):
        return
    pp = ctypes.POINTER(_p)
    lib.ugemm_grouped_plan_create.argtypes = [_i, ctypes.POINTER(Problem), _i,
                                              ctypes.POINTER(TileConfig), _i, pp]
    lib.ugemm_grouped_plan_create.restype = _i
    for name in ("ugemm_grouped_run", "ugemm_grouped_check"):
        getattr(lib, name).argtypes = [_p, _p]
        getattr(lib, name).restype = _i
    lib.ugemm_grouped_plan_destroy.argtypes = [_p]
    lib.ugemm_grouped_plan_destroy.restype = _i
    lib.ugemm_grouped_flops.argtypes = [_p]
    lib.ugemm_grouped_flops.restype = ctypes.c_double
    lib.ugemm_grouped_config.argtypes = [_p, ctypes.POINTER(TileConfig)]
    lib.ugemm_grouped_config.restype = _i
    lib.ugemm_sgemm_grouped.argtypes = [_i, ctypes.POINTER(Problem), _i, _p]
    lib.ugemm_sgemm_grouped.restype = _i
    lib.ugemm_tune_grouped.argtypes = [_i, ctypes.POINTER(Problem), _i, _i,
                                       ctypes.POINTER(TileConfig), ctypes.POINTER(ctypes.c_double)]
    lib.ugemm_tune_grouped.restype = _i
    lib._grouped_ready = True


def make_problems(specs):
    """specs: iterable of dicts with ta, tb, M, N, K, alpha, beta, A, lda, B, ldb, C, ldc
    (A/B/C torch CUDA tensors or device addresses)."""
    specs = list(specs)
    arr = (Problem * len(specs))()
    ptr = (lambda t: t if isinstance(t, int) else t.data_ptr())
    for i, s in enumerate(specs):
        bias = s.get("bias")
        arr[i] = Problem(s["ta"].encode(), s["tb"].encode(), s["M"], s["N"], s["K"], s["alpha"],
                         s["beta"], ptr(s["A"]), s["lda"], ptr(s["B"]), s["ldb"], ptr(s["C"]),
                         s["ldc"], 0 if bias is None else ptr(bias), s.get("act", 0),
                         s.get("slope", 0.1))
    return arr


class GroupedPlan:
    """A grouped GEMM plan (ugemm_grouped_plan); run() is stream-ordered."""

    def __init__(self, problems, precision="bf16x6", config=None, graph=False):
        lib = load()
        _grouped_sigs(lib)
        self._lib = lib
        self.problems = problems if isinstance(problems, ctypes.Array) else make_problems(problems)
        cfg = None
        if config is not None:
            cfg = ctypes.byref(config if isinstance(config, TileConfig) else TileConfig(**config))
        h = _p()
        _check(lib.ugemm_grouped_plan_create(len(self.problems), self.problems, _prec(precision),
                                             cfg, PLAN_GRAPH if graph else 0, ctypes.byref(h)))
        self.handle = h

    def run(self, stream=None):
        _check(self._lib.ugemm_grouped_run(self.handle, _stream_ptr(stream)))

    def check(self, stream=None):
        _check(self._lib.ugemm_grouped_check(self.handle, _stream_ptr(stream)))

    @property
    def flops(self) -> float:
        return float(self._lib.ugemm_grouped_flops(self.handle))

    @property
    def config(self) -> dict:
        c = TileConfig()
        _check(self._lib.ugemm_grouped_config(self.handle, ctypes.byref(c)))
        return c.as_dict()

    def close(self):
        if self.handle:
            self._lib.ugemm_grouped_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune_grouped(problems, precision="bf16x6", force=False):
    """Autotune the tile configuration of a problem set; returns (config dict, ms)."""
    lib = load()
    _grouped_sigs(lib)
    arr = problems if isinstance(problems, ctypes.Array) else make_problems(problems)
    best = TileConfig()
    ms = ctypes.c_double()
    _check(lib.ugemm_tune_grouped(len(arr), arr, _prec(precision), 1 if force else 0,
                                  ctypes.byref(best), ctypes.byref(ms)))
    return best.as_dict(), ms.value


def sgemm_grouped(problems, precision="bf16x6", stream=None):
    lib = load()
    _grouped_sigs(lib)
    arr = problems if isinstance(problems, ctypes.Array) else make_problems(problems)
    _check(lib.ugemm_sgemm_grouped(len(arr), arr, _prec(precision), _stream_ptr(stream)))


# --------------------------------------------------------------------------
# im2col convolution stack
# --------------------------------------------------------------------------
CONV_FORWARD, CONV_BACKWARD = 1, 2
CONV_IM2COL = 2  # create flag: materialise the im2col matrix (UGEMM_CONV_IM2COL)
CONV_BUFFERS = {"x": 0, "w": 1, "y": 2, "col": 3, "dw": 4, "dcol": 5, "dx": 6, "dy": 7, "bias": 8,
                "dbias": 9}


class ConvLayer(ctypes.Structure):
    """ugemm_conv_layer."""
    _fields_ = [("cin", _i), ("cout", _i), ("height", _i), ("width", _i), ("ksize", _i),
                ("pad", _i), ("stride", _i), ("act", _i), ("slope", _f)]


def _conv_sigs(lib):
    if getattr(lib, "_conv_ready", False):
        return
    lib.ugemm_im2col.argtypes = [_p, _i, _i, _i, _i, _i, _i, _i, _p, _p]
    lib.ugemm_im2col.restype = _i
    lib.ugemm_col2im.argtypes = [_p, _i, _i, _i, _i, _i, _i, _i, _p, _p]
    lib.ugemm_col2im.restype = _i
    lib.ugemm_conv_stack_create.argtypes = [_i, ctypes.POINTER(ConvLayer), _i, _i, _i,
                                            ctypes.POINTER(_p)]
    lib.ugemm_conv_stack_create.restype = _i
    lib.ugemm_conv_stack_buffer.argtypes = [_p, _i, _i, ctypes.POINTER(_p), ctypes.POINTER(_sz)]
    lib.ugemm_conv_stack_buffer.restype = _i
    lib.ugemm_conv_stack_run.argtypes = [_p, _i, _p]
    lib.ugemm_conv_stack_run.restype = _i
    lib.ugemm_conv_stack_flops.argtypes = [_p, _i]
    lib.ugemm_conv_stack_flops.restype = ctypes.c_double
    lib.ugemm_conv_stack_destroy.argtypes = [_p]
    lib.ugemm_conv_stack_destroy.restype = _i
    lib._conv_ready = True


def im2col(x, channels, batch, height, width, ksize, pad, stride, col, stream=None):
    lib = load()
    _conv_sigs(lib)
    ptr = (lambda t: t if isinstance(t, int) else t.data_ptr())
    _check(lib.ugemm_im2col(ptr(x), channels, batch, height, width, ksize, pad, stride, ptr(col),
                            _stream_ptr(stream)))


def col2im(col, channels, batch, height, width, ksize, pad, stride, x, stream=None):
    lib = load()
    _conv_sigs(lib)
    ptr = (lambda t: t if isinstance(t, int) else t.data_ptr())
    _check(lib.ugemm_col2im(ptr(col), channels, batch, height, width, ksize, pad, stride, ptr(x),
                            _stream_ptr(stream)))


class ConvStack:
    """ugemm_conv_stack: layers as (cin, cout, height, width, stride[, ksize, pad]); with
    leaky=slope every layer computes LeakyReLU(W*col + bias) (slope 0.1 is the reference's).
    im2col=True materialises each layer's im2col matrix (buffer "col") before its GEMMs;
    by default the GEMMs gather it from the layer input and there is no col buffer."""

    def __init__(self, layers, batch, precision="bf16x6", graph=True, leaky=None, im2col=False):
        lib = load()
        _conv_sigs(lib)
        self._lib = lib
        arr = (ConvLayer * len(layers))()
        for i, l in enumerate(layers):
            cin, cout, h, w, stride = l[:5]
            k = l[5] if len(l) > 5 else 3
            pad = l[6] if len(l) > 6 else 1
            arr[i] = ConvLayer(cin, cout, h, w, k, pad, stride, 0 if leaky is None else 1,
                               0.0 if leaky is None else float(leaky))
        self.layers = arr
        self.batch = batch
        h = _p()
        flags = (PLAN_GRAPH if graph else 0) | (CONV_IM2COL if im2col else 0)
        _check(lib.ugemm_conv_stack_create(len(arr), arr, batch, _prec(precision), flags,
                                           ctypes.byref(h)))
        self.handle = h

    def buffer(self, layer: int, which: str):
        """(device address, element count) of a buffer."""
        p, n = _p(), _sz()
        _check(self._lib.ugemm_conv_stack_buffer(self.handle, layer, CONV_BUFFERS[which],
                                                 ctypes.byref(p), ctypes.byref(n)))
        return p.value, n.value

    def tensor(self, layer: int, which: str, shape):
        """A torch view of a stack buffer (no copy)."""
        import torch
        addr, n = self.buffer(layer, which)
        numel = 1
        for s in shape:
            numel *= s
        assert numel == n, (which, shape, n)
        return _torch_view(addr, shape, torch)

    def run(self, what: int = CONV_FORWARD | CONV_BACKWARD, stream=None):
        _check(self._lib.ugemm_conv_stack_run(self.handle, what, _stream_ptr(stream)))

    def flops(self, what: int = CONV_FORWARD | CONV_BACKWARD) -> float:
        return float(self._lib.ugemm_conv_stack_flops(self.handle, what))

    def close(self):
        if self.handle:
            self._lib.ugemm_conv_stack_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _torch_view(addr: int, shape, torch):
    """Wrap library-owned float32 device memory as a torch tensor (no copy)."""
    class _Holder:
        pass
    numel = 1
    for s in shape:
        numel *= s
    h = _Holder()
    h.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f4", "data": (addr, False),
                                  "version": 3, "strides": None}
    return torch.as_tensor(h, device="cuda")


# --------------------------------------------------------------------------
# SAXPY / SGEMV (ugemm.h:86-160) on device pointers
# --------------------------------------------------------------------------
def _blas2_sigs(lib):
    if getattr(lib, "_blas2_ready", False):
        return
    lib.ugemm_saxpy.argtypes = [_i, _f, _p, _i, _p, _i, _p]
    lib.ugemm_saxpy.restype = _i
    lib.ugemm_sgemv.argtypes = [_c, _i, _i, _f, _p, _i, _p, _i, _f, _p, _i, _p]
    lib.ugemm_sgemv.restype = _i
    lib._blas2_ready = True


def saxpy(N, alpha, x, incx, y, incy, stream=None):
    lib = load()
    _blas2_sigs(lib)
    ptr = (lambda t: t if isinstance(t, int) else t.data_ptr())
    _check(lib.ugemm_saxpy(N, alpha, ptr(x), incx, ptr(y), incy, _stream_ptr(stream)))


def sgemv(trans, M, N, alpha, A, lda, x, incx, beta, y, incy, stream=None):
    lib = load()
    _blas2_sigs(lib)
    ptr = (lambda t: t if isinstance(t, int) else t.data_ptr())
    _check(lib.ugemm_sgemv(trans.encode(), M, N, alpha, ptr(A), lda, ptr(x), incx, beta, ptr(y),
                           incy, _stream_ptr(stream)))
