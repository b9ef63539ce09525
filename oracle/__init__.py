"""CPU oracle for the ugemm SGEMM path -- TEST INFRASTRUCTURE ONLY.

This package restates the reference's CPU GEMMs (ugemm.h, gemm_cpu.h,
sgemm_avx256.h, check_sgemm.c, sgemm_ocl1.h im2col) in portable C
(``ugemm_oracle.c``, ``ugemm_oracle_port.c``) and loads them through ctypes.
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
and reference legs may import it; the product library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_STRICT = os.path.join(HERE, "_ref", "libugemm_ref_strict.so")
REF_FAST = os.path.join(HERE, "_ref", "libugemm_ref_fast.so")

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_c = ctypes.c_char
_i = ctypes.c_int
_f = ctypes.c_float
_d = ctypes.c_double

_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so with oracle/Makefile (portable; both hosts)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


def build_ref(ref_dir: str | None = None) -> bool:
    """Compile the reference's own CPU GEMMs (x86-64 with the reference tree
    only) from `ref_dir`, else from $UGEMM_REF_DIR; False if neither names a
    directory."""
    import platform
    ref_dir = ref_dir or os.environ.get("UGEMM_REF_DIR")
    if platform.machine() != "x86_64" or not ref_dir or not os.path.isdir(ref_dir):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={ref_dir}"], check=True)
    return True


def _gemm_sig(ptr, real):
    return [_c, _c, _c, _i, _i, _i, real, ptr, _i, ptr, _i, real, ptr, _i]


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB_PATH)
        for name in ("oracle_sgemm_cpu", "oracle_sgemm_c"):
            getattr(lib, name).argtypes = _gemm_sig(_f32p, _f)
            getattr(lib, name).restype = _i
        for name in ("oracle_dgemm_cpu", "oracle_dgemm_c"):
            getattr(lib, name).argtypes = _gemm_sig(_f64p, _d)
            getattr(lib, name).restype = _i
        lib.oracle_sgemm_avx256.argtypes = [_i, _i, _i, _f, _f32p, _i, _f32p, _i, _f, _f32p, _i]
        lib.oracle_sgemm_avx256.restype = None
        lib.oracle_sgemm_avx256_mt.argtypes = [_i, _c, _c, _i, _i, _i, _f, _f32p, _i, _f32p, _i,
                                               _f, _f32p, _i]
        lib.oracle_sgemm_avx256_mt.restype = _i
        lib.oracle_sgemm_sse.argtypes = _gemm_sig(_f32p, _f)
        lib.oracle_sgemm_sse.restype = None
        for name in ("oracle_gemm_rnn", "oracle_gemm_rnt", "oracle_gemm_rtn"):
            getattr(lib, name).argtypes = [_i, _i, _i, _f, _f32p, _f32p, _f, _f32p]
            getattr(lib, name).restype = None
        lib.oracle_cmp_results.argtypes = [_i, _i, _f32p, _f32p, _i, _f64p]
        lib.oracle_cmp_results.restype = _i
        lib.oracle_im2col.argtypes = [_f32p, _i, _i, _i, _i, _i, _i, _f32p]
        lib.oracle_im2col.restype = None
        lib.oracle_bias_leaky.argtypes = [_f32p, _i, _i, _f32p]
        lib.oracle_bias_leaky.restype = None
        lib.oracle_saxpy_cpu.argtypes = [_i, _f, _f32p, _i, _f32p, _i]
        lib.oracle_saxpy_cpu.restype = None
        lib.oracle_sgemv_cpu.argtypes = [_c, _i, _i, _f, _f32p, _i, _f32p, _i, _f, _f32p, _i]
        lib.oracle_sgemv_cpu.restype = None
        _lib = lib
    return _lib


def load_ref(fast: bool) -> ctypes.CDLL:
    """The reference's own functions (oracle/_ref); raises if not built."""
    lib = ctypes.CDLL(REF_FAST if fast else REF_STRICT)
    for name in ("sgemm_cpu", "sgemm_c", "sgemm_avx", "ref_sgemm_sse"):
        getattr(lib, name).argtypes = _gemm_sig(_f32p, _f)
        getattr(lib, name).restype = None
    for name in ("dgemm_cpu", "_dgemm_c", "dgemm_avx"):
        getattr(lib, name).argtypes = _gemm_sig(_f64p, _d)
        getattr(lib, name).restype = None
    lib.ref_cmp_results.argtypes = [_i, _i, _f32p, _f32p, _i]
    lib.ref_cmp_results.restype = None
    lib.saxpy_cpu.argtypes = [_i, _f, _f32p, _i, _f32p, _i]
    lib.saxpy_cpu.restype = None
    lib.sgemv_cpu.argtypes = [_c, _i, _i, _f, _f32p, _i, _f32p, _i, _f, _f32p, _i]
    lib.sgemv_cpu.restype = None
    return lib


# ----------------------------------------------------------------------------
# numpy-facing helpers (row-major 'R' unless major='C')
# ----------------------------------------------------------------------------
def op_shape(trans: str, rows: int, cols: int):
    """Stored shape of an operand whose op() is rows x cols (row-major)."""
    return (rows, cols) if trans == "N" else (cols, rows)


def sgemm(fn: str, ta: str, tb: str, M: int, N: int, K: int, alpha: float, A, B, beta: float,
          C, major: str = "R"):
    """Run one of oracle_sgemm_cpu / oracle_sgemm_c on row-major numpy arrays.

    ``A``, ``B``, ``C`` are 2-D C-contiguous float32 arrays; lda/ldb/ldc are
    their row lengths.  C is updated in place and returned.
    """
    lib = load()
    f = getattr(lib, fn)
    rc = f(major.encode(), ta.encode(), tb.encode(), M, N, K, alpha, A, A.shape[1], B, B.shape[1],
           beta, C, C.shape[1])
    if rc != 0:
        raise RuntimeError(f"{fn} failed with {rc}")
    return C


def dgemm(ta: str, tb: str, M: int, N: int, K: int, alpha: float, A, B, beta: float, C,
          major: str = "R", fn: str = "oracle_dgemm_c"):
    lib = load()
    rc = getattr(lib, fn)(major.encode(), ta.encode(), tb.encode(), M, N, K, alpha, A, A.shape[1],
                          B, B.shape[1], beta, C, C.shape[1])
    if rc != 0:
        raise RuntimeError(f"{fn} failed with {rc}")
    return C


def sgemm_avx256_mt(nthreads: int, ta: str, tb: str, M: int, N: int, K: int, alpha: float, A, B,
                    beta: float, C):
    lib = load()
    rc = lib.oracle_sgemm_avx256_mt(nthreads, ta.encode(), tb.encode(), M, N, K, alpha, A,
                                    A.shape[1], B, B.shape[1], beta, C, C.shape[1])
    if rc != 0:
        raise RuntimeError(f"oracle_sgemm_avx256_mt failed with {rc}")
    return C


def cmp_results(ref, res):
    """check_sgemm.c:56-85 metric: (label, stdErr, stdRef, maxErr, argmax)."""
    lib = load()
    out = np.zeros(4, dtype=np.float64)
    M, N = ref.shape
    label = lib.oracle_cmp_results(M, N, np.ascontiguousarray(ref, dtype=np.float32),
                                   np.ascontiguousarray(res, dtype=np.float32), N, out)
    return {0: "", 1: "Sucks !", 2: "FAIL !!!"}[label], out[0], out[1], out[2], int(out[3])


def im2col(im, ksize: int, pad: int, stride: int):
    """sgemm_ocl1.h:81-119 on one CHW image (float32)."""
    lib = load()
    c, h, w = im.shape
    ho = (h + 2 * pad - ksize) // stride + 1
    wo = (w + 2 * pad - ksize) // stride + 1
    col = np.empty((c * ksize * ksize, ho * wo), dtype=np.float32)
    lib.oracle_im2col(np.ascontiguousarray(im, dtype=np.float32), c, h, w, ksize, pad, stride, col)
    return col


def normwise_error(C, C64) -> float:
    """||C - C64||_F / ||C64||_F computed in float64."""
    C = np.asarray(C, dtype=np.float64)
    C64 = np.asarray(C64, dtype=np.float64)
    return float(np.linalg.norm(C - C64) / np.linalg.norm(C64))


def bias_leaky(out, bias):
    """sgemm_gl1.h:210-217 applied in place to a channels x pixels float32 array."""
    lib = load()
    c, n = out.shape
    lib.oracle_bias_leaky(out, c, n, np.ascontiguousarray(bias, dtype=np.float32))
    return out
