"""The C-ABI library builds, loads without a GPU and exports every symbol the
public headers declare; host-side argument checks need no GPU."""
import ctypes
import os
import re
import shutil

import numpy as np
import pytest

import ugemm_gb300 as ug

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = []
    inc = os.path.join(ROOT, "include")
    for fn in sorted(os.listdir(inc)):
        if fn.endswith(".h"):
            text = open(os.path.join(inc, fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"^\s*(?:UGEMM_API\s+)?(?:const\s+)?[a-z_]+\s*\**\s*([a-z_][a-z0-9_]*)\s*\(", text,
                                re.M)
    return names


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(ug.LIB_PATH):
        if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
            pytest.skip("nvcc not available to build the library")
        ug.build()
    return ug.load()


def test_exports_every_header_symbol(lib):
    names = header_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
    assert set(ug.EXPORTS) <= set(names)


def test_only_c_abi_symbols_are_exported(lib):
    # Internal C++ symbols are hidden; no torch types leak through the ABI.
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", ug.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    ours = {n for n in exported if n.startswith(("ugemm_", "sgemm_"))}
    assert set(header_functions()) <= ours


def header_enum(prefix):
    text = open(os.path.join(ROOT, "include", "sgemm_cuda.h")).read()
    return {m.group(1): int(m.group(2))
            for m in re.finditer(r"\b(" + prefix + r"[A-Z0-9_]+)\s*=\s*(\d+)", text)}


def test_python_constants_match_the_header():
    """The host mirror's status codes and arithmetic forms are the header's."""
    forms = header_enum("UGEMM_PREC_")
    assert forms == {f"UGEMM_PREC_{k.upper()}": v for k, v in ug.PRECISIONS.items()}
    status = header_enum("UGEMM_ERR_")
    for name, value in status.items():
        assert getattr(ug, name[len("UGEMM_"):]) == value, name


def test_status_strings(lib):
    assert lib.ugemm_status_string(0) == b"ok"
    assert b"argument" in lib.ugemm_status_string(ug.ERR_ARG)
    assert lib.ugemm_status_string(99) == b"unknown status"


def test_argument_checks_need_no_gpu(lib):
    f = lib.ugemm_sgemm_dev
    # bad transpose flag
    assert f(b"R", b"X", b"N", 4, 4, 4, 1.0, 16, 4, 16, 4, 0.0, 16, 4, 0, None) == ug.ERR_ARG
    # bad major
    assert f(b"Q", b"N", b"N", 4, 4, 4, 1.0, 16, 4, 16, 4, 0.0, 16, 4, 0, None) == ug.ERR_ARG
    # negative size
    assert f(b"R", b"N", b"N", -1, 4, 4, 1.0, 16, 4, 16, 4, 0.0, 16, 4, 0, None) == ug.ERR_ARG
    # lda < K for a row-major 'N' A
    assert f(b"R", b"N", b"N", 4, 4, 8, 1.0, 16, 4, 16, 4, 0.0, 16, 4, 0, None) == ug.ERR_ARG
    # ldc < N
    assert f(b"R", b"N", b"N", 4, 8, 4, 1.0, 16, 4, 16, 8, 0.0, 16, 4, 0, None) == ug.ERR_ARG
    # NULL C
    assert f(b"R", b"N", b"N", 4, 4, 4, 1.0, 16, 4, 16, 4, 0.0, None, 4, 0, None) == ug.ERR_ARG
    assert b"leading" in lib.ugemm_last_error_message() or lib.ugemm_last_error() == ug.ERR_ARG
    # empty problems are a no-op before any device work
    assert f(b"R", b"N", b"N", 0, 4, 4, 1.0, None, 4, None, 4, 0.0, None, 4, 0, None) == ug.OK


def test_noalloc_refuses_forms_it_does_not_run(lib):
    """The allocation-free entry point runs the bf16 split forms; the others
    are refused before any device work (host-only check)."""
    f = lib.ugemm_sgemm_dev_noalloc
    f.argtypes = [ctypes.c_char, ctypes.c_char, ctypes.c_char, ctypes.c_int, ctypes.c_int,
                  ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                  ctypes.c_void_p]
    f.restype = ctypes.c_int
    for prec in (ug.PREC_SIMT, ug.PREC_FP16X3):
        assert f(b"R", b"N", b"N", 4, 4, 4, 1.0, 16, 4, 16, 4, 0.0, 16, 4, prec, None) == \
            ug.ERR_UNSUPPORTED
        assert b"bf16 split forms" in lib.ugemm_last_error_message()


def test_compat_requires_init(lib):
    assert lib.sgemm_cuda_status(b"N", b"N", 2, 2, 2, 1.0, None, None, 0.0, None) == ug.ERR_NOT_INIT


def test_workspace_query_is_host_only(lib):
    # split-precision form: 3 bf16 pieces of A (M x Kp) and B (N x Kp)
    # (fewer tiles than SMs, shallow k: neither split-K nor a wave tail)
    n = ug.workspace_bytes("N", "N", 1536, 1536, 512, 512, 1536, "bf16x6")
    assert n == 2 * 3 * 1536 * 512 * 2
    # a deep k under a small output runs as split-K slices: partial tiles too
    pieces = 3 * (64 + 200) * 40000 * 2
    assert ug.workspace_bytes("N", "N", 64, 200, 40000, 40000, 200, "bf16x6") > pieces + 2 * 64 * 200 * 4
    assert ug.workspace_bytes("N", "N", 1024, 1024, 1024, 1024, 1024, "simt") == 0
    # unaligned lda forces a packed copy in the SIMT form
    assert ug.workspace_bytes("N", "N", 64, 64, 63, 63, 64, "simt") > 0


def test_fp16x3_workspace_has_two_pieces_and_scale_words(lib):
    # two fp16 pieces per element, each operand followed by a trailer of one
    # word per row (rounded up to 256 bytes) that receives the row's largest
    # magnitude, from which the row's scale follows
    n = ug.workspace_bytes("N", "N", 1536, 1536, 512, 512, 1536, "fp16x3")
    assert n == 2 * (2 * 1536 * 512 * 2 + 1536 * 4)
    assert n < ug.workspace_bytes("N", "N", 1536, 1536, 512, 512, 1536, "bf16x6")
    # K rounds up to 32 (the 64-deep stages read the rest as TMA zero fill)
    assert ug.workspace_bytes("T", "T", 1536, 1536, 33, 1536, 33, "fp16x3") == \
        2 * (2 * 1536 * 64 * 2 + 1536 * 4)
    # rows that are not a multiple of 64: the trailer rounds up to 256 bytes
    assert ug.workspace_bytes("N", "N", 1000, 1000, 512, 512, 1000, "fp16x3") == \
        2 * (2 * 1000 * 512 * 2 + 4096)


def test_tf32x3_workspace_has_two_four_byte_pieces(lib):
    # two tf32 pieces (FP32 containers) per element, no scale words
    n = ug.workspace_bytes("N", "N", 1536, 1536, 512, 512, 1536, "tf32x3")
    assert n == 2 * (2 * 1536 * 512 * 4)
    assert ug.workspace_bytes("T", "T", 1000, 1000, 33, 1000, 33, "tf32x3") == \
        2 * (2 * 1000 * 64 * 4)


def test_fast_division_constants_are_exact():
    """The implicit im2col gather divides pixel and tap indices by run-time
    constants with q = (umulhi(x, m) + x) >> s (internal.h FastDiv);
    the constants are exact for every divisor the conv geometry can produce
    and every index below 2^31."""
    rng = np.random.default_rng(0)
    divisors = list(range(1, 300)) + [3136, 784, 196, 49, 12544, 100352, 2**20 + 7, 2**30 + 3]
    xs = np.concatenate([np.arange(0, 70000, dtype=np.uint64),
                         rng.integers(0, 2**31, 200000, dtype=np.uint64),
                         np.array([2**31 - 1, 2**31 - 2], dtype=np.uint64)])
    for d in divisors:
        s = 0
        while (1 << s) < d:
            s += 1
        m = ((1 << 32) * ((1 << s) - d)) // d + 1
        assert 0 < m <= 0xFFFFFFFF
        q = (((xs * np.uint64(m)) >> np.uint64(32)) + xs) >> np.uint64(s)
        assert np.array_equal(q, xs // np.uint64(d)), d
