"""The allocation-free entry point, ugemm_sgemm_dev_noalloc.

Callers that must not allocate device memory while they run (a fixed
device-memory budget, a framework that owns every allocation, a
latency-critical loop) use this entry point: its scratch is a fixed array in
the library's device memory instead of a workspace grown with cudaMalloc.
These tests call it through the C ABI and require, on two calls in a row
(the second reuses the array the first one filled), the same bits as the
ordinary entry point, ugemm_sgemm_dev, and FP32 accuracy against the GPU
FP64 oracle; they cover a shape whose last wave of tiles runs as the
wave-tail launch (its partial tiles also live in the array), column-major
calls, the two-piece BF16X3 form, alpha = 0, the error word through
ugemm_check, and the refusal of a problem larger than the array.  This file
is collected last on purpose.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import ugemm_gb300 as ug  # noqa: E402

TOL = 2e-6  # normwise bound the other GEMM parity tests use


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ug.build()
    lib = ug.load()
    f = lib.ugemm_sgemm_dev_noalloc
    f.argtypes = [ctypes.c_char, ctypes.c_char, ctypes.c_char, ctypes.c_int, ctypes.c_int,
                  ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                  ctypes.c_void_p]
    f.restype = ctypes.c_int
    return lib


def operands(major, ta, tb, M, N, K, seed):
    """Row-major storage of the operands; a column-major call reads the same
    memory as the transposed matrices."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    if major == "C":  # column-major X (r x c) is row-major X^T (c x r)
        a_shape = (K, M) if ta == "N" else (M, K)
        b_shape = (N, K) if tb == "N" else (K, N)
        c_shape = (N, M)
    else:
        a_shape = (M, K) if ta == "N" else (K, M)
        b_shape = (K, N) if tb == "N" else (N, K)
        c_shape = (M, N)
    A = torch.rand(a_shape, device="cuda", generator=g) * 2 - 1
    B = torch.rand(b_shape, device="cuda", generator=g) * 2 - 1
    C = torch.rand(c_shape, device="cuda", generator=g) * 2 - 1
    return A, B, C


def reference(major, ta, tb, A, B, C0, alpha, beta):
    if major == "C":  # C^T = op(B)^T op(A)^T in row-major storage
        return ug.ref64(tb, ta, B, A, C0, alpha, beta)
    return ug.ref64(ta, tb, A, B, C0, alpha, beta)


CASES = [
    # major, ta, tb, M, N, K, alpha, beta, precision
    ("R", "N", "T", 1000, 700, 900, 1.5, 0.5, "bf16x6"),
    ("R", "T", "N", 515, 1030, 333, 1.5, 0.5, "bf16x6"),
    # 17 x 9 = 153 tiles of 128 x 256 on 152 SMs: the last wave runs as the wave tail
    ("R", "N", "N", 2176, 2304, 1024, 1.0, 0.0, "bf16x6"),
    ("C", "T", "N", 700, 600, 500, 0.75, 1.25, "bf16x6"),
    ("R", "N", "N", 640, 384, 512, 1.0, 0.5, "bf16x3"),
    ("R", "N", "N", 320, 200, 100, 0.0, 0.5, "bf16x9"),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "-".join(map(str, c[:6])) + "-" + c[8])
def test_noalloc_matches_workspace_entry_point_twice(lib, case):
    major, ta, tb, M, N, K, alpha, beta, prec = case
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):  # the second call reuses the array the first one filled
        A, B, C0 = operands(major, ta, tb, M, N, K, seed=100 * call + M + N + K)
        lda, ldb, ldc = A.stride(0), B.stride(0), C0.stride(0)
        want = C0.clone()
        ug.sgemm_dev(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, want, ldc, precision=prec,
                     major=major)
        got = C0.clone()
        rc = lib.ugemm_sgemm_dev_noalloc(major.encode(), ta.encode(), tb.encode(), M, N, K,
                                         alpha, A.data_ptr(), lda, B.data_ptr(), ldb, beta,
                                         got.data_ptr(), ldc, ug.PRECISIONS[prec], stream)
        assert rc == ug.OK, lib.ugemm_last_error_message()
        ug.check()  # no kernel wait of either call gave up
        assert torch.equal(got, want), (call, float((got - want).abs().max()))
        ref = reference(major, ta, tb, A, B, C0, alpha, beta)
        err = float(torch.linalg.norm(got.double() - ref) / torch.linalg.norm(ref))
        bound = 1e-2 if prec == "bf16x3" else TOL  # BF16X3 keeps ~16 bits: a study form
        assert err < bound, (call, err)


def test_noalloc_error_word_is_reported_once(lib):
    """A code planted in the entry point's own error word (a host copy; no
    fault, no hang) does not stop the next call, and ugemm_check reports it
    once."""
    stream = torch.cuda.current_stream().cuda_stream
    A, B, C0 = operands("R", "N", "N", 600, 500, 700, seed=3)
    ref = ug.ref64("N", "N", A, B)

    def call():
        C = torch.full_like(C0, float("nan"))
        rc = lib.ugemm_sgemm_dev_noalloc(b"R", b"N", b"N", 600, 500, 700, 1.0, A.data_ptr(), 700,
                                         B.data_ptr(), 500, 0.0, C.data_ptr(), 500,
                                         ug.PREC_BF16X6, stream)
        assert rc == ug.OK, lib.ugemm_last_error_message()
        torch.cuda.synchronize()
        assert float(torch.linalg.norm(C.double() - ref) / torch.linalg.norm(ref)) < TOL

    call()  # the first call on the device sets up the array's and the word's addresses
    ug.check()
    assert lib.ugemm_debug_set_error_word(1, 4) == ug.OK
    call()
    with pytest.raises(ug.UgemmError) as err:
        ug.check()
    assert err.value.status == ug.ERR_TIMEOUT and "code 4" in str(err.value)
    ug.check()


def test_noalloc_refuses_problems_beyond_its_array(lib):
    M = N = K = 4096  # 6 * 8192 * 4096 bytes of pieces > 64 MiB
    A = torch.zeros((M, K), device="cuda")
    C = torch.zeros((M, N), device="cuda")
    rc = lib.ugemm_sgemm_dev_noalloc(b"R", b"N", b"N", M, N, K, 1.0, A.data_ptr(), K,
                                     A.data_ptr(), N, 0.0, C.data_ptr(), N, ug.PREC_BF16X6,
                                     torch.cuda.current_stream().cuda_stream)
    assert rc == ug.ERR_ARENA_TOO_SMALL
    assert b"fixed array" in lib.ugemm_last_error_message()
