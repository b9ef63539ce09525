"""The allocation-free entry point, ugemm_sgemm_dev_noalloc.

Callers that must not allocate device memory while they run (a fixed
device-memory budget, a framework that owns every allocation, a
latency-critical loop) use this entry point: its scratch is a fixed array in
the library's device memory instead of a workspace grown with cudaMalloc.
These tests call it through the C ABI and compare its output with the
ordinary entry point, ugemm_sgemm_dev, on two calls in a row (the second call
reuses the array the first one filled), and check that a problem larger than
the fixed array is refused.  This file is collected last on purpose.
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


def operands(ta, tb, M, N, K, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.rand((M, K) if ta == "N" else (K, M), device="cuda", generator=g) * 2 - 1
    B = torch.rand((K, N) if tb == "N" else (N, K), device="cuda", generator=g) * 2 - 1
    C = torch.rand((M, N), device="cuda", generator=g) * 2 - 1
    return A, B, C


def test_noalloc_matches_workspace_entry_point_twice(lib):
    stream = torch.cuda.current_stream().cuda_stream
    for call, (ta, tb, M, N, K, seed) in enumerate([("N", "T", 1000, 700, 900, 1),
                                                    ("T", "N", 515, 1030, 333, 2)]):
        A, B, C0 = operands(ta, tb, M, N, K, seed)
        want = C0.clone()
        ug.sgemm_dev(ta, tb, M, N, K, 1.5, A, A.stride(0), B, B.stride(0), 0.5, want, N,
                     precision="bf16x6")
        got = C0.clone()
        rc = lib.ugemm_sgemm_dev_noalloc(b"R", ta.encode(), tb.encode(), M, N, K, 1.5,
                                         A.data_ptr(), A.stride(0), B.data_ptr(), B.stride(0),
                                         0.5, got.data_ptr(), N, ug.PREC_BF16X6, stream)
        assert rc == ug.OK, lib.ugemm_last_error_message()
        torch.cuda.synchronize()
        err = float(torch.linalg.norm(got.double() - want.double()) /
                    torch.linalg.norm(want.double()))
        assert err < TOL, (call, err)


def test_noalloc_refuses_problems_beyond_its_array(lib):
    M = N = K = 4096  # 6 * 8192 * 4096 bytes of pieces > 64 MiB
    A = torch.zeros((M, K), device="cuda")
    C = torch.zeros((M, N), device="cuda")
    rc = lib.ugemm_sgemm_dev_noalloc(b"R", b"N", b"N", M, N, K, 1.0, A.data_ptr(), K,
                                     A.data_ptr(), N, 0.0, C.data_ptr(), N, ug.PREC_BF16X6,
                                     torch.cuda.current_stream().cuda_stream)
    assert rc == ug.ERR_ARENA_TOO_SMALL
    assert b"fixed array" in lib.ugemm_last_error_message()
