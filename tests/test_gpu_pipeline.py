"""GPU parity of the pipelined host-pointer path: large ugemm_sgemm /
sgemm_cuda calls run as k slabs accumulated on the device, then row bands
that finish the rest of k and go back while later bands compute; the
result must equal an FP64 GEMM of the same operands, for every transpose
pair, beta == 0 and beta != 0, padded leading dimensions, in both forms.
The operands here are plain numpy arrays -- pageable memory, as the
reference's callers pass (sgemm_test.c's static arrays) -- which the path
reads with copy kernels where the device addresses pageable memory; pinned
buffers (copy engines) must give the same bits."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import ugemm_gb300 as ug  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ug.build()
    ug.load()


def fp64(ta, tb, alpha, A, B, beta, C, M, N, K):
    dev = torch.device("cuda")
    a = torch.from_numpy(A).to(dev, torch.float64)
    b = torch.from_numpy(B).to(dev, torch.float64)
    a = a[:M, :K] if ta == "N" else a[:K, :M].T
    b = b[:K, :N] if tb == "N" else b[:N, :K].T
    c = torch.from_numpy(C[:, :N]).to(dev, torch.float64)
    return (alpha * (a @ b) + beta * c).cpu().numpy()


@pytest.mark.parametrize("prec", ["bf16x6", "fp16x3", "simt"])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
@pytest.mark.parametrize("beta", [0.0, 0.5])
def test_banded_host_gemm_matches_fp64(prec, ta, tb, beta):
    rng = np.random.default_rng(ord(ta) * 7 + ord(tb) + int(beta * 10))
    M, N, K = 4100, 3000, 2500
    pad = 4 if prec == "simt" else 3  # SIMT bands need 16-byte pitches; split takes any
    A = rng.uniform(-1, 1, (M, K + pad) if ta == "N" else (K, M + pad)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N + pad) if tb == "N" else (N, K + pad)).astype(np.float32)
    C = rng.uniform(-1, 1, (M, N + 5)).astype(np.float32)
    ref = fp64(ta, tb, 1.25, A, B, beta, C, M, N, K)
    out = C.copy()
    ug.ugemm_sgemm("R", ta, tb, M, N, K, 1.25, A, A.shape[1], B, B.shape[1], beta, out,
                   out.shape[1], precision=prec)
    err = float(np.linalg.norm(out[:, :N].astype(np.float64) - ref) / np.linalg.norm(ref))
    assert err < 2e-6, (prec, ta, tb, beta, err)
    assert np.array_equal(out[:, N:], C[:, N:])  # padding of C untouched


def test_compat_sgemm_cuda_large_call():
    """sgemm_cuda (tight leading dimensions) through the banded path."""
    M, N, K = 4096, 4096, 2048
    rng = np.random.default_rng(3)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (N, K)).astype(np.float32)  # 'T'
    C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    ref = fp64("N", "T", 1.0, A, B, 0.5, C, M, N, K)
    ug.sgemm_cuda_init(0, 0, (M * K + K * N + M * N) * 10 * 4)
    try:
        ug.sgemm_cuda("N", "T", M, N, K, 1.0, A, B, 0.5, C)
    finally:
        ug.sgemm_cuda_finish()
    assert float(np.linalg.norm(C.astype(np.float64) - ref) / np.linalg.norm(ref)) < 2e-6


@pytest.mark.parametrize("prec", ["fp16x3", "bf16x6"])
def test_compat_8192_on_pageable_numpy_arrays(prec):
    """sgemm_cuda at 8192^3 on plain numpy arrays (pageable), the arena sized
    as sgemm_test.c sizes it, against the GPU FP64 oracle; the same call on
    pinned copies of the operands gives the same bits."""
    M = N = K = 8192
    rng = np.random.default_rng(8192)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    C0 = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    dev = torch.device("cuda")
    ref = ug.ref64("N", "N", torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev),
                   torch.from_numpy(C0).to(dev), 1.5, 0.5)
    C = C0.copy()
    ug.sgemm_cuda_init(0, 0, (M * K + K * N + M * N) * 10 * 4)
    try:
        ug.set_precision(prec)
        ug.sgemm_cuda("N", "N", M, N, K, 1.5, A, B, 0.5, C)
        hA, hB = torch.from_numpy(A).pin_memory(), torch.from_numpy(B).pin_memory()
        hC = torch.from_numpy(C0).pin_memory()
        ug._check(ug.load().sgemm_cuda_status(b"N", b"N", M, N, K, 1.5, hA.data_ptr(),
                                              hB.data_ptr(), 0.5, hC.data_ptr()))
    finally:
        ug.set_precision("auto")
        ug.sgemm_cuda_finish()
    got = torch.from_numpy(C).to(dev, torch.float64)
    err = float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))
    assert err < 2e-6, err
    assert np.array_equal(C, hC.numpy())


def run_counted(prec, ta, tb, M, N, K, alpha, beta, seed):
    """One host-pointer call with the launch profiler on; returns the
    normwise error against FP64 and the pre-pass launch count."""
    rng = np.random.default_rng(seed)
    A = rng.uniform(-1, 1, (M, K) if ta == "N" else (K, M)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N) if tb == "N" else (N, K)).astype(np.float32)
    C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    ref = fp64(ta, tb, alpha, A, B, beta, C, M, N, K)
    out = C.copy()
    ug.profile_enable(True)
    try:
        ug.ugemm_sgemm("R", ta, tb, M, N, K, alpha, A, A.shape[1], B, B.shape[1], beta, out, N,
                       precision=prec)
        prof = ug.profile_collect()
    finally:
        ug.profile_enable(False)
    err = float(np.linalg.norm(out.astype(np.float64) - ref) / np.linalg.norm(ref))
    return err, prof["split_prepass"][1]


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "T")])
def test_slab_then_band_schedule(ta, tb):
    """4100 x 3000 x 2500: k1 = 1024 in one slab, the other 1476 of k in
    five bands (1152, 1152, 1152, then the last 644 rows halved: 384 + 260):
    the slab splits A and B, the rest of B splits once, every band splits
    its rows."""
    err, prep = run_counted("bf16x6", ta, tb, 4100, 3000, 2500, 1.25, 0.5, 11)
    assert err < 2e-6, err
    assert prep == 2 * 1 + 1 + 5


@pytest.mark.parametrize("prec", ["bf16x6", "simt"])
@pytest.mark.parametrize("beta", [0.0, -0.75])
def test_bands_only_schedule_for_shallow_k(prec, beta):
    """K < 2048: no slab phase; B whole first, then ten bands (six of 1024
    rows, four of 512) that read their C directly (beta applied by the GEMM
    itself)."""
    err, prep = run_counted(prec, "N", "T", 8192, 2048, 1024, 0.5, beta, 12)
    assert err < 2e-6, (prec, beta, err)
    assert prep == (1 + 10 if prec == "bf16x6" else 0)


def test_deep_k_many_slabs():
    """K = 20000: slabs of 1280, 3840 and 4864 accumulate k1 = 9984 before
    three bands (1024, 512, 512 rows) take the other 10016."""
    K = 20000
    err, prep = run_counted("bf16x6", "T", "N", 2048, 1024, K, 1.0, 0.5, 13)
    assert err < max(2e-6, 2.5e-8 * K ** 0.5), err
    assert prep == 2 * 3 + 1 + 3
