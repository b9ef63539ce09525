"""GPU parity: the CUDA forms (SIMT, split-precision tcgen05) through the C
ABI against the CPU oracle and an FP64 reference, on the reference's own
golden fixtures, its known-answer test, ragged shapes, every transpose pair,
leading-dimension padding and the beta == 0 contract."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import ugemm_gb300 as ug  # noqa: E402

FORMS = ("simt", "bf16x6", "bf16x9", "fp16x3", "tf32x3")
# Normwise relative error bound vs FP64 for the FP32-accurate forms at the
# small sizes below (FP32 unit roundoff is 6e-8; observed errors ~1e-7).
TOL_FP32 = 2e-6


@pytest.fixture(scope="module", autouse=True)
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ug.build()
    ug.load()
    torch.cuda.init()
    yield


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def run(ta, tb, M, N, K, alpha, A, B, beta, C, prec, lda=None, ldb=None, ldc=None):
    """Row-major GEMM on device copies of numpy arrays; returns C as numpy."""
    a, b, c = dev(A), dev(B), dev(C)
    ug.sgemm_dev(ta, tb, M, N, K, alpha, a, lda or A.shape[1], b, ldb or B.shape[1], beta, c,
                 ldc or C.shape[1], precision=prec)
    torch.cuda.synchronize()
    return c.cpu().numpy()


def ref64(ta, tb, M, N, K, alpha, A, B, beta, C):
    return oracle.dgemm(ta, tb, M, N, K, alpha, A.astype(np.float64), B.astype(np.float64), beta,
                        C.astype(np.float64))


def inputs(rng, ta, tb, M, N, K):
    A = rng.uniform(-1, 1, oracle.op_shape(ta, M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, oracle.op_shape(tb, K, N)).astype(np.float32)
    C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    return A, B, C


def test_device_is_gb300():
    sms, major, minor = ug.device_info()
    assert (major, minor) == (10, 3)
    assert sms >= 100


@pytest.mark.parametrize("prec", FORMS)
def test_known_answer_rnn_3x3x2(golden, prec):
    """sgemm_test.c:186-200."""
    A, B = golden["kat/rnn3x3x2/A"], golden["kat/rnn3x3x2/B"]
    C = np.zeros((3, 3), dtype=np.float32)
    out = run("N", "N", 3, 3, 2, 1.0, A, B, 0.0, C, prec)
    assert np.array_equal(out, golden["kat/rnn3x3x2/out"])


@pytest.mark.parametrize("prec", FORMS)
def test_golden_fixtures_host_api(golden, prec):
    """Every FP32 golden case (reference sgemm_cpu output) through ugemm_sgemm."""
    cases = [c for c in golden["cases"] if str(c).startswith("s/")]
    for name in cases:
        g = lambda k: golden[f"{name}/{k}"]  # noqa: E731
        M, N, K = (int(x) for x in g("meta"))
        alpha, beta = (float(x) for x in g("ab"))
        major, ta, tb = bytes(g("flags")).decode()
        A, B, C = g("A"), g("B"), g("C").copy()
        ug.ugemm_sgemm(major, ta, tb, M, N, K, alpha, A, A.shape[1], B, B.shape[1], beta, C,
                       C.shape[1], precision=prec)
        ref = g("sgemm_cpu")
        scale = max(np.abs(ref).max(), 1e-30)
        assert np.abs(C - ref).max() / scale < 1e-5, (name, prec)


@pytest.mark.parametrize("prec", FORMS)
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
def test_ragged_shapes_vs_fp64(prec, ta, tb):
    rng = np.random.default_rng(11)
    for (M, N, K) in [(1, 1, 1), (17, 17, 17), (33, 65, 129), (130, 257, 70), (255, 129, 300),
                      (129, 300, 33)]:
        for (alpha, beta) in [(1.0, 0.0), (1.5, 0.5)]:
            A, B, C = inputs(rng, ta, tb, M, N, K)
            out = run(ta, tb, M, N, K, alpha, A, B, beta, C, prec)
            err = oracle.normwise_error(out, ref64(ta, tb, M, N, K, alpha, A, B, beta, C))
            assert err < TOL_FP32, (prec, ta, tb, M, N, K, alpha, beta, err)


def test_bf16x3_is_truncated_but_close():
    """Two pieces carry ~16 bits: error well above FP32, well below bf16."""
    rng = np.random.default_rng(5)
    A, B, C = inputs(rng, "N", "N", 200, 300, 256)
    out = run("N", "N", 200, 300, 256, 1.0, A, B, 0.0, C, "bf16x3")
    err = oracle.normwise_error(out, ref64("N", "N", 200, 300, 256, 1.0, A, B, 0.0, C))
    assert 1e-7 < err < 1e-4


@pytest.mark.parametrize("prec", FORMS)
def test_config1_1024_matches_cpu_oracle(prec):
    """1024^3, alpha=1, beta=0, U[-1,1): vs the reference's AVX256 SGEMM
    (restated) and blocked sgemm_c, reported as max-abs-diff / max-abs and
    the check_sgemm.c cmp_results line."""
    rng = np.random.default_rng(20261204)
    n = 1024
    A = rng.uniform(-1, 1, (n, n)).astype(np.float32)
    B = rng.uniform(-1, 1, (n, n)).astype(np.float32)
    C = np.zeros((n, n), dtype=np.float32)
    out = run("N", "N", n, n, n, 1.0, A, B, 0.0, C, prec)
    cpu = oracle.sgemm_avx256_mt(8, "N", "N", n, n, n, 1.0, A, B, 0.0, C.copy())
    rel = np.abs(out - cpu).max() / np.abs(cpu).max()
    assert rel < 1e-5, rel
    blk = oracle.sgemm("oracle_sgemm_c", "N", "N", n, n, n, 1.0, A, B, 0.0, C.copy())
    assert np.abs(out - blk).max() / np.abs(blk).max() < 1e-5
    label, std_err, std_ref, max_err, _ = oracle.cmp_results(cpu, out)
    assert std_err / std_ref < 1e-6
    print(f"{prec}: max-abs-diff/max-abs={rel:.3e} cmp_results stdErr/stdRef={std_err/std_ref:.3e} "
          f"{label}")


@pytest.mark.parametrize("prec", FORMS)
def test_beta_zero_does_not_read_c(prec):
    """sgemm_ocl2.h:86-88: with beta == 0 a NaN-filled C must not leak."""
    rng = np.random.default_rng(2)
    A, B, _ = inputs(rng, "N", "N", 64, 96, 40)
    C = np.full((64, 96), np.nan, dtype=np.float32)
    out = run("N", "N", 64, 96, 40, 1.0, A, B, 0.0, C, prec)
    assert np.isfinite(out).all()


@pytest.mark.parametrize("prec", FORMS)
def test_leading_dimensions_and_unaligned_operands(prec):
    """lda/ldb not multiples of 4 (TMA-incompatible: packed copy) and a padded
    ldc whose padding must stay untouched."""
    rng = np.random.default_rng(4)
    M, N, K = 70, 50, 37
    lda, ldb, ldc = K + 3, N + 1, N + 5
    Af = rng.uniform(-1, 1, (M, lda)).astype(np.float32)
    Bf = rng.uniform(-1, 1, (K, ldb)).astype(np.float32)
    Cf = rng.uniform(-1, 1, (M, ldc)).astype(np.float32)
    out = run("N", "N", M, N, K, 1.25, Af, Bf, 0.75, Cf, prec, lda=lda, ldb=ldb, ldc=ldc)
    ref = ref64("N", "N", M, N, K, 1.25, np.ascontiguousarray(Af[:, :K]),
                np.ascontiguousarray(Bf[:, :N]), 0.75, np.ascontiguousarray(Cf[:, :N]))
    assert oracle.normwise_error(out[:, :N], ref) < TOL_FP32
    assert np.array_equal(out[:, N:], Cf[:, N:])


def test_column_major_calls():
    """major='C' (ugemm.h:226-284) goes through the operand swap."""
    rng = np.random.default_rng(8)
    M, N, K = 45, 38, 29
    for ta in "NT":
        for tb in "NT":
            # column-major storage = row-major arrays of the transposed shape
            A = rng.uniform(-1, 1, oracle.op_shape(ta, M, K)[::-1]).astype(np.float32)
            B = rng.uniform(-1, 1, oracle.op_shape(tb, K, N)[::-1]).astype(np.float32)
            C = rng.uniform(-1, 1, (N, M)).astype(np.float32)
            ref = C.copy()
            oracle.sgemm("oracle_sgemm_cpu", ta, tb, M, N, K, 1.5, A, B, 0.5, ref, major="C")
            out = C.copy()
            ug.ugemm_sgemm("C", ta, tb, M, N, K, 1.5, A, A.shape[1], B, B.shape[1], 0.5, out,
                           out.shape[1], precision="simt")
            assert np.abs(out - ref).max() / np.abs(ref).max() < 1e-5


def test_compat_api_sgemm_test_pattern():
    """sgemm_test.c:202-258: A[i]=B[i]=i+1, C=1, 1023x1000x1023, RNN/RNT/RTN,
    through sgemm_cuda_init / sgemm_cuda / sgemm_cuda_finish."""
    M, N, K = 1023, 1000, 1023
    ug.sgemm_cuda_init(0, 0, (M * K + K * N + M * N) * 10 * 4)
    try:
        A = (np.arange(M * K, dtype=np.float64) + 1).astype(np.float32)
        B = (np.arange(K * N, dtype=np.float64) + 1).astype(np.float32)
        for prec in ("simt", "bf16x6"):
            ug.set_precision(prec)
            for ta, tb in (("N", "N"), ("N", "T"), ("T", "N")):
                a = A.reshape(oracle.op_shape(ta, M, K))
                b = B.reshape(oracle.op_shape(tb, K, N))
                C = np.ones((M, N), dtype=np.float32)
                ug.sgemm_cuda(ta, tb, M, N, K, 1.0, a, b, 0.0, C)
                ref = (a.astype(np.float64) if ta == "N" else a.astype(np.float64).T) @ \
                      (b.astype(np.float64) if tb == "N" else b.astype(np.float64).T)
                assert oracle.normwise_error(C, ref) < 1e-6, (prec, ta, tb)
    finally:
        ug.set_precision("auto")
        ug.sgemm_cuda_finish()


def test_compat_arena_too_small_is_an_error():
    ug.sgemm_cuda_init(0, 0, 1024)
    try:
        a = np.ones((64, 64), dtype=np.float32)
        c = np.zeros((64, 64), dtype=np.float32)
        with pytest.raises(ug.UgemmError) as e:
            ug.sgemm_cuda("N", "N", 64, 64, 64, 1.0, a, a, 0.0, c)
        assert e.value.status == ug.ERR_ARENA_TOO_SMALL
    finally:
        ug.sgemm_cuda_finish()


def test_double_init_is_an_error():
    ug.sgemm_cuda_init(0, 0, 1 << 20)
    try:
        with pytest.raises(ug.UgemmError):
            ug.sgemm_cuda_init(0, 0, 1 << 20)
    finally:
        ug.sgemm_cuda_finish()


def test_zero_k_and_zero_alpha_scale_c():
    rng = np.random.default_rng(9)
    A, B, C = inputs(rng, "N", "N", 33, 44, 5)
    out = run("N", "N", 33, 44, 0, 1.0, A, B, 0.5, C, "simt")
    np.testing.assert_array_equal(out, (C * np.float32(0.5)).astype(np.float32))
    out = run("N", "N", 33, 44, 5, 0.0, A, B, 0.0, C, "bf16x6")
    assert not out.any()


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
@pytest.mark.parametrize("beta", [0.5, 0.0])
def test_deep_narrow_gemm_runs_split_k(ta, tb, beta):
    """A small output with a deep k (a weight-gradient shape) has fewer tiles
    than the GPU has SMs: the split form cuts k into slices whose partial
    tiles one reduce launch sums; beta == 0 still never reads C."""
    M, N, K = 64, 200, 40000
    g = torch.Generator(device="cuda").manual_seed(11)
    A = torch.rand(oracle.op_shape(ta, M, K), device="cuda", generator=g) * 2 - 1
    B = torch.rand(oracle.op_shape(tb, K, N), device="cuda", generator=g) * 2 - 1
    C0 = torch.rand((M, N + 3), device="cuda", generator=g) * 2 - 1
    if beta == 0.0:
        C0[:, :N] = float("nan")
    C = C0.clone()
    ug.profile_enable(True)
    try:
        ug.sgemm_dev(ta, tb, M, N, K, 1.5, A, A.shape[1], B, B.shape[1], beta, C, N + 3,
                     precision="bf16x6")
        prof = ug.profile_collect()
    finally:
        ug.profile_enable(False)
    assert prof["aux"][1] == 1  # the split-K reduce
    a64 = A.double() if ta == "N" else A.double().T
    b64 = B.double() if tb == "N" else B.double().T
    ref = 1.5 * (a64 @ b64)
    if beta != 0.0:
        ref = ref + beta * C0[:, :N].double()
    err = float(torch.linalg.norm(C[:, :N].double() - ref) / torch.linalg.norm(ref))
    assert err < 2e-6, err
    assert torch.equal(C[:, N:], C0[:, N:])


def test_fp32_peak_probe_is_a_plausible_rate():
    """The measured FP32 FMA peak the benchmark divides the SIMT form by:
    positive, below the nominal rate of 128 FMA lanes per SM at the
    device's maximum clock, and above half of it."""
    props = torch.cuda.get_device_properties(0)
    nominal = props.multi_processor_count * 128 * 2 * 2.07e9 / 1e12
    peak = ug.fp32_peak(50.0)
    assert 0.5 * nominal < peak < 1.05 * nominal, (peak, nominal)


@pytest.mark.parametrize("K", [1000, 1001, 8192, 8200])
def test_fp16x3_one_pass_row_split_matches_two_pass(K):
    """op(A) with rows contiguous in k (NN, K <= 8192) takes its FP16x3 row
    maxima and pieces in one pass; the same op(A) stored transposed (TN)
    takes the maximum pass and the split pass.  Same words, same pieces:
    C must be bit-identical, including a zero row, a row with an infinity
    (its maximum ignores it) and a row 2^30 below the others; an odd K
    with rows padded by NaNs that must not be read; K = 8200 takes the two
    passes on both sides."""
    rng = np.random.default_rng(K)
    M, N = 256, 192
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    A[3] = 0.0
    A[7, 5] = np.inf
    A[11] *= np.float32(2.0 ** -30)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    # rows padded to a multiple of 4 floats (16-byte aligned), as the one
    # pass needs; the padding holds garbage that must not be read
    lda = -(-K // 4) * 4
    Ap = np.full((M, lda), np.nan, np.float32)
    Ap[:, :K] = A
    nn = run("N", "N", M, N, K, 1.25, Ap, B, 0.5, C, "fp16x3", lda=lda)
    tn = run("T", "N", M, N, K, 1.25, np.ascontiguousarray(A.T), B, 0.5, C, "fp16x3", lda=M)
    assert np.array_equal(nn.view(np.int32), tn.view(np.int32))
    finite = np.isfinite(A).all(axis=1)
    ref = ref64("N", "N", int(finite.sum()), N, K, 1.25, A[finite], B, 0.5, C[finite])
    got = nn[finite].astype(np.float64)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < TOL_FP32
    assert not np.isfinite(nn[7]).any()
