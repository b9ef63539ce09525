"""The FP16x3 split form: every row of op(A) and every column of op(B) is
scaled by a power of two chosen from its own largest magnitude and written as
two fp16 pieces.  These cases check the scale logic where it matters --
operands far above fp16's range, far below it, one outlier element, rows and
columns 2^30 apart, an infinity, an all-zero operand -- against the GPU FP64
oracle, row by row as well as normwise, and that the form matches BF16x6 and
the FP32 SIMT form on ordinary inputs."""
import math

import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import ugemm_gb300 as ug  # noqa: E402

TOL = 2e-6  # normwise bound of the other FP32-accurate GEMM parity tests


@pytest.fixture(scope="module", autouse=True)
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ug.build()
    ug.load()


def gemm(ta, tb, A, B, C0, alpha, beta, prec):
    M = A.shape[0] if ta == "N" else A.shape[1]
    K = A.shape[1] if ta == "N" else A.shape[0]
    N = B.shape[1] if tb == "N" else B.shape[0]
    C = C0.clone()
    ug.sgemm_dev(ta, tb, M, N, K, alpha, A, A.stride(0), B, B.stride(0), beta, C, N,
                 precision=prec)
    torch.cuda.synchronize()
    return C


def ref64(ta, tb, A, B, C0, alpha, beta):
    return ug.ref64(ta, tb, A, B, C0, alpha, beta)


def nerr(got, ref):
    return float(torch.linalg.norm(got.double() - ref) / torch.linalg.norm(ref))


def worst_row(got, ref):
    """max_i ||C_i - ref_i|| / ||ref_i|| over the rows with a non-zero reference."""
    d = (got.double() - ref).norm(dim=1)
    n = ref.norm(dim=1)
    return float((d[n > 0] / n[n > 0]).max())


def worst_col(got, ref):
    return worst_row(got.T, ref.T)


def uniform(shape, g, scale=1.0):
    return (torch.rand(shape, device="cuda", generator=g) * 2 - 1) * scale


@pytest.mark.parametrize("ea,eb", [(100, -90), (-60, -60), (60, 60), (0, 0), (20, -3)])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T")])
def test_operands_far_from_fp16_range(ea, eb, ta, tb):
    """Operands scaled by 2^ea and 2^eb: without the power-of-two scale fp16
    would overflow (|x| > 65504) or lose every piece to underflow."""
    g = torch.Generator(device="cuda").manual_seed(1000 + ea * 7 + eb)
    M, N, K = 300, 260, 700
    A = uniform((M, K) if ta == "N" else (K, M), g, math.ldexp(1.0, ea))
    B = uniform((K, N) if tb == "N" else (N, K), g, math.ldexp(1.0, eb))
    scale_c = math.ldexp(1.0, ea + eb)
    C0 = uniform((M, N), g, scale_c)
    ref = ref64(ta, tb, A, B, C0, 1.25, 0.5)
    got = gemm(ta, tb, A, B, C0, 1.25, 0.5, "fp16x3")
    assert torch.isfinite(got).all()
    assert nerr(got, ref) < TOL, (ea, eb, ta, tb, nerr(got, ref))


def test_outlier_element_leaves_the_other_rows_accurate():
    """One element 2^40 times the others: it sets the scale of its own row of
    A only, so every other row of C keeps FP32 accuracy (an operand-wide
    scale would flush all of them to zero, and a normwise check, dominated by
    the outlier's row, would not see it)."""
    g = torch.Generator(device="cuda").manual_seed(5)
    M, N, K = 257, 129, 513
    A = uniform((M, K), g)
    A[17, 33] = math.ldexp(1.0, 40)
    B = uniform((K, N), g)
    C0 = torch.zeros((M, N), device="cuda")
    ref = ref64("N", "N", A, B, C0, 1.0, 0.0)
    got = gemm("N", "N", A, B, C0, 1.0, 0.0, "fp16x3")
    simt = gemm("N", "N", A, B, C0, 1.0, 0.0, "simt")
    assert nerr(got, ref) < TOL
    assert worst_row(got, ref) <= worst_row(simt, ref), (worst_row(got, ref), worst_row(simt, ref))
    assert worst_row(got, ref) < TOL


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
def test_rows_and_columns_far_apart(ta, tb):
    """Every other row of op(A) and every third column of op(B) scaled by
    2^-30: each row and column gets its own scale, so every row and column
    of C is as accurate as the FP32 SIMT form's."""
    g = torch.Generator(device="cuda").manual_seed(40 + ord(ta) + 2 * ord(tb))
    M, N, K = 300, 390, 1100
    opA = uniform((M, K), g)
    opB = uniform((K, N), g)
    opA[::2] *= math.ldexp(1.0, -30)
    opB[:, ::3] *= math.ldexp(1.0, -30)
    A = opA.contiguous() if ta == "N" else opA.T.contiguous()
    B = opB.contiguous() if tb == "N" else opB.T.contiguous()
    C0 = torch.zeros((M, N), device="cuda")
    ref = ref64(ta, tb, A, B, C0, 1.0, 0.0)
    got = gemm(ta, tb, A, B, C0, 1.0, 0.0, "fp16x3")
    simt = gemm(ta, tb, A, B, C0, 1.0, 0.0, "simt")
    for f in (worst_row, worst_col):
        assert f(got, ref) <= f(simt, ref), (f.__name__, f(got, ref), f(simt, ref))
    assert worst_row(got, ref) < TOL


def test_infinity_does_not_set_the_scale():
    """An infinite element propagates into its own row of C only: the scale
    follows the finite elements, so the rest of a large-valued operand
    (1e6: unscaled it would overflow fp16) stays accurate."""
    g = torch.Generator(device="cuda").manual_seed(8)
    M, N, K = 130, 140, 300
    A = uniform((M, K), g, 1e6)
    A[0, 5] = float("inf")
    B = uniform((K, N), g)
    C0 = torch.zeros((M, N), device="cuda")
    got = gemm("N", "N", A, B, C0, 1.0, 0.0, "fp16x3")
    assert not torch.isfinite(got[0]).any()
    ref = ref64("N", "N", A[1:], B, C0[1:], 1.0, 0.0)
    assert torch.isfinite(got[1:]).all()
    assert nerr(got[1:], ref) < TOL


def test_zero_operand_gives_beta_c():
    g = torch.Generator(device="cuda").manual_seed(6)
    A = torch.zeros((200, 300), device="cuda")
    B = uniform((300, 150), g)
    C0 = uniform((200, 150), g)
    got = gemm("N", "N", A, B, C0, 2.0, 0.5, "fp16x3")
    assert torch.equal(got, C0 * 0.5)


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
def test_matches_bf16x6_and_simt_accuracy(ta, tb):
    """On U[-1,1) inputs FP16x3 is within the FP32-accurate bound and no
    worse than the plain FP32 SIMT form."""
    g = torch.Generator(device="cuda").manual_seed(ord(ta) * 3 + ord(tb))
    M, N, K = 1030, 770, 2100
    A = uniform((M, K) if ta == "N" else (K, M), g)
    B = uniform((K, N) if tb == "N" else (N, K), g)
    C0 = uniform((M, N), g)
    ref = ref64(ta, tb, A, B, C0, 1.5, 0.5)
    errs = {p: nerr(gemm(ta, tb, A, B, C0, 1.5, 0.5, p), ref) for p in ("fp16x3", "bf16x6", "simt")}
    assert errs["fp16x3"] < TOL, errs
    assert errs["fp16x3"] <= errs["simt"], errs


def test_repeated_calls_are_bit_identical():
    """The scale is recomputed from scratch on every call (the max word is
    cleared first), so a second call on other data is not affected by the
    first, and the same call twice gives the same bits."""
    g = torch.Generator(device="cuda").manual_seed(9)
    big = uniform((512, 512), g, 1e15)
    small = uniform((512, 512), g)
    C0 = torch.zeros((512, 512), device="cuda")
    gemm("N", "N", big, big, C0, 1.0, 0.0, "fp16x3")
    first = gemm("N", "N", small, small, C0, 1.0, 0.0, "fp16x3")
    second = gemm("N", "N", small, small, C0, 1.0, 0.0, "fp16x3")
    assert torch.equal(first, second)
    assert nerr(first, ref64("N", "N", small, small, C0, 1.0, 0.0)) < TOL
