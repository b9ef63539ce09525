"""The GPU FP64 oracle (ugemm_dgemm_oracle_dev) every FP32 form is measured
against, pinned to the reference's own FP64 GEMMs.

* Golden vectors: outputs of the reference's dgemm_cpu (ugemm.h:162),
  _dgemm_c (gemm_cpu.h:284) and dgemm_avx (dgemm_avx.h:844), compiled from
  the reference sources; the GPU oracle sums with fused multiply-adds in k
  order, so it agrees to FP64 rounding, not bit for bit.
* Large shapes: row bands of the 8192^3 config-2 problems (U[-1,1), the
  wide-range set with exponents in [-8, 8] and in [-40, 40]) and the ragged
  4095 x 4097 x 1023 problem, NN / NT / TN, against the CPU restatement of
  _dgemm_c (bit-identical to the reference's, tests/test_oracle_golden.py).
* torch's float64 matmul, which the tests used as the oracle before, is
  compared with it at 8192^3; its measured agreement is printed."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import oracle  # noqa: E402
import ugemm_gb300 as ug  # noqa: E402

BAND = 32  # rows of a large problem checked on the CPU (a few seconds each)


@pytest.fixture(scope="module", autouse=True)
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ug.build()
    ug.load()


def draw(shape, kind, g):
    if kind == "uniform":
        return torch.rand(shape, device="cuda", generator=g) * 2 - 1
    span = 8 if kind == "wide" else 40
    mant = 1 + torch.rand(shape, device="cuda", generator=g)
    sign = torch.where(torch.rand(shape, device="cuda", generator=g) < 0.5, -1.0, 1.0)
    expo = torch.randint(-span, span + 1, shape, device="cuda", generator=g).float()
    return sign * mant * torch.exp2(expo)


def golden_cases(golden):
    return sorted({k.rsplit("/", 1)[0] for k in golden.files if k.startswith("d/")})


def test_matches_the_reference_fp64_gemms(golden):
    cases = golden_cases(golden)
    assert len(cases) >= 8
    for name in cases:
        g = lambda k: golden[f"{name}/{k}"]  # noqa: E731
        M, N, K = (int(x) for x in g("meta"))
        major, ta, tb = bytes(g("flags")).decode()
        A = torch.from_numpy(np.ascontiguousarray(g("A"))).cuda()
        B = torch.from_numpy(np.ascontiguousarray(g("B"))).cuda()
        C = torch.from_numpy(np.ascontiguousarray(g("C"))).cuda()
        ug.dgemm_oracle(ta, tb, M, N, K, 1.5, A, A.shape[1], B, B.shape[1], 0.5, C, C.shape[1],
                        major=major)
        got = C.cpu().numpy()
        for key in ("dgemm_cpu", "dgemm_c", "dgemm_avx"):
            ref = g(key)
            scale = np.abs(ref).max() + 1.0
            assert np.abs(got - ref).max() <= 4 * K * 2.0 ** -53 * scale, (name, key)


@pytest.mark.parametrize("kind", ["uniform", "wide", "wide40"])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N")])
@pytest.mark.parametrize("shape", [(8192, 8192, 8192), (4095, 4097, 1023)])
def test_row_band_matches_the_cpu_restatement(shape, ta, tb, kind):
    M, N, K = shape
    g = torch.Generator(device="cuda").manual_seed(M + N + K + ord(ta) + 3 * ord(tb))
    A = draw((M, K) if ta == "N" else (K, M), kind, g)
    B = draw((K, N) if tb == "N" else (N, K), kind, g)
    C0 = draw((M, N), kind, g)
    got = ug.ref64(ta, tb, A, B, C0, 1.5, 0.5)[:BAND].cpu().numpy()
    # the band's rows of op(A) as an 'N' operand
    a_band = (A[:BAND] if ta == "N" else A[:, :BAND].T).double().contiguous().cpu().numpy()
    b = B.double().cpu().numpy()
    ref = C0[:BAND].double().cpu().numpy().copy()
    oracle.dgemm("N", tb, BAND, N, K, 1.5, a_band, b, 0.5, ref, fn="oracle_dgemm_c")
    err = oracle.normwise_error(got, ref)
    print(f"{shape} {ta}{tb} {kind}: GPU FP64 oracle vs CPU _dgemm_c {err:.2e}")
    assert err < 1e-14, err


@pytest.mark.parametrize("kind", ["uniform", "wide40"])
def test_torch_float64_matmul_against_the_oracle(kind):
    """Records how far torch's float64 matmul (cuBLAS DGEMM) is from the
    oracle at 8192^3; the tests and the benchmark no longer depend on it."""
    M = N = K = 8192
    g = torch.Generator(device="cuda").manual_seed(7)
    A, B = draw((M, K), kind, g).double(), draw((K, N), kind, g).double()
    ours = ug.ref64("N", "N", A, B)
    theirs = A @ B
    torch.cuda.synchronize()
    err = float(torch.linalg.norm(theirs - ours) / torch.linalg.norm(ours))
    rows = float(((theirs - ours).norm(dim=1) / ours.norm(dim=1)).max())
    print(f"torch float64 vs FP64 oracle, 8192^3 {kind}: normwise {err:.2e}, worst row {rows:.2e}")
    assert err < 1e-6  # far below any FP32 form's error either way
