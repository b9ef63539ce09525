"""North-star config 2: split-precision tensor-core SGEMM vs plain FP32 SIMT
at 8192^3 and the ragged 4095 x 4097 x 1023, alpha = 1.5, beta = 0.5, all
four transpose pairs, on U[-1,1) inputs and on wide-range sets (mantissa
U[1,2), random sign, exponent uniform in [-8, 8], and in [-40, 40]); error
of every form against the GPU FP64 oracle (ugemm_dgemm_oracle_dev),
normwise, in the worst row and in the worst column (which a form that loses
whole rows or columns to a scale cannot pass).  Every split form (BF16x6,
FP16x3, TF32x3) must be at least as accurate as the FP32 SIMT form in all
three on every case.  The hardest is exponents spread over [-40, 40] at
k = 1023: each element of C is dominated by a few products, which SIMT's
fused multiply-add computes exactly, so SIMT's error is at its smallest;
the split forms meet it with their main accumulator drained every 64 k at
that depth."""
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import ugemm_gb300 as ug  # noqa: E402

ALPHA, BETA = 1.5, 0.5


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


def rowwise(C, ref):
    """max_i ||C_i - ref_i|| / ||ref_i|| and the same over columns."""
    d = C.double() - ref
    return (float((d.norm(dim=1) / ref.norm(dim=1)).max()),
            float((d.norm(dim=0) / ref.norm(dim=0)).max()))


def errors(ta, tb, M, N, K, kind, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = draw((M, K) if ta == "N" else (K, M), kind, g)
    B = draw((K, N) if tb == "N" else (N, K), kind, g)
    C0 = draw((M, N), kind, g)
    ref = ug.ref64(ta, tb, A, B, C0, ALPHA, BETA)
    out = {}
    for prec in ("simt", "bf16x6", "fp16x3", "tf32x3"):
        C = C0.clone()
        ug.sgemm_dev(ta, tb, M, N, K, ALPHA, A, A.stride(0), B, B.stride(0), BETA, C, N,
                     precision=prec)
        ug.check()
        norm = float(torch.linalg.norm(C.double() - ref) / torch.linalg.norm(ref))
        out[prec] = (norm, *rowwise(C, ref))
    return out


@pytest.mark.parametrize("kind", ["uniform", "wide", "wide40"])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
@pytest.mark.parametrize("shape", [(8192, 8192, 8192), (4095, 4097, 1023)])
def test_split_at_least_as_accurate_as_simt(shape, ta, tb, kind):
    M, N, K = shape
    e = errors(ta, tb, M, N, K, kind, seed=M + 2 * N + 3 * K + ord(ta) + 5 * ord(tb) + len(kind))
    print(f"{shape} {ta}{tb} {kind}: (normwise, worst row, worst column) " +
          " ".join(f"{p} {v[0]:.2e}/{v[1]:.2e}/{v[2]:.2e}" for p, v in e.items()))
    for prec in ("bf16x6", "fp16x3", "tf32x3"):
        for i in range(3):
            assert e[prec][i] <= e["simt"][i], (prec, i, e)
    assert e["simt"][0] < 1e-5
