"""North-star config 2: split-precision tensor-core SGEMM vs plain FP32 SIMT
at 8192^3 and the ragged 4095 x 4097 x 1023, alpha = 1.5, beta = 0.5, all
four transpose pairs, on U[-1,1) inputs and on a wide-range set (mantissa
U[1,2), random sign, exponent uniform in [-8, 8]); normwise error of both
forms against an FP64 GEMM on the GPU.  Both split forms (BF16x6 and FP16x3)
must be at least as accurate as the FP32 SIMT form on every case."""
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
    mant = 1 + torch.rand(shape, device="cuda", generator=g)
    sign = torch.where(torch.rand(shape, device="cuda", generator=g) < 0.5, -1.0, 1.0)
    expo = torch.randint(-8, 9, shape, device="cuda", generator=g).float()
    return sign * mant * torch.exp2(expo)


def errors(ta, tb, M, N, K, kind, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = draw((M, K) if ta == "N" else (K, M), kind, g)
    B = draw((K, N) if tb == "N" else (N, K), kind, g)
    C0 = draw((M, N), kind, g)
    ref = ALPHA * ((A.double() if ta == "N" else A.double().T) @
                   (B.double() if tb == "N" else B.double().T)) + BETA * C0.double()
    out = {}
    for prec in ("simt", "bf16x6", "fp16x3"):
        C = C0.clone()
        ug.sgemm_dev(ta, tb, M, N, K, ALPHA, A, A.stride(0), B, B.stride(0), BETA, C, N,
                     precision=prec)
        torch.cuda.synchronize()
        out[prec] = float(torch.linalg.norm(C.double() - ref) / torch.linalg.norm(ref))
    return out


@pytest.mark.parametrize("kind", ["uniform", "wide"])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
@pytest.mark.parametrize("shape", [(8192, 8192, 8192), (4095, 4097, 1023)])
def test_split_at_least_as_accurate_as_simt(shape, ta, tb, kind):
    M, N, K = shape
    e = errors(ta, tb, M, N, K, kind, seed=M + 2 * N + 3 * K + ord(ta) + 5 * ord(tb))
    print(f"{shape} {ta}{tb} {kind}: simt {e['simt']:.3e} bf16x6 {e['bf16x6']:.3e} "
          f"fp16x3 {e['fp16x3']:.3e}")
    assert e["bf16x6"] <= e["simt"], e
    assert e["fp16x3"] <= e["simt"], e
    assert e["simt"] < 1e-5
