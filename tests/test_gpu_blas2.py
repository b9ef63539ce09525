"""GPU SAXPY / SGEMV against the reference's saxpy_cpu / sgemv_cpu golden
outputs (ugemm.h:86-160) and against FP64 at larger sizes."""
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


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_saxpy_golden(golden):
    for name in [c for c in golden["cases"] if str(c).startswith("axpy/")]:
        g = lambda k: golden[f"{name}/{k}"]  # noqa: E731
        n, incx, incy = (int(v) for v in g("meta"))
        y = dev(g("y"))
        ug.saxpy(n, 0.75, dev(g("x")), incx, y, incy)
        torch.cuda.synchronize()
        np.testing.assert_allclose(y.cpu().numpy(), g("out"), rtol=0, atol=2e-7)


def test_sgemv_golden(golden):
    for name in [c for c in golden["cases"] if str(c).startswith("gemv/")]:
        g = lambda k: golden[f"{name}/{k}"]  # noqa: E731
        M, N, lda, inc = (int(v) for v in g("meta"))
        y = dev(g("y"))
        ug.sgemv(bytes(g("flags")).decode(), M, N, 1.5, dev(g("A")), lda, dev(g("x")), inc, 0.5, y,
                 inc)
        torch.cuda.synchronize()
        ref = g("out")
        assert np.abs(y.cpu().numpy() - ref).max() / np.abs(ref).max() < 1e-5, name


@pytest.mark.parametrize("trans", ["N", "T"])
def test_sgemv_large_vs_fp64(trans):
    M, N = 5000, 3001
    lda = (M if trans == "N" else N) + 3
    cols = N if trans == "N" else M
    A = torch.rand((cols, lda), device="cuda") * 2 - 1   # column-major: one column per row of storage
    x = torch.rand(N, device="cuda") * 2 - 1
    y0 = torch.rand(M, device="cuda") * 2 - 1
    y = y0.clone()
    ug.sgemv(trans, M, N, 1.5, A, lda, x, 1, 0.5, y, 1)
    torch.cuda.synchronize()
    Am = A[:, :M].double().T if trans == "N" else A[:, :N].double()  # M x N
    ref = 1.5 * (Am @ x.double()) + 0.5 * y0.double()
    assert float(torch.linalg.norm(y.double() - ref) / torch.linalg.norm(ref)) < 2e-6


def test_saxpy_large_and_strided():
    n = (1 << 22) + 3
    x = torch.rand(n, device="cuda")
    y = torch.rand(n, device="cuda")
    ref = y.double() + 0.25 * x.double()
    ug.saxpy(n, 0.25, x, 1, y, 1)
    torch.cuda.synchronize()
    assert float((y.double() - ref).abs().max()) < 1e-6
    xs = torch.rand(3 * 1000, device="cuda")
    ys = torch.rand(2 * 1000, device="cuda")
    ref = ys.clone()
    ref[::2] += 2.0 * xs[::3]
    ug.saxpy(1000, 2.0, xs, 3, ys, 2)
    torch.cuda.synchronize()
    assert torch.allclose(ys, ref, atol=1e-6)
