"""GPU parity of the adjoint (ugemm_sgemm_backward).

Loss L = sum(W * C) with C = alpha*op(A)*op(B) + beta*C0, so dC = W and
  dA = alpha * W * op(B)^T   (in A's storage layout),
  dB = alpha * op(A)^T * W   (in B's storage layout).
Checked (i) against FP64 central finite differences of L (h = 1e-3) on random
entries -- L is linear in each entry, so only one row (column) of C has to be
recomputed in FP64 per difference -- and (ii) against the CPU reference
gradient computed by the oracle (the reference's AVX256 SGEMM restated, all
host cores).
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import ugemm_gb300 as ug  # noqa: E402

H = 1e-3


@pytest.fixture(scope="module", autouse=True)
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ug.build()
    ug.load()


def op(x, t):
    return x if t == "N" else x.T


def fd_grad_a(A64, B64, W64, ta, tb, alpha, idx):
    """Central differences of L w.r.t. stored A entries idx (list of (r, c))."""
    out = []
    opB = op(B64, tb)
    for (r, c) in idx:
        i, k = (r, c) if ta == "N" else (c, r)   # the entry of op(A) it feeds
        row = op(A64, ta)[i].clone()
        vals = []
        for s in (+1, -1):
            row_s = row.clone()
            row_s[k] += s * H
            vals.append(float((W64[i] * (alpha * (row_s @ opB))).sum()))
        out.append((vals[0] - vals[1]) / (2 * H))
    return np.array(out)


def fd_grad_b(A64, B64, W64, ta, tb, alpha, idx):
    out = []
    opA = op(A64, ta)
    for (r, c) in idx:
        k, j = (r, c) if tb == "N" else (c, r)
        col = op(B64, tb)[:, j].clone()
        vals = []
        for s in (+1, -1):
            col_s = col.clone()
            col_s[k] += s * H
            vals.append(float((W64[:, j] * (alpha * (opA @ col_s))).sum()))
        out.append((vals[0] - vals[1]) / (2 * H))
    return np.array(out)


def run_backward(ta, tb, M, N, K, alpha, prec, seed, beta_acc=0.0):
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.rand(oracle.op_shape(ta, M, K), device="cuda", generator=g) * 2 - 1
    B = torch.rand(oracle.op_shape(tb, K, N), device="cuda", generator=g) * 2 - 1
    W = torch.randn((M, N), device="cuda", generator=g)
    dA0 = torch.randn(A.shape, device="cuda", generator=g)
    dB0 = torch.randn(B.shape, device="cuda", generator=g)
    dA, dB = dA0.clone(), dB0.clone()
    ug.sgemm_backward(ta, tb, M, N, K, alpha, A, A.shape[1], B, B.shape[1], W, N, beta_acc, dA,
                      dA.shape[1], beta_acc, dB, dB.shape[1], precision=prec)
    torch.cuda.synchronize()
    return A, B, W, dA0, dB0, dA, dB


@pytest.mark.parametrize("prec", ["simt", "bf16x6", "fp16x3", "tf32x3"])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
def test_backward_small_vs_fp64(prec, ta, tb):
    M, N, K = 150, 97, 203
    alpha, beta_acc = 1.5, 0.5
    A, B, W, dA0, dB0, dA, dB = run_backward(ta, tb, M, N, K, alpha, prec, 1, beta_acc)
    A64, B64, W64 = A.double(), B.double(), W.double()
    gA = alpha * (W64 @ op(B64, tb).T)          # d/d op(A)
    gB = alpha * (op(A64, ta).T @ W64)          # d/d op(B)
    refA = op(gA, ta) + beta_acc * dA0.double()
    refB = op(gB, tb) + beta_acc * dB0.double()
    for got, ref in ((dA, refA), (dB, refB)):
        err = float(torch.linalg.norm(got.double() - ref) / torch.linalg.norm(ref))
        assert err < 2e-6, (prec, ta, tb, err)


@pytest.mark.parametrize("shape", [(4096, 4096, 4096), (2048, 8192, 1024)])
@pytest.mark.parametrize("prec", ["bf16x6", "fp16x3", "simt"])
def test_backward_config3_fd_and_cpu_gradient(shape, prec):
    """North-star config 3: loss sum(W*C), A,B ~ U[-1,1), W ~ N(0,1), NN."""
    M, N, K = shape
    alpha = 1.0
    A, B, W, _, _, dA, dB = run_backward("N", "N", M, N, K, alpha, prec, 3)
    A64, B64, W64 = A.double(), B.double(), W.double()
    rng = np.random.default_rng(17)
    ia = [(int(rng.integers(M)), int(rng.integers(K))) for _ in range(64)]
    ib = [(int(rng.integers(K)), int(rng.integers(N))) for _ in range(64)]
    fa = fd_grad_a(A64, B64, W64, "N", "N", alpha, ia)
    fb = fd_grad_b(A64, B64, W64, "N", "N", alpha, ib)
    ga = np.array([float(dA[r, c]) for r, c in ia])
    gb = np.array([float(dB[r, c]) for r, c in ib])
    # FD of a bilinear loss in FP64 is exact to ~1e-12 relative; the FP32
    # gradient entries carry FP32 accumulation error over N (resp. M) terms.
    sa = np.abs(fa).max()
    sb = np.abs(fb).max()
    assert np.abs(ga - fa).max() / sa < 1e-5
    assert np.abs(gb - fb).max() / sb < 1e-5
    # CPU reference gradient (oracle, all host cores) on a row band
    rows = 256
    An, Bn, Wn = A[:rows].cpu().numpy(), B.cpu().numpy(), W[:rows].cpu().numpy()
    cpu_da = oracle.sgemm_avx256_mt(16, "N", "T", rows, K, N, alpha, Wn, Bn, 0.0,
                                    np.zeros((rows, K), dtype=np.float32))
    got_da = dA[:rows].cpu().numpy()
    assert np.abs(got_da - cpu_da).max() / np.abs(cpu_da).max() < 1e-5
    cols = 256
    Wc = np.ascontiguousarray(W[:, :cols].cpu().numpy())
    An = A.cpu().numpy()
    cpu_db = oracle.sgemm_avx256_mt(16, "T", "N", K, cols, M, alpha, An, Wc, 0.0,
                                    np.zeros((K, cols), dtype=np.float32))
    got_db = dB[:, :cols].cpu().numpy()
    assert np.abs(got_db - cpu_db).max() / np.abs(cpu_db).max() < 1e-5


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "T")])
def test_backward_with_deep_narrow_gradient(ta, tb):
    """dA of a wide, short problem is a small output with a deep k: the split
    form runs dA as k slices beside dB, in one launch plus one reduce."""
    M, N, K = 200, 20000, 96
    alpha, beta_acc = 0.75, 0.5
    A, B, W, dA0, dB0, dA, dB = run_backward(ta, tb, M, N, K, alpha, "bf16x6", 5, beta_acc)
    A64, B64, W64 = A.double(), B.double(), W.double()
    refA = op(alpha * (W64 @ op(B64, tb).T), ta) + beta_acc * dA0.double()
    refB = op(alpha * (op(A64, ta).T @ W64), tb) + beta_acc * dB0.double()
    for got, ref in ((dA, refA), (dB, refB)):
        err = float(torch.linalg.norm(got.double() - ref) / torch.linalg.norm(ref))
        assert err < 2e-6, (ta, tb, err)
