"""Fused bias + LeakyReLU epilogue (gl_convolution_LReLU's post-GEMM loop,
sgemm_gl1.h:210-217, moved into the GEMM kernels): single GEMMs in both
forms, grouped problems, and a conv stack with activations whose backward
masks the gradient and produces the bias gradient."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import ugemm_gb300 as ug  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ug.build()
    ug.load()


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("prec", ["simt", "bf16x6"])
@pytest.mark.parametrize("M,N,K", [(64, 3136, 576), (130, 257, 70), (1000, 1200, 900)])
def test_fused_bias_leaky_matches_reference_loop(prec, M, N, K):
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    W = torch.randn((M, K), device="cuda", generator=g) * 0.1
    X = torch.rand((K, N), device="cuda", generator=g)
    bias = torch.randn(M, device="cuda", generator=g)
    Y = ug.gemm_ex(W, X, bias=bias, act=1, slope=0.1, precision=prec)
    torch.cuda.synchronize()
    ref = (W.double() @ X.double()).cpu().numpy().astype(np.float32)
    oracle.bias_leaky(ref, bias.cpu().numpy())
    assert rel(Y.cpu().numpy(), ref.astype(np.float64)) < 2e-6
    # no activation, bias only, with alpha/beta
    C0 = torch.rand((M, N), device="cuda", generator=g)
    Y2 = ug.gemm_ex(W, X, C0.clone(), bias=bias, act=0, alpha=1.5, beta=0.5, precision=prec)
    ref2 = 1.5 * (W.double() @ X.double()) + 0.5 * C0.double() + bias.double()[:, None]
    assert float(torch.linalg.norm(Y2.double() - ref2) / torch.linalg.norm(ref2)) < 2e-6


@pytest.mark.parametrize("prec", ["bf16x6", "simt"])
def test_grouped_problems_with_epilogue(prec):
    g = torch.Generator(device="cuda").manual_seed(9)
    specs, refs = [], []
    for (M, N, K) in [(64, 500, 200), (200, 64, 33), (128, 128, 128)]:
        A = torch.randn((M, K), device="cuda", generator=g)
        B = torch.randn((K, N), device="cuda", generator=g)
        C = torch.empty((M, N), device="cuda")
        bias = torch.randn(M, device="cuda", generator=g)
        specs.append(dict(ta="N", tb="N", M=M, N=N, K=K, alpha=1.0, beta=0.0, A=A, lda=K, B=B,
                          ldb=N, C=C, ldc=N, bias=bias, act=1, slope=0.1))
        pre = A.double() @ B.double() + bias.double()[:, None]
        refs.append(torch.where(pre > 0, pre, pre * 0.1))
    ug.sgemm_grouped(specs, precision=prec)
    torch.cuda.synchronize()
    for s, r in zip(specs, refs):
        assert float(torch.linalg.norm(s["C"].double() - r) / torch.linalg.norm(r)) < 2e-6


def test_conv_stack_with_leaky_relu_forward_and_backward():
    from ugemm_gb300 import workloads
    batch = 4
    layers = workloads.conv_layers(batch)[:5]
    shapes = workloads.conv_gemm_shapes(batch)[:5]
    st = ug.ConvStack(layers, batch, precision="bf16x6", graph=True, leaky=0.1, im2col=True)
    g = torch.Generator(device="cuda").manual_seed(2)
    cin, _, h, w, _ = layers[0]
    st.tensor(0, "x", (cin, batch * h * w)).copy_(torch.rand((cin, batch * h * w), device="cuda",
                                                             generator=g))
    for l, (ci, co, _, _, _) in enumerate(layers):
        st.tensor(l, "w", (co, ci * 9)).copy_(torch.randn((co, ci * 9), device="cuda", generator=g)
                                              * (2.0 / (ci * 9)) ** 0.5)
        st.tensor(l, "bias", (co,)).copy_(torch.randn(co, device="cuda", generator=g) * 0.1)
    st.run(ug.CONV_FORWARD)
    torch.cuda.synchronize()
    ys = []
    for l, (M, N, K) in enumerate(shapes):
        pre = st.tensor(l, "w", (M, K)).double() @ st.tensor(l, "col", (K, N)).double() + \
            st.tensor(l, "bias", (M,)).double()[:, None]
        ref = torch.where(pre > 0, pre, 0.1 * pre)
        y = st.tensor(l, "y", (M, N)).clone()
        ys.append(y)
        assert float(torch.linalg.norm(y.double() - ref) / torch.linalg.norm(ref)) < 2e-6
    st.run(ug.CONV_BACKWARD)
    torch.cuda.synchronize()
    for l, (M, N, K) in enumerate(shapes):
        # the incoming gradient (layer l+1's dX, or the last layer's own output) is masked
        raw = ys[l].double() if l + 1 == len(shapes) else None
        dy = st.tensor(l, "dy", (M, N)).double()   # masked in place by the backward run
        if raw is not None:
            masked = torch.where(ys[l].double() > 0, raw, 0.1 * raw)
            assert float(torch.linalg.norm(dy - masked) / torch.linalg.norm(masked)) < 1e-6
        dbias = st.tensor(l, "dbias", (M,)).double()
        assert float(torch.linalg.norm(dbias - dy.sum(1)) / torch.linalg.norm(dy.sum(1))) < 1e-5
        col = st.tensor(l, "col", (K, N)).double()
        w_ = st.tensor(l, "w", (M, K)).double()
        for got, ref in ((st.tensor(l, "dw", (M, K)), dy @ col.T),
                         (st.tensor(l, "dcol", (K, N)), w_.T @ dy)):
            assert float(torch.linalg.norm(got.double() - ref) / torch.linalg.norm(ref)) < 2e-6
    st.close()


@pytest.mark.parametrize("M,N,K", [(4096, 4096, 1024), (64, 200, 20000), (2048, 3000, 2048)])
def test_fused_epilogue_through_split_k_and_wave_tail(M, N, K):
    """Shapes whose split-form GEMM runs partly outside the single kernel: a
    partial last wave run as two k slices (4096 x 4096), a deep narrow
    problem run as split-K slices (64 x 200 x 20000): the bias (per row of C,
    offset to the sliced rows) and the activation are applied by the reduce."""
    g = torch.Generator(device="cuda").manual_seed(M + K)
    W = torch.randn((M, K), device="cuda", generator=g) * (1.0 / K ** 0.5)
    X = torch.rand((K, N), device="cuda", generator=g)
    bias = torch.randn(M, device="cuda", generator=g)
    C0 = torch.rand((M, N), device="cuda", generator=g)
    Y = ug.gemm_ex(W, X, C0.clone(), bias=bias, act=1, slope=0.1, alpha=1.25, beta=0.5,
                   precision="bf16x6")
    torch.cuda.synchronize()
    pre = 1.25 * (W.double() @ X.double()) + 0.5 * C0.double() + bias.double()[:, None]
    ref = torch.where(pre > 0, pre, 0.1 * pre)
    assert float(torch.linalg.norm(Y.double() - ref) / torch.linalg.norm(ref)) < 2e-6


def test_grouped_split_k_problem_with_epilogue():
    g = torch.Generator(device="cuda").manual_seed(21)
    specs, refs = [], []
    for (M, N, K) in [(64, 300, 30000), (200, 64, 64)]:
        A = torch.randn((M, K), device="cuda", generator=g) * (1.0 / K ** 0.5)
        B = torch.randn((K, N), device="cuda", generator=g)
        C = torch.empty((M, N), device="cuda")
        bias = torch.randn(M, device="cuda", generator=g)
        specs.append(dict(ta="N", tb="N", M=M, N=N, K=K, alpha=1.0, beta=0.0, A=A, lda=K, B=B,
                          ldb=N, C=C, ldc=N, bias=bias, act=1, slope=0.1))
        pre = A.double() @ B.double() + bias.double()[:, None]
        refs.append(torch.where(pre > 0, pre, pre * 0.1))
    for prec in ("bf16x6", "simt"):
        ug.sgemm_grouped(specs, precision=prec)
        torch.cuda.synchronize()
        for s, r in zip(specs, refs):
            err = float(torch.linalg.norm(s["C"].double() - r) / torch.linalg.norm(r))
            assert err < max(2e-6, 2.5e-8 * s["K"] ** 0.5), (prec, s["M"], s["K"], err)
