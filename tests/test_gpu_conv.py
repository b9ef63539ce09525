"""GPU parity of im2col / col2im and the 12-layer im2col convolution stack
(spec config 5): forward, dX and dW of every layer as grouped GEMMs in
one CUDA graph, each layer's GEMMs checked against FP64."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import ugemm_gb300 as ug  # noqa: E402
from ugemm_gb300 import workloads  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ug.build()
    ug.load()


@pytest.mark.parametrize("c,h,w,k,pad,stride", [(3, 7, 9, 3, 1, 1), (2, 8, 8, 3, 1, 2),
                                                (4, 5, 6, 1, 0, 1), (2, 6, 5, 4, 2, 2),
                                                (16, 56, 56, 3, 1, 1)])
def test_im2col_single_image_matches_reference_semantics(c, h, w, k, pad, stride):
    """B = 1: the CHW image and column layout of sgemm_ocl1.h:81-119, bit exact."""
    rng = np.random.default_rng(c * 100 + h)
    im = rng.uniform(0, 1, (c, h, w)).astype(np.float32)
    ref = oracle.im2col(im, k, pad, stride)
    col = torch.empty(ref.shape, device="cuda")
    ug.im2col(torch.from_numpy(im).cuda(), c, 1, h, w, k, pad, stride, col)
    torch.cuda.synchronize()
    assert np.array_equal(col.cpu().numpy(), ref)


def test_im2col_batched_and_col2im_adjoint():
    C, B, H, W, k, pad, stride = 5, 3, 9, 7, 3, 1, 2
    Ho, Wo = (H + 2 * pad - k) // stride + 1, (W + 2 * pad - k) // stride + 1
    x = torch.rand((C, B, H, W), device="cuda")
    col = torch.empty((C * k * k, B * Ho * Wo), device="cuda")
    ug.im2col(x, C, B, H, W, k, pad, stride, col)
    # batched columns are the per-image columns side by side
    for b in range(B):
        one = torch.empty((C * k * k, Ho * Wo), device="cuda")
        ug.im2col(x[:, b].contiguous(), C, 1, H, W, k, pad, stride, one)
        assert torch.equal(col.view(C * k * k, B, Ho * Wo)[:, b], one)
    y = torch.rand_like(col)
    dx = torch.empty_like(x)
    ug.col2im(y, C, B, H, W, k, pad, stride, dx)
    torch.cuda.synchronize()
    lhs = float((col.double() * y.double()).sum())
    rhs = float((x.double() * dx.double()).sum())
    assert abs(lhs - rhs) / abs(lhs) < 1e-6


def test_conv_via_im2col_matches_torch_conv():
    """The layer GEMM W * im2col(X) is the convolution (FP64 check)."""
    C, B, H, W, Co = 8, 2, 12, 10, 6
    x = torch.rand((C, B, H, W), device="cuda")
    wt = torch.randn((Co, C, 3, 3), device="cuda")
    col = torch.empty((C * 9, B * (H // 2) * (W // 2)), device="cuda")
    ug.im2col(x, C, B, H, W, 3, 1, 2, col)
    y = ug.gemm(wt.reshape(Co, -1).contiguous(), col, precision="bf16x6")
    ref = torch.nn.functional.conv2d(x.permute(1, 0, 2, 3).double(), wt.double(), padding=1,
                                     stride=2)
    ref = ref.permute(1, 0, 2, 3).reshape(Co, -1)
    assert float(torch.linalg.norm(y.double() - ref) / torch.linalg.norm(ref)) < 2e-6


def fill_stack(stack, layers, batch, seed=0):
    g = torch.Generator(device="cuda").manual_seed(seed)
    cin, _, h, w, _ = layers[0]
    x0 = stack.tensor(0, "x", (cin, batch * h * w))
    x0.copy_(torch.rand(x0.shape, device="cuda", generator=g))          # U[0,1) activations
    for l, (ci, co, _, _, _) in enumerate(layers):
        wt = stack.tensor(l, "w", (co, ci * 9))
        wt.copy_(torch.randn(wt.shape, device="cuda", generator=g) * (2.0 / (ci * 9)) ** 0.5)


def rel(a, b):
    return float(torch.linalg.norm(a.double() - b) / torch.linalg.norm(b))


def tol(k):
    """Normwise bound for an FP32 GEMM of depth k: FP32 SIMT accumulation
    error grows like sqrt(k) (4.6e-6 measured at k = 100352)."""
    return max(2e-6, 2.5e-8 * k ** 0.5)


def col2im64(dcol, ci, batch, h, w, s):
    """FP64 adjoint of im2col (torch fold) in the stack's C x (B*H*W) layout."""
    ho, wo = (h + 2 - 3) // s + 1, (w + 2 - 3) // s + 1
    cols = dcol.reshape(ci * 9, batch, ho * wo).permute(1, 0, 2).contiguous()
    out = torch.nn.functional.fold(cols, (h, w), kernel_size=3, padding=1, stride=s)
    return out.permute(1, 0, 2, 3).reshape(ci, batch * h * w)


def layer_col(stack, layers, batch, l, explicit):
    """col_l = im2col(X_l): the stack's buffer (explicit stacks) or computed
    here by the standalone im2col (implicit stacks store none)."""
    ci, _, h, w, s = layers[l]
    ho, wo = (h + 2 - 3) // s + 1, (w + 2 - 3) // s + 1
    shape = (ci * 9, batch * ho * wo)
    if explicit:
        return stack.tensor(l, "col", shape)
    col = torch.empty(shape, device="cuda")
    ug.im2col(stack.tensor(l, "x", (ci, batch * h * w)), ci, batch, h, w, 3, 1, s, col)
    torch.cuda.synchronize()
    return col


@pytest.mark.parametrize("prec,explicit", [("bf16x6", False), ("fp16x3", False), ("simt", False),
                                           ("bf16x6", True)])
def test_config5_conv_stack_per_layer_fp64(prec, explicit):
    batch = 32
    layers = workloads.conv_layers(batch)
    shapes = workloads.conv_gemm_shapes(batch)
    stack = ug.ConvStack(layers, batch, precision=prec, graph=True, im2col=explicit)
    fill_stack(stack, layers, batch)
    stack.run(ug.CONV_FORWARD | ug.CONV_BACKWARD)
    torch.cuda.synchronize()
    for l, (M, N, K) in enumerate(shapes):
        ci, _, h, w_, s = layers[l]
        col = layer_col(stack, layers, batch, l, explicit).double()
        w = stack.tensor(l, "w", (M, K)).double()
        y = stack.tensor(l, "y", (M, N))
        dy = stack.tensor(l, "dy", (M, N)).double()
        dcol_ref = w.T @ dy
        errs = [rel(y, w @ col) if l + 1 < len(shapes) else 0.0,   # last y is its own dY slot
                rel(stack.tensor(l, "dw", (M, K)), dy @ col.T),
                rel(stack.tensor(l, "dx", (ci, batch * h * w_)),
                    col2im64(dcol_ref, ci, batch, h, w_, s))]
        # GEMM depths: forward K, dW N, dX up to 9 M (direct: one GEMM of depth 9 M)
        depths = [K, N, 9 * M]
        try:
            dcol = stack.tensor(l, "dcol", (K, N))    # stride-2 and explicit layers
            errs.append(rel(dcol, dcol_ref))
            depths.append(M)
        except ug.UgemmError as e:
            assert e.status == ug.ERR_UNSUPPORTED and not explicit and s == 1
        for e, depth in zip(errs, depths):
            assert e < tol(depth), (prec, l, errs)
    if explicit:  # dX of layer 0 is col2im of its dcol
        ci, _, h, w_, s = layers[0]
        dx = stack.tensor(0, "dx", (ci, batch * h * w_))
        ref = torch.empty_like(dx)
        ug.col2im(stack.tensor(0, "dcol", (ci * 9, shapes[0][1])), ci, batch, h, w_, 3, 1, s, ref)
        torch.cuda.synchronize()
        assert torch.equal(dx, ref)
    assert stack.flops() == pytest.approx(3 * sum(2.0 * m * n * k for m, n, k in shapes))
    stack.close()


def test_conv_stack_graph_replay_is_deterministic():
    batch = 4
    layers = workloads.conv_layers(batch)[:6]
    stack = ug.ConvStack(layers, batch, precision="bf16x6", graph=True)
    fill_stack(stack, layers, batch, seed=3)
    stack.run()
    torch.cuda.synchronize()
    first = stack.tensor(0, "dw", (64, 576)).clone()
    stack.run()
    torch.cuda.synchronize()
    assert torch.equal(stack.tensor(0, "dw", (64, 576)), first)
    stack.close()


@pytest.mark.parametrize("prec", ["bf16x6", "fp16x3", "tf32x3", "simt"])
def test_implicit_im2col_equals_explicit(prec):
    """Gathering col inside the operand pass reads exactly the values the
    im2col pass would have stored: every Y and the top layer's dW are
    bit-identical; dX of the stride-1 layers is one direct GEMM (summed in
    another order) instead of dcol + col2im, which the lower layers' dW
    inherit."""
    batch = 4
    layers = workloads.conv_layers(batch)[:7]   # includes a stride-2 layer
    out = []
    for explicit in (False, True):
        stack = ug.ConvStack(layers, batch, precision=prec, graph=True, im2col=explicit)
        fill_stack(stack, layers, batch, seed=5)
        stack.run()
        torch.cuda.synchronize()
        res = []
        for l, (ci, co, h, w, s) in enumerate(layers):
            for name in ("y", "dw", "dx"):
                addr, n = stack.buffer(l, name)
                res.append((name, ug._torch_view(addr, (n,), torch).clone()))
        out.append(res)
        if not explicit:
            with pytest.raises(ug.UgemmError) as e:
                stack.buffer(0, "col")
            assert e.value.status == ug.ERR_UNSUPPORTED
        stack.close()
    for (name, a), (_, b) in zip(*out):
        if name == "y":
            assert torch.equal(a, b)
        else:  # dX (and through it the lower layers' dW) differ by rounding only
            err = float(torch.linalg.norm((a - b).double()) / torch.linalg.norm(b.double()))
            assert err < 2e-6, (name, err)
    assert torch.equal(out[0][-2][1], out[1][-2][1])  # the top layer's dW: same dY


def test_conv_stack_rejects_mismatched_layers():
    with pytest.raises(ug.UgemmError):
        ug.ConvStack([(3, 8, 16, 16, 1), (4, 8, 16, 16, 1)], 2)
