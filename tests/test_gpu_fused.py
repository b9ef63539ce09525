"""Fused grouped launches: the GEMM kernel copies the FP32 operand tiles
into shared memory itself and converter threads split them into the three
bf16 pieces in the layout the piece copies would have had, instead of a
pre-pass writing the pieces to memory first.  The pieces, the tile schedule,
the MMA order and the order in which chunk sums are added are the pre-pass
launch's, so with the same tile shape (128 wide: separate converter warps;
256 wide: the epilogue warps convert and keep chunk sums in global memory)
the results must be the same bits; they are also checked against FP64."""
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import ugemm_gb300 as ug  # noqa: E402
from ugemm_gb300 import workloads  # noqa: E402

from test_gpu_grouped import make_group, worst_error  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ug.build()
    ug.load()


def run_plan(specs, prec, fused, chunk_k=256, expect=None, block_n=128):
    for s in specs:
        s["C"].copy_(s["C0"])
    plan = ug.GroupedPlan(specs, precision=prec,
                          config={"block_n": block_n, "chunk_k": chunk_k, "fused": int(fused)})
    assert plan.config["fused"] == int(fused if expect is None else expect)
    plan.run()
    plan.check()
    plan.close()
    return [s["C"].clone() for s in specs]


def with_c0(specs):
    for s in specs:
        s["C0"] = s["C"].clone()
    return specs


@pytest.mark.parametrize("block_n", [128, 256])
@pytest.mark.parametrize("prec", ["bf16x6", "bf16x9"])
def test_fused_config4_group_is_bit_identical(prec, block_n):
    """The 256-problem group (M, N, K log-uniform in [32, 1024], NN/NT/TN),
    leading dimensions rounded up to 16 bytes."""
    specs, refs = make_group(workloads.grouped_shapes(), seed=2, align=4)
    with_c0(specs)
    pre = run_plan(specs, prec, fused=False, block_n=block_n)
    fus = run_plan(specs, prec, fused=True, block_n=block_n)
    for a, b in zip(pre, fus):
        assert torch.equal(a, b)
    assert worst_error(specs, refs) < 2e-6


@pytest.mark.parametrize("block_n", [128, 256])
@pytest.mark.parametrize("chunk_k", [64, 256])
def test_fused_split_k_epilogue_transposes(chunk_k, block_n):
    """Deep-k problems cut into split-K slices, a fused bias + LeakyReLU
    epilogue, padded leading dimensions, every transpose pair, wide problems
    computed transposed, ragged edges in every dimension."""
    shapes = [("N", "N", 64, 200, 9000), ("T", "T", 300, 100, 5000), ("N", "T", 17, 1000, 300),
              ("T", "N", 130, 145, 77), ("N", "N", 1, 4000, 33), ("T", "T", 40, 700, 129),
              ("N", "T", 129, 257, 1)]
    specs, refs = make_group(shapes, seed=9, alpha=0.75, beta=-1.5, pad=3, align=4)
    g = torch.Generator(device="cuda").manual_seed(10)
    for s in specs[:3]:
        s["bias"] = torch.rand((s["M"],), device="cuda", generator=g)
        s["act"], s["slope"] = 1, 0.1
    with_c0(specs)
    pre = run_plan(specs, "bf16x6", fused=False, chunk_k=chunk_k, block_n=block_n)
    fus = run_plan(specs, "bf16x6", fused=True, chunk_k=chunk_k, block_n=block_n)
    for a, b in zip(pre, fus):
        assert torch.equal(a, b)
    # the problems without an epilogue against FP64
    plain = [i for i, s in enumerate(specs) if "bias" not in s]
    assert worst_error([specs[i] for i in plain], [refs[i] for i in plain]) < 2e-6


def test_fused_falls_back_where_tma_cannot_copy():
    """A K = 0 problem in the group: the plan takes the pre-pass (reported in
    its config) and the results are still right."""
    shapes = [("N", "N", 64, 64, 64), ("N", "N", 17, 300, 0)]
    specs, refs = make_group(shapes, seed=4, alpha=1.0, beta=0.5, align=4)
    with_c0(specs)
    run_plan(specs, "bf16x6", fused=True, expect=False)
    assert worst_error(specs, refs) < 2e-6
    # the FP16x3 form (two pieces) has no fused launch
    with_c0(specs)
    run_plan(specs[:1], "fp16x3", fused=True, expect=False)
