"""GPU parity of the grouped GEMM (spec batching form): 256 uneven
problems with mixed transposes in one persistent launch, split-precision and
SIMT forms, plain and CUDA-graph replay, and the autotuner's cache."""
import json
import os

import numpy as np
import pytest

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


def make_group(shapes, seed=1, alpha=1.0, beta=0.0, pad=0, align=1):
    """Problems with leading dimensions of (columns + pad) rounded up to a
    multiple of align."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    specs, refs = [], []

    def ld(cols):
        return -(-(cols + pad) // align) * align

    for (ta, tb, M, N, K) in shapes:
        ashape = (M, K) if ta == "N" else (K, M)
        bshape = (K, N) if tb == "N" else (N, K)
        A = torch.rand((ashape[0], ld(ashape[1])), device="cuda", generator=g) * 2 - 1
        B = torch.rand((bshape[0], ld(bshape[1])), device="cuda", generator=g) * 2 - 1
        C = torch.rand((M, ld(N)), device="cuda", generator=g) * 2 - 1
        a = A[:, :ashape[1]].double()
        b = B[:, :bshape[1]].double()
        ref = alpha * ((a if ta == "N" else a.T) @ (b if tb == "N" else b.T)) + beta * C[:, :N].double()
        specs.append(dict(ta=ta, tb=tb, M=M, N=N, K=K, alpha=alpha, beta=beta, A=A, lda=A.stride(0),
                          B=B, ldb=B.stride(0), C=C, ldc=C.stride(0)))
        refs.append(ref)
    return specs, refs


def worst_error(specs, refs):
    worst = 0.0
    for s, ref in zip(specs, refs):
        got = s["C"][:, :s["N"]].double()
        worst = max(worst, float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref)))
    return worst


@pytest.mark.parametrize("prec", ["bf16x6", "fp16x3", "simt"])
@pytest.mark.parametrize("graph", [False, True])
def test_config4_grouped_256_problems(prec, graph):
    shapes = workloads.grouped_shapes()
    specs, refs = make_group(shapes, alpha=1.0, beta=0.0)
    plan = ug.GroupedPlan(specs, precision=prec, graph=graph)
    plan.run()
    plan.check()
    assert worst_error(specs, refs) < 2e-6
    assert abs(plan.flops - sum(2.0 * m * n * k for _, _, m, n, k in shapes)) < 1
    # replay: same result (beta == 0, deterministic schedule)
    before = [s["C"].clone() for s in specs[:8]]
    plan.run()
    plan.check()
    for s, b in zip(specs[:8], before):
        assert torch.equal(s["C"], b)
    plan.close()


@pytest.mark.parametrize("prec", ["bf16x6", "bf16x9", "fp16x3", "tf32x3", "simt"])
def test_grouped_edge_cases(prec):
    """Tiny, ragged, K = 0, alpha = 0 and padded leading dimensions."""
    shapes = [("N", "N", 1, 1, 1), ("T", "T", 3, 5, 7), ("N", "T", 129, 257, 33),
              ("T", "N", 200, 64, 1000), ("N", "N", 17, 300, 0), ("N", "T", 64, 64, 64)]
    specs, refs = make_group(shapes, seed=2, alpha=1.5, beta=0.5, pad=3)
    # alpha == 0 on the last problem
    specs[-1]["alpha"] = 0.0
    refs[-1] = 0.5 * specs[-1]["C"][:, :64].double()
    keep = [s["C"][:, s["N"]:].clone() for s in specs]
    ug.sgemm_grouped(specs, precision=prec)
    torch.cuda.synchronize()
    for s, ref, k in zip(specs, refs, keep):
        got = s["C"][:, :s["N"]].double()
        err = float(torch.linalg.norm(got - ref) / max(torch.linalg.norm(ref), 1e-30))
        assert err < 2e-6, (prec, s["M"], s["N"], s["K"], err)
        assert torch.equal(s["C"][:, s["N"]:], k)  # padding untouched


@pytest.mark.parametrize("prec", ["bf16x6", "fp16x3", "simt"])
def test_grouped_split_k_slices_deep_problems(prec):
    """Weight-gradient-shaped problems (small output, k in the tens of
    thousands) beside shallow ones: the plan cuts the deep ones into k
    slices whose partial tiles one reduce launch sums (with beta * C)."""
    shapes = [("N", "T", 64, 200, 40000), ("T", "N", 100, 50, 30000), ("N", "N", 300, 40, 256),
              ("N", "T", 33, 900, 64)]
    specs, refs = make_group(shapes, seed=7, alpha=1.25, beta=0.5, pad=1)
    c0 = [s["C"].clone() for s in specs]
    keep = [s["C"][:, s["N"]:].clone() for s in specs]
    plan = ug.GroupedPlan(specs, precision=prec)
    ug.profile_enable(True)
    try:
        plan.run()
        prof = ug.profile_collect()
    finally:
        ug.profile_enable(False)
    plan.check()
    assert prof["aux"][1] == 1  # the split-K reduce ran once
    for s, ref, k in zip(specs, refs, keep):
        got = s["C"][:, :s["N"]].double()
        err = float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))
        # FP32 accumulation depth of a slice, not of the whole k
        assert err < max(2e-6, 2.5e-8 * s["K"] ** 0.5), (prec, s["M"], s["N"], s["K"], err)
        assert torch.equal(s["C"][:, s["N"]:], k)  # padding untouched
    # replay from the same C: bit-identical (fixed slice order)
    first = [s["C"].clone() for s in specs]
    for s, c in zip(specs, c0):
        s["C"].copy_(c)
    plan.run()
    plan.check()
    for s, f in zip(specs, first):
        assert torch.equal(s["C"], f)
    plan.close()


@pytest.mark.parametrize("prec", ["bf16x6", "bf16x9", "fp16x3"])
def test_grouped_wide_and_narrow_problems(prec):
    """Few rows and many columns (computed transposed by the split form) and
    narrow right-edge tiles (MMAs as wide as the columns, in steps of 16)."""
    shapes = [("N", "N", 17, 1000, 300), ("T", "T", 40, 700, 129), ("N", "T", 500, 24, 64),
              ("T", "N", 130, 145, 77), ("N", "N", 1, 4000, 33), ("N", "T", 16, 16, 16)]
    specs, refs = make_group(shapes, seed=8, alpha=0.75, beta=-1.5, pad=5)
    keep = [s["C"][:, s["N"]:].clone() for s in specs]
    # both tile widths; a grid smaller than the GPU deals the tiles to 37 CTAs
    for bn, ctas in ((128, 0), (256, 0), (256, 37)):
        plan = ug.GroupedPlan(specs, precision=prec, config={"block_n": bn, "chunk_k": 256,
                                                             "max_ctas": ctas})
        c0 = [s["C"].clone() for s in specs]
        plan.run()
        plan.check()
        assert worst_error(specs, refs) < 2e-6, (bn, ctas)
        for s, k in zip(specs, keep):
            assert torch.equal(s["C"][:, s["N"]:], k)
        for s, c in zip(specs, c0):  # beta != 0: restore C for the next tile width
            s["C"].copy_(c)
        plan.close()


def test_grouped_rejects_bad_problems():
    specs, _ = make_group([("N", "N", 8, 8, 8)])
    specs[0]["lda"] = 4  # < K
    with pytest.raises(ug.UgemmError) as e:
        ug.GroupedPlan(specs)
    assert e.value.status == ug.ERR_ARG


def test_autotuner_caches_its_choice(tmp_path, monkeypatch):
    cache = tmp_path / "tune.jsonl"
    monkeypatch.setenv("UGEMM_TUNE_CACHE", str(cache))
    shapes = workloads.grouped_shapes(count=24, seed=5)
    specs, refs = make_group(shapes, seed=3)
    best, ms = ug.tune_grouped(specs, precision="bf16x6", force=True)
    assert best["block_n"] in (128, 256) and best["chunk_k"] in (128, 256)
    assert ms > 0
    lines = [json.loads(x) for x in cache.read_text().splitlines()]
    line = lines[-1]
    assert all(line[k] == v for k, v in best.items())
    # every candidate is recorded with its time, the schedule knobs were
    # searched (split-K threshold, tile deal, transposed tiles, grid size),
    # and the choice is the fastest of them
    cands = line["candidates"]
    fields = ("block_n", "chunk_k", "max_ctas", "split_k", "deal", "transpose", "fused")
    assert len(cands) >= 11
    for i, name in enumerate(fields[2:], start=2):
        assert len({c[i] for c in cands}) >= 2, name
    fastest = min(cands, key=lambda c: c[7])
    assert fastest[7] == pytest.approx(line["ms"], rel=1e-6)
    assert dict(zip(fields, fastest[:7])) == best
    # cached: returned without timing, and picked up by a plan without config
    again, ms2 = ug.tune_grouped(specs, precision="bf16x6")
    assert again == best and ms2 == pytest.approx(ms, rel=1e-5)
    plan = ug.GroupedPlan(specs, precision="bf16x6")
    assert plan.config["block_n"] == best["block_n"]
    plan.run()
    plan.check()
    assert worst_error(specs, refs) < 2e-6
    plan.close()
    simt_best, _ = ug.tune_grouped(specs, precision="simt", force=True)
    assert simt_best["block_n"] in (64, 128)
    simt_line = json.loads(cache.read_text().splitlines()[-1])
    assert min(c[7] for c in simt_line["candidates"]) == pytest.approx(simt_line["ms"], rel=1e-6)
