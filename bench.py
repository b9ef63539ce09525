"""Benchmark of the ugemm GB300 SGEMM backend.

One step = one SGEMM C = 1.5*A*B + 0.5*C at M=N=K=8192, FP32 row-major, NN,
inputs U[-1,1) (seeded, resident in HBM; each operand is 256 MiB, larger than
the 129 MB L2, so no explicit flush between steps).  The headline `value` is
the split-precision tensor-core form in TFLOPS (2*M*N*K per step): of the two
split forms measured (BF16x6, FP16x3 and TF32x3 on tcgen05), the fastest one whose
error against FP64 is at most the plain FP32 SIMT form's -- normwise and in
its worst row, on the benchmark's inputs and on a 4096^3 problem whose
exponents span [-40, 40] (worst row and worst column too).  The SIMT form,
every form's errors against the GPU FP64 oracle (ugemm_dgemm_oracle_dev),
the end-to-end number through the
reference-facing host-pointer API (sgemm_cuda, pinned host buffers, copies
inside the timed region) and the CPU baseline (the reference's AVX256 SGEMM,
restated portably, on all host cores) go in the same JSON line.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) each rank runs an independent replica (the GEMM is
not sharded: the spec path is one GPU); value = all ranks' flops / the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TFLOPS @8192³: split-TC vs plain FP32 SIMT at equal FP64 err; grouped TFLOPS"
SEED = 20261205


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p, "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
                "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(steps: int = 1):
    """The reference's AVX256 SGEMM (restated portably in oracle/) on all host
    cores, on a bounded row band of the 8192^3 NN problem."""
    import numpy as np

    import oracle
    n = 8192
    rows = int(os.environ.get("UGEMM_CPU_ROWS", "512"))
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(SEED)
    A = rng.uniform(-1, 1, (rows, n)).astype(np.float32)
    B = rng.uniform(-1, 1, (n, n)).astype(np.float32)
    C = rng.uniform(-1, 1, (rows, n)).astype(np.float32)
    oracle.load()
    times = []
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        oracle.sgemm_avx256_mt(threads, "N", "N", rows, n, n, 1.5, A, B, 0.5, C)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    tflops = 2.0 * rows * n * n / t / 1e12
    return {"value": round(tflops, 5), "unit": "TFLOPS", "cores": threads, "kind": "port",
            "sample": f"rows 0..{rows - 1} of the 8192x8192x8192 NN problem (alpha=1.5, beta=0.5), "
                      f"median of {len(times)} runs, {threads} threads, oracle AVX256 port",
            "seconds_per_run": round(t, 4)}


def grouped_forms(ug, torch, stream, steps):
    """TFLOPS of the 256-problem grouped SGEMM (config 4) in both forms, each
    a tuned plan replayed as a CUDA graph, timed with CUDA events.  Operand
    rows are padded to a multiple of 4 floats (16 bytes), as a caller that
    wants the fused launches (operands copied by TMA, which needs 16-byte
    strides) allocates them; the tuner may still pick a pre-pass launch."""
    from ugemm_gb300 import workloads
    shapes = workloads.grouped_shapes()
    gen = torch.Generator(device="cuda").manual_seed(SEED + 7)
    specs, refs = [], []

    def padded(rows, cols):
        return (torch.rand((rows, -(-cols // 4) * 4), device="cuda", generator=gen) * 2 - 1)[:, :cols]

    for (ta, tb, M, N, K) in shapes:
        A = padded(M, K) if ta == "N" else padded(K, M)
        B = padded(K, N) if tb == "N" else padded(N, K)
        C = torch.zeros((M, N), device="cuda")
        specs.append(dict(ta=ta, tb=tb, M=M, N=N, K=K, alpha=1.0, beta=0.0, A=A, lda=A.stride(0),
                          B=B, ldb=B.stride(0), C=C, ldc=N))
        refs.append(ug.ref64(ta, tb, A, B))
    out = {"problems": len(shapes), "flops": sum(2.0 * m * n * k for _, _, m, n, k in shapes),
           "operand_rows": "padded to 16 bytes"}
    for prec in ("bf16x6", "fp16x3", "simt"):
        cfg, _ = ug.tune_grouped(specs, precision=prec)
        plan = ug.GroupedPlan(specs, precision=prec, config=cfg, graph=True)
        for _ in range(3):
            plan.run(stream)
        plan.check(stream)
        err = max(float(torch.linalg.norm(s["C"].double() - r) / torch.linalg.norm(r))
                  for s, r in zip(specs, refs))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        reps = max(steps, 20)
        e0.record(stream)
        for _ in range(reps):
            plan.run(stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        launches = 1 if plan.config.get("fused") else (3 if prec == "fp16x3" else 2)
        out[prec] = {"tflops": round(out["flops"] / (ms * 1e-3) / 1e12, 3), "ms": round(ms, 4),
                     "max_normwise_err_fp64": err, "config": plan.config,
                     "launches_per_run": launches}
        plan.close()
    best = max(("bf16x6", "fp16x3"), key=lambda p: out[p]["tflops"])
    out["split_over_simt"] = round(out[best]["tflops"] / out["simt"]["tflops"], 3)
    out["best_split"] = best
    return out


def backward_forms(ug, torch, stream, steps):
    """Config 3: forward + hand-written adjoint (dA, dB) at 4096^3 and
    2048 x 8192 x 1024, TFLOPS of the backward pair (4MNK) in both forms."""
    out = {}
    for (M, N, K) in ((4096, 4096, 4096), (2048, 8192, 1024)):
        g = torch.Generator(device="cuda").manual_seed(SEED + M + N + K)
        A = torch.rand((M, K), device="cuda", generator=g) * 2 - 1
        B = torch.rand((K, N), device="cuda", generator=g) * 2 - 1
        W = torch.randn((M, N), device="cuda", generator=g)
        dA = torch.empty_like(A)
        dB = torch.empty_like(B)
        row = {}
        for prec in ("bf16x6", "fp16x3", "simt"):
            def bwd():
                ug.sgemm_backward("N", "N", M, N, K, 1.0, A, K, B, N, W, N, 0.0, dA, K, 0.0, dB, N,
                                  precision=prec, stream=stream)
            for _ in range(3):
                bwd()
            reps = max(5, steps // 10)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                bwd()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            ref_a = ug.ref64("N", "T", W, B)
            err = float(torch.linalg.norm(dA.double() - ref_a) / torch.linalg.norm(ref_a))
            row[prec] = {"tflops": round(4.0 * M * N * K / (ms * 1e-3) / 1e12, 2),
                         "ms": round(ms, 3), "dA_normwise_err_fp64": err}
        out[f"{M}x{N}x{K}"] = row
    return out


def conv_forms(ug, torch, stream, steps):
    """Config 5: the 12-layer im2col conv stack, forward + dX + dW as grouped
    GEMMs replayed from one CUDA graph; TFLOPS over the GEMM flops."""
    from ugemm_gb300 import workloads
    batch = 32
    layers = workloads.conv_layers(batch)
    out = {"layers": len(layers), "batch": batch, "im2col": "implicit (gathered in the operand pass)"}
    for name, prec, explicit in (("bf16x6", "bf16x6", False), ("fp16x3", "fp16x3", False),
                                 ("simt", "simt", False), ("bf16x6_explicit_im2col", "bf16x6", True)):
        st = ug.ConvStack(layers, batch, precision=prec, graph=True, im2col=explicit)
        g = torch.Generator(device="cuda").manual_seed(SEED + 5)
        cin, _, h, w, _ = layers[0]
        st.tensor(0, "x", (cin, batch * h * w)).copy_(
            torch.rand((cin, batch * h * w), device="cuda", generator=g))
        for l, (ci, co, _, _, _) in enumerate(layers):
            st.tensor(l, "w", (co, ci * 9)).copy_(
                torch.randn((co, ci * 9), device="cuda", generator=g) * (2.0 / (ci * 9)) ** 0.5)
        for _ in range(2):
            st.run(stream=stream)
        reps = max(3, steps // 20)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            st.run(stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out[name] = {"tflops": round(st.flops() / (ms * 1e-3) / 1e12, 2), "ms": round(ms, 3),
                     "gemm_gflop": round(st.flops() / 1e9, 1)}
        st.close()
    return out


def profile_case(args):
    """One kernel family on a size ncu can capture (no timing, no JSON line):
    'split' (BF16x6) / 'split_fp16' (FP16x3) / 'simt' = size^3 NN SGEMM;
    'grouped_*' = the 256-problem group;
    'conv_split' = the 12-layer conv stack (implicit im2col, split form) at
    batch --size (16: operands above L2, about 2 GB on the device)."""
    import torch

    import ugemm_gb300 as ug
    from ugemm_gb300 import workloads
    ug.build()
    ug.load()
    n = args.size
    reps = max(1, args.steps)
    if args.profile_case == "conv_split":
        layers = workloads.conv_layers(n)
        st = ug.ConvStack(layers, n, precision="bf16x6", graph=False)
        cin, _, h, w, _ = layers[0]
        st.tensor(0, "x", (cin, n * h * w)).uniform_()
        for l, (ci, co, _, _, _) in enumerate(layers):
            st.tensor(l, "w", (co, ci * 9)).normal_(0.0, (2.0 / (ci * 9)) ** 0.5)
        for _ in range(reps):
            st.run()
        st.close()
    elif args.profile_case in ("split", "split_fp16", "simt"):
        A = torch.rand((n, n), device="cuda") * 2 - 1
        B = torch.rand((n, n), device="cuda") * 2 - 1
        C = torch.zeros((n, n), device="cuda")
        prec = {"split": "bf16x6", "split_fp16": "fp16x3", "simt": "simt"}[args.profile_case]
        for _ in range(reps):
            ug.sgemm_dev("N", "N", n, n, n, 1.0, A, n, B, n, 0.0, C, n, precision=prec)
    else:
        # the 256-problem group, operand rows padded to 16 bytes as in the
        # benchmark; grouped_fused: the fused launch (128-wide tiles)
        def padded(rows, cols):
            return (torch.rand((rows, -(-cols // 4) * 4), device="cuda") * 2 - 1)[:, :cols]

        specs = []
        for (ta, tb, M, N, K) in workloads.grouped_shapes():
            A = padded(M, K) if ta == "N" else padded(K, M)
            B = padded(K, N) if tb == "N" else padded(N, K)
            C = torch.zeros((M, N), device="cuda")
            specs.append(dict(ta=ta, tb=tb, M=M, N=N, K=K, alpha=1.0, beta=0.0, A=A,
                              lda=A.stride(0), B=B, ldb=B.stride(0), C=C, ldc=N))
        prec = "simt" if args.profile_case == "grouped_simt" else "bf16x6"
        cfg = dict(block_n=128, chunk_k=256, fused=1) if args.profile_case == "grouped_fused" else None
        plan = ug.GroupedPlan(specs, precision=prec, config=cfg)
        if cfg and not plan.config["fused"]:
            raise RuntimeError("grouped_fused: the plan could not take the fused launch")
        for _ in range(reps):
            plan.run()
        plan.check()
        plan.close()
    torch.cuda.synchronize()
    print(f"profile case {args.profile_case} size {n}: {reps} runs done")


def pick_headline(ms_forms: dict, errs: dict, err_simt, fallback: str = "bf16x6") -> str:
    """The split form the headline reports: the fastest one whose error
    against FP64 is at most the plain FP32 SIMT form's on the same inputs
    ("split-TC vs plain FP32 SIMT at equal FP64 error") in every measure
    given -- a number, or a tuple such as (normwise, worst row, ...) compared
    entry by entry; `fallback` if none qualifies."""
    def as_tuple(e):
        return tuple(e) if isinstance(e, (tuple, list)) else (e,)
    eligible = [p for p in ms_forms
                if all(a <= b for a, b in zip(as_tuple(errs[p]), as_tuple(err_simt)))]
    return min(eligible or [fallback], key=lambda p: ms_forms.get(p, float("inf")))


def wide_range_errors(ug, torch, forms, n=4096, span=40):
    """(normwise, worst row, worst column) error of every form on an n^3 NN
    problem whose elements have exponents uniform in [-span, span] (mantissa
    U[1,2), random sign), against the GPU FP64 oracle."""
    g = torch.Generator(device="cuda").manual_seed(SEED + 40)

    def draw():
        mant = 1 + torch.rand((n, n), device="cuda", generator=g)
        sign = torch.where(torch.rand((n, n), device="cuda", generator=g) < 0.5, -1.0, 1.0)
        return sign * mant * torch.exp2(torch.randint(-span, span + 1, (n, n), device="cuda",
                                                      generator=g).float())
    A, B = draw(), draw()
    ref = ug.ref64("N", "N", A, B)
    out = {}
    for prec in forms:
        C = torch.empty((n, n), device="cuda")
        ug.sgemm_dev("N", "N", n, n, n, 1.0, A, n, B, n, 0.0, C, n, precision=prec)
        ug.check()
        d = C.double() - ref
        out[prec] = (float(d.norm() / ref.norm()), float((d.norm(dim=1) / ref.norm(dim=1)).max()),
                     float((d.norm(dim=0) / ref.norm(dim=0)).max()))
    return out


def max_over_ranks(x: float, world: int, device) -> float:
    """The slowest rank's value; every rank of the job must call it."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, seconds: float, world: int) -> float:
    """Weak scaling: every rank processed `units_per_rank` within `seconds`
    (the slowest rank's time), so the job's rate is world times that."""
    return units_per_rank * world / seconds


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    steps = max(1, args.steps)
    for _ in range(min(args.warmup, 1)):
        cpu_sample(1)
    base = cpu_sample(steps)
    line = {"metric": METRIC, "value": base["value"], "unit": "TFLOPS", "impl": "reference",
            "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic U[-1,1) (seeded)",
            "config": {"workload": "sgemm 8192x8192x8192 NN alpha=1.5 beta=0.5 (row band sample)",
                       "model": "sgemm", "global_batch": 1, "seq_len": 0, "parallelism": "none"},
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": "TFLOPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=8192)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--profile-case", default=None,
                    choices=["split", "split_fp16", "simt", "grouped_split", "grouped_fused",
                             "grouped_simt", "conv_split"],
                    help="run only this case --steps times (for ncu captures) and exit")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.profile_case:
        profile_case(args)
        return

    import numpy as np
    import torch
    import torch.distributed as dist

    import ugemm_gb300 as ug

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    ug.build()
    ug.load()

    n = args.size
    M = N = K = n
    alpha, beta = 1.5, 0.5
    flops = 2.0 * M * N * K
    gen = torch.Generator(device="cuda").manual_seed(SEED + rank)
    A = torch.rand((M, K), device="cuda", generator=gen) * 2 - 1
    B = torch.rand((K, N), device="cuda", generator=gen) * 2 - 1
    C0 = torch.rand((M, N), device="cuda", generator=gen) * 2 - 1
    C = C0.clone()
    stream = torch.cuda.current_stream()

    def step(prec):
        ug.sgemm_dev("N", "N", M, N, K, alpha, A, K, B, N, beta, C, N, precision=prec,
                     stream=stream)

    def barrier():
        if world > 1:
            dist.barrier()

    def timed(prec, steps, warmup):
        for _ in range(max(warmup, 3)):
            step(prec)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step(prec)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        ms = max_over_ranks(e0.elapsed_time(e1), world, torch.device("cuda", local))
        return ms / steps

    # --- accuracy of each form against the GPU FP64 oracle on the same inputs
    # (normwise and worst row), and on a wide-exponent-range problem
    ref = ug.ref64("N", "N", A, B, C0, alpha, beta)

    def form_error(prec):
        out = C0.clone()
        ug.sgemm_dev("N", "N", M, N, K, alpha, A, K, B, N, beta, out, N, precision=prec,
                     stream=stream)
        ug.check(stream)
        d = out.double() - ref
        return (float(torch.linalg.norm(d) / torch.linalg.norm(ref)),
                float((d.norm(dim=1) / ref.norm(dim=1)).max()))

    # 16-bit-rate piece products per FP32 product (TF32 MMAs run at half the
    # 16-bit dense rate: three TF32 products cost six)
    split_forms = {"bf16x6": 6, "fp16x3": 3, "tf32x3": 6}
    errs_main = {prec: form_error(prec) for prec in list(split_forms) + ["simt"]}
    del ref
    torch.cuda.empty_cache()
    errs_wide = wide_range_errors(ug, torch, list(split_forms) + ["simt"])
    torch.cuda.empty_cache()
    # every measure the headline form must meet: (normwise, worst row) on the
    # benchmark's inputs, then (normwise, worst row, worst column) on the wide set
    gate = {p: errs_main[p] + errs_wide[p] for p in errs_main}
    errs = {p: errs_main[p][0] for p in errs_main}  # normwise on the benchmark's inputs
    err_simt = errs["simt"]

    # --- headline: split-precision tensor-core forms, device-resident inputs
    sampler = ClockSampler(local)
    sampler.start()
    ms_forms = {prec: timed(prec, args.steps, args.warmup) for prec in split_forms}
    clocks = sampler.stop()
    ms_simt = timed("simt", max(2, args.steps // 2), 3)
    # the faster split form at equal or better error than FP32 SIMT (every
    # rank decides alike: the slowest rank's times)
    head = pick_headline(ms_forms, gate, gate["simt"])
    ms_split, err_split = ms_forms[head], errs[head]

    # --- per-kernel attribution with CUDA events on the launching stream
    ug.profile_enable(True)
    for _ in range(3):
        step(head)
    prof = ug.profile_collect()
    ug.profile_enable(False)
    # per step: the operand pre-pass (two launches), and the GEMM proper --
    # the persistent kernel plus, when the tiles' last wave is short, the
    # wave-tail launch and its reduce
    gemm_ms = (prof["split_gemm"][0] + prof["grouped"][0] + prof["aux"][0]) / 3.0
    prep_ms = prof["split_prepass"][0] / 3.0
    launches_per_step = sum(v[1] for v in prof.values()) / 3.0

    # --- batching form: 256 uneven problems, one persistent launch, CUDA graph
    grouped = grouped_forms(ug, torch, stream, args.steps)
    backward = backward_forms(ug, torch, stream, args.steps)
    conv = conv_forms(ug, torch, stream, args.steps)

    # --- end to end through the reference-facing host API (sgemm_cuda)
    hA = A.cpu().pin_memory()
    hB = B.cpu().pin_memory()
    hC = C0.cpu().pin_memory()
    # the reference's test sizes the device buffer at ten times the three
    # matrices (sgemm_test.c:29); the pipelined host path keeps the whole
    # problem resident in it
    size = (M * K + K * N + M * N) * 10 * 4
    lib = ug.load()
    lib.sgemm_cuda_init(0, local, size)
    ug._check(lib.ugemm_last_error())
    lib.sgemm_cuda_set_precision(ug.PRECISIONS[head])
    e2e_steps = max(2, args.steps // 2)

    def e2e_time(a_ptr, b_ptr, c_ptr):
        def call():
            ug._check(lib.sgemm_cuda_status(b"N", b"N", M, N, K, alpha, a_ptr, b_ptr, beta, c_ptr))
        for _ in range(2):
            call()
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            call()
        return max_over_ranks((time.perf_counter() - t0) / e2e_steps, world,
                              torch.device("cuda", local))

    e2e_s = e2e_time(hA.data_ptr(), hB.data_ptr(), hC.data_ptr())
    # the reference's callers pass pageable memory (sgemm_test.c's static
    # arrays): the same call on plain numpy arrays
    nA, nB, nC = hA.numpy().copy(), hB.numpy().copy(), hC.numpy().copy()
    e2e_pageable_s = e2e_time(nA.ctypes.data, nB.ctypes.data, nC.ctypes.data)
    del nA, nB, nC
    lib.sgemm_cuda_finish()

    pk, pk_kind = peaks()
    tflops_split = flops / (ms_split * 1e-3) / 1e12
    tflops_simt = flops / (ms_simt * 1e-3) / 1e12
    achieved = flops / (gemm_ms * 1e-3) / 1e12
    peak_split = pk["bf16_tflops"] / split_forms[head]
    sm_max = pk.get("sm_max_mhz", 2070.0)
    fp32_peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12
    # the FP32 FMA rate measured on this GPU (no FP32 figure is in the
    # measured-peaks file): 200 ms of independent FMA chains
    fp32_measured = ug.fp32_peak(200.0)
    traffic = None  # DRAM bytes of the GEMM phase from the committed ncu capture (8192^3)
    try:
        with open(os.path.join(ROOT, "profiles", "split_tc_kernel_sgemm8192_traffic.json")) as f:
            traffic = json.load(f).get(head) if n == 8192 else None
    except (OSError, ValueError):
        pass

    line = {
        "metric": METRIC,
        "value": round(whole_job_rate(flops, ms_split * 1e-3, world) / 1e12, 3),
        "unit": "TFLOPS",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_split, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": f"f32 ({head} split on tcgen05, FP32 accumulate)",
        "data": "synthetic U[-1,1) (seeded, torch.Generator on device)",
        "config": {"workload": f"sgemm {n}x{n}x{n} NN alpha=1.5 beta=0.5 row-major",
                   "model": "sgemm", "global_batch": 1, "seq_len": 0,
                   "parallelism": f"replicas{world}", "l2": "inputs larger than L2 (no flush)"},
        "forms": {
            "headline": head,
            **{f"split_{p}": {"tflops": round(flops / (ms_forms[p] * 1e-3) / 1e12, 3),
                              "ms": round(ms_forms[p], 4), "normwise_err_fp64": errs[p],
                              "worst_row_err_fp64": errs_main[p][1],
                              "wide40_4096_err_fp64": dict(zip(("normwise", "worst_row",
                                                                 "worst_col"), errs_wide[p])),
                              "piece_products_16bit_rate": split_forms[p]} for p in split_forms},
            "simt_fp32": {"tflops": round(tflops_simt, 3), "normwise_err_fp64": err_simt,
                          "worst_row_err_fp64": errs_main["simt"][1],
                          "wide40_4096_err_fp64": dict(zip(("normwise", "worst_row", "worst_col"),
                                                           errs_wide["simt"])),
                          "frac_of_fp32_peak_measured": round(tflops_simt / fp32_measured, 4),
                          "fp32_peak_measured_tflops": round(fp32_measured, 2),
                          "frac_of_fp32_peak_nominal": round(tflops_simt / fp32_peak, 4),
                          "fp32_peak_nominal_tflops": round(fp32_peak, 2)},
            "split_over_simt": round(tflops_split / tflops_simt, 3),
            "split_err_over_simt_err": round(err_split / err_simt, 4),
            "split_prepass_ms": round(prep_ms, 4), "split_gemm_ms": round(gemm_ms, 4),
            "grouped": grouped,
            "backward": backward,
            "conv_stack": conv,
        },
        "roofline": {"bound": "tensor", "achieved": round(achieved, 3),
                     "peak": round(peak_split, 3), "unit": "TFLOP/s",
                     "frac": round(achieved / peak_split, 4), "traffic": traffic,
                     "kernel": f"split_tc_kernel ({head}; with its wave-tail launch and reduce)",
                     "peak_basis": f"bf16_tflops ({pk_kind} cuBLAS burst {pk['bf16_tflops']}; "
                                   f"fp16 runs at the same dense rate) / {split_forms[head]} "
                                   "piece products; achieved = 2MNK / kernel time"},
        "e2e": {"value": round(whole_job_rate(flops, e2e_s, world) / 1e12, 3), "unit": "TFLOPS",
                "h2d_bytes_per_step": 3 * M * N * 4, "d2h_bytes_per_step": M * N * 4,
                "api": "sgemm_cuda (compat, host pointers, pinned)",
                "pageable": {"value": round(whole_job_rate(flops, e2e_pageable_s, world) / 1e12, 3),
                             "unit": "TFLOPS", "ms": round(e2e_pageable_s * 1e3, 3),
                             "api": "sgemm_cuda on plain numpy arrays (pageable host memory)"},
                "ms": round(e2e_s * 1e3, 3)},
        "gpu_launches": int(round(launches_per_step * args.steps)),
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_sample(5)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
