"""Generate tests/golden/ugemm_golden.npz from the reference's OWN CPU code.

Run in a container that has the reference tree (x86-64): it compiles
``oracle/_ref/*.so`` from the reference sources (``make -C oracle ref``) and
calls the reference functions through ctypes:

* ``sgemm_cpu``  (ugemm.h:287)   all 4 transposes x 'R'/'C' x (alpha, beta)
* ``sgemm_c``    (gemm_cpu.h:284) the same cases, K up to 800 (KC=384 blocks)
* ``sgemm_avx``  (sgemm_avx256.h:392) NN row-major, N and K across the 96/35
  block edges
* ``sgemm_sse`` (sgemm_sse.h:400) 8x8-tile Goto GEMM, both majors, all transposes
* ``dgemm_cpu`` / ``_dgemm_c`` / ``dgemm_avx`` (ugemm.h:162, gemm_cpu.h:284,
  dgemm_avx.h:844) FP64
* ``cmp_results`` (check_sgemm.c:56) printed lines
* the known-answer test in the comment at sgemm_test.c:186-200

Inputs are drawn from numpy's PCG64 with fixed seeds and stored beside the
outputs, so the fixture file alone is enough on a machine without the
reference.  Usage: ``python tests/golden/make_golden.py <reference tree>``.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ugemm_golden.npz")

GEMM_SHAPES = [(3, 3, 2), (16, 16, 16), (17, 17, 17), (33, 29, 47), (5, 6, 400)]
AVX_SHAPES = [(3, 3, 2), (17, 17, 17), (5, 96, 35), (8, 100, 71), (11, 200, 40), (4, 193, 36),
              (2, 97, 70)]
D_SHAPES = [(3, 3, 2), (17, 19, 23), (5, 6, 400)]
ALPHA_BETA = [(1.0, 0.0), (1.5, 0.5)]


def stored(major: str, trans: str, rows: int, cols: int):
    """numpy shape of an operand whose op() is rows x cols, for 'R'/'C' storage."""
    shape = oracle.op_shape(trans, rows, cols)
    return shape if major == "R" else shape[::-1]


def capture_stdout(fn):
    """Run fn() and return what it printed on fd 1."""
    r, w = os.pipe()
    saved = os.dup(1)
    sys.stdout.flush()
    os.dup2(w, 1)
    try:
        fn()
    finally:
        os.dup2(saved, 1)
        os.close(w)
        os.close(saved)
    out = os.read(r, 1 << 16).decode()
    os.close(r)
    return out


def main() -> None:
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else None
    if not oracle.build_ref(ref_dir):
        raise SystemExit("usage: make_golden.py <reference tree> (or set UGEMM_REF_DIR; "
                         "x86-64 only)")
    strict = oracle.load_ref(fast=False)
    fast = oracle.load_ref(fast=True)
    rng = np.random.default_rng(20261203)
    data: dict[str, np.ndarray] = {}
    cases = []

    def add(name, **arrs):
        for k, v in arrs.items():
            data[f"{name}/{k}"] = v
        cases.append(name)

    # --- FP32 naive and blocked: every transpose, both majors, two (alpha, beta)
    for (M, N, K) in GEMM_SHAPES:
        for major in "RC":
            for ta in "NT":
                for tb in "NT":
                    for ai, (alpha, beta) in enumerate(ALPHA_BETA):
                        if M * N * K > 5000 and ai == 0:
                            continue  # larger shapes: the (1.5, 0.5) case only, to keep the file small
                        A = rng.uniform(-1, 1, stored(major, ta, M, K)).astype(np.float32)
                        B = rng.uniform(-1, 1, stored(major, tb, K, N)).astype(np.float32)
                        C = rng.uniform(-1, 1, (M, N) if major == "R" else (N, M)).astype(np.float32)
                        outs = {}
                        for fn in ("sgemm_cpu", "sgemm_c"):
                            Cr = C.copy()
                            getattr(strict, fn)(major.encode(), ta.encode(), tb.encode(), M, N, K,
                                                alpha, A, A.shape[1], B, B.shape[1], beta, Cr,
                                                Cr.shape[1])
                            outs[fn] = Cr
                        add(f"s/{major}{ta}{tb}/{M}x{N}x{K}/{ai}", A=A, B=B, C=C,
                            meta=np.array([M, N, K], dtype=np.int64),
                            ab=np.array([alpha, beta], dtype=np.float32),
                            flags=np.frombuffer((major + ta + tb).encode(), dtype=np.uint8),
                            sgemm_cpu=outs["sgemm_cpu"], sgemm_c=outs["sgemm_c"])

    # --- AVX256 SGEMM (NN row-major), built with contraction like the reference
    for (M, N, K) in AVX_SHAPES:
        for ai, (alpha, beta) in enumerate(ALPHA_BETA):
            A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
            B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
            C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
            Cr = C.copy()
            fast.sgemm_avx(b"R", b"N", b"N", M, N, K, alpha, A, K, B, N, beta, Cr, N)
            add(f"avx/{M}x{N}x{K}/{ai}", A=A, B=B, C=C, meta=np.array([M, N, K], dtype=np.int64),
                ab=np.array([alpha, beta], dtype=np.float32), sgemm_avx=Cr)

    # --- FP64 references
    for (M, N, K) in D_SHAPES:
        for ta in "NT":
            for tb in "NT":
                A = rng.uniform(-1, 1, oracle.op_shape(ta, M, K))
                B = rng.uniform(-1, 1, oracle.op_shape(tb, K, N))
                C = rng.uniform(-1, 1, (M, N))
                outs = {}
                for fn in ("dgemm_cpu", "_dgemm_c", "dgemm_avx"):
                    Cr = C.copy()
                    getattr(strict, fn)(b"R", ta.encode(), tb.encode(), M, N, K, 1.5, A, A.shape[1],
                                        B, B.shape[1], 0.5, Cr, N)
                    outs[fn.lstrip("_")] = Cr
                add(f"d/{ta}{tb}/{M}x{N}x{K}", A=A, B=B, C=C, meta=np.array([M, N, K], dtype=np.int64),
                    flags=np.frombuffer(f"R{ta}{tb}".encode(), dtype=np.uint8), **outs)

    # --- cmp_results lines (check_sgemm.c:56-85)
    for i, (M, N) in enumerate([(16, 24), (7, 33)]):
        ref = rng.uniform(-1, 1, (M, N)).astype(np.float32)
        res = (ref + rng.normal(0, 10.0 ** (-3 - 2 * i), (M, N))).astype(np.float32)
        line = capture_stdout(lambda: strict.ref_cmp_results(M, N, ref, res, N))
        add(f"cmp/{i}", ref=ref, res=res, line=np.frombuffer(line.encode(), dtype=np.uint8))

    # --- saxpy_cpu / sgemv_cpu (ugemm.h:86-160)
    for i, (n, incx, incy) in enumerate([(37, 1, 1), (50, 2, 3)]):
        x = rng.uniform(-1, 1, n * incx).astype(np.float32)
        y = rng.uniform(-1, 1, n * incy).astype(np.float32)
        yr = y.copy()
        strict.saxpy_cpu(n, 0.75, x, incx, yr, incy)
        add(f"axpy/{i}", x=x, y=y, meta=np.array([n, incx, incy], dtype=np.int64), out=yr)
    for i, (trans, M, N, lda, inc) in enumerate([("N", 33, 21, 40, 1), ("T", 19, 45, 50, 1),
                                                 ("N", 17, 9, 17, 2)]):
        A = rng.uniform(-1, 1, lda * (N if trans == "N" else M)).astype(np.float32)
        x = rng.uniform(-1, 1, N * inc).astype(np.float32)
        y = rng.uniform(-1, 1, M * inc).astype(np.float32)
        yr = y.copy()
        strict.sgemv_cpu(trans.encode(), M, N, 1.5, A, lda, x, inc, 0.5, yr, inc)
        add(f"gemv/{i}", A=A, x=x, y=y, flags=np.frombuffer(trans.encode(), dtype=np.uint8),
            meta=np.array([M, N, lda, inc], dtype=np.int64), out=yr)

    # --- sgemm_sse (sgemm_sse.h:400-451), built with contraction like the
    # reference: two k blocks (k = 400 > 384) in every major/transpose
    # combination, and two row blocks (m = 390 > 384) with edge tiles
    sse_cases = [(major, ta, tb, 13, 11, 400, 1.5, 0.5) for major in "RC" for ta in "NT"
                 for tb in "NT"]
    sse_cases += [("R", "N", "N", 390, 9, 20, 1.0, 0.0), ("C", "T", "N", 390, 9, 20, 0.75, 1.0)]
    for n_case, (major, ta, tb, M, N, K, alpha, beta) in enumerate(sse_cases):
        A = rng.uniform(-1, 1, stored(major, ta, M, K)).astype(np.float32)
        B = rng.uniform(-1, 1, stored(major, tb, K, N)).astype(np.float32)
        C = rng.uniform(-1, 1, (M, N) if major == "R" else (N, M)).astype(np.float32)
        Cr = C.copy()
        fast.ref_sgemm_sse(major.encode(), ta.encode(), tb.encode(), M, N, K, alpha, A, A.shape[1],
                           B, B.shape[1], beta, Cr, Cr.shape[1])
        add(f"sse/{n_case}", A=A, B=B, C=C, meta=np.array([M, N, K], dtype=np.int64),
            ab=np.array([alpha, beta], dtype=np.float32),
            flags=np.frombuffer((major + ta + tb).encode(), dtype=np.uint8), sgemm_sse=Cr)

    # --- known-answer test, sgemm_test.c:186-200 (RNN 3x3x2)
    A = np.array([[1, 2], [3, 4], [5, 6]], dtype=np.float32)
    B = np.array([[1, 2, 3], [4, 5, 6]], dtype=np.float32)
    C = np.zeros((3, 3), dtype=np.float32)
    strict.sgemm_cpu(b"R", b"N", b"N", 3, 3, 2, 1.0, A, 2, B, 3, 0.0, C, 3)
    add("kat/rnn3x3x2", A=A, B=B, out=C)

    data["cases"] = np.array(cases)
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT}: {len(cases)} cases, {os.path.getsize(OUT)} bytes")


if __name__ == "__main__":
    main()
