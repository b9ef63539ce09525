"""Pin the CPU oracle against fixtures produced by the reference's own code.

tests/golden/ugemm_golden.npz was written by tests/golden/make_golden.py,
which compiled the reference's ugemm.h / gemm_cpu.h / sgemm_avx256.h /
dgemm_avx.h / check_sgemm.c and ran them.  Every FP32 restatement must match
bit for bit; FP64 to the last ulp of the same operation order.
"""
import numpy as np
import pytest

import oracle


def _cases(golden, prefix):
    return [c for c in golden["cases"] if str(c).startswith(prefix)]


def test_oracle_builds_and_loads():
    lib = oracle.load()
    for sym in ("oracle_sgemm_cpu", "oracle_dgemm_cpu", "oracle_sgemm_c", "oracle_dgemm_c",
                "oracle_sgemm_avx256", "oracle_sgemm_avx256_mt", "oracle_sgemm_sse",
                "oracle_cmp_results", "oracle_im2col"):
        assert hasattr(lib, sym)


def test_sgemm_naive_and_blocked_bit_exact(golden):
    cases = _cases(golden, "s/")
    assert len(cases) >= 40
    for name in cases:
        g = lambda k: golden[f"{name}/{k}"]  # noqa: E731
        M, N, K = (int(x) for x in g("meta"))
        alpha, beta = (float(x) for x in g("ab"))
        major, ta, tb = bytes(g("flags")).decode()
        for fn, key in (("oracle_sgemm_cpu", "sgemm_cpu"), ("oracle_sgemm_c", "sgemm_c")):
            C = g("C").copy()
            oracle.sgemm(fn, ta, tb, M, N, K, alpha, g("A"), g("B"), beta, C, major=major)
            assert np.array_equal(C, g(key)), (name, fn)


def test_avx256_port_bit_exact(golden):
    cases = _cases(golden, "avx/")
    assert len(cases) >= 10
    lib = oracle.load()
    for name in cases:
        g = lambda k: golden[f"{name}/{k}"]  # noqa: E731
        M, N, K = (int(x) for x in g("meta"))
        alpha, beta = (float(x) for x in g("ab"))
        C = g("C").copy()
        lib.oracle_sgemm_avx256(M, N, K, alpha, g("A"), K, g("B"), N, beta, C, N)
        assert np.array_equal(C, g("sgemm_avx")), name


def test_sse_goto_gemm_bit_exact(golden):
    """sgemm_sse (sgemm_sse.h:400-451): both majors, all transposes, two k
    blocks, two row blocks, edge tiles, alpha/beta special cases."""
    cases = _cases(golden, "sse/")
    assert len(cases) >= 10
    lib = oracle.load()
    for name in cases:
        g = lambda k: golden[f"{name}/{k}"]  # noqa: E731
        M, N, K = (int(x) for x in g("meta"))
        alpha, beta = (float(x) for x in g("ab"))
        major, ta, tb = bytes(g("flags")).decode()
        A, B, C = g("A"), g("B"), g("C").copy()
        lib.oracle_sgemm_sse(major.encode(), ta.encode(), tb.encode(), M, N, K, alpha, A,
                             A.shape[1], B, B.shape[1], beta, C, C.shape[1])
        assert np.array_equal(C, g("sgemm_sse")), name


@pytest.mark.parametrize("loop,ta,tb", [("rnn", "N", "N"), ("rnt", "N", "T"), ("rtn", "T", "N")])
def test_gpu_test_cpu_loops(golden, loop, ta, tb):
    """sgemm_test.c:40-105 (not compilable here: it needs OpenCL headers).
    On small-integer inputs every product and sum is exact in FP32, so the
    loops must equal the naive oracle exactly whatever their order; plus the
    known-answer test of sgemm_test.c:186-200 through gemm_rnn."""
    lib = oracle.load()
    rng = np.random.default_rng(7)
    M, N, K = 23, 17, 31
    A = rng.integers(-8, 9, oracle.op_shape(ta, M, K)).astype(np.float32)
    B = rng.integers(-8, 9, oracle.op_shape(tb, K, N)).astype(np.float32)
    for alpha, beta in ((1.0, 0.0), (2.0, 0.5), (1.0, 1.0)):
        C0 = rng.integers(-8, 9, (M, N)).astype(np.float32)
        got = C0.copy()
        getattr(lib, f"oracle_gemm_{loop}")(M, N, K, alpha, A, B, beta, got)
        ref = oracle.sgemm("oracle_sgemm_cpu", ta, tb, M, N, K, alpha, A, B, beta, C0.copy())
        assert np.array_equal(got, ref), (loop, alpha, beta)
    if loop == "rnn":
        g = lambda k: golden[f"kat/rnn3x3x2/{k}"]  # noqa: E731
        C = np.zeros((3, 3), dtype=np.float32)
        lib.oracle_gemm_rnn(3, 3, 2, 1.0, g("A"), g("B"), 0.0, C)
        assert np.array_equal(C, g("out"))


@pytest.mark.parametrize("threads", [1, 3, 4])
def test_avx256_threaded_harness_matches_single(golden, threads):
    """Row bands do not change per-element arithmetic; transposes are exact."""
    rng = np.random.default_rng(7)
    M, N, K = 67, 131, 75
    for ta in "NT":
        for tb in "NT":
            A = rng.uniform(-1, 1, oracle.op_shape(ta, M, K)).astype(np.float32)
            B = rng.uniform(-1, 1, oracle.op_shape(tb, K, N)).astype(np.float32)
            C0 = rng.uniform(-1, 1, (M, N)).astype(np.float32)
            An = np.ascontiguousarray(A if ta == "N" else A.T)
            Bn = np.ascontiguousarray(B if tb == "N" else B.T)
            ref = C0.copy()
            oracle.load().oracle_sgemm_avx256(M, N, K, 1.5, An, K, Bn, N, 0.5, ref, N)
            C = C0.copy()
            oracle.sgemm_avx256_mt(threads, ta, tb, M, N, K, 1.5, A, B, 0.5, C)
            assert np.array_equal(C, ref)


def test_dgemm_matches_reference(golden):
    cases = _cases(golden, "d/")
    assert len(cases) >= 8
    for name in cases:
        g = lambda k: golden[f"{name}/{k}"]  # noqa: E731
        M, N, K = (int(x) for x in g("meta"))
        major, ta, tb = bytes(g("flags")).decode()
        for fn, key in (("oracle_dgemm_cpu", "dgemm_cpu"), ("oracle_dgemm_c", "dgemm_c")):
            C = g("C").copy()
            oracle.dgemm(ta, tb, M, N, K, 1.5, g("A"), g("B"), 0.5, C, major=major, fn=fn)
            assert np.array_equal(C, g(key)), (name, fn)
        # dgemm_avx (dgemm_avx.h:844) sums in another order: agree to FP64 rounding
        C = g("C").copy()
        oracle.dgemm(ta, tb, M, N, K, 1.5, g("A"), g("B"), 0.5, C, fn="oracle_dgemm_cpu")
        np.testing.assert_allclose(C, g("dgemm_avx"), rtol=0, atol=1e-12 * K)


def test_cmp_results_matches_reference_line(golden):
    for name in _cases(golden, "cmp/"):
        g = lambda k: golden[f"{name}/{k}"]  # noqa: E731
        label, std_err, std_ref, max_err, max_i = oracle.cmp_results(g("ref"), g("res"))
        N = g("ref").shape[1]
        line = "%.3e/%.3e=%.3e. %.3e at [%3d,%3d] %18.10e vs %18.10e %s\n" % (
            std_err, std_ref, std_err / std_ref, max_err, max_i // N, max_i % N,
            float(g("ref").flat[max_i]), float(g("res").flat[max_i]), label)
        assert line == bytes(g("line")).decode()


def test_known_answer_rnn_3x3x2(golden):
    """sgemm_test.c:186-200: [[1,2],[3,4],[5,6]] x [[1,2,3],[4,5,6]]."""
    A = golden["kat/rnn3x3x2/A"]
    B = golden["kat/rnn3x3x2/B"]
    C = np.zeros((3, 3), dtype=np.float32)
    oracle.sgemm("oracle_sgemm_cpu", "N", "N", 3, 3, 2, 1.0, A, B, 0.0, C)
    expect = np.array([[9, 12, 15], [19, 26, 33], [29, 40, 51]], dtype=np.float32)
    assert np.array_equal(C, expect)
    assert np.array_equal(golden["kat/rnn3x3x2/out"], expect)


def test_im2col_matches_direct_convolution():
    """im2col (sgemm_ocl1.h:81-119) followed by a GEMM is a convolution.

    The reference's im2col is an OpenCL kernel that cannot run here; its
    restatement is pinned by this property against a direct FP64 convolution.
    """
    rng = np.random.default_rng(3)
    for (c, h, w, k, pad, stride) in [(3, 7, 9, 3, 1, 1), (2, 8, 8, 3, 1, 2), (4, 5, 6, 1, 0, 1),
                                      (2, 6, 5, 4, 2, 2)]:
        im = rng.uniform(0, 1, (c, h, w)).astype(np.float32)
        wt = rng.normal(0, 1, (5, c, k, k))
        col = oracle.im2col(im, k, pad, stride)
        ho = (h + 2 * pad - k) // stride + 1
        wo = (w + 2 * pad - k) // stride + 1
        got = wt.reshape(5, -1) @ col.astype(np.float64)
        padded = np.pad(im.astype(np.float64), ((0, 0), (pad, pad), (pad, pad)))
        ref = np.zeros((5, ho, wo))
        for i in range(ho):
            for j in range(wo):
                patch = padded[:, i * stride:i * stride + k, j * stride:j * stride + k]
                ref[:, i, j] = np.tensordot(wt, patch, axes=([1, 2, 3], [0, 1, 2]))
        np.testing.assert_allclose(got, ref.reshape(5, -1), rtol=1e-12, atol=1e-12)


def test_saxpy_and_sgemv_restatements_bit_exact(golden):
    lib = oracle.load()
    for name in [c for c in golden["cases"] if str(c).startswith("axpy/")]:
        g = lambda k: golden[f"{name}/{k}"]  # noqa: E731
        n, incx, incy = (int(v) for v in g("meta"))
        y = g("y").copy()
        lib.oracle_saxpy_cpu(n, 0.75, g("x"), incx, y, incy)
        assert np.array_equal(y, g("out")), name
    for name in [c for c in golden["cases"] if str(c).startswith("gemv/")]:
        g = lambda k: golden[f"{name}/{k}"]  # noqa: E731
        M, N, lda, inc = (int(v) for v in g("meta"))
        y = g("y").copy()
        lib.oracle_sgemv_cpu(bytes(g("flags")), M, N, 1.5, g("A"), lda, g("x"), inc, 0.5, y, inc)
        assert np.array_equal(y, g("out")), name


def test_bias_leaky_restatement():
    """sgemm_gl1.h:210-217 on a few values, including the double-precision leak."""
    out = np.array([[1.0, -1.0, -3.0], [0.5, -0.25, 2.0]], dtype=np.float32)
    oracle.bias_leaky(out, np.array([0.5, -1.0], dtype=np.float32))
    expect = np.array([[1.5, np.float32(-0.5 * 0.1), np.float32(-2.5 * 0.1)],
                       [np.float32(-0.5 * 0.1), np.float32(-1.25 * 0.1), 1.0]], dtype=np.float32)
    assert np.array_equal(out, expect)
