"""CPU model of the split-precision representations the tensor-core forms use
(numpy, no GPU): how much of an FP32 operand each split keeps, and the
FP16x3 power-of-two scale rule.

* BF16x6: x = x0 + x1 + x2 in bf16 is exact; dropping a1b2, a2b1, a2b2
  leaves ~2^-24 relative per product.
* FP16x3: x 2^e = h0 + h1 + r in fp16 with |r| <= 2^-22 |x 2^e|; dropping
  h1 g1 and r leaves ~2^-22 relative per product -- 6.5e-8 normwise on the
  config-2 input sets, a third of what the FP32 SIMT form loses to
  rounding already at K = 1023 (5.7e-7 measured).
The scale rule restated here is the kernels' f16_scale_exp, applied to every
row of op(A) and every column of op(B) on its own: the row's largest finite
magnitude m lands in [2^14, 2^15), so nothing overflows fp16 (largest 65504)
and the lower piece of every element near m is normal; C[i][j] is the
accumulator times 2^-(eA[i] + eB[j]).  Per-row scales keep rows and columns
of very different magnitudes accurate (a single operand-wide scale would
flush every element more than 2^38 below the operand's largest to zero)."""
import numpy as np
import pytest


def scale_exp(m):
    """e such that m 2^e lies in [2^14, 2^15); 0 for zero or non-finite m.
    From the largest finite float (-113) to the smallest subnormal (163)."""
    if m == 0 or not np.isfinite(m):
        return 0
    return 14 - int(np.floor(np.log2(np.float64(m))))


def split_fp16(x):
    """Per-row FP16x3 pieces of x (rows x K): h0, h1 and each row's exponent."""
    x = np.atleast_2d(x)
    e = np.array([scale_exp(np.abs(r[np.isfinite(r)]).max() if np.isfinite(r).any() else 0.0)
                  for r in x], dtype=np.int64)
    xs = (x.astype(np.float64) * 2.0 ** e[:, None]).astype(np.float32)
    with np.errstate(invalid="ignore", over="ignore"):  # inf - inf: the NaN lower piece
        h0 = xs.astype(np.float16).astype(np.float32)
        h1 = (xs - h0).astype(np.float16).astype(np.float32)
    return h0.astype(np.float64), h1.astype(np.float64), e


def fp16x3_product(A, B):
    """The FP16x3 form's product in exact arithmetic (no accumulation error):
    per-row pieces of A, per-column pieces of B, three piece products."""
    a0, a1, ea = split_fp16(A)
    b0, b1, eb = split_fp16(B.T)
    acc = a0 @ b0.T + a0 @ b1.T + a1 @ b0.T
    return acc * 2.0 ** (-(ea[:, None] + eb[None, :]))


def rowwise(C, R):
    """Largest relative error of a row: max_i ||C_i - R_i|| / ||R_i||."""
    return float(np.max(np.linalg.norm(C - R, axis=1) / np.linalg.norm(R, axis=1)))


def bf16(x):
    """Round-to-nearest-even to bf16, returned as float32."""
    b = x.astype(np.float32).view(np.uint32).astype(np.uint64)
    r = ((b >> 16) & 1) + 0x7FFF
    return ((b + r) & 0xFFFF0000).astype(np.uint32).view(np.float32)


def tf32(x):
    """Round to nearest (ties away from zero) to TF32's 10 stored significand
    bits, as FP32 (the PTX cvt.rna.tf32.f32 rounding)."""
    b = x.astype(np.float32).view(np.uint32).astype(np.uint64)
    return (((b + 0x1000) & 0xFFFFE000) & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def split_tf32(x):
    x0 = tf32(x)
    x1 = tf32((x - x0).astype(np.float32))
    return x0.astype(np.float64), x1.astype(np.float64)


def split_bf16(x):
    x0 = bf16(x)
    x1 = bf16((x - x0).astype(np.float32))
    x2 = bf16((x - x0 - x1).astype(np.float32))
    return [p.astype(np.float64) for p in (x0, x1, x2)]


def draw(kind, shape, rng, span=8):
    if kind == "uniform":
        return rng.uniform(-1, 1, shape).astype(np.float32)
    mant = rng.uniform(1, 2, shape)
    sign = rng.choice([-1.0, 1.0], shape)
    expo = rng.integers(-span, span + 1, shape)
    return (sign * mant * 2.0 ** expo).astype(np.float32)


@pytest.mark.parametrize("kind", ["uniform", "wide"])
def test_split_errors_against_fp64(kind):
    rng = np.random.default_rng(3)
    A, B = draw(kind, (64, 1023), rng), draw(kind, (1023, 48), rng)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    norm = np.linalg.norm(exact)
    fp16x3 = fp16x3_product(A, B)
    x0, x1, x2 = split_bf16(A)
    y0, y1, y2 = split_bf16(B)
    bf16x6 = x0 @ y0 + x0 @ y1 + x1 @ y0 + x0 @ y2 + x2 @ y0 + x1 @ y1
    assert np.array_equal(x0 + x1 + x2, A.astype(np.float64))  # three bf16 pieces are exact
    t0, t1 = split_tf32(A)
    u0, u1 = split_tf32(B)
    tf32x3 = t0 @ u0 + t0 @ u1 + t1 @ u0
    e16 = np.linalg.norm(fp16x3 - exact) / norm
    ebf = np.linalg.norm(bf16x6 - exact) / norm
    etf = np.linalg.norm(tf32x3 - exact) / norm
    assert etf < 1.2e-7, etf      # the same 22 bits as FP16x3, no scaling
    assert e16 < 1.2e-7, e16      # ~6.5e-8: the 2^-22 dropped terms
    assert ebf < 1e-8, ebf        # ~4.5e-9: the 2^-24 dropped terms


def fp32_rowwise(A, B):
    """Row-wise error of an FP32 GEMM that rounds after every k step (the
    SIMT form's accumulation), the bar the split forms must meet."""
    acc = np.zeros((A.shape[0], B.shape[1]), np.float32)
    for k in range(A.shape[1]):
        acc = (acc.astype(np.float64) + A[:, k:k + 1].astype(np.float64) * B[k:k + 1, :]).astype(
            np.float32)
    return acc.astype(np.float64)


def adversarial(name, rng):
    M, N, K = 48, 40, 512
    A, B = draw("uniform", (M, K), rng), draw("uniform", (K, N), rng)
    if name == "outlier":       # one element 2^40 times the rest
        A[17, 33] = 2.0 ** 40
    elif name == "rows":        # every other row of A, every third column of B at 2^-30
        A[::2] *= np.float32(2.0 ** -30)
        B[:, ::3] *= np.float32(2.0 ** -30)
    else:                       # exponents uniform in [-40, 40]
        A, B = draw("wide", (M, K), rng, 40), draw("wide", (K, N), rng, 40)
    return A, B


@pytest.mark.parametrize("name", ["outlier", "rows", "wide40"])
def test_per_row_scales_keep_every_row_accurate(name):
    """The cases a single operand-wide scale gets wrong (rows far below the
    operand's largest element lose every bit): with per-row scales every row
    of C is at least as accurate as an FP32 k-loop's."""
    rng = np.random.default_rng(11)
    A, B = adversarial(name, rng)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    ours = rowwise(fp16x3_product(A, B), exact)
    fp32 = rowwise(fp32_rowwise(A, B), exact)
    assert ours <= fp32, (name, ours, fp32)
    assert ours < 2e-7, (name, ours)


@pytest.mark.parametrize("m", [1.0, 0.999, 1023.9, 65504.0, 3e38, 1e-30, 1e-40, 0.125, 32767.0,
                               1e-45])
def test_scale_puts_the_largest_element_in_range(m):
    e = scale_exp(np.float32(m))
    scaled = np.float64(np.float32(m)) * 2.0 ** e
    assert 2.0 ** 14 <= scaled < 2.0 ** 15  # subnormal rows too: the scale is up to 2^163
    assert np.isfinite(np.float16(scaled))
    assert -113 <= e <= 163


def test_scale_ignores_non_finite_and_zero():
    assert scale_exp(0.0) == 0
    assert scale_exp(np.inf) == 0
    assert scale_exp(np.nan) == 0
    x = np.array([1e6, -3.0, np.inf, 7.5], dtype=np.float32)
    h0, h1, e = split_fp16(x)
    assert e[0] == scale_exp(1e6)         # the infinity does not set the scale
    assert np.isfinite(h0[0, [0, 1, 3]]).all()  # the finite elements stay finite
    assert np.isinf(h0[0, 2])
