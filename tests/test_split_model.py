"""CPU model of the split-precision representations the tensor-core forms use
(numpy, no GPU): how much of an FP32 operand each split keeps, and the
FP16x3 power-of-two scale rule.

* BF16x6: x = x0 + x1 + x2 in bf16 is exact; dropping a1b2, a2b1, a2b2
  leaves ~2^-24 relative per product.
* FP16x3: x 2^e = h0 + h1 + r in fp16 with |r| <= 2^-22 |x 2^e|; dropping
  h1 g1 and r leaves ~2^-22 relative per product -- 6.5e-8 normwise on the
  config-2 input sets, a third of what the FP32 SIMT form loses to
  rounding already at K = 1023 (5.7e-7 measured).
The scale rule restated here is the kernels' f16_scale_exp: the largest
finite magnitude m lands in [2^14, 2^15), so nothing overflows fp16
(largest 65504) and the lower piece of every element near m is normal."""
import numpy as np
import pytest


def scale_exp(m):
    """2^e such that m 2^e lies in [2^14, 2^15); 0 for zero or non-finite m,
    clamped to [-113, 126] so that 2^e and 2^-e are normal floats."""
    if m == 0 or not np.isfinite(m):
        return 0
    e = 14 - int(np.floor(np.log2(np.float64(m))))
    return max(-113, min(126, e))


def split_fp16(x):
    finite = np.abs(x[np.isfinite(x)])
    e = scale_exp(finite.max() if finite.size else 0.0)
    xs = (x.astype(np.float64) * 2.0 ** e).astype(np.float32)
    with np.errstate(invalid="ignore", over="ignore"):  # inf - inf: the NaN lower piece
        h0 = xs.astype(np.float16).astype(np.float32)
        h1 = (xs - h0).astype(np.float16).astype(np.float32)
    return h0.astype(np.float64), h1.astype(np.float64), e


def bf16(x):
    """Round-to-nearest-even to bf16, returned as float32."""
    b = x.astype(np.float32).view(np.uint32).astype(np.uint64)
    r = ((b >> 16) & 1) + 0x7FFF
    return ((b + r) & 0xFFFF0000).astype(np.uint32).view(np.float32)


def split_bf16(x):
    x0 = bf16(x)
    x1 = bf16((x - x0).astype(np.float32))
    x2 = bf16((x - x0 - x1).astype(np.float32))
    return [p.astype(np.float64) for p in (x0, x1, x2)]


def draw(kind, shape, rng):
    if kind == "uniform":
        return rng.uniform(-1, 1, shape).astype(np.float32)
    mant = rng.uniform(1, 2, shape)
    sign = rng.choice([-1.0, 1.0], shape)
    expo = rng.integers(-8, 9, shape)
    return (sign * mant * 2.0 ** expo).astype(np.float32)


@pytest.mark.parametrize("kind", ["uniform", "wide"])
def test_split_errors_against_fp64(kind):
    rng = np.random.default_rng(3)
    A, B = draw(kind, (64, 1023), rng), draw(kind, (1023, 48), rng)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    norm = np.linalg.norm(exact)
    a0, a1, ea = split_fp16(A)
    b0, b1, eb = split_fp16(B)
    fp16x3 = (a0 @ b0 + a0 @ b1 + a1 @ b0) * 2.0 ** (-ea - eb)
    x0, x1, x2 = split_bf16(A)
    y0, y1, y2 = split_bf16(B)
    bf16x6 = x0 @ y0 + x0 @ y1 + x1 @ y0 + x0 @ y2 + x2 @ y0 + x1 @ y1
    assert np.array_equal(x0 + x1 + x2, A.astype(np.float64))  # three bf16 pieces are exact
    e16 = np.linalg.norm(fp16x3 - exact) / norm
    ebf = np.linalg.norm(bf16x6 - exact) / norm
    assert e16 < 1.2e-7, e16      # ~6.5e-8: the 2^-22 dropped terms
    assert ebf < 1e-8, ebf        # ~4.5e-9: the 2^-24 dropped terms


@pytest.mark.parametrize("m", [1.0, 0.999, 1023.9, 65504.0, 3e38, 1e-30, 1e-40, 0.125, 32767.0])
def test_scale_puts_the_largest_element_in_range(m):
    e = scale_exp(np.float32(m))
    scaled = np.float64(np.float32(m)) * 2.0 ** e
    if np.float32(m) >= 2.0 ** -112:
        assert 2.0 ** 14 <= scaled < 2.0 ** 15
    else:  # denormal operands: clamped, still far below fp16's largest value
        assert scaled < 2.0 ** 15
    assert np.isfinite(np.float16(scaled))
    assert -113 <= e <= 126


def test_scale_ignores_non_finite_and_zero():
    assert scale_exp(0.0) == 0
    assert scale_exp(np.inf) == 0
    assert scale_exp(np.nan) == 0
    x = np.array([1e6, -3.0, np.inf, 7.5], dtype=np.float32)
    h0, h1, e = split_fp16(x)
    assert e == scale_exp(1e6)            # the infinity does not set the scale
    assert np.isfinite(h0[[0, 1, 3]]).all()  # the finite elements stay finite
    assert np.isinf(h0[2])
