"""The rounding identity the mixed extension band relies on (csrc/vsl_tiled.cuh,
extend_node_mixed): for finite FP32 values a and b, the FP64 difference a - b rounded to FP32
equals the FP32 difference a - b.  The band node therefore takes a segment between two FP32
values of its line in FP32 and only the segments that touch an FP64 value (the node's
shadow, a crossing value, a neighbour's shadow) in FP64, with the same bits as taking all six
in FP64.

Why it holds: a - b is a multiple of the smaller operand's unit in the last place and below
2^(e+2), e the larger exponent, so it needs at most e - e_b + 25 significant bits and is exact
in FP64 unless the exponents lie more than 28 apart; then |b| < 2^(e-28), and a - b lies
within that of the FP32 value a, at least 2^(e-25) - 2^(e-28) from any FP32 rounding
boundary, which the FP64 rounding (at most 2^(e-53)) cannot cross.
"""
import numpy as np
import pytest


def _fp64_then_fp32(a, b):
    with np.errstate(all="ignore"):
        return (a.astype(np.float64) - b.astype(np.float64)).astype(np.float32)


def _fp32(a, b):
    with np.errstate(all="ignore"):
        return a - b


def _same_bits(x, y):
    return np.array_equal(x.view(np.uint32), y.view(np.uint32))


@pytest.mark.parametrize("case", ["any_bits", "near_equal", "level_set", "wide_spread"])
def test_fp64_difference_rounded_is_fp32_difference(case):
    rng = np.random.default_rng(7)
    n = 2_000_000
    if case == "any_bits":  # every sign and exponent, subnormals and overflow included
        a = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32).view(np.float32)
        b = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32).view(np.float32)
    elif case == "near_equal":  # cancellation: operands a few thousand units apart
        a = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32).view(np.float32)
        b = (a.view(np.uint32) + rng.integers(-3000, 3000, n).astype(np.uint32)).view(np.float32)
    elif case == "level_set":  # values and differences of a distance field and its crossings
        a = (rng.standard_normal(n) * 10.0 ** rng.integers(-12, 2, n)).astype(np.float32)
        b = (rng.standard_normal(n) * 10.0 ** rng.integers(-12, 2, n)).astype(np.float32)
    else:  # exponent spreads around 28: where the FP64 difference stops being exact
        a = (rng.random(n) + 1).astype(np.float32)
        sign = np.where(rng.random(n) < 0.5, -1.0, 1.0)
        b = ((rng.random(n) + 1) * 2.0 ** -rng.integers(20, 40, n) * sign).astype(np.float32)
    keep = np.isfinite(a) & np.isfinite(b)
    a, b = a[keep], b[keep]
    assert _same_bits(_fp64_then_fp32(a, b), _fp32(a, b))


def test_signed_zeros_and_equal_operands():
    vals = np.array([0.0, -0.0, 1.0, -1.0, 2.0**-149, -(2.0**-149), 3.4e38, -3.4e38], dtype=np.float32)
    a, b = np.meshgrid(vals, vals)
    a, b = a.ravel(), b.ravel()
    assert _same_bits(_fp64_then_fp32(a, b), _fp32(a, b))
