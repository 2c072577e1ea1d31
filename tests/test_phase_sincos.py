"""The argument reduction of the float phase sin/cos (csrc/bem_common.cuh,
phase_sincos): Cody & Waite by 2 pi with 2 pi split into two floats and the
1.5*2^23 shifter for round(x / 2 pi), emulated step by step in IEEE single
precision.  Over the phases the kernels use (|k r| <= 10^3) the reduced
argument lies in [-pi, pi] (up to 1e-4 where x / 2 pi is near a half
integer and the rounding of the quotient decides) and differs from the exact remainder by less than
2e-6 (the hardware sin/cos that follow are accurate to ~2^-21 there).  The
device results are covered by the mixed-precision parity tests."""
import numpy as np

f32 = np.float32


def fma(a, b, c):
    # single rounding of a*b + c (the product of two floats is exact in FP64)
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def reduce(x):
    sh = fma(f32(x), f32(0.159154943), f32(12582912.0))
    q = f32(sh - f32(12582912.0))
    r = fma(q, f32(-6.28318548202514648), f32(x))
    return fma(q, f32(1.74845553146951e-07), r), q


def test_reduction_range_and_error():
    rng = np.random.default_rng(3)
    xs = np.concatenate([rng.uniform(-1000, 1000, 20000), rng.uniform(-7, 7, 4000),
                         np.arange(-160, 161) * np.pi]).astype(np.float32)
    worst = 0.0
    for x in xs:
        r, q = reduce(x)
        assert abs(float(r)) <= np.pi + 1e-4
        exact = np.remainder(np.float64(x) + np.pi, 2 * np.pi) - np.pi
        d = abs(np.remainder(float(r) - exact + np.pi, 2 * np.pi) - np.pi)
        worst = max(worst, d)
    assert worst < 2e-6, worst
