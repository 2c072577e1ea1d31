"""The float sin/cos of the mixed-precision kernels (Cody-Waite reduction by
pi/2 + Taylor polynomials, csrc/bem_common.cuh phase_sincos), emulated step by
step in IEEE single precision and bounded against FP64 sin/cos over the phase
range the kernels use (|k r| <= 10^3).  The device results are covered by the
mixed-precision parity tests."""
import numpy as np

f32 = np.float32


def fma(a, b, c):
    # single rounding of a*b + c, as the device FMA
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def phase_sincos(x):
    sh = fma(f32(x), f32(0.636619772), f32(12582912.0))
    qi = int(np.array(sh, dtype=np.float32).view(np.int32))
    q = f32(sh - f32(12582912.0))
    r = fma(q, f32(-1.57079637050628662), f32(x))
    r = fma(q, f32(4.37113882867379e-08), r)
    r = fma(q, f32(1.71512451000588e-15), r)
    r2 = f32(r * r)
    ps = fma(r2, f32(2.755731922e-6), f32(-1.984126984e-4))
    ps = fma(ps, r2, f32(8.333333333e-3))
    ps = fma(ps, r2, f32(-0.1666666667))
    sn = fma(f32(ps * r2), r, r)
    pc = fma(r2, f32(-2.755731922e-7), f32(2.480158730e-5))
    pc = fma(pc, r2, f32(-1.388888889e-3))
    pc = fma(pc, r2, f32(4.166666667e-2))
    pc = fma(pc, r2, f32(-0.5))
    cs = fma(pc, r2, f32(1.0))
    so, co = (cs, sn) if qi & 1 else (sn, cs)
    return (-so if qi & 2 else so), (-co if (qi + 1) & 2 else co)


def test_phase_sincos_error_bound():
    rng = np.random.default_rng(3)
    xs = np.concatenate([rng.uniform(-1000, 1000, 4000), rng.uniform(-4, 4, 2000),
                         np.arange(-20, 21) * (np.pi / 2)]).astype(np.float32)
    err = 0.0
    for x in xs:
        s, c = phase_sincos(x)
        xd = float(x)
        err = max(err, abs(float(s) - np.sin(xd)), abs(float(c) - np.cos(xd)))
    # a few float ulps of values of magnitude <= 1
    assert err < 3e-7, err
