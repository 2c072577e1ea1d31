"""Test infrastructure (oracle only): FP64 series solutions for scattering by
a rigid (sound-hard) or soft (sound-soft) sphere.

Conventions follow NumCalc: time factor e^{-i w t}, free-space Green's
function G = e^{ikr}/(4 pi r) (``NC_ConstantsVariables.h:92-94``), pressure
p = i rho w phi (``NC_Main.cpp:376``).  A point source of NC.inp amplitude Q
then radiates p_inc = Q G(x, s), a plane wave of amplitude Q and unit
direction d radiates p_inc = Q e^{ik d.x} (``NC_EquationSystem.cpp:1731-1812``
with the 1/(i rho w) of ``NC_EquationSystem.cpp:1936,1957``).

The series are the classical ones (e.g. Beranek & Mellow, Acoustics: Sound
Fields and Transducers, sec. 12.4), the same physics the reference's
``tests/resources/test_numcalc/analytical_references/sphere_*.m`` scripts
evaluate in the e^{+jwt} convention; here everything is written directly in
the e^{-iwt} convention with scipy's spherical Bessel functions.
"""
from __future__ import annotations

import numpy as np
from scipy.special import eval_legendre, spherical_jn, spherical_yn


def _h1(n, x, derivative=False):
    return spherical_jn(n, x, derivative) + 1j * spherical_yn(n, x, derivative)


def _nterms(k, rmax):
    return int(np.ceil(k * rmax + 10.0 * (k * rmax) ** (1.0 / 3.0) + 20))


def point_source_sphere(points, source, a, k, Q=1.0, rigid=True, nmax=None):
    """Total pressure at ``points`` (|x| >= a) for a point source at ``source``."""
    pts = np.atleast_2d(points).astype(float)
    s = np.asarray(source, float)
    rs = np.linalg.norm(s)
    r = np.linalg.norm(pts, axis=1)
    cosg = np.clip(pts @ s / (r * rs), -1.0, 1.0)
    nmax = nmax or _nterms(k, max(rs, r.max()))
    ka = k * a
    out = np.zeros(len(pts), complex)
    rl = np.minimum(r, rs)
    rg = np.maximum(r, rs)
    for n in range(nmax + 1):
        if rigid:
            c = spherical_jn(n, ka, True) / _h1(n, ka, True)
        else:
            c = spherical_jn(n, ka) / _h1(n, ka)
        term = (spherical_jn(n, k * rl) - c * _h1(n, k * rl)) * _h1(n, k * rg)
        out += (2 * n + 1) * eval_legendre(n, cosg) * term
    return Q * 1j * k / (4 * np.pi) * out


def plane_wave_sphere(points, direction, a, k, Q=1.0, rigid=True, nmax=None):
    """Total pressure for an incident plane wave Q e^{ik d.x}."""
    pts = np.atleast_2d(points).astype(float)
    d = np.asarray(direction, float)
    d = d / np.linalg.norm(d)
    r = np.linalg.norm(pts, axis=1)
    cost = np.clip(pts @ d / r, -1.0, 1.0)
    nmax = nmax or _nterms(k, r.max())
    ka = k * a
    out = np.zeros(len(pts), complex)
    for n in range(nmax + 1):
        if rigid:
            c = spherical_jn(n, ka, True) / _h1(n, ka, True)
        else:
            c = spherical_jn(n, ka) / _h1(n, ka)
        out += (1j ** n) * (2 * n + 1) * eval_legendre(n, cost) * (
            spherical_jn(n, k * r) - c * _h1(n, k * r))
    return Q * out
