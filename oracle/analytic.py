"""ORACLE - analytic sphere solutions used by the reference's tests and examples.

Restated from BoundaryIntegralEquations.jl:
  * incoming_wave                 src/analytical/3d_scattering.jl:4-12
  * plane_wave_scattering_sphere  src/analytical/3d_scattering.jl:20-44
    (total pressure on a rigid sphere, series summed until the relative size of
    the last term is below Ieps)
  * interior pulsating sphere     examples/3d_pulsating_sphere.jl:34-35
"""
from __future__ import annotations

import numpy as np
from scipy.special import eval_legendre, hankel1, jv


def incoming_wave(angles, P0, xyzb, k):
    A = np.sin(angles[0]) * np.cos(angles[1])
    B = np.sin(angles[0]) * np.sin(angles[1])
    Cc = np.cos(angles[0])
    dps = (A * xyzb[0] + B * xyzb[1] + Cc * xyzb[2]) / np.sqrt(A**2 + B**2 + Cc**2)
    return P0 * np.exp(-1j * (k * dps))


def plane_wave_scattering_sphere(k, a, r, theta, Ieps):
    ka, kr = k * a, k * r
    theta = np.asarray(theta, dtype=np.float64)
    ptot = np.zeros(theta.shape, dtype=np.complex128)
    n = 0
    rel = Ieps * 10.0
    acc = []
    while rel > Ieps:
        apri = (n * jv(n - 0.5, ka) - (n + 1) * jv(n + 1.5, ka)) / \
               (n * hankel1(n - 0.5, ka) - (n + 1) * hankel1(n + 1.5, ka))
        P = eval_legendre(n, np.cos(theta))
        factor = (-1j) ** n * (2 * n + 1) * np.sqrt(np.pi / 2.0 / kr)
        it = factor * (jv(n + 0.5, kr) - apri * hankel1(n + 0.5, kr)) * P
        ptot = ptot + it
        with np.errstate(divide="ignore", invalid="ignore"):
            rel = float(np.max(np.abs(it / ptot)))
        acc.append(rel)
        n += 1
    return ptot, acc


def pulsating_sphere_interior(k, a, Z0, vr, r):
    """p(r) = i Z0 vr (a / r) ka sin(kr) / (ka cos(ka) - sin(ka)), r <= a."""
    r = np.asarray(r, dtype=np.float64)
    return 1j * Z0 * vr * (a / r) * (k * a * np.sin(k * r)) / (k * a * np.cos(k * a) - np.sin(k * a))
