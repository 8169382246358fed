"""Wavenumbers of the visco-thermal ("lossy") three-wavenumber system.

The reference computes the acoustic, thermal and viscous wavenumbers from the
ambient state of air in `visco_thermal_constants` (src/utils/lossy_constants.jl:
1-34, with the Rasmussen air-property tables of src/utils/ambient_to_properties.jl).
This module gives their leading-order forms for fixed textbook air properties,
in the reference's S = +1 sign convention:

    k   = omega / c
    k_v = sqrt(i omega rho / mu)        (viscous; kv2 = S i kp / lvp)
    k_h = sqrt(i omega / alpha)         (thermal; kh2 ~ S i kp / lh)

so that Im k_v / Re k_v = Im k_h / Re k_h = 1.  These fix the three
wavenumbers of the multi-right-hand-side workload; no other part of the
lossy system (its boundary conditions, the tangential-derivative coupling of
LossyGlobalOuter) is built here.
"""
from __future__ import annotations

import numpy as np

AIR_20C = {"rho": 1.204, "c": 343.2, "mu": 1.81e-5, "alpha": 2.2e-5}


def boundary_layer_wavenumbers(freq: float = 100.0, air: dict = AIR_20C):
    """[k, k_v, k_h] (complex) at frequency `freq` in Hz."""
    w = 2.0 * np.pi * freq
    k = w / air["c"]
    kv = np.sqrt(1j * w * air["rho"] / air["mu"])
    kh = np.sqrt(1j * w / air["alpha"])
    return [complex(k), complex(kv), complex(kh)]
