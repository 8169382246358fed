"""Visco-thermal system, host parts (no GPU): the air properties and constants
and the tangential derivative matrices of libbiegpu against the oracle, and the
oracle against the identities the reference's own tests check."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
from biegpu import _capi
from biegpu import mesh as bm
from oracle import lossy as olossy


def test_oracle_air_at_20C_50RH():
    # properties of humid air at 101325 Pa, 20 C, 50 % RH (water vapour raises
    # c0 by ~0.8 m/s over dry air's 343.2 m/s and lowers the density)
    rho, c0, cf, gamma, eta, alfa, Cp, Cv, landa, beta = olossy.ambient_to_properties(1000.0)
    assert abs(c0 - 343.99) < 0.05
    assert abs(rho - 1.1992) < 0.001
    assert abs(gamma - 1.401) < 0.002
    assert abs(eta - 1.81e-5) < 0.01e-5
    assert abs(Cp - 1012.0) < 5.0
    assert abs(landa - 0.0252) < 0.0005
    assert cf > c0 and 0.0 < alfa < 0.01
    assert abs(beta - rho * (Cp - Cv)) < 1e-12 * beta


@pytest.mark.parametrize("S", [1.0, -1.0])
def test_oracle_constant_identities(S):
    # test/3d/losses_test.jl:44-45 (mu_a, mu_h), and k_v^2 = S i kp / lvp
    rho, c, kp, ka, kh, kv, tau_a, tau_h, phi_a, phi_h, eta, mu = olossy.visco_thermal_constants(100.0, S=S)
    mu_a = phi_a - tau_a * phi_h / tau_h
    mu_h = tau_a * phi_h / tau_h
    assert abs(mu_a + mu_h - phi_a) < 1e-14 * abs(phi_a)
    assert abs(kv**2 - S * 1j * kp * rho * c / mu) < 1e-12 * abs(kv) ** 2
    assert abs(ka - kp) < 1e-3 * kp          # acoustic wavenumber close to omega / c
    assert abs(kh.real) > 100 * kp and abs(kv.real) > 100 * kp


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.mark.parametrize("freq,S,air", [(100.0, 1.0, None), (1000.0, -1.0, None), (5000.0, 1.0, (90000.0, 35.0, 80.0)),
                                        (20.0, 1.0, (101325.0, -10.0, 0.0))])
def test_constants_match_oracle(freq, S, air):
    pa, t, Hr = air if air else (101325.0, 20.0, 50.0)
    got = biegpu.visco_thermal_constants(freq, S=S, pa=pa, t=t, Hr=Hr)
    ref = olossy.visco_thermal_constants(freq, S=S, pa=pa, t=t, Hr=Hr)
    for g, r in zip(got, ref):
        assert rel(g, r) <= 1e-13
    gp = biegpu.ambient_to_properties(freq, pa, t, Hr)
    rp = olossy.ambient_to_properties(freq, pa, t, Hr)
    for g, r in zip(gp, rp):
        assert rel(g, r) <= 1e-13


def test_constants_argument_errors():
    L = _capi.lib()
    k = _capi.LossyConstants()
    import ctypes as C
    assert L.bie_visco_thermal_constants(-1.0, 1.0, 101325.0, 20.0, 50.0, C.byref(k)) == _capi.BIE_ERR_INVALID
    assert L.bie_visco_thermal_constants(100.0, 0.0, 101325.0, 20.0, 50.0, C.byref(k)) == _capi.BIE_ERR_INVALID
    assert L.bie_visco_thermal_constants(100.0, 1.0, -5.0, 20.0, 50.0, C.byref(k)) == _capi.BIE_ERR_INVALID
    assert L.bie_visco_thermal_constants(100.0, 1.0, 101325.0, 20.0, 50.0, None) == _capi.BIE_ERR_INVALID


MESHES = {
    "linear": lambda: bm.icosphere(3),
    "quadratic": lambda: bm.icosphere(2, geometry="quadratic"),
    "quadratic_geometry_linear_physics": lambda: bm.icosphere(2, geometry="quadratic", physics="linear"),
    "ellipsoid": lambda: bm.ellipsoid(3),
}


@pytest.mark.parametrize("name", list(MESHES))
def test_tangential_derivatives_match_oracle(name):
    mesh = MESHES[name]()
    D = biegpu.tangential_derivatives(mesh)
    R = olossy.tangential_derivatives(mesh)
    for a, b in zip(D, R):
        A, B = a.toarray(), b.toarray()
        assert np.abs(A - B).max() <= 1e-12 * np.abs(B).max()
    # test/3d/meshing_test.jl:35-39: constant pressure has zero derivatives
    one = np.ones(mesh.n_sources)
    for a in D:
        assert np.sum(np.abs(a @ one)) / mesh.n_sources <= 1e-13


def test_tangential_derivatives_are_tangential_on_a_sphere():
    # on a sphere of linear elements the averaged nodal gradient of x is close
    # to e_x minus its normal part (the averaging error is O(h))
    mesh = bm.icosphere(8)
    Dx, Dy, Dz = biegpu.tangential_derivatives(mesh)
    x = mesh.sources[0]
    g = np.stack([Dx @ x, Dy @ x, Dz @ x])
    n = -mesh.normals   # the mesh's normals point into the sphere
    expect = np.array([1.0, 0.0, 0.0])[:, None] - n * n[0][None, :]
    assert np.abs(g - expect).max() < 0.05


def test_tangential_derivatives_bad_mesh():
    import ctypes as C
    mesh = bm.icosphere(2)
    d, keep = biegpu.lossy._mesh_desc(mesh)
    keep[1][0, 0] = 0   # 1-based index out of range
    nnz = C.c_int64()
    assert _capi.lib().bie_tangential_derivatives(C.byref(d), C.byref(nnz), None, None, None, None, None) \
        == _capi.BIE_ERR_INVALID
