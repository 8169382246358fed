"""ORACLE - test infrastructure only (never imported by the product path).

CPU restatement of the reference's visco-thermal ("lossy") system:

  * ``ambient_to_properties``   - src/utils/ambient_to_properties.jl:1-134
    (Rasmussen, "Calculation methods for the physical properties of air used
    in the calibration of microphones", DTU report PL-11b, 1997, annex A);
  * ``visco_thermal_constants`` - src/utils/lossy_constants.jl:1-34;
  * ``tangential_derivatives``  - src/3d/interpolation_function_derivatives.jl:
    10-18, 36-118 (Dx, Dy, Dz of the physics interpolation, averaged over the
    elements of each node);
  * ``LossyOuter``              - LossyGlobalOuter of src/3d/LossyGlobalMatrix.jl:
    76-172 (constructor), 179-197 (product) and 241-253 (_full1), with the
    nested gmres calls replaced by direct solves (the reference's gmres converge
    to the same vectors within their tolerance).

Parity pins: the reference's own tests of this part check identities, which
tests/test_lossy_host.py reproduces (mu_a = phi_a - phi_h tau_a / tau_h,
test/3d/losses_test.jl:44-45; D 1 = 0 for constant pressure,
test/3d/meshing_test.jl:35-39; the solved-mode identities of
test/3d/losses_test.jl:46-58); the air properties are pinned to the published
values of humid air at 20 C, 50 % RH, 101325 Pa (c0 = 343.99 m/s,
rho = 1.1992 kg/m^3, gamma = 1.401, mu = 1.81e-5 Pa s).
"""
from __future__ import annotations

import math

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp
import scipy.sparse.linalg as spla

# Rasmussen's table A.1, one coefficient list per property (the column order
# of the reference's matrix `aa`).
_ENHANCE = (1.00062, 3.14e-8, 5.6e-7)
_Z = (1.58123e-6, -2.9331e-8, 1.1043e-10, 5.707e-6, -2.051e-8, 1.9898e-4, -2.376e-6, 1.83e-11, -0.765e-8)
_C0 = (331.5024, 0.603055, -0.000528, 51.471935, 0.1495874, -0.000782, -1.82e-7, 3.73e-8, -2.93e-10,
       -85.20931, -0.228525, 5.91e-5, -2.835149, -2.15e-13, 29.179762, 0.000486)
_GAMMA = (1.400822, -1.75e-5, -1.73e-7, -0.0873629, -0.0001665, -3.26e-6, 2.047e-8, -1.26e-10, 5.939e-14,
          -0.1199717, -0.0008693, 1.979e-6, -0.01104, -3.478e-16, 0.0450616, 1.82e-6)
_VISC = (84.986, 7.0, 113.157, -1.0, -3.7501e-3, -100.015)
_COND = (60.054, 1.846, 2.06e-6)
_CP = (0.251625, -9.2525e-5, 2.1334e-7, -1.0043e-10, 0.12477, -2.283e-5, 1.267e-7, 0.01116, 4.61e-6, 1.74e-8)


def _table_poly16(a, t, xw, ps, xc):
    """The 16-term form shared by the speed of sound and the ratio of specific heats."""
    return (a[0] + a[1] * t + a[2] * t**2 + (a[3] + a[4] * t + a[5] * t**2) * xw
            + (a[6] + a[7] * t + a[8] * t**2) * ps + (a[9] + a[10] * t + a[11] * t**2) * xc
            + a[12] * xw**2 + a[13] * ps**2 + a[14] * xc**2 + a[15] * xw * ps * xc)


def ambient_to_properties(f=1000.0, ps=101325.0, t=20.0, H=50.0):
    """(rho, c0, cf, CpCv, eta, alfa, Cp, Cv, landa, beta), ambient_to_properties.jl:1-134."""
    T0, T20, psr = 273.15, 293.15, 101325.0
    T = T0 + t
    psv = psr * 10.0 ** (4.6151 - 6.8346 * ((T0 + 0.01) / T) ** 1.261)
    fpst = _ENHANCE[0] + _ENHANCE[1] * ps + _ENHANCE[2] * t**2
    xw = H * psv * fpst / (100.0 * ps)
    z = _Z
    Z = (1.0 - ps / T * (z[0] + z[1] * t + z[2] * t**2 + (z[3] + z[4]) * xw + (z[5] + z[6]) * xw**2)
         + (ps / T) ** 2 * (z[7] + z[8] * xw**2))
    xc = 0.0004
    rho = (3.48349 + 1.44 * (xc - 0.0004)) * 1e-3 * ps / (Z * T) * (1.0 - 0.3780 * xw)
    c0 = _table_poly16(_C0, t, xw, ps, xc)
    gamma = _table_poly16(_GAMMA, t, xw, ps, xc)
    v = _VISC
    eta = (v[0] + v[1] * T + (v[2] + v[3] * T) * xw + v[4] * T**2 + v[5] * xw**2) * 1e-8
    # the reference takes the humidity terms of the conductivity from the
    # viscosity coefficients (rows 4 and 5 of column 6); kept for parity
    landa = (_COND[0] + _COND[1] * T + _COND[2] * T**2 + (v[3] + v[4] * T) * xw) * 1e-8
    p = _CP
    Cp = (p[0] + p[1] * T + p[2] * T**2 + p[3] * T**3 + (p[4] + p[5] * T + p[6] * T**2) * xw
          + (p[7] + p[8] * T + p[9] * T**2) * xw**2)
    frO = ps / psr * (24.0 + 4.04e6 * xw * (0.2 + 1e3 * xw) / (3.91 + 1e3 * xw))
    frN = ps / psr * (T / T20) ** (-0.5) * (9.0 + 28.0e3 * xw * math.exp(-4.170 * ((T / T20) ** (-1.0 / 3.0) - 1.0)))
    a_O = 0.01275 * f**2 * math.exp(-2239.1 / T) / (frO + f**2 / frO) * (T20 / T) ** 2.5
    a_N = 0.1068 * f**2 * math.exp(-3352.0 / T) / (frN + f**2 / frN) * (T20 / T) ** 2.5
    cf = 1.0 / (1.0 / c0 - a_O / (2 * math.pi * frO) - a_N / (2 * math.pi * frN))
    alfa = 18.4e-12 * f**2 * (ps / psr) ** (-1) * (T / T20) ** 0.5 + a_O + a_N
    Cp = Cp * 4.1868 * 1000.0
    landa = landa * 4.1868 * 1000.0
    Cv = Cp / gamma
    beta = rho * (Cp - Cv)
    return rho, c0, cf, gamma, eta, alfa, Cp, Cv, landa, beta


def visco_thermal_constants(freq=1000.0, S=-1.0, pa=101325.0, t=20.0, Hr=50.0):
    """(rho, c, kp, ka, kh, kv, tau_a, tau_h, phi_a, phi_h, eta, mu), lossy_constants.jl:1-34."""
    rho, c, _, cpcv, mu, _, Cp, _, landa, beta = ambient_to_properties(freq, pa, t, Hr)
    eta = 0.6 * mu
    lh = landa / (rho * Cp * c)
    lv = (eta + 4.0 * mu / 3.0) / (rho * c)
    lvp = mu / (rho * c)
    lvh = lv + (cpcv - 1.0) * lh
    lvhp = (cpcv - 1.0) * (lh - lv)
    kp = 2 * math.pi * freq / c
    j = 1j
    ka2 = kp**2 / (1.0 - S * j * kp * lvh - kp**2 * lh * lvhp)
    kh2 = S * j * kp / (lh * (1.0 + S * j * kp * lvhp))
    kv2 = S * j * kp / lvp
    ka, kh, kv = np.sqrt(ka2), np.sqrt(kh2), np.sqrt(kv2)
    tau_a = (cpcv - 1.0) / (beta * cpcv * (1.0 + S * j * lh * ka2 / kp))
    tau_h = (cpcv - 1.0) / (beta * cpcv * (1.0 + S * j * lh * kh2 / kp))
    phi_a = -S * j / (rho * 2.0 * math.pi * freq * (1.0 + S * j * lv * ka2 / kp))
    phi_h = -S * j / (rho * 2.0 * math.pi * freq * (1.0 + S * j * lv * kh2 / kp))
    return (rho, c, kp, complex(ka), complex(kh), complex(kv), complex(tau_a), complex(tau_h),
            complex(phi_a), complex(phi_h), eta, mu)


# nodal (u, v) of the element nodes and the shape-function derivatives there
_NODAL_UV = {"linear": ((0.0, 0.0), (1.0, 0.0), (0.0, 1.0)),
             "quadratic": ((0.0, 0.0), (1.0, 0.0), (0.0, 1.0), (0.5, 0.0), (0.5, 0.5), (0.0, 0.5))}


def _dshape(kind, u, v):
    """dN/du, dN/dv of the 3- or 6-node triangle (surface_functions.jl:191-236, 322-366)."""
    if kind == "linear":
        return np.array([-1.0, 1.0, 0.0]), np.array([-1.0, 0.0, 1.0])
    l = 1.0 - u - v
    du = np.array([1.0 - 4.0 * l, 4.0 * u - 1.0, 0.0, 4.0 * (l - u), 4.0 * v, -4.0 * v])
    dv = np.array([1.0 - 4.0 * l, 0.0, 4.0 * v - 1.0, -4.0 * u, 4.0 * u, 4.0 * (l - v)])
    return du, dv


def tangential_derivatives(mesh):
    """(Dx, Dy, Dz) as scipy CSR (N x N), interpolation_function_derivatives(mesh)."""
    X = mesh.coordinates
    T = mesh.topology - 1
    P = mesh.physics_topology - 1
    NP, E = P.shape
    N = mesh.n_sources
    count = np.bincount(P.ravel(), minlength=N).astype(np.float64)
    rows, cols, vx, vy, vz = [], [], [], [], []
    for a, (ua, va) in enumerate(_NODAL_UV[mesh.physics_function][:NP]):
        su, sv = _dshape(mesh.shape_function, ua, va)
        pu, pv = _dshape(mesh.physics_function, ua, va)
        L = np.zeros((3, NP))
        L[0], L[1] = pu, pv
        Xe = X[:, T]                                  # 3 x NS x E
        tu = np.einsum("kse,s->ek", Xe, su)           # E x 3
        tv = np.einsum("kse,s->ek", Xe, sv)
        M = np.stack([tu, tv, np.cross(tu, tv)], axis=1)   # E x 3 x 3 (rows)
        Gr = np.linalg.solve(M, np.broadcast_to(L, (E, 3, NP)))   # E x 3 x NP
        row = P[a]
        w = 1.0 / count[row]
        for b in range(NP):
            rows.append(row)
            cols.append(P[b])
            vx.append(Gr[:, 0, b] * w)
            vy.append(Gr[:, 1, b] * w)
            vz.append(Gr[:, 2, b] * w)
    r, c = np.concatenate(rows), np.concatenate(cols)
    mk = lambda v: sp.csr_matrix((np.concatenate(v), (r, c)), shape=(N, N))  # noqa: E731
    return mk(vx), mk(vy), mk(vz)


class LossyOuter:
    """LossyGlobalOuter(mesh, freq; depth, n=m=quad, S=1, exterior) on the CPU
    with dense acoustic matrices (fmm_on = false) or the fast-operator
    algorithm (fmm_on = true, exact far-field sums)."""

    def __init__(self, mesh, freq, depth=1, quad=3, S=1.0, exterior=True, fmm_on=False):
        import oracle
        (self.rho, self.c, self.kp, self.ka, self.kh, self.kv, self.tau_a, self.tau_h, self.phi_a,
         self.phi_h, self.eta, self.mu) = visco_thermal_constants(freq=freq, S=S)
        self.mu_a = self.phi_a - self.tau_a * self.phi_h / self.tau_h
        self.mu_h = self.tau_a * self.phi_h / self.tau_h
        N = mesh.n_sources
        self.n = N
        if fmm_on:
            self.Ga = oracle.fast_operator(mesh, self.ka, "G", n_gauss=quad, offset=0.2, depth=depth)
            self.Ha = oracle.fast_operator(mesh, self.ka, "F", n_gauss=quad, offset=0.2, depth=depth) \
                + 0.5 * np.eye(N)
            C0 = np.full(N, 0.5, dtype=np.complex128)
        else:
            F, G, Cv = oracle.assemble(mesh, self.ka, n=quad, m=quad)
            C0 = Cv if exterior else 1.0 - Cv
            self.Ha = (F if exterior else -F) + np.diag(C0)
            self.Ga = G
        sgn = 1.0 if exterior else -1.0

        def sparse(k):
            rp, cl, Fv, Gv = oracle.nearfield(mesh, k, depth=depth, offset=0.0)
            Fm = sp.csr_matrix((Fv, cl, rp), shape=(N, N))
            Gm = sp.csr_matrix((Gv, cl, rp), shape=(N, N))
            return (sgn * Fm + sp.diags(C0)).tocsc(), Gm.tocsc()

        self.Hh, self.Gh = sparse(self.kh)
        self.Av, self.Bv = sparse(self.kv)
        self.Dx, self.Dy, self.Dz = tangential_derivatives(mesh)
        self.nrm = np.asarray(mesh.normals, dtype=np.float64)
        self._gh = spla.splu(self.Gh)
        self._bv = spla.splu(self.Bv)
        # inner operator R_N = Dr Nd - Nd' Gv^-1 Hv Nd as a dense matrix
        I = np.eye(N)
        self.RN = np.column_stack([self.inner(I[:, j]) for j in range(N)])
        self._rn = sla.lu_factor(self.RN)

    # blocks of the reference (Nd = -[diag nx; diag ny; diag nz])
    def Dc(self, x):
        return [self.Dx @ x, self.Dy @ x, self.Dz @ x]

    def Dr(self, q):
        return self.Dx @ q[0] + self.Dy @ q[1] + self.Dz @ q[2]

    def Nd(self, x):
        return [-self.nrm[0] * x, -self.nrm[1] * x, -self.nrm[2] * x]

    def NdT(self, q):
        return -(self.nrm[0] * q[0] + self.nrm[1] * q[1] + self.nrm[2] * q[2])

    def Gv_solve_Hv(self, q):
        return [self._bv.solve(self.Av @ qc) for qc in q]

    def inner(self, z):
        p = self.Nd(z)
        return self.Dr(p) - self.NdT(self.Gv_solve_Hv(p))

    def inner_solve(self, r):
        return sla.lu_solve(self._rn, r)

    def matvec(self, x):
        x = np.asarray(x, dtype=np.complex128)
        y = -self.phi_a * (self.Ha @ x)
        sh = self._gh.solve(self.Hh @ x)
        q = self.Dc(x)
        r = self.Dr(q) - self.NdT(self.Gv_solve_Hv(q))
        return y + self.Ga @ (self.mu_h * sh + self.mu_a * self.inner_solve(r))

    def rhs(self, v0):
        """Ga gmres(inner, Dr v0 - Nd' gmres(Gv, Hv v0)) of test/3d/losses_test.jl:33
        (v0: list of three N-vectors)."""
        r = self.Dr(v0) - self.NdT(self.Gv_solve_Hv(v0))
        return self.Ga @ self.inner_solve(r)

    def full(self):
        N = self.n
        I = np.eye(N, dtype=np.complex128)
        return np.column_stack([self.matvec(I[:, j]) for j in range(N)])
