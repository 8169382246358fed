"""ORACLE - test infrastructure only (never imported by the product path).

Forward-mode derivative of the far-field objective through the CPU assembly
(the check the adjoint gradient is held to besides finite differences).

The objective is the one of ``oracle.farfield_objective``:
    (F + Diagonal(1 - C) - i rho c k G_Y) p = p_I,
    p_f = p_I(x_f) + (-F_x + i rho c k G_{x,Y}) p,   J = sum |p_f|^2,
with F, G, C the dense collocation assembly of assemble_parallel!
(src/3d/assembly_collocation.jl:213-252, 270-353: rule clustered at the
nearest node, jacobian!'s negated normal src/3d/jacobian.jl:63-87, kernels
greens3d! / freens3d! / freens3dk0! of src/3d/kernels.jl:13-55).  Here the
assembly of 3-node triangles with nodal physics is restated with dual numbers
(value + derivative along one direction of the vertex coordinates, the
collocation points moving with the vertices), vectorised over all (target,
element, quadrature point) triples; the nearest-node rule choice is piecewise
constant and taken from the values.  Derivatives along impedance directions
use the C oracle directly: G_Y is linear in the admittances Y_e = 1 / Z_e.
For small meshes only (memory grows as targets x elements x 12 points).
"""
from __future__ import annotations

import numpy as np

import oracle


class Dual:
    """a + eps b with eps^2 = 0; a, b numpy arrays of one shape (real or complex)."""

    __slots__ = ("v", "d")

    def __init__(self, v, d=None):
        self.v = np.asarray(v)
        self.d = np.zeros_like(self.v) if d is None else np.broadcast_to(np.asarray(d), self.v.shape) * 1

    @staticmethod
    def lift(x):
        return x if isinstance(x, Dual) else Dual(x)

    def __add__(self, o):
        o = Dual.lift(o)
        return Dual(self.v + o.v, self.d + o.d)

    __radd__ = __add__

    def __sub__(self, o):
        o = Dual.lift(o)
        return Dual(self.v - o.v, self.d - o.d)

    def __rsub__(self, o):
        return Dual.lift(o) - self

    def __neg__(self):
        return Dual(-self.v, -self.d)

    def __mul__(self, o):
        o = Dual.lift(o)
        return Dual(self.v * o.v, self.d * o.v + self.v * o.d)

    __rmul__ = __mul__

    def __truediv__(self, o):
        o = Dual.lift(o)
        return Dual(self.v / o.v, (self.d * o.v - self.v * o.d) / (o.v * o.v))

    def __rtruediv__(self, o):
        return Dual.lift(o) / self

    def __getitem__(self, idx):
        return Dual(self.v[idx], self.d[idx])

    def sum(self, axis):
        return Dual(self.v.sum(axis=axis), self.d.sum(axis=axis))


def dsqrt(x: Dual) -> Dual:
    s = np.sqrt(x.v)
    return Dual(s, x.d / (2.0 * s))


def dexp(x: Dual) -> Dual:
    e = np.exp(x.v)
    return Dual(e, e * x.d)


def _cross(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def assemble_linear_dual(mesh, k, Vdir, targets=None, n=2, m=2, g_weight=None):
    """(F, G, C) as Dual arrays (M x N, M x N, M) for 3-node triangles with
    nodal physics on the vertices.  The vertices move along ``Vdir`` (3 x Nc);
    targets=None means the collocation points (= the vertices, moving with
    them), else fixed field points (3 x M)."""
    if mesh.shape_function != "linear" or mesh.physics_function != "linear":
        raise ValueError("linear triangles with nodal physics only")
    k = complex(k)
    Xc = mesh.coordinates
    T = mesh.topology - 1                  # 3 x E
    P = mesh.physics_topology - 1          # 3 x E (into sources)
    N, E = mesh.n_sources, T.shape[1]
    if not np.array_equal(mesh.sources, Xc):
        raise ValueError("the collocation points must be the vertices")
    Vd = np.asarray(Vdir, dtype=np.float64)
    if targets is None:
        tv, td = Xc, Vd
    else:
        tv = np.asarray(targets, dtype=np.float64)
        td = np.zeros_like(tv)
    M = tv.shape[1]
    # element vertices as duals, 3 coordinates x E
    Xe = [Dual(Xc[:, T[a]], Vd[:, T[a]]) for a in range(3)]
    tang = [Xe[1][c] - Xe[0][c] for c in range(3)]
    sang = [Xe[2][c] - Xe[0][c] for c in range(3)]
    nn = _cross(tang, sang)
    jac = dsqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2])
    nrm = [-(nn[c] / jac) for c in range(3)]              # jacobian!'s negated normal
    # nearest node of every (target, element) pair (values only; first wins)
    src = mesh.sources[:, P]                              # 3 x 3 x E (coord, node, element)
    d2 = np.sum((src[:, :, None, :] - tv[:, None, :, None]) ** 2, axis=0)   # node x M x E
    choice = np.argmin(d2, axis=0)                        # M x E (first minimum wins)
    t = [Dual(tv[c][:, None, None], td[c][:, None, None]) for c in range(3)]   # M x 1 x 1
    Fv = np.zeros((M, N), dtype=np.complex128)
    Fd = np.zeros_like(Fv)
    Gv = np.zeros_like(Fv)
    Gd = np.zeros_like(Fv)
    Cv = np.zeros(M)
    Cd = np.zeros(M)
    gw = None if g_weight is None else np.asarray(g_weight, dtype=np.complex128)
    four_pi = 4.0 * np.pi
    for r in range(3):
        u, v, w = oracle.rule(n, m, r + 1)
        mask = (choice == r)[:, :, None]                  # M x E x 1
        if not mask.any():
            continue
        Nq = np.stack([1.0 - u - v, u, v])                # node x Q
        xq = [sum(Xe[a][c][None, :, None] * Nq[a][None, None, :] for a in range(3)) for c in range(3)]  # 1 x E x Q
        jw = jac[None, :, None] * w[None, None, :]
        D = [xq[c] - t[c] for c in range(3)]              # M x E x Q
        rr = dsqrt(D[0] * D[0] + D[1] * D[1] + D[2] * D[2])
        dn = D[0] * nrm[0][None, :, None] + D[1] * nrm[1][None, :, None] + D[2] * nrm[2][None, :, None]
        ek = dexp(1j * k * rr)
        r3 = rr * rr * rr
        g = ek / (four_pi * rr) * jw
        f = ek * (1j * k * rr - 1.0) * dn / (four_pi * r3) * jw
        cq = -dn / (four_pi * r3) * jw
        Cv += np.sum(np.where(mask, cq.v, 0.0), axis=(1, 2))
        Cd += np.sum(np.where(mask, cq.d, 0.0), axis=(1, 2))
        for a in range(3):
            ga = Dual(np.where(mask, g.v, 0.0) * Nq[a], np.where(mask, g.d, 0.0) * Nq[a]).sum(axis=2)   # M x E
            fa = Dual(np.where(mask, f.v, 0.0) * Nq[a], np.where(mask, f.d, 0.0) * Nq[a]).sum(axis=2)
            if gw is not None:
                ga = ga * gw[None, :]
            cols = P[a]
            for arr, val in ((Gv, ga.v), (Gd, ga.d), (Fv, fa.v), (Fd, fa.d)):
                np.add.at(arr.T, cols, val.T)
    return Dual(Fv, Fd), Dual(Gv, Gd), Dual(Cv, Cd)


def farfield_directional_derivative(mesh, k, Z, field_points, Vdir=None, dZ=None, rho_c=1.21 * 343.0,
                                    direction=(0.0, 0.0, 1.0), n=2, m=2):
    """(J, dJ): the objective and its derivative along vertex displacements
    ``Vdir`` (3 x Nc) and/or impedance changes ``dZ`` (E complex; the derivative
    is the real directional derivative along Re and Im parts)."""
    k = complex(k)
    d = np.asarray(direction, dtype=np.float64)
    d = d / np.linalg.norm(d)
    Z = np.asarray(Z, dtype=np.complex128)
    Y = 1.0 / Z
    X = np.asarray(field_points, dtype=np.float64)
    Vd = np.zeros_like(mesh.coordinates) if Vdir is None else np.asarray(Vdir, dtype=np.float64)
    F, G, C = assemble_linear_dual(mesh, k, Vd, n=n, m=m, g_weight=Y)
    Fx, Gx, _ = assemble_linear_dual(mesh, k, Vd, targets=X, n=n, m=m, g_weight=Y)
    a = 1j * rho_c * k
    Av = F.v + np.diag(1.0 - C.v) - a * G.v
    Ad = F.d - np.diag(C.d) - a * G.d
    Bv = -Fx.v + a * Gx.v
    Bd = -Fx.d + a * Gx.d
    src = mesh.sources
    pIv = np.exp(-1j * k * (d @ src))
    pId = -1j * k * (d @ Vd) * pIv
    if dZ is not None:
        dY = -np.asarray(dZ, dtype=np.complex128) / (Z * Z)
        _, GdY, _ = oracle.assemble(mesh, k, n=n, m=m, fOn=False, cOn=False, g_weight=np.ascontiguousarray(dY))
        _, GxdY, _ = oracle.assemble(mesh, k, targets=X, n=n, m=m, fOn=False, cOn=False,
                                     g_weight=np.ascontiguousarray(dY))
        Ad = Ad - a * GdY
        Bd = Bd + a * GxdY
    p = np.linalg.solve(Av, pIv)
    dp = np.linalg.solve(Av, pId - Ad @ p)
    pf = np.exp(-1j * k * (d @ X)) + Bv @ p
    dpf = Bd @ p + Bv @ dp
    return float(np.sum(np.abs(pf) ** 2)), float(2.0 * np.real(np.vdot(pf, dpf)))
