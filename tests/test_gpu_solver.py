"""Matrix-free operator products (K3) and device GMRES (K5) against the CPU
oracle and the analytic sphere solutions.

Tolerances: FP64 matrix-free products match the dense oracle product to a
relative 2-norm error <= 1e-12; mixed products <= 1e-6; GMRES solutions match
a dense direct solve to <= 1e-6 relative (IterativeSolvers' default reltol is
sqrt(eps) on the residual)."""
from __future__ import annotations

import numpy as np
import pytest

import biegpu
import oracle
import oracle.analytic as an
from biegpu import Diagonal, GPUFOperator, GPUGOperator, I, gmres
from biegpu import mesh as bm

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def rand_c(n, seed):
    r = np.random.default_rng(seed)
    return r.normal(size=n) + 1j * r.normal(size=n)


@pytest.mark.parametrize("geo,f,k", [("linear", 6, 3.0), ("quadratic", 4, 5.0), ("linear", 5, 2.0 + 0.5j)])
def test_matvec_matches_dense_oracle(geo, f, k):
    mesh = bm.icosphere(f, geometry=geo)
    F, G, _ = oracle.assemble(mesh, k, n=2, m=2, cOn=False)
    x, v = rand_c(mesh.n_sources, 1), rand_c(mesh.n_sources, 2)
    for prec, tol in (("fp64", 1e-12), ("mixed", 1e-6)):
        Ff = GPUFOperator(mesh, k, precision=prec)
        Gf = GPUGOperator(mesh, k, precision=prec)
        assert rel(Ff @ x, F @ x) <= tol
        assert rel(Gf @ v, G @ v) <= tol


def test_matvec_field_points():
    mesh = bm.icosphere(6)
    z = np.linspace(0.1, 0.9, 20)
    X = np.vstack([0 * z, 0 * z, z])
    Fp, Gp, _ = oracle.assemble(mesh, 1.5, targets=X, n=2, m=2, cOn=False)
    p = rand_c(mesh.n_sources, 3)
    for prec, tol in (("fp64", 1e-12), ("mixed", 1e-6)):
        Ff = GPUFOperator(mesh, 1.5, precision=prec)
        assert rel(Ff.evaluate_targets(p, X), Fp @ p) <= tol
        Gf = GPUGOperator(mesh, 1.5, precision=prec)
        assert rel(Gf.evaluate_targets(p, X), Gp @ p) <= tol


def test_gmres_dense_exterior_system():
    # test/3d/assembly_test.jl:37-38 pattern: (Fp + Diagonal(1 - Cp)) p = pI
    mesh = bm.icosphere(6, geometry="quadratic")
    k = 2.0
    Fp, _, Cp = biegpu.assemble_parallel(mesh, k, mesh.sources, n=2, m=2, gOn=False)
    pI = an.incoming_wave([np.pi / 2, 0.0], 1.0, mesh.sources, k)
    ctx = biegpu.get_context(mesh, n=2, m=2)
    x, res = gmres(Fp + Diagonal(1.0 - Cp), pI, ctx=ctx, log=True)
    xd = np.linalg.solve(Fp + np.diag(1.0 - Cp), pI)
    assert res.converged
    assert res.relres <= 1.5e-8
    assert rel(x, xd) <= 1e-6


def test_gmres_refinement_dense():
    mesh = bm.icosphere(6, geometry="quadratic")
    k = 3.0
    Fp, _, Cp = biegpu.assemble_parallel(mesh, k, mesh.sources, n=2, m=2, gOn=False)
    A = Fp + np.diag(1.0 - Cp)
    b = rand_c(mesh.n_sources, 5)
    ctx = biegpu.get_context(mesh, n=2, m=2)
    x, res = gmres(Fp + Diagonal(1.0 - Cp), b, ctx=ctx, refine=True, log=True)
    assert res.converged and res.refinements >= 1
    assert rel(x, np.linalg.solve(A, b)) <= 1e-6


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gmres_matrix_free_interior(prec):
    # examples/3d_pulsating_sphere.jl:46-50: Hf = Diagonal(1 - C) - Ff, b = Gf * vs
    mesh = bm.icosphere(5, geometry="quadratic")
    k, Z0 = 1.0, 1.21 * 343.0
    F, G, C = oracle.assemble(mesh, k, n=2, m=2)
    vs = 1j * Z0 * k * np.ones(mesh.n_sources)
    p_dense = np.linalg.solve(np.diag(1.0 - C) - F, G @ vs)
    Ff = GPUFOperator(mesh, k, precision=prec)
    Gf = GPUGOperator(mesh, k, precision=prec)
    bf = Gf @ vs
    x, res = gmres(Diagonal(1.0 - C) - Ff, bf, log=True)
    assert res.converged
    assert rel(x, p_dense) <= (1e-7 if prec == "fp64" else 2e-6)


def test_rigid_sphere_gpu_pipeline_vs_analytic():
    """Rigid-sphere scattering with the GPU assembly + GPU GMRES on a P2
    icosphere, against the analytic series (assembly_test.jl's check)."""
    mesh = bm.icosphere(8, geometry="quadratic")
    k = 2 * np.pi * 100 / 340
    Fp, _, Cp = biegpu.assemble_parallel(mesh, k, mesh.sources, gOn=False, precision="mixed")
    pI = an.incoming_wave([np.pi / 2, 0.0], 1.0, mesh.sources, k)
    x = gmres(Fp + Diagonal(1.0 - Cp), pI, ctx=biegpu.get_context(mesh))
    theta = np.arccos(np.clip(mesh.sources[0], -1, 1))
    pa, _ = an.plane_wave_scattering_sphere(k, 1.0, 1.0, theta, 1e-6)
    assert rel(x, pa) <= 2.8e-5 * 10   # quadratic/geometry row of the reference table, coarser mesh


def test_pulsating_sphere_full_size_matrix_free():
    """Pulsating-sphere workload (f=32, 10242 nodes): matrix-free mixed
    operators + GPU GMRES + field evaluation vs the analytic interior pressure."""
    mesh = bm.icosphere(32)
    k, Z0 = 2 * np.pi * 200 / 343, 1.21 * 343.0
    _, _, C = biegpu.assemble_parallel(mesh, k, mesh.sources, n=2, m=2, fOn=False, gOn=False)
    Ff = GPUFOperator(mesh, k, precision="mixed")
    Gf = GPUGOperator(mesh, k, precision="mixed")
    vs = 1j * Z0 * k * np.ones(mesh.n_sources)
    p, res = gmres(Diagonal(1.0 - C) - Ff, Gf @ vs, log=True)
    assert res.converged
    z = np.linspace(0.1, 0.9, 20)
    X = np.vstack([0 * z, 0 * z, z])
    pf = Ff.evaluate_targets(p, X) + Gf.evaluate_targets(vs, X)
    pa = an.pulsating_sphere_interior(k, 1.0, Z0, 1.0, z)
    assert rel(pf, pa) <= 0.1    # flat-facet geometry error, O(h) (0.14 at f=20 with the oracle)


def _torch_dev():
    import torch
    return torch, torch.device("cuda:0")


@pytest.mark.parametrize("refine,prec", [(False, "fp64"), (True, "fp64"), (False, "mixed")])
def test_gmres_host_entry_matches_device_entry_dense(refine, prec):
    """bie_gmres (host buffers: numpy in, numpy out) against bie_gmres_device
    (CUDA tensors) on the same dense system: same iterate sequence, so the
    solutions agree to rounding and the iteration counts match."""
    torch, dev = _torch_dev()
    mesh = bm.icosphere(5, geometry="quadratic")
    Fp, _, Cp = biegpu.assemble_parallel(mesh, 2.5, mesh.sources, n=2, m=2, gOn=False)
    b = rand_c(mesh.n_sources, 8)
    ctx = biegpu.get_context(mesh, n=2, m=2)
    xh, rh = gmres(Fp + Diagonal(1.0 - Cp), b, ctx=ctx, refine=refine, precision=prec, log=True)
    Ad = torch.as_tensor(np.asfortranarray(Fp).T.copy(), device=dev)
    xd, rd = gmres(Ad + Diagonal(torch.as_tensor(1.0 - Cp, device=dev)), torch.as_tensor(b, device=dev),
                   ctx=ctx, refine=refine, precision=prec, log=True)
    assert isinstance(xh, np.ndarray)
    assert rh.converged and rd.converged
    assert abs(rh.iterations - rd.iterations) <= 1
    assert rel(xh, xd.cpu().numpy()) <= (1e-12 if prec == "fp64" and not refine else 1e-6)
    assert rel(xh, np.linalg.solve(Fp + np.diag(1.0 - Cp), b)) <= 1e-6


def test_gmres_host_entry_given_a32_and_start():
    """A caller-supplied complex64 matrix and a non-zero start vector through
    the host entry: a start at the solution converges in no more than one
    Arnoldi step."""
    mesh = bm.icosphere(4, geometry="quadratic")
    Fp, _, Cp = biegpu.assemble_parallel(mesh, 1.5, mesh.sources, n=2, m=2, gOn=False)
    A = Fp + np.diag(1.0 - Cp)
    b = rand_c(mesh.n_sources, 9)
    ctx = biegpu.get_context(mesh, n=2, m=2)
    x, res = gmres(Fp + Diagonal(1.0 - Cp), b, ctx=ctx, refine=True, A32=np.asfortranarray(Fp, np.complex64),
                   log=True)
    assert res.converged and rel(x, np.linalg.solve(A, b)) <= 1e-6
    xs = np.linalg.solve(A, b)
    x2, res2 = gmres(Fp + Diagonal(1.0 - Cp), b, ctx=ctx, x0=xs, log=True)
    assert res2.converged and res2.iterations <= 1
    assert rel(x2, xs) <= 1e-12


def test_gmres_host_entry_matrix_free_and_not_converged():
    mesh = bm.icosphere(5, geometry="quadratic")
    k = 1.0
    _, _, C = oracle.assemble(mesh, k, n=2, m=2, fOn=False, gOn=False)
    Ff = GPUFOperator(mesh, k, precision="fp64")
    b = rand_c(mesh.n_sources, 10)
    x, res = gmres(Diagonal(1.0 - C) - Ff, b, log=True)
    torch, dev = _torch_dev()
    xd, rd = gmres(Diagonal(torch.as_tensor(1.0 - C, device=dev)) - Ff, torch.as_tensor(b, device=dev), log=True)
    assert res.converged and abs(res.iterations - rd.iterations) <= 1
    assert rel(x, xd.cpu().numpy()) <= 1e-12
    # maxiter reached: x is still returned with the info filled, as gmres does
    x3, r3 = gmres(Diagonal(1.0 - C) - Ff, b, maxiter=2, log=True)
    assert not r3.converged and r3.iterations == 2 and np.all(np.isfinite(x3))
