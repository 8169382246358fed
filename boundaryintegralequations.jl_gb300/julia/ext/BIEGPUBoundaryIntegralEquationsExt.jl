"""
Methods of BoundaryIntegralEquations' own functions for the GPU backend, so
that a reference script switches to libbiegpu by adding `GPU()` after the
arguments it already passes:

    F, G, C = assemble_parallel!(mesh, k, mesh.sources, GPU(); n=2, m=2)
    Ff = FMMFOperator(mesh, k, GPU(); n_gauss=3, nearfield=true, offset=0.2, depth=1)
    Gf = FMMGOperator(mesh, k, GPU(); n_gauss=3, nearfield=true, offset=0.2, depth=1)

Keyword arguments and their defaults are the reference's
(src/3d/assembly_collocation.jl:259-268, src/3d/fast_multipole_method.jl:
473-488); `precision` (:fp64, :df64 or :mixed) is the one addition.  The
results have the reference's types: `Matrix{ComplexF64}` / `Vector{ComplexF64}`
for the assembly (sparse matrices with `sparse=true`), `LinearMap`s for the
operators, which compose with `Diagonal(1 .- C)` and `gmres` unchanged.
"""
module BIEGPUBoundaryIntegralEquationsExt

using BIEGPU
import BoundaryIntegralEquations
const BIE = BoundaryIntegralEquations

function BIE.assemble_parallel!(mesh::BIE.Mesh3d, k, in_sources, ::BIEGPU.GPU; fOn=true, gOn=true, cOn=true,
                                sparse=false, m=4, n=4, progress=true, depth=2, offset=nothing,
                                precision=:fp64)
    if sparse
        return BIEGPU.sparse_assemble_parallel_gpu!(mesh, k; depth=depth, offset=offset, fOn=fOn, gOn=gOn)
    end
    return BIEGPU.assemble_parallel_gpu!(mesh, k, in_sources; fOn=fOn, gOn=gOn, cOn=cOn, m=m, n=n,
                                         progress=progress, precision=precision)
end

BIE.FMMFOperator(mesh::BIE.Mesh3d, k, ::BIEGPU.GPU; n_gauss=3, tol=1e-6, nearfield=true, offset=0.2, depth=1,
                 precision=:mixed) =
    BIEGPU.FastFOperator(mesh, k; tol=tol, n_gauss=n_gauss, nearfield=nearfield, offset=offset, depth=depth,
                         precision=precision)

BIE.FMMGOperator(mesh::BIE.Mesh3d, k, ::BIEGPU.GPU; n_gauss=3, tol=1e-6, nearfield=true, offset=0.2, depth=1,
                 precision=:mixed) =
    BIEGPU.FastGOperator(mesh, k; tol=tol, n_gauss=n_gauss, nearfield=nearfield, offset=offset, depth=depth,
                         precision=precision)

end # module
