"""
    BIEGPU

Julia glue for libbiegpu.so, the GB300 (sm_103a) collocation-BEM hot path.
It keeps the BoundaryIntegralEquations.jl API for the path:

* `assemble_parallel_gpu!(mesh, k, sources; fOn, gOn, cOn, m, n, precision)`
  returns `(F, G, C)` like `assemble_parallel!`
  (src/3d/assembly_collocation.jl:259-268);
* `GPUFOperator(mesh, k)` / `GPUGOperator(mesh, k)` are `LinearMap`s that can
  replace `FMMFOperator` / `FMMGOperator` (src/3d/fast_multipole_method.jl:
  220-318, 374-488) in `gmres(Diagonal(1 .- C) - Ff, Gf*vs)`.

The library is reached with `ccall`; every array is passed as a pointer to
Julia-owned column-major memory (`GC.@preserve`).  Set `ENV["BIEGPU_LIB"]` to
the path of libbiegpu.so.
"""
module BIEGPU

using LinearAlgebra
using SparseArrays
using LinearMaps
import ChainRulesCore

const libbiegpu = get(ENV, "BIEGPU_LIB", "libbiegpu.so")

const BIE_OK = Cint(0)
const BIE_TRI_LINEAR = Cint(1)
const BIE_TRI_QUADRATIC = Cint(2)
const BIE_F = Cint(1)
const BIE_G = Cint(2)
const BIE_C = Cint(4)
const BIE_PREC_FP64 = Cint(0)
const BIE_PREC_MIXED = Cint(1)

# bie_mesh_desc (include/biegpu.h)
struct MeshDesc
    n_coordinates::Int64
    coordinates::Ptr{Float64}
    n_elements::Int64
    shape_kind::Int32
    physics_kind::Int32
    topology::Ptr{Int64}
    physics_topology::Ptr{Int64}
    n_sources::Int64
    sources::Ptr{Float64}
    quad_n::Int32
    quad_m::Int32
    physics_beta::Float64
end

"""
    GPU()

Backend tag of the drop-in methods: with BoundaryIntegralEquations loaded, the
package extension BIEGPUBoundaryIntegralEquationsExt adds
`assemble_parallel!(mesh, k, sources, GPU(); kwargs...)`,
`FMMFOperator(mesh, k, GPU(); kwargs...)` and `FMMGOperator(mesh, k, GPU(); kwargs...)`
to the reference's own functions, with the reference's keyword arguments.
"""
struct GPU end

struct BIEError <: Exception
    code::Cint
    msg::String
end
Base.showerror(io::IO, e::BIEError) = print(io, "libbiegpu error ", e.code, ": ", e.msg)

function check(status::Cint)
    status == BIE_OK && return nothing
    msg = unsafe_string(ccall((:bie_last_error, libbiegpu), Cstring, ()))
    throw(BIEError(status, msg))
end

element_kind(n_nodes::Integer) = n_nodes == 3 ? BIE_TRI_LINEAR :
                                 n_nodes == 6 ? BIE_TRI_QUADRATIC :
                                 throw(ArgumentError("only 3- and 6-node triangles are supported"))

# physics kind and node offset of `mesh.physics_function`: the discontinuous
# triangles (src/3d/SurfaceFunction.jl:81-105) by type name, else by node count
function physics_kind(pf, n_nodes::Integer)
    name = nameof(typeof(pf))
    name === :DiscontinuousTriangularConstant && return (Int32(3), 0.0)
    name === :DiscontinuousTriangularLinear && return (Int32(4), Float64(pf.beta))
    name === :DiscontinuousTriangularQuadratic && return (Int32(5), Float64(pf.beta))
    return (element_kind(n_nodes), 0.0)
end

# bie_rule_table (include/biegpu.h)
struct RuleTable
    n_points::Int64
    u::Ptr{Float64}
    v::Ptr{Float64}
    w::Ptr{Float64}
end

"""
    Context(mesh; n=4, m=4, device=0, rules=nothing)

Uploads the mesh (coordinates, topology, sources, physics topology) and builds
the clustered quadrature rules on the device.  One context per (mesh, n, m).
`rules`, when given, is a vector of `(u, v, w)` tuples, one per element node
that can be the nearest to a collocation point (3 for linear geometry, the
physics nodes per element for quadratic geometry); they replace the rules
built from (n, m) (`bie_ctx_create_rules`).  `reference_rules` collects them
from the shape functions of the reference's own `create_rotated_element`.
"""
mutable struct Context
    handle::Ptr{Cvoid}
    n_sources::Int
    function Context(mesh; n=4, m=4, device=0, rules=nothing)
        coords = Matrix{Float64}(mesh.coordinates)
        topo = Matrix{Int64}(mesh.topology)
        ptopo = Matrix{Int64}(mesh.physics_topology)
        src = Matrix{Float64}(mesh.sources)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        pk, pb = physics_kind(mesh.physics_function, size(ptopo, 1))
        GC.@preserve coords topo ptopo src begin
            desc = Ref(MeshDesc(size(coords, 2), pointer(coords), size(topo, 2),
                                element_kind(size(topo, 1)), pk,
                                pointer(topo), pointer(ptopo), size(src, 2), pointer(src),
                                Int32(n), Int32(m), pb))
            if rules === nothing
                check(ccall((:bie_ctx_create, libbiegpu), Cint,
                            (Ref{Ptr{Cvoid}}, Ref{MeshDesc}, Cint), h, desc, device))
            else
                keep = [(Vector{Float64}(u), Vector{Float64}(v), Vector{Float64}(w)) for (u, v, w) in rules]
                GC.@preserve keep begin
                    tabs = [RuleTable(length(t[3]), pointer(t[1]), pointer(t[2]), pointer(t[3])) for t in keep]
                    check(ccall((:bie_ctx_create_rules, libbiegpu), Cint,
                                (Ref{Ptr{Cvoid}}, Ref{MeshDesc}, Ptr{RuleTable}, Cint, Cint),
                                h, desc, tabs, length(tabs), device))
                end
            end
        end
        ctx = new(h[], size(src, 2))
        finalizer(c -> ccall((:bie_ctx_destroy, libbiegpu), Cint, (Ptr{Cvoid},), c.handle), ctx)
        return ctx
    end
end

"""
    reference_rules(create_rotated_element, rotated_midpoint_triangular_quadpoints,
                    shape_function, n, m, n_rules)

The reference's own clustered rules as `(u, v, w)` tuples for
`Context(mesh; rules=...)`: `create_rotated_element(shape_function, n, m, node)`
for the corners (src/3d/assembly_collocation.jl:122-136, 287-289, 372-374) and
`rotated_midpoint_triangular_quadpoints(n, m, node)` for the edge midpoints
4-6 of quadratic elements (:385-387).  Pass the reference's functions.
"""
function reference_rules(create_rotated_element, rotated_midpoint_triangular_quadpoints,
                         shape_function, n, m, n_rules)
    map(1:n_rules) do r
        if r <= 3
            e = create_rotated_element(shape_function, n, m, r)
            (copy(e.gauss_u), copy(e.gauss_v), copy(e.weights))
        else
            x, y, w = rotated_midpoint_triangular_quadpoints(n, m, r)
            (Vector{Float64}(x), Vector{Float64}(y), Vector{Float64}(w))
        end
    end
end

# :df64 (assembly only): FP64-grade results from double-float arithmetic on
# the FP32 pipes (BIE_PREC_DF64)
precision_code(p::Symbol) = p === :fp64 ? BIE_PREC_FP64 : p === :mixed ? BIE_PREC_MIXED :
                            p === :df64 ? Cint(6) :
                            throw(ArgumentError("precision must be :fp64, :mixed or :df64"))

"""
    assemble_parallel_gpu!(mesh, k, sources; fOn=true, gOn=true, cOn=true, m=4, n=4,
                           precision=:fp64, ctx=Context(mesh; n=n, m=m))

GPU drop-in for `assemble_parallel!` (dense collocation assembly): returns
`(F, G, C)` as `Matrix{ComplexF64}` (length(sources) x N) and `Vector{ComplexF64}`.
"""
function assemble_parallel_gpu!(mesh, k, sources; fOn=true, gOn=true, cOn=true, m=4, n=4,
                                progress=false, precision=:fp64, ctx=nothing)
    c = ctx === nothing ? Context(mesh; n=n, m=m) : ctx
    kk = ComplexF64(k)
    tg = Matrix{Float64}(sources)
    M = size(tg, 2)
    N = c.n_sources
    F = fOn ? Matrix{ComplexF64}(undef, M, N) : Matrix{ComplexF64}(undef, 0, 0)
    G = gOn ? Matrix{ComplexF64}(undef, M, N) : Matrix{ComplexF64}(undef, 0, 0)
    C = cOn ? Vector{ComplexF64}(undef, M) : Vector{ComplexF64}(undef, 0)
    flags = (fOn ? BIE_F : Cint(0)) | (gOn ? BIE_G : Cint(0)) | (cOn ? BIE_C : Cint(0))
    same = sources === mesh.sources
    GC.@preserve tg F G C begin
        check(ccall((:bie_assemble, libbiegpu), Cint,
                    (Ptr{Cvoid}, Float64, Float64, Ptr{Float64}, Int64, Cint, Cint,
                     Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{ComplexF64}),
                    c.handle, real(kk), imag(kk), same ? C_NULL : pointer(tg), M, flags,
                    precision_code(precision), fOn ? pointer(F) : C_NULL,
                    gOn ? pointer(G) : C_NULL, cOn ? pointer(C) : C_NULL))
    end
    return F, G, C
end

# ---------------------------------------------------------------------------
# LinearMaps operators (matrix-free F and G)
# ---------------------------------------------------------------------------
struct GPUOperator{W} <: LinearMaps.LinearMap{ComplexF64}
    ctx::Context
    k::ComplexF64
    precision::Cint
end

const GPUFOperator = GPUOperator{:F}
const GPUGOperator = GPUOperator{:G}

GPUFOperator(mesh, k; n=2, m=2, precision=:mixed, ctx=Context(mesh; n=n, m=m)) =
    GPUOperator{:F}(ctx, ComplexF64(k), precision_code(precision))
GPUGOperator(mesh, k; n=2, m=2, precision=:mixed, ctx=Context(mesh; n=n, m=m)) =
    GPUOperator{:G}(ctx, ComplexF64(k), precision_code(precision))

Base.size(A::GPUOperator) = (A.ctx.n_sources, A.ctx.n_sources)

function LinearMaps._unsafe_mul!(y::AbstractVector, A::GPUOperator{W}, x::AbstractVector) where {W}
    xv = Vector{ComplexF64}(x)
    yv = Vector{ComplexF64}(undef, length(y))
    GC.@preserve xv yv begin
        px = pointer(xv); py = pointer(yv)
        check(ccall((:bie_matvec, libbiegpu), Cint,
                    (Ptr{Cvoid}, Float64, Float64, Ptr{Float64}, Int64, Ptr{ComplexF64},
                     Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{ComplexF64}, Cint),
                    A.ctx.handle, real(A.k), imag(A.k), C_NULL, 0,
                    W === :F ? px : C_NULL, W === :G ? px : C_NULL,
                    W === :F ? py : C_NULL, W === :G ? py : C_NULL, A.precision))
    end
    copyto!(y, yv)
    return y
end

"""
    evaluate_targets(A::GPUOperator, x, targets)

The operator applied at other points (3 x M), like `evaluate_targets` of the
FMM operators (src/3d/fast_multipole_method.jl:326-344, 497-519).
"""
function evaluate_targets(A::GPUOperator{W}, x, targets) where {W}
    xv = Vector{ComplexF64}(x)
    tg = Matrix{Float64}(targets)
    y = Vector{ComplexF64}(undef, size(tg, 2))
    GC.@preserve xv tg y begin
        check(ccall((:bie_matvec, libbiegpu), Cint,
                    (Ptr{Cvoid}, Float64, Float64, Ptr{Float64}, Int64, Ptr{ComplexF64},
                     Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{ComplexF64}, Cint),
                    A.ctx.handle, real(A.k), imag(A.k), pointer(tg), size(tg, 2),
                    W === :F ? pointer(xv) : C_NULL, W === :G ? pointer(xv) : C_NULL,
                    W === :F ? pointer(y) : C_NULL, W === :G ? pointer(y) : C_NULL, A.precision))
    end
    return y
end

"""
    LinearMaps._unsafe_mul!(Y, A::GPUOperator, X::AbstractMatrix)

All columns at once through `bie_matvec_multi` (the matrix method of the FMM
operators, src/3d/fast_multipole_method.jl:249-287, 427-471): matrix strips
generated on the device and multiplied on the tensor cores (`multi_precision`,
default FP16 hi + lo, ~1e-5 relative), or one product per column with
`multi_precision=:none`.
"""
const MULTI_PRECISION = Dict(:fp16 => Cint(2), :bf16 => Cint(3), :fp16_split => Cint(4),
                             :bf16_split => Cint(5))
const multi_precision = Ref(:fp16_split)

function LinearMaps._unsafe_mul!(Y::AbstractMatrix, A::GPUOperator{W}, X::AbstractMatrix) where {W}
    Xm = Matrix{ComplexF64}(X)
    Ym = Matrix{ComplexF64}(undef, size(Y))
    prec = multi_precision[] === :none ? A.precision : MULTI_PRECISION[multi_precision[]]
    GC.@preserve Xm Ym begin
        px = pointer(Xm); py = pointer(Ym)
        check(ccall((:bie_matvec_multi, libbiegpu), Cint,
                    (Ptr{Cvoid}, Float64, Float64, Int64, Ptr{ComplexF64}, Ptr{ComplexF64},
                     Ptr{ComplexF64}, Ptr{ComplexF64}, Cint, Int64),
                    A.ctx.handle, real(A.k), imag(A.k), size(Xm, 2),
                    W === :F ? px : C_NULL, W === :G ? px : C_NULL,
                    W === :F ? py : C_NULL, W === :G ? py : C_NULL, prec, 0))
    end
    copyto!(Y, Ym)
    return Y
end

# Solve of many right-hand sides at once: (F + Diagonal(1 - C)) X = B, which
# the reference solves column by column with gmres (test/3d/assembly_test.jl:37-38)
struct MultisolveOpts
    precision::Cint
    restart::Cint
    maxiter::Cint
    max_refine::Cint
    reltol::Float64
    inner_reltol::Float64
end

struct MultisolveInfo
    passes::Cint
    inner_steps::Cint
    converged::Cint
    tensor_products::Cint
    exact_products::Cint
    reserved::Cint
    max_relres::Float64
    setup_ms::Float64
    tensor_ms::Float64
    exact_ms::Float64
end

"""
    X, info = solve_multi_gpu(ctx, k, B; precision=:fp16_split, reltol=0.0, restart=0, maxiter=0,
                              max_refine=0, inner_reltol=0.0)

`X[:, j] = gmres(Fp + Diagonal(1 .- Cp), B[:, j])` for every column of `B` in
one call (`bie_solve_multi`): lockstep GMRES on tensor-core products of the
mixed-precision F, refined with exact complex64 residuals until each column's
relative residual is at most `reltol` (0: sqrt(eps)).  `info.converged` counts
the columns that met it.
"""
function solve_multi_gpu(ctx::Context, k, B::AbstractMatrix; precision=:fp16_split, reltol=0.0, restart=0,
                         maxiter=0, max_refine=0, inner_reltol=0.0)
    Bm = Matrix{ComplexF64}(B)
    size(Bm, 1) == ctx.n_sources || throw(DimensionMismatch("B needs one row per collocation node"))
    X = Matrix{ComplexF64}(undef, size(Bm))
    opts = Ref(MultisolveOpts(MULTI_PRECISION[precision], restart, maxiter, max_refine, reltol, inner_reltol))
    info = Ref{MultisolveInfo}()
    GC.@preserve Bm X check(ccall((:bie_solve_multi, libbiegpu), Cint,
                                  (Ptr{Cvoid}, Float64, Float64, Int64, Ptr{ComplexF64}, Ptr{ComplexF64},
                                   Ref{MultisolveOpts}, Ref{MultisolveInfo}),
                                  ctx.handle, real(k), imag(k), size(Bm, 2), Bm, X, opts, info))
    return X, info[]
end

# ---------------------------------------------------------------------------
# Near field: sparse_assemble_parallel! (src/3d/assembly_collocation_losses.jl:200-405)
# ---------------------------------------------------------------------------
"""
    sparse_assemble_parallel_gpu!(mesh, k; depth=1, offset=nothing, fOn=true, gOn=true)

Accurate near-field F and G on the connected_sources pattern as
`SparseMatrixCSC{ComplexF64}` (adaptive singular rules; offset = 0 unless given).
"""
function sparse_assemble_parallel_gpu!(mesh, k; depth=1, offset=nothing, fOn=true, gOn=true,
                                       coarse=false, n_gauss=3, ctx=nothing)
    c = ctx === nothing ? Context(mesh; n=2, m=2) : ctx
    N = c.n_sources
    nnz = Ref{Int64}(0)
    check(ccall((:bie_nearfield_pattern, libbiegpu), Cint,
                (Ptr{Cvoid}, Cint, Ref{Int64}, Ptr{Int64}, Ptr{Int64}), c.handle, depth, nnz, C_NULL, C_NULL))
    rowptr = Vector{Int64}(undef, N + 1)
    cols = Vector{Int64}(undef, nnz[])
    check(ccall((:bie_nearfield_pattern, libbiegpu), Cint,
                (Ptr{Cvoid}, Cint, Ref{Int64}, Ptr{Int64}, Ptr{Int64}), c.handle, depth, nnz, rowptr, cols))
    kk = ComplexF64(k)
    Fv = Vector{ComplexF64}(undef, fOn ? nnz[] : 0)
    Gv = Vector{ComplexF64}(undef, gOn ? nnz[] : 0)
    check(ccall((:bie_nearfield_assemble, libbiegpu), Cint,
                (Ptr{Cvoid}, Float64, Float64, Cint, Float64, Cint, Cint, Cint,
                 Ptr{ComplexF64}, Ptr{ComplexF64}),
                c.handle, real(kk), imag(kk), depth, offset === nothing ? 0.0 : Float64(offset),
                coarse ? 1 : 0, n_gauss, (fOn ? BIE_F : 0) | (gOn ? BIE_G : 0),
                fOn ? pointer(Fv) : C_NULL, gOn ? pointer(Gv) : C_NULL))
    # CSR rows -> CSC of the transpose, transposed back
    I = Int[]; J = Int[]
    for i in 1:N, p in rowptr[i]+1:rowptr[i+1]
        push!(I, i); push!(J, cols[p] + 1)
    end
    F = fOn ? sparse(I, J, Fv, N, N) : spzeros(ComplexF64, N, N)
    G = gOn ? sparse(I, J, Gv, N, N) : spzeros(ComplexF64, N, N)
    return F, G
end

# ---------------------------------------------------------------------------
# Frequency sweep (replaces the per-frequency loop of examples/sweep_meta.jl:219-233)
# ---------------------------------------------------------------------------
struct SweepOpts
    precision::Int32
    refine::Int32
    restart::Int32; maxiter::Int32; reltol::Float64; abstol::Float64
    gprecision::Int32; grefine::Int32; inner_reltol::Float64; max_refine::Int32
    initially_nonzero::Int32
    eager::Int32                 # 0: the sweep of each mesh replays one CUDA graph
    target_error::Float64        # mixed: re-solve at FP64 grade where 5e-7 x sensitivity exceeds it
    sensitivity::Ptr{Float64}    # optional nmesh x nk output of the sensitivity estimates
end
struct SweepInfo
    solves::Int64; converged::Int64; iterations::Int64; assemble_ms::Float64; solve_ms::Float64
    record_ms::Float64; graph_launches::Int64; accurate_solves::Int64
end

"""
    sweep_gpu(meshes, ks, ws; precision=:mixed) -> Vector{Matrix{ComplexF64}}

For every mesh m and wavenumber k_j: assemble F, G, C on the device and solve
(F + Diagonal(1 .- C)) p = G w_m with GMRES; returns one N_m x length(ks)
matrix per mesh.  With `precision=:mixed`, solves whose estimated error
exceeds `target_error` (near the mesh's interior resonances) are solved again
at FP64 grade.
"""
function sweep_gpu(meshes, ks, ws; precision=:mixed, refine=true, ctxs=nothing, target_error=1e-6)
    cs = ctxs === nothing ? [Context(m; n=2, m=2) for m in meshes] : ctxs
    kv = ComplexF64.(ks)
    wv = [Vector{ComplexF64}(w) for w in ws]
    ps = [Matrix{ComplexF64}(undef, c.n_sources, length(kv)) for c in cs]
    tgt = precision == :mixed ? Float64(target_error) : 0.0
    opts = Ref(SweepOpts(precision_code(precision), refine, 0, 0, 0.0, 0.0, 0, 0, 0.0, 0, 0, 0, tgt, C_NULL))
    info = Ref{SweepInfo}()
    GC.@preserve cs kv wv ps begin
        hs = [c.handle for c in cs]
        wp = [pointer(w) for w in wv]
        pp = [pointer(p) for p in ps]
        check(ccall((:bie_sweep, libbiegpu), Cint,
                    (Ptr{Ptr{Cvoid}}, Cint, Ptr{ComplexF64}, Cint, Ptr{Ptr{ComplexF64}},
                     Ptr{Ptr{ComplexF64}}, Ref{SweepOpts}, Ref{SweepInfo}, Ptr{Int32}),
                    hs, length(cs), kv, length(kv), wp, pp, opts, info, C_NULL))
    end
    return ps
end

# ---------------------------------------------------------------------------
# Adjoint gradient (bie_adjoint) and its ChainRulesCore rule
# ---------------------------------------------------------------------------
struct AdjointOpts
    rho_c::Float64
    dir::NTuple{3,Float64}
    reltol::Float64
    precision::Int32   # 0: FP64 forward assembly, 6: double-float (BIE_PREC_DF64)
end
struct AdjointInfo
    forward_iterations::Int32; forward_converged::Int32
    adjoint_iterations::Int32; adjoint_converged::Int32
end

"""
    farfield_objective(coordinates, Z, mesh, k, field; rho_c=1.21*343, dir=(0,0,1), gradient=false)

J = sum |p(x_f)|^2 of plane-wave scattering by the surface of `mesh` with its
vertices moved to `coordinates` (3 x N_c) and element impedances `Z`; with
`gradient=true` also dJ/dcoordinates (3 x N_c) and dJ/dZ (dJ/dRe Z + i dJ/dIm Z).
"""
function farfield_objective(coordinates, Z, mesh, k, field; rho_c=1.21 * 343.0, dir=(0.0, 0.0, 1.0),
                            gradient=false, reltol=1e-13, precision=:fp64)
    moved = (coordinates=Matrix{Float64}(coordinates), topology=mesh.topology,
             physics_topology=mesh.physics_topology, sources=Matrix{Float64}(coordinates))
    c = Context(moved; n=2, m=2)
    Zv = Vector{ComplexF64}(Z)
    X = Matrix{Float64}(field)
    J = Ref{Float64}(0.0)
    pf = Vector{ComplexF64}(undef, size(X, 2))
    dX = gradient ? zeros(Float64, size(coordinates)) : Matrix{Float64}(undef, 0, 0)
    dZ = gradient ? zeros(ComplexF64, length(Zv)) : Vector{ComplexF64}(undef, 0)
    d = collect(Float64, dir); d ./= norm(d)
    # precision: forward-model assembly, :fp64 or :df64 (double-float)
    opts = Ref(AdjointOpts(rho_c, (d[1], d[2], d[3]), reltol, precision_code(precision)))
    info = Ref{AdjointInfo}()
    GC.@preserve Zv X pf dX dZ begin
        check(ccall((:bie_adjoint, libbiegpu), Cint,
                    (Ptr{Cvoid}, Float64, Float64, Ptr{ComplexF64}, Ptr{Float64}, Int64, Ref{AdjointOpts},
                     Ref{Float64}, Ptr{ComplexF64}, Ptr{Float64}, Ptr{ComplexF64}, Ref{AdjointInfo}),
                    c.handle, Float64(real(k)), Float64(imag(k)), Zv, X, size(X, 2), opts, J, pf,
                    gradient ? pointer(dX) : C_NULL, gradient ? pointer(dZ) : C_NULL, info))
    end
    return gradient ? (J[], dX, dZ) : J[]
end

# The pullback scales the adjoint gradients by the incoming cotangent of J; the
# complex cotangent of Z follows ChainRules' convention (dJ/dRe Z + i dJ/dIm Z).
function ChainRulesCore.rrule(::typeof(farfield_objective), coordinates, Z, mesh, k, field; kwargs...)
    J, dX, dZ = farfield_objective(coordinates, Z, mesh, k, field; kwargs..., gradient=true)
    function farfield_objective_pullback(dJ)
        s = ChainRulesCore.unthunk(dJ)
        return (ChainRulesCore.NoTangent(), s .* dX, s .* dZ, ChainRulesCore.NoTangent(),
                ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent())
    end
    return J, farfield_objective_pullback
end

# ---------------------------------------------------------------------------
# Fast operators: the FMMFOperator / FMMGOperator algorithm (Gauss-rule far
# field summed exactly on the GPU + near-field correction),
# src/3d/fast_multipole_method.jl:163-194, 306-324, 473-490
# ---------------------------------------------------------------------------
mutable struct GPUFastOperator{W} <: LinearMaps.LinearMap{ComplexF64}
    ctx::Context
    handle::Ptr{Cvoid}
    precision::Cint
end

function GPUFastOperator{W}(mesh, k; tol=1e-6, n_gauss=3, nearfield=true, offset=0.2, depth=1,
                            precision=:mixed, ctx=Context(mesh; n=2, m=2)) where {W}
    kk = ComplexF64(k)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:bie_fastop_create, libbiegpu), Cint,
                (Ptr{Cvoid}, Float64, Float64, Cint, Cint, Cint, Float64, Cint, Ref{Ptr{Cvoid}}),
                ctx.handle, real(kk), imag(kk), W === :F ? BIE_F : BIE_G, n_gauss, nearfield ? 1 : 0,
                offset, depth, h))
    op = GPUFastOperator{W}(ctx, h[], precision_code(precision))
    finalizer(o -> ccall((:bie_fastop_destroy, libbiegpu), Cint, (Ptr{Cvoid},), o.handle), op)
    return op
end

"Drop-in for FMMFOperator(mesh, k; n_gauss, nearfield, offset, depth) (`tol` is accepted, the sum is exact)."
const FastFOperator = GPUFastOperator{:F}
"Drop-in for FMMGOperator(mesh, k; n_gauss, nearfield, offset, depth)."
const FastGOperator = GPUFastOperator{:G}

Base.size(A::GPUFastOperator) = (A.ctx.n_sources, A.ctx.n_sources)

function LinearMaps._unsafe_mul!(y::AbstractVector, A::GPUFastOperator, x::AbstractVector)
    xv = Vector{ComplexF64}(x)
    yv = Vector{ComplexF64}(undef, length(y))
    GC.@preserve xv yv check(ccall((:bie_fastop_apply, libbiegpu), Cint,
                                   (Ptr{Cvoid}, Ptr{ComplexF64}, Ptr{ComplexF64}, Cint),
                                   A.handle, xv, yv, A.precision))
    copyto!(y, yv)
    return y
end

function evaluate_targets(A::GPUFastOperator, x, targets)
    xv = Vector{ComplexF64}(x)
    tg = Matrix{Float64}(targets)
    y = Vector{ComplexF64}(undef, size(tg, 2))
    GC.@preserve xv tg y check(ccall((:bie_fastop_evaluate_targets, libbiegpu), Cint,
                                     (Ptr{Cvoid}, Ptr{Float64}, Int64, Ptr{ComplexF64}, Ptr{ComplexF64}, Cint),
                                     A.handle, tg, size(tg, 2), xv, y, A.precision))
    return y
end

# ---------------------------------------------------------------------------
# k-derivative assembly (taylor_assemble!, src/3d/rosebem.jl:56-157)
# ---------------------------------------------------------------------------
"""
    taylor_assemble_gpu!(mesh, k0, sources; M=0, fOn=true, gOn=true, cOn=true, n=3, m=3, U=I)

`(From, Grom, C)` with From[:, :, m+1] the m-th k-derivative of F at k0 (and G),
projected on U as the reference does (From = U' F U).
"""
function taylor_assemble_gpu!(mesh, k0, sources; M=0, fOn=true, gOn=true, cOn=true, n=3, m=3, U=I,
                              ctx=nothing)
    c = ctx === nothing ? Context(mesh; n=n, m=m) : ctx
    kk = ComplexF64(k0)
    tg = Matrix{Float64}(sources)
    Mt = size(tg, 2)
    N = c.n_sources
    F = fOn ? Array{ComplexF64}(undef, Mt, N, M + 1) : Array{ComplexF64}(undef, 0, 0, 0)
    G = gOn ? Array{ComplexF64}(undef, Mt, N, M + 1) : Array{ComplexF64}(undef, 0, 0, 0)
    C = cOn ? Vector{ComplexF64}(undef, Mt) : Vector{ComplexF64}(undef, 0)
    flags = (fOn ? BIE_F : Cint(0)) | (gOn ? BIE_G : Cint(0)) | (cOn ? BIE_C : Cint(0))
    same = sources === mesh.sources
    GC.@preserve tg F G C check(ccall((:bie_taylor_assemble, libbiegpu), Cint,
                                      (Ptr{Cvoid}, Float64, Float64, Ptr{Float64}, Int64, Cint, Cint,
                                       Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{ComplexF64}),
                                      c.handle, real(kk), imag(kk), same ? C_NULL : pointer(tg), Mt, flags, M,
                                      fOn ? pointer(F) : C_NULL, gOn ? pointer(G) : C_NULL,
                                      cOn ? pointer(C) : C_NULL))
    if !(U isa UniformScaling)
        F = fOn ? cat([U' * F[:, :, j] * U for j in 1:M+1]...; dims=3) : F
        G = gOn ? cat([U' * G[:, :, j] * U for j in 1:M+1]...; dims=3) : G
    end
    return F, G, C
end

# ---------------------------------------------------------------------------
# Visco-thermal system (LossyGlobalOuter, src/3d/LossyGlobalMatrix.jl:76-197)
# ---------------------------------------------------------------------------
struct GmresOptsC
    restart::Int32; maxiter::Int32; reltol::Float64; abstol::Float64
    precision::Int32; refine::Int32; inner_reltol::Float64; max_refine::Int32; initially_nonzero::Int32
end
GmresOptsC(; reltol=0.0, restart=0, maxiter=0) = GmresOptsC(restart, maxiter, reltol, 0.0, 0, 0, 0.0, 0, 0)

struct GmresInfoC
    iterations::Int32; restarts::Int32; refinements::Int32; converged::Int32
    matvecs::Int64; residual_norm::Float64; rhs_norm::Float64
end

# bie_operator (include/biegpu.h)
struct OperatorC
    kind::Int32
    A::Ptr{ComplexF64}
    A32::Ptr{ComplexF32}
    k_re::Float64; k_im::Float64
    scale_re::Float64; scale_im::Float64
    diag::Ptr{ComplexF64}
    fast::Ptr{Cvoid}
end

function _gmres_host(ctx::Context, op::OperatorC, b, reltol, restart, maxiter, precision, refine)
    bv = Vector{ComplexF64}(b)
    x = zeros(ComplexF64, length(bv))
    opts = GmresOptsC(restart, maxiter, reltol, 0.0, precision_code(precision), refine ? 1 : 0, 0.0, 0, 0)
    info = Ref{GmresInfoC}()
    st = GC.@preserve bv x ccall((:bie_gmres, libbiegpu), Cint,
                                 (Ptr{Cvoid}, Ref{OperatorC}, Ptr{ComplexF64}, Ptr{ComplexF64},
                                  Ref{GmresOptsC}, Ref{GmresInfoC}), ctx.handle, op, bv, x, opts, info)
    st == Cint(-3) || check(st)   # not converged: x is still returned, as gmres does
    return x
end

"""
    gmres_gpu(ctx, H::AbstractMatrix, b; diag=nothing, scale=1, refine=false,
              precision=:fp64, reltol=0, restart=0, maxiter=0)

`gmres(scale * H + Diagonal(diag), b)` for a dense matrix on the host (e.g.
`gmres(Fp + Diagonal(1 .- Cp), pI)`, test/3d/assembly_test.jl:37-38 →
`gmres_gpu(ctx, Fp, pI; diag=1 .- Cp)`), solved by the library's device GMRES
(`bie_gmres`; IterativeSolvers defaults for zero arguments).  `refine=true`
runs complex64 inner iterations with FP64 residual refinement.
"""
function gmres_gpu(ctx::Context, H::AbstractMatrix, b; diag=nothing, scale=1.0, refine=false,
                   precision=:fp64, reltol=0.0, restart=0, maxiter=0)
    Hm = Matrix{ComplexF64}(H)
    dv = diag === nothing ? ComplexF64[] : Vector{ComplexF64}(diag)
    s = ComplexF64(scale)
    GC.@preserve Hm dv begin
        op = OperatorC(0, pointer(Hm), C_NULL, 0.0, 0.0, real(s), imag(s),
                       diag === nothing ? C_NULL : pointer(dv), C_NULL)
        return _gmres_host(ctx, op, b, reltol, restart, maxiter, precision, refine)
    end
end

"""
    gmres_gpu(Ff::GPUFOperator, b; diag=nothing, scale=1, ...)

`gmres(scale * Ff + Diagonal(diag), b)` matrix-free (the F rows generated on
the fly in every product), e.g. `gmres(Diagonal(1 .- C) - Ff, Gf * vs)`
(examples/3d_pulsating_sphere.jl:46-50) → `gmres_gpu(Ff, Gf * vs; diag=1 .- C, scale=-1)`.
"""
function gmres_gpu(Ff::GPUOperator{:F}, b; diag=nothing, scale=1.0, refine=false, reltol=0.0,
                   restart=0, maxiter=0)
    dv = diag === nothing ? ComplexF64[] : Vector{ComplexF64}(diag)
    s = ComplexF64(scale)
    prec = Ff.precision == BIE_PREC_MIXED ? :mixed : :fp64
    GC.@preserve dv begin
        op = OperatorC(1, C_NULL, C_NULL, real(Ff.k), imag(Ff.k), real(s), imag(s),
                       diag === nothing ? C_NULL : pointer(dv), C_NULL)
        return _gmres_host(Ff.ctx, op, b, reltol, restart, maxiter, prec, refine)
    end
end

struct LossyOpts
    S::Float64; custom_air::Int32; pa::Float64; t::Float64; Hr::Float64
    depth::Int32; interior::Int32; fmm_on::Int32; n_gauss::Int32; fmm_offset::Float64
    normals::Ptr{Float64}; solve::GmresOptsC
end

const LOSSY_BLOCKS = (outer=0, Ha=1, Ga=2, Hh=3, Gh=4, Hv=5, Gv=6, Dc=7, Dr=8, Nd=9, NdT=10, inner=11)

"A block of the device-resident lossy system as a `LinearMap` (products on the GPU)."
struct GPULossyBlock <: LinearMaps.LinearMap{ComplexF64}
    owner::Any
    code::Cint
    dims::Tuple{Int,Int}
end
Base.size(A::GPULossyBlock) = A.dims

function LinearMaps._unsafe_mul!(y::AbstractVector, A::GPULossyBlock, x::AbstractVector)
    xv = Vector{ComplexF64}(x)
    yv = Vector{ComplexF64}(undef, size(A, 1))
    GC.@preserve xv yv check(ccall((:bie_lossy_apply, libbiegpu), Cint,
                                   (Ptr{Cvoid}, Cint, Ptr{ComplexF64}, Ptr{ComplexF64}),
                                   A.owner.handle, A.code, xv, yv))
    copyto!(y, yv)
    return y
end

"""
    gmres_gpu(A::GPULossyBlock, b; reltol=0, restart=0, maxiter=0)

`gmres(A, b)` with the device GMRES of the library (IterativeSolvers defaults
for zeros); square blocks only.
"""
function gmres_gpu(A::GPULossyBlock, b; reltol=0.0, restart=0, maxiter=0)
    bv = Vector{ComplexF64}(b)
    x = similar(bv)
    opts = Ref(GmresOptsC(; reltol=reltol, restart=restart, maxiter=maxiter))
    info = Ref{GmresInfoC}()
    st = GC.@preserve bv x ccall((:bie_lossy_solve, libbiegpu), Cint,
                                 (Ptr{Cvoid}, Cint, Ptr{ComplexF64}, Ptr{ComplexF64}, Ref{GmresOptsC},
                                  Ref{GmresInfoC}), A.owner.handle, A.code, bv, x, opts, info)
    st == Cint(-3) || check(st)   # not converged: x is still returned, as gmres does
    return x
end

"""
    GPULossyGlobalOuter(mesh, freq; depth=1, n=3, exterior=true, fmm_on=false, S=1)

Drop-in for `LossyGlobalOuter(mesh, freq; depth, n, exterior, fmm_on)`: the
acoustic, thermal and viscous BEM blocks, the tangential derivatives and the
normals live on the device and the product (with its nested gmres calls) runs
there.  The fields `Ha, Ga, Hh, Gh, Hv, Gv, Dc, Dr, Nd, inner` are
`GPULossyBlock`s (`Nd'` is `NdT`), and `phi_a, phi_h, tau_a, tau_h, mu_a,
mu_h` the constants, as in the reference's struct.
"""
mutable struct GPULossyGlobalOuter <: LinearMaps.LinearMap{ComplexF64}
    ctx::Context
    handle::Ptr{Cvoid}
    n::Int
    normals::Matrix{Float64}
    Ha::GPULossyBlock; Ga::GPULossyBlock; Hh::GPULossyBlock; Gh::GPULossyBlock
    Hv::GPULossyBlock; Gv::GPULossyBlock; Dc::GPULossyBlock; Dr::GPULossyBlock
    Nd::GPULossyBlock; NdT::GPULossyBlock; inner::GPULossyBlock
    phi_a::ComplexF64; phi_h::ComplexF64; tau_a::ComplexF64; tau_h::ComplexF64
    mu_a::ComplexF64; mu_h::ComplexF64
    GPULossyGlobalOuter() = new()
end

function GPULossyGlobalOuter(mesh, freq; depth=1, n=3, exterior=true, fmm_on=false, S=1.0, fmm_offset=0.2,
                             reltol=0.0, restart=0, maxiter=0, ctx=Context(mesh; n=n, m=n))
    L = GPULossyGlobalOuter()
    L.ctx = ctx
    N = ctx.n_sources
    L.n = N
    L.normals = Matrix{Float64}(mesh.normals)
    opts = Ref(LossyOpts(S, 0, 0.0, 0.0, 0.0, depth, exterior ? 0 : 1, fmm_on ? 1 : 0, n, fmm_offset,
                         pointer(L.normals), GmresOptsC(; reltol=reltol, restart=restart, maxiter=maxiter)))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve L check(ccall((:bie_lossy_create, libbiegpu), Cint,
                               (Ptr{Cvoid}, Float64, Ref{LossyOpts}, Ref{Ptr{Cvoid}}), ctx.handle, freq, opts, h))
    L.handle = h[]
    finalizer(o -> ccall((:bie_lossy_destroy, libbiegpu), Cint, (Ptr{Cvoid},), o.handle), L)
    k = Ref{NTuple{23,Float64}}()
    check(ccall((:bie_lossy_constants_of, libbiegpu), Cint, (Ptr{Cvoid}, Ref{NTuple{23,Float64}}), L.handle, k))
    v = k[]
    cx(i) = complex(v[i], v[i+1])
    L.tau_a, L.tau_h, L.phi_a, L.phi_h = cx(10), cx(12), cx(14), cx(16)
    L.mu_a, L.mu_h = cx(20), cx(22)
    blk(name, d) = GPULossyBlock(L, Cint(LOSSY_BLOCKS[name]), d)
    L.Ha, L.Ga, L.Hh, L.Gh = blk(:Ha, (N, N)), blk(:Ga, (N, N)), blk(:Hh, (N, N)), blk(:Gh, (N, N))
    L.Hv, L.Gv = blk(:Hv, (3N, 3N)), blk(:Gv, (3N, 3N))
    L.Dc, L.Dr = blk(:Dc, (3N, N)), blk(:Dr, (N, 3N))
    L.Nd, L.NdT, L.inner = blk(:Nd, (3N, N)), blk(:NdT, (N, 3N)), blk(:inner, (N, N))
    return L
end

Base.size(L::GPULossyGlobalOuter) = (L.n, L.n)

function LinearMaps._unsafe_mul!(y::AbstractVector, L::GPULossyGlobalOuter, x::AbstractVector)
    xv = Vector{ComplexF64}(x)
    yv = Vector{ComplexF64}(undef, L.n)
    GC.@preserve xv yv check(ccall((:bie_lossy_apply, libbiegpu), Cint,
                                   (Ptr{Cvoid}, Cint, Ptr{ComplexF64}, Ptr{ComplexF64}),
                                   L.handle, Cint(LOSSY_BLOCKS.outer), xv, yv))
    copyto!(y, yv)
    return y
end

"""
    set_one_launch!(L, mode=:auto)

The sparse thermal / viscous solves inside `L`'s products (`bie_lossy_set_one_launch`):
`:auto` one launch each (a cooperative grid over the SMs for more than 2048
rows, else a thread-block cluster), `:cluster`, `:grid`, or `:off` for the
launch-per-operation device GMRES.
"""
function set_one_launch!(L::GPULossyGlobalOuter, mode::Symbol=:auto)
    code = Dict(:off => 0, :auto => 1, :cluster => 2, :grid => 3)[mode]
    check(ccall((:bie_lossy_set_one_launch, libbiegpu), Cint, (Ptr{Cvoid}, Cint), L.handle, code))
    return L
end

"`gmres(L, b)` for the whole lossy system with the library's device GMRES."
gmres_gpu(L::GPULossyGlobalOuter, b; kwargs...) = gmres_gpu(GPULossyBlock(L, Cint(0), (L.n, L.n)), b; kwargs...)

version() = unsafe_string(ccall((:bie_version, libbiegpu), Cstring, ()))

"""
    order, counts = element_slicing(mesh, level)

The element slicing of the assembly kernels, computed on the host
(`bie_element_slicing`, no GPU): `order` holds the 1-based element numbers in
the order the kernels process them (a recursive coordinate bisection of the
element centroids); `counts` the nodes of each kind at slicing level `level`
(2^level slices, 0..7) as a NamedTuple: shared between slices (with their
side slots), of one slice with several contributions summed in the
shared-memory ring or widened afterwards, with one contribution, untouched.
"""
function element_slicing(mesh, level::Integer)
    coords = Matrix{Float64}(mesh.coordinates)
    topo = Matrix{Int64}(mesh.topology)
    ptopo = Matrix{Int64}(mesh.physics_topology)
    src = Matrix{Float64}(mesh.sources)
    pk, pb = physics_kind(mesh.physics_function, size(ptopo, 1))
    order = Vector{Int32}(undef, size(topo, 2))
    counts = zeros(Int64, 6)
    GC.@preserve coords topo ptopo src begin
        desc = Ref(MeshDesc(size(coords, 2), pointer(coords), size(topo, 2), element_kind(size(topo, 1)), pk,
                            pointer(topo), pointer(ptopo), size(src, 2), pointer(src), Int32(1), Int32(1), pb))
        check(ccall((:bie_element_slicing, libbiegpu), Cint,
                    (Ref{MeshDesc}, Cint, Ptr{Int32}, Ptr{Int64}, Ptr{UInt32}, Ptr{Int32}),
                    desc, level, order, counts, C_NULL, C_NULL))
    end
    return order, (shared=counts[1], side_slots=counts[2], ring=counts[3], widened=counts[4],
                   single=counts[5], untouched=counts[6])
end

export GPU, Context, reference_rules, assemble_parallel_gpu!, GPUFOperator, GPUGOperator, evaluate_targets,
       sparse_assemble_parallel_gpu!, sweep_gpu, farfield_objective, FastFOperator, FastGOperator,
       taylor_assemble_gpu!, GPULossyGlobalOuter, GPULossyBlock, gmres_gpu, solve_multi_gpu, set_one_launch!,
       element_slicing

end # module
