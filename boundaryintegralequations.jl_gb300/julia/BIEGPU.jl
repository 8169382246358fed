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
using LinearMaps

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
end

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

"""
    Context(mesh; n=4, m=4, device=0)

Uploads the mesh (coordinates, topology, sources, physics topology) and builds
the clustered quadrature rules on the device.  One context per (mesh, n, m).
"""
mutable struct Context
    handle::Ptr{Cvoid}
    n_sources::Int
    function Context(mesh; n=4, m=4, device=0)
        coords = Matrix{Float64}(mesh.coordinates)
        topo = Matrix{Int64}(mesh.topology)
        ptopo = Matrix{Int64}(mesh.physics_topology)
        src = Matrix{Float64}(mesh.sources)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        GC.@preserve coords topo ptopo src begin
            desc = Ref(MeshDesc(size(coords, 2), pointer(coords), size(topo, 2),
                                element_kind(size(topo, 1)), element_kind(size(ptopo, 1)),
                                pointer(topo), pointer(ptopo), size(src, 2), pointer(src),
                                Int32(n), Int32(m)))
            check(ccall((:bie_ctx_create, libbiegpu), Cint,
                        (Ref{Ptr{Cvoid}}, Ref{MeshDesc}, Cint), h, desc, device))
        end
        ctx = new(h[], size(src, 2))
        finalizer(c -> ccall((:bie_ctx_destroy, libbiegpu), Cint, (Ptr{Cvoid},), c.handle), ctx)
        return ctx
    end
end

precision_code(p::Symbol) = p === :fp64 ? BIE_PREC_FP64 : p === :mixed ? BIE_PREC_MIXED :
                            throw(ArgumentError("precision must be :fp64 or :mixed"))

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

version() = unsafe_string(ccall((:bie_version, libbiegpu), Cstring, ()))

export Context, assemble_parallel_gpu!, GPUFOperator, GPUGOperator, evaluate_targets

end # module
