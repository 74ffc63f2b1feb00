# FerriteGB300.jl -- Julia binding of libferrite_gb300 (the C ABI in include/ferrite_gb300.h).
#
# Replaces Ferrite's assembly loop
#     assembler = start_assemble(K, f); for cell in CellIterator(dh) ... assemble!(...) end
# with one ccall that fills K.nzval and f. Everything is passed as Ferrite's own memory.
# (Julia is not available where this repository is built and tested; the same entry points are
# exercised from Python through ctypes with byte-identical arrays.)
module FerriteGB300

using Ferrite, SparseArrays
import ChainRulesCore
using ChainRulesCore: NoTangent, unthunk

const LIB = get(ENV, "FERRITE_GB300_LIB", joinpath(@__DIR__, "..", "lib", "libferrite_gb300.so"))

const FE_HEAT, FE_LINEAR_ELASTIC, FE_NEO_HOOKE = Int32(1), Int32(2), Int32(3)
const FE_PREC_MIXED, FE_PREC_FP64 = Int32(0), Int32(1)
const FE_FILLZERO = UInt32(1)
const FE_ASYNC = UInt32(8)
const FE_STAGED_OUTPUT = UInt32(512)
const FE_FP32_SUM = UInt32(1024)   # plain FP32 sums per entry instead of the compensated default

# raw address of a host Vector or a device array (CuArray's CuPtr is a 64-bit primitive)
_ptr(x, ::Type{T}=Float64) where {T} = x === nothing ? Ptr{T}(C_NULL) : reinterpret(Ptr{T}, pointer(x))

struct GridDesc
    dim::Int32
    n_nodes::Int64
    nodes::Ptr{Float64}
    n_cells::Int64
end

struct SubdomainDesc
    cell_type::Int32
    ip_order::Int32
    n_components::Int32
    n_qp::Int32
    qr_weights::Ptr{Float64}
    N::Ptr{Float64}
    dNdxi::Ptr{Float64}
    M::Ptr{Float64}
    dMdxi::Ptr{Float64}
    n_cells::Int64
    cellset::Ptr{Int64}
    cell_nodes::Ptr{Int64}
end

struct DofDesc
    ndofs::Int64
    cell_dofs::Ptr{Int64}
    cell_dofs_offset::Ptr{Int64}
end

struct CscDesc
    n::Int64
    nnz::Int64
    colptr::Ptr{Int64}
    rowval::Ptr{Int64}
end

struct AssembleParams
    physics::Int32
    precision::Int32
    flags::UInt32
    p0::Float64
    p1::Float64
    body::NTuple{3,Float64}
    cell_scale::Ptr{Float64}
    u::Ptr{Float64}
    cond_threshold::Float64
    stream::Ptr{Cvoid}
end

struct ErrorInfo
    code::Int32
    cell::Int64
    detJ::Float64
    row::Int64
    col::Int64
    message::NTuple{256,UInt8}
end

celltype_code(::Type{Triangle}) = Int32(1)
celltype_code(::Type{Quadrilateral}) = Int32(2)
celltype_code(::Type{Tetrahedron}) = Int32(3)
celltype_code(::Type{Hexahedron}) = Int32(4)
celltype_code(::Type{Wedge}) = Int32(5)

mutable struct Handle
    ptr::Ptr{Cvoid}
    keep::Vector{Any}
    dim::Int
    n_nodes::Int
    n_cells::Int
end

function check(rc, h)
    rc == 0 && return
    info = Ref{ErrorInfo}()
    ccall((:fe_last_error, LIB), Cint, (Ptr{Cvoid}, Ptr{ErrorInfo}), h, info)
    msg = String(filter(!=(0x00), collect(info[].message)))
    rc == 3 && throw(ArgumentError("det(J) is not positive: det(J) = $(info[].detJ) (cell $(info[].cell))"))
    rc == 4 && error(msg)
    error("ferrite_gb300 error $rc: $msg")
end

"""
    Handle(dh, cellvalues_per_sdh, K)

fe_create for a closed DofHandler, one scalar-interpolation CellValues per SubDofHandler (the
field is `ip^n_components`), and the pattern of `K = allocate_matrix(dh)`.
"""
Handle(dh::DofHandler, cvs::Vector, K::SparseMatrixCSC{Float64,Int}) = Handle(dh, cvs, K.colptr, K.rowval)

# A SparseMatrixCSR{1} of allocate_matrix(SparseMatrixCSR, dh) (ext/FerriteSparseMatrixCSR.jl):
# Handle(dh, cvs, K.rowptr, K.colval); its arrays equal the CSC ones (symmetric pattern).
function Handle(dh::DofHandler, cvs::Vector, colptr::Vector{Int64}, rowval::Vector{Int64})
    grid = Ferrite.get_grid(dh)
    nodes = reinterpret(Float64, grid.nodes)            # AoS Vec{dim} memory
    keep = Any[nodes]
    subs = SubdomainDesc[]
    for (sdh, cv) in zip(dh.subdofhandlers, cvs)
        cells = sort!(collect(sdh.cellset))
        ct = typeof(grid.cells[first(cells)])
        conn = reduce(vcat, [collect(Int64, grid.cells[c].nodes) for c in cells])
        fv, gm = cv.fun_values, cv.geo_mapping
        N = Matrix{Float64}(fv.Nξ)                       # [n_base, n_qp] == C [n_qp][n_base]
        dN = reinterpret(Float64, fv.dNdξ)               # Vec{rdim} per (base, qp)
        M = Matrix{Float64}(gm.M)
        dM = reinterpret(Float64, gm.dMdξ)
        w = Vector{Float64}(getweights(cv.qr))
        cs = Vector{Int64}(cells)
        ip = Ferrite.getfieldinterpolation(sdh, first(sdh.field_names))
        nc = ip isa VectorizedInterpolation ? ip.vdim : 1
        order = Ferrite.getorder(Ferrite.get_base_interpolation(ip))
        append!(keep, (conn, N, dN, M, dM, w, cs))
        push!(subs, SubdomainDesc(celltype_code(ct), Int32(order), Int32(nc), Int32(length(w)),
                                  pointer(w), pointer(N), pointer(dN), pointer(M), pointer(dM),
                                  length(cs), pointer(cs), pointer(conn)))
    end
    offs = Vector{Int64}(dh.cell_dofs_offset)
    cd = Vector{Int64}(dh.cell_dofs)
    append!(keep, (offs, cd))
    g = Ref(GridDesc(Int32(Ferrite.getspatialdim(grid)), length(grid.nodes), pointer(nodes), length(grid.cells)))
    d = Ref(DofDesc(ndofs(dh), pointer(cd), pointer(offs)))
    p = Ref(CscDesc(length(colptr) - 1, length(rowval), pointer(colptr), pointer(rowval)))
    out = Ref{Ptr{Cvoid}}(C_NULL)
    rc = GC.@preserve keep subs colptr rowval ccall((:fe_create, LIB), Cint,
        (Ptr{GridDesc}, Int32, Ptr{SubdomainDesc}, Ptr{DofDesc}, Ptr{CscDesc}, Ptr{Ptr{Cvoid}}),
        g, Int32(length(subs)), subs, d, p, out)
    check(rc, C_NULL)
    h = Handle(out[], keep, Int(Ferrite.getspatialdim(grid)), length(grid.nodes), length(grid.cells))
    finalizer(x -> ccall((:fe_destroy, LIB), Cvoid, (Ptr{Cvoid},), x.ptr), h)
    return h
end

"""
    assemble_csc!(K, f, h; physics, p0, p1, body, cell_scale, u, precision, fillzero)

The whole `start_assemble(K, f)` + cell loop + `assemble!` in one call. K.nzval and f may be
host arrays or device arrays (CuArray pointers). `staged_output=true`: host arrays go through
a device buffer and the copy engine even when page-locked.
"""
function assemble_csc!(K::SparseMatrixCSC{Float64,Int}, f::Vector{Float64}, h::Handle;
                       physics=FE_LINEAR_ELASTIC, p0=1.0, p1=0.3, body=(0.0, 0.0, 0.0),
                       cell_scale=nothing, u=nothing, precision=FE_PREC_MIXED, fillzero=true,
                       staged_output=false)
    cs = cell_scale === nothing ? Ptr{Float64}(C_NULL) : pointer(cell_scale)
    up = u === nothing ? Ptr{Float64}(C_NULL) : pointer(u)
    flags = (fillzero ? FE_FILLZERO : UInt32(0)) | (staged_output ? FE_STAGED_OUTPUT : UInt32(0))
    par = Ref(AssembleParams(physics, precision, flags, p0, p1,
                             Tuple(Float64.(body)), cs, up, 0.0, C_NULL))
    rc = GC.@preserve K f cell_scale u ccall((:fe_assemble, LIB), Cint,
        (Ptr{Cvoid}, Ptr{AssembleParams}, Ptr{Float64}, Ptr{Float64}), h.ptr, par, K.nzval, f)
    check(rc, h.ptr)
    return K, f
end

"""
    assemble_csr!(K, f, h; ...)

`start_assemble(K::SparseMatrixCSR, f)` + the cell loop + `assemble!` of
ext/FerriteSparseMatrixCSR.jl for a handle made with `Handle(dh, cvs, K.rowptr, K.colval)`:
every physics here has a symmetric K, so the CSC values of the same arrays are the CSR values
(up to the rounding of Ke(I, J) against Ke(J, I)).
"""
function assemble_csr!(K, f::Vector{Float64}, h::Handle; physics=FE_LINEAR_ELASTIC, p0=1.0, p1=0.3,
                       body=(0.0, 0.0, 0.0), cell_scale=nothing, u=nothing, precision=FE_PREC_MIXED, fillzero=true)
    cs = cell_scale === nothing ? Ptr{Float64}(C_NULL) : pointer(cell_scale)
    up = u === nothing ? Ptr{Float64}(C_NULL) : pointer(u)
    par = Ref(AssembleParams(physics, precision, fillzero ? FE_FILLZERO : UInt32(0), p0, p1,
                             Tuple(Float64.(body)), cs, up, 0.0, C_NULL))
    rc = GC.@preserve K f cell_scale u ccall((:fe_assemble, LIB), Cint,
        (Ptr{Cvoid}, Ptr{AssembleParams}, Ptr{Float64}, Ptr{Float64}), h.ptr, par, K.nzval, f)
    check(rc, h.ptr)
    return K, f
end

struct ElementLayout
    ke_stride::NTuple{3,Int64}
    fe_stride::NTuple{2,Int64}
end

"""
    assemble_elements!(Kes, fes, h; physics, p0, p1, ...)

The GPU how-to's element assembly (gpu_assembly.jl:270-303): `Kes[cellid, :, :]` and
`fes[cellid, :]` for every cell, in the how-to's arrays `Kes = CUDA.zeros(Float32, ncells, nbf,
nbf)`, `fes = CUDA.zeros(Float32, ncells, nbf)` (Float64 arrays with FE_PREC_FP64).
"""
function assemble_elements!(Kes, fes, h::Handle; physics=FE_LINEAR_ELASTIC, p0=1.0, p1=0.3,
                            body=(0.0, 0.0, 0.0), cell_scale=nothing, u=nothing, precision=FE_PREC_MIXED)
    n, nbf = size(Kes, 1), size(Kes, 2)
    lay = Ref(ElementLayout((1, n, n * nbf), (1, n)))
    cs = cell_scale === nothing ? Ptr{Float64}(C_NULL) : pointer(cell_scale)
    up = u === nothing ? Ptr{Float64}(C_NULL) : pointer(u)
    par = Ref(AssembleParams(physics, precision, UInt32(0), p0, p1, Tuple(Float64.(body)), cs, up, 0.0, C_NULL))
    rc = GC.@preserve Kes fes cell_scale u ccall((:fe_assemble_elements, LIB), Cint,
        (Ptr{Cvoid}, Ptr{AssembleParams}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{ElementLayout}),
        h.ptr, par, pointer(Kes), pointer(fes), lay)
    check(rc, h.ptr)
    return Kes, fes
end

# Matrix-free product with the element matrices of assemble_elements!
mutable struct ElementOperator
    ptr::Ptr{Cvoid}
    h::Handle
end

"""
    ElementOperator(h, Kes; precision=FE_PREC_MIXED)

The operator u -> sum_c A_c' Kes[c, :, :] A_c u for the how-to's `Kes` (column-major
`CUDA.zeros(Float32, ncells, nbf, nbf)`; Float64 with FE_PREC_FP64), which the how-to leaves
to the user (gpu_assembly.jl:265-311).
"""
function ElementOperator(h::Handle, Kes; precision=FE_PREC_MIXED)
    n, nbf = size(Kes, 1), size(Kes, 2)
    lay = Ref(ElementLayout((1, n, n * nbf), (0, 0)))
    out = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:fe_element_operator_create, LIB), Cint, (Ptr{Cvoid}, Ptr{ElementLayout}, Int32, Ptr{Ptr{Cvoid}}),
               h.ptr, lay, Int32(precision), out)
    check(rc, h.ptr)
    op = ElementOperator(out[], h)
    finalizer(x -> ccall((:fe_element_operator_destroy, LIB), Cvoid, (Ptr{Cvoid},), x.ptr), op)
    return op
end

"""
    element_mul!(y, op::ElementOperator, Kes, u; fillzero=true)

y = sum_c A_c' Ke_c A_c u (y += ... with fillzero=false) on device arrays; asynchronous on the
default stream.
"""
function element_mul!(y, op::ElementOperator, Kes, u; fillzero::Bool=true)
    rc = GC.@preserve y Kes u op ccall((:fe_element_matvec, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, UInt32, Ptr{Cvoid}),
        op.ptr, pointer(Kes), pointer(u), pointer(y), fillzero ? FE_FILLZERO : UInt32(0), C_NULL)
    check(rc, op.h.ptr)
    return y
end

# Dirichlet constraints of a closed ConstraintHandler on the handle's pattern
mutable struct Constraints
    ptr::Ptr{Cvoid}
    h::Handle
    inhomogeneities::Vector{Float64}
end

function Constraints(h::Handle, K::SparseMatrixCSC{Float64,Int}, ch::ConstraintHandler)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    pd = Vector{Int64}(ch.prescribed_dofs)
    rc = GC.@preserve K pd ccall((:fe_dirichlet_create, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Int64}, Int64, Ptr{Int64}, Ptr{Ptr{Cvoid}}), h.ptr, K.rowval, length(pd), pd, out)
    check(rc, h.ptr)
    c = Constraints(out[], h, Vector{Float64}(ch.inhomogeneities))
    finalizer(x -> ccall((:fe_dirichlet_destroy, LIB), Cvoid, (Ptr{Cvoid},), x.ptr), c)
    return c
end

"""
    apply!(nzval, f, c::Constraints; applyzero=false)

`Ferrite.apply!(K, f, ch)` / `apply_zero!(K, f, ch)` (ConstraintHandler.jl:711-744) on device
arrays (`nzval = nonzeros(K_gpu)`, `f` a CuArray); asynchronous on the default stream.
"""
function apply!(nzval, f, c::Constraints; applyzero::Bool=false)
    rc = GC.@preserve nzval f c ccall((:fe_apply, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int32, Ptr{Cvoid}),
        c.ptr, pointer(nzval), f === nothing ? C_NULL : pointer(f), c.inhomogeneities, Int32(applyzero), C_NULL)
    check(rc, c.h.ptr)
    return nzval, f
end

"""
    sparsity_pattern_device!(colptr, grid, subs, dofs, rowval=nothing) -> nnz

`allocate_matrix(dh)` by GPU kernels (fe_sparsity_pattern_device) into device arrays, e.g. the
`colPtr`/`rowVal` of a `CuSparseMatrixCSC` (the same arrays as `allocate_matrix(dh)`): call
once with `rowval === nothing` for colptr and nnz, then with a `CuArray{Int64}(undef, nnz)`.
`grid`, `subs` and `dofs` are the descriptors `Handle` builds. The facet tables below are
`[nf][nqp]...` row-major, i.e. Julia arrays of size (nqp, nf), (nbase, nqp, nf), (dim, ngeo,
nqp, nf).
"""
function sparsity_pattern_device!(colptr, grid::Ref{GridDesc}, subs::Vector{SubdomainDesc}, dofs::Ref{DofDesc}, rowval=nothing)
    nnz = Ref{Int64}(0)
    rc = GC.@preserve colptr rowval subs ccall((:fe_sparsity_pattern_device, LIB), Cint,
        (Ptr{GridDesc}, Int32, Ptr{SubdomainDesc}, Ptr{DofDesc}, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}),
        grid, length(subs), subs, dofs, pointer(colptr), rowval === nothing ? C_NULL : pointer(rowval), nnz)
    rc == 0 || error("fe_sparsity_pattern_device failed with code $rc")
    return nnz[]
end

struct FacetDesc
    n_qp::Int32
    n_ref_facets::Int32
    qr_weights::Ptr{Float64}
    N::Ptr{Float64}
    dMdxi::Ptr{Float64}
    n_facets::Int64
    cells::Ptr{Int64}
    facets::Ptr{Int32}
end

mutable struct FacetSet
    ptr::Ptr{Cvoid}
    h::Handle
end

"""
    FacetSet(h, facetset, fv)

A facet set (`getfacetset(grid, name)`: FacetIndex(cell, facet) pairs) with its FacetValues
tables (`fv.fun_values.Nξ`, `fv.geo_mapping.dMdξ`, `getweights(fv.fqr, f)` per reference facet).
"""
function FacetSet(h::Handle, facetset, w::Array{Float64,2}, N::Array{Float64,3}, dM::Array{Float64,4})
    cells = Int64[first(fi) for fi in facetset]
    facets = Int32[last(fi) for fi in facetset]
    d = Ref(FacetDesc(Int32(size(w, 1)), Int32(size(w, 2)), pointer(w), pointer(N), pointer(dM),
                      length(cells), pointer(cells), pointer(facets)))
    out = Ref{Ptr{Cvoid}}(C_NULL)
    rc = GC.@preserve w N dM cells facets ccall((:fe_facet_set_create, LIB), Cint,
        (Ptr{Cvoid}, Ptr{FacetDesc}, Ptr{Ptr{Cvoid}}), h.ptr, d, out)
    check(rc, h.ptr)
    fs = FacetSet(out[], h)
    finalizer(x -> ccall((:fe_facet_set_destroy, LIB), Cvoid, (Ptr{Cvoid},), x.ptr), fs)
    return fs
end

"""
    assemble_facet_load!(f, fs; pressure, traction)

`f += ∫ N_i ⋅ (pressure n + traction) dΓ` over the set (benchmark/helper.jl:331-348,
hyperelasticity.jl:278-290 with pressure = -tn); f a CuArray.
"""
function assemble_facet_load!(f, fs::FacetSet; pressure=0.0, traction=(0.0, 0.0, 0.0), fillzero::Bool=false)
    t = collect(Float64.(traction))
    rc = GC.@preserve f t ccall((:fe_assemble_facet_load, LIB), Cint,
        (Ptr{Cvoid}, Float64, Ptr{Float64}, UInt32, Ptr{Float64}, Ptr{Cvoid}),
        fs.ptr, pressure, t, fillzero ? FE_FILLZERO : UInt32(0), pointer(f), C_NULL)
    check(rc, fs.h.ptr)
    return f
end

# ---------------------------------------------------------------------------------------
# Adjoint: vector-Jacobian products of Phi = lambda' (K(X, s) u - f(X))
# ---------------------------------------------------------------------------------------
struct AdjointParams
    physics::Int32
    precision::Int32
    flags::UInt32
    p0::Float64
    p1::Float64
    body::NTuple{3,Float64}
    cell_scale::Ptr{Float64}
    dscale::Ptr{Float64}
    stream::Ptr{Cvoid}
end

"""
    assemble_adjoint!(d_s, d_X, h, u, λ; physics, p0, p1, body, cell_scale, dscale, precision)

fe_assemble_adjoint: `d_s[c] = dscale[c] * λ_c' (∂K_c/∂s_c) u_c` for every cell (the SIMP
sensitivity of topology_optimization.jl:347-383 with `s = ρ^p`, `dscale = p ρ^(p-1)`; with
`dscale = nothing` it is ∂Φ/∂s itself), and `d_X = ∂Φ/∂X` for the node coordinates (node-major
like `grid.nodes`; `d_X = nothing` skips it). Heat and linear elasticity on linear cells.
Arrays may be host `Vector`s or device arrays.
"""
function assemble_adjoint!(d_s, d_X, h::Handle, u, λ; physics=FE_LINEAR_ELASTIC, p0=1.0, p1=0.3,
                           body=(0.0, 0.0, 0.0), cell_scale=nothing, dscale=nothing, precision=FE_PREC_MIXED)
    par = Ref(AdjointParams(physics, precision, UInt32(0), p0, p1, Tuple(Float64.(body)),
                            _ptr(cell_scale), _ptr(dscale), C_NULL))
    rc = GC.@preserve d_s d_X u λ cell_scale dscale ccall((:fe_assemble_adjoint, LIB), Cint,
        (Ptr{Cvoid}, Ptr{AdjointParams}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h.ptr, par, _ptr(u), _ptr(λ), _ptr(d_s), _ptr(d_X))
    check(rc, h.ptr)
    return d_s, d_X
end

"""
    coordinate_sensitivity(h, u, λ; kwargs...) -> d_X

`∂Φ/∂X` of `Φ = λ' (K(X, s) u - f(X))` at the handle's node coordinates, as a
`(dim, n_nodes)` matrix (the layout of `reinterpret(Float64, grid.nodes)`).
"""
function coordinate_sensitivity(h::Handle, u::Vector{Float64}, λ::Vector{Float64}; kwargs...)
    d_s = zeros(h.n_cells)
    d_X = zeros(h.dim, h.n_nodes)
    assemble_adjoint!(d_s, d_X, h, u, λ; kwargs...)
    return d_X
end

"""
    residual(h, K, s, u; physics, p0, p1, body, precision) -> r = K(s) u - f

Assembles K and f with the per-cell material factor `s` (`cell_scale`: E_c = s_c p0) into K
and a fresh f, and returns the residual. Differentiable in `s` and `u` through the
ChainRulesCore.rrule below, whose pullback for a cotangent `λ` is one adjoint kernel launch,
`s̄ = λ' ∂(K u - f)/∂s` (geometry recomputed on the device, nothing stored), and
`ū = K' λ = K λ` (K is symmetric). This replaces differentiating Ferrite's cell loop
(topology_optimization.jl:347-383): with `s = ρ.^p` the chain rule through `s` gives the SIMP
sensitivities. For the node coordinates see `coordinate_sensitivity`.
"""
function residual(h::Handle, K::SparseMatrixCSC{Float64,Int}, s::Vector{Float64}, u::Vector{Float64};
                  physics=FE_LINEAR_ELASTIC, p0=1.0, p1=0.3, body=(0.0, 0.0, 0.0), precision=FE_PREC_MIXED)
    f = zeros(size(K, 1))
    assemble_csc!(K, f, h; physics=physics, p0=p0, p1=p1, body=body, cell_scale=s, precision=precision)
    return K * u - f
end

function ChainRulesCore.rrule(::typeof(residual), h::Handle, K::SparseMatrixCSC{Float64,Int}, s::Vector{Float64},
                              u::Vector{Float64}; physics=FE_LINEAR_ELASTIC, p0=1.0, p1=0.3, body=(0.0, 0.0, 0.0),
                              precision=FE_PREC_MIXED)
    r = residual(h, K, s, u; physics=physics, p0=p0, p1=p1, body=body, precision=precision)
    # K(s) of this evaluation: the caller may re-assemble into K before the pullback runs
    Ks = SparseMatrixCSC(size(K, 1), size(K, 2), K.colptr, K.rowval, copy(nonzeros(K)))
    function residual_pullback(r̄)
        λ = Vector{Float64}(unthunk(r̄))
        s̄ = zeros(length(s))
        assemble_adjoint!(s̄, nothing, h, u, λ; physics=physics, p0=p0, p1=p1, body=body, cell_scale=s,
                          precision=precision)
        ū = Ks * λ
        return NoTangent(), NoTangent(), NoTangent(), s̄, ū
    end
    return r, residual_pullback
end

# ---------------------------------------------------------------------------------------
# CUDA graphs of repeated assemblies and the plan autotuner
# ---------------------------------------------------------------------------------------
mutable struct AssemblyGraph
    id::Int32
    h::Handle
    stream::Ptr{Cvoid}
    keep::Vector{Any}
end

"""
    capture_graph(h, steps, nzvals, fs; stream) -> AssemblyGraph

fe_graph_capture: the assemblies `steps[k]` (NamedTuples with `physics, p0, p1, body, u,
cell_scale, precision`) into `nzvals[k]`, `fs[k]` (device arrays) recorded as one CUDA graph on
`stream` (a created stream's handle, e.g. `CUDA.stream().handle`). Replaying re-reads the
buffers, so a `u` updated in place re-assembles with the new values: the Newton loop of
hyperelasticity.jl:386-420 without per-step launch overhead.
"""
function capture_graph(h::Handle, steps::AbstractVector, nzvals::AbstractVector, fs::AbstractVector; stream::Ptr{Cvoid})
    params = AssembleParams[]
    for s in steps
        push!(params, AssembleParams(Int32(get(s, :physics, FE_LINEAR_ELASTIC)), Int32(get(s, :precision, FE_PREC_MIXED)),
                                     FE_FILLZERO, Float64(get(s, :p0, 1.0)), Float64(get(s, :p1, 0.3)),
                                     Tuple(Float64.(get(s, :body, (0.0, 0.0, 0.0)))), _ptr(get(s, :cell_scale, nothing)),
                                     _ptr(get(s, :u, nothing)), 0.0, stream))
    end
    nzp = Ptr{Float64}[_ptr(x) for x in nzvals]
    fp = Ptr{Float64}[_ptr(x) for x in fs]
    id = Ref{Int32}(0)
    rc = GC.@preserve steps nzvals fs params nzp fp ccall((:fe_graph_capture, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Int32, Ptr{AssembleParams}, Ptr{Ptr{Float64}}, Ptr{Ptr{Float64}}, Ptr{Int32}),
        h.ptr, stream, Int32(length(params)), params, nzp, fp, id)
    check(rc, h.ptr)
    g = AssemblyGraph(id[], h, stream, Any[steps, nzvals, fs])
    finalizer(x -> ccall((:fe_graph_destroy, LIB), Cint, (Ptr{Cvoid}, Int32), x.h.ptr, x.id), g)
    return g
end

"""
    replay!(g::AssemblyGraph; async=false)

fe_graph_replay: all captured assemblies, reading the current contents of their buffers.
"""
function replay!(g::AssemblyGraph; async::Bool=false)
    rc = GC.@preserve g ccall((:fe_graph_replay, LIB), Cint, (Ptr{Cvoid}, Int32, Ptr{Cvoid}, UInt32),
                              g.h.ptr, g.id, g.stream, async ? FE_ASYNC : UInt32(0))
    check(rc, g.h.ptr)
    return g
end

const FE_TUNE_MAX = 16
struct TuneResult
    n_candidates::Int32
    stage_cap::NTuple{FE_TUNE_MAX,Int32}
    ms::NTuple{FE_TUNE_MAX,Float64}
    n_tiles::NTuple{FE_TUNE_MAX,Int64}
    n_cell_visits::NTuple{FE_TUNE_MAX,Int64}
    best_stage_cap::Int32
    best_ms::Float64
    form_mask::NTuple{FE_TUNE_MAX,UInt32}
    best_form_mask::UInt32
end

"""
    autotune!(h, nzval, f; stage_caps=nothing, reps=3, physics, p0, p1, body, cell_scale, u, precision)

fe_autotune: re-plan the handle for each candidate staging capacity (tile size), time `reps`
assemblies of these parameters for every assignment of the SubDofHandlers (cell types) to the
fused or two-phase form, and keep the fastest plan and form. Returns a NamedTuple with the
candidates, their times, the chosen capacity and form mask (bit s: SubDofHandler s two-phase).
"""
function autotune!(h::Handle, nzval, f; stage_caps=nothing, reps::Integer=3, physics=FE_LINEAR_ELASTIC, p0=1.0,
                   p1=0.3, body=(0.0, 0.0, 0.0), cell_scale=nothing, u=nothing, precision=FE_PREC_MIXED)
    par = Ref(AssembleParams(physics, precision, FE_FILLZERO, p0, p1, Tuple(Float64.(body)), _ptr(cell_scale),
                             _ptr(u), 0.0, C_NULL))
    caps = stage_caps === nothing ? Int32[] : Vector{Int32}(stage_caps)
    res = Ref{TuneResult}()
    rc = GC.@preserve nzval f cell_scale u caps ccall((:fe_autotune, LIB), Cint,
        (Ptr{Cvoid}, Ptr{AssembleParams}, Ptr{Float64}, Ptr{Float64}, Int32, Ptr{Int32}, Int32, Ptr{TuneResult}),
        h.ptr, par, _ptr(nzval), _ptr(f), Int32(length(caps)), isempty(caps) ? Ptr{Int32}(C_NULL) : pointer(caps),
        Int32(reps), res)
    check(rc, h.ptr)
    r = res[]
    n = Int(r.n_candidates)
    return (stage_caps=collect(r.stage_cap[1:n]), ms=collect(r.ms[1:n]), n_tiles=collect(r.n_tiles[1:n]),
            form_masks=collect(r.form_mask[1:n]), best_stage_cap=Int(r.best_stage_cap), best_ms=r.best_ms,
            best_form_mask=r.best_form_mask)
end

end # module
