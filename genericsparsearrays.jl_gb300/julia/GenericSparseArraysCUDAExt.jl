# GenericSparseArraysCUDAExt -- CUDA package extension of GenericSparseArrays.jl that sends
# sparse x dense mul!, three-argument dot, COO -> CSR/CSC conversion, sparse + dense / sparse
# sums, dropzeros and sparse x sparse products on CuArray-backed matrices to libgsa
# (include/gsa.h).  It adds methods that are more specific than the package's generated
# KernelAbstractions methods (src/matrix_csr/matrix_csr.jl:145-211,
# src/matrix_csc/matrix_csc.jl:144-213, src/matrix_coo/matrix_coo.jl:155-221,
# src/conversions/conversions.jl:171-212,282-323) for element types Float32, Float64,
# ComplexF32, ComplexF64, Int32, Int64 and index types Int32, Int64 when A, B and C share one
# element type; every other combination keeps the package's own methods.
#
# Loading: weak dependency CUDA (see the [weakdeps]/[extensions] entries in INTEGRATION.md);
# the library path comes from ENV["GSA_LIBRARY"] or deps/libgsa.so next to the package.
module GenericSparseArraysCUDAExt

using CUDA
using LinearAlgebra
using GenericSparseArrays
using GenericSparseArrays: GenericSparseMatrixCSR, GenericSparseMatrixCSC, GenericSparseMatrixCOO
using SparseArrays: SparseArrays

const libgsa = get(ENV, "GSA_LIBRARY", joinpath(@__DIR__, "..", "deps", "libgsa.so"))

const GSAValue = Union{Float32, Float64, ComplexF32, ComplexF64, Int32, Int64}
const GSAIndex = Union{Int32, Int64}

gsa_dtype(::Type{Float32}) = Cint(0)
gsa_dtype(::Type{Float64}) = Cint(1)
gsa_dtype(::Type{ComplexF32}) = Cint(2)
gsa_dtype(::Type{ComplexF64}) = Cint(3)
gsa_dtype(::Type{Int32}) = Cint(4)
gsa_dtype(::Type{Int64}) = Cint(5)
gsa_itype(::Type{Int32}) = Cint(0)
gsa_itype(::Type{Int64}) = Cint(1)

const CSRCu{T, Ti} = GenericSparseMatrixCSR{T, Ti, <:CuVector{Ti}, <:CuVector{Ti}, <:CuVector{T}}
const CSCCu{T, Ti} = GenericSparseMatrixCSC{T, Ti, <:CuVector{Ti}, <:CuVector{Ti}, <:CuVector{T}}
const COOCu{T, Ti} = GenericSparseMatrixCOO{T, Ti, <:CuVector{Ti}, <:CuVector{Ti}, <:CuVector{T}}

function gsa_check(status::Cint)
    status == 0 && return nothing
    msg = unsafe_string(ccall((:gsa_last_error_string, libgsa), Cstring, ()))
    status == 2 && throw(DimensionMismatch(msg))
    status in (1, 3, 6) && throw(ArgumentError(msg))
    return error("libgsa status $status: $msg")
end

# op(A) code and parent, following trans_adj_wrappers (src/core.jl:102-113)
_opA(A) = (A, Cint(0))
_opA(A::Transpose) = (parent(A), Cint(1))
_opA(A::Adjoint{<:Real}) = (parent(A), Cint(1))
_opA(A::Adjoint) = (parent(A), Cint(2))

# op(B) as (parent, ld, code): the parent is column-major, ld = stride(parent, 2)
_ld(P::CuVector) = max(length(P), 1)
_ld(P::CuMatrix) = max(stride(P, 2), size(P, 1), 1)
_opB(B::CuVecOrMat) = (B, _ld(B), Cint(0))
_opB(B::Transpose{<:Any, <:CuVecOrMat}) = (parent(B), _ld(parent(B)), Cint(1))
_opB(B::Adjoint{<:Real, <:CuVecOrMat}) = (parent(B), _ld(parent(B)), Cint(1))
_opB(B::Adjoint{<:Any, <:CuVecOrMat}) = (parent(B), _ld(parent(B)), Cint(2))

_ptrs(A::GenericSparseMatrixCSR) = (A.rowptr, A.colval)
_ptrs(A::GenericSparseMatrixCSC) = (A.colptr, A.rowval)
_ptrs(A::GenericSparseMatrixCOO) = (A.rowind, A.colind)
_entry(::GenericSparseMatrixCSR) = :gsa_csr_mul
_entry(::GenericSparseMatrixCSC) = :gsa_csc_mul

# Plans (gsa_plan_create): made once per compressed structure and kept beside it, keyed on
# the pointer array (the structure must not change in place while its plan lives); a
# finalizer on the key frees the plan's device memory.
const _PLANS = WeakKeyDict{Any, Ptr{Cvoid}}()
const _PLANS_LOCK = ReentrantLock()

function _plan(A::Union{GenericSparseMatrixCSR, GenericSparseMatrixCSC, GenericSparseMatrixCOO})
    ptr = A isa GenericSparseMatrixCSR ? A.rowptr : (A isa GenericSparseMatrixCSC ? A.colptr : A.rowind)
    lock(_PLANS_LOCK) do
        get!(_PLANS, ptr) do
            Ti = eltype(ptr)
            h = Ref{Ptr{Cvoid}}(C_NULL)
            if A isa GenericSparseMatrixCOO  # row pointers when the rows are sorted
                gsa_check(ccall((:gsa_coo_plan_create, libgsa), Cint,
                    (CUstream, Cint, Int64, Int64, Int64, CuPtr{Ti}, Cint, Ref{Ptr{Cvoid}}),
                    CUDA.stream(), gsa_itype(Ti), size(A, 1), size(A, 2), length(A.nzval), ptr, Cint(1), h))
            else
                outer = A isa GenericSparseMatrixCSR ? size(A, 1) : size(A, 2)
                gsa_check(ccall((:gsa_plan_create, libgsa), Cint,
                    (CUstream, Cint, Int64, Int64, CuPtr{Ti}, Cint, Ref{Ptr{Cvoid}}),
                    CUDA.stream(), gsa_itype(Ti), outer, length(A.nzval), ptr, Cint(1), h))
            end
            finalizer(_ -> ccall((:gsa_plan_destroy, libgsa), Cint, (Ptr{Cvoid},), h[]), ptr)
            h[]
        end
    end
end

_planned_entry(::GenericSparseMatrixCSR) = :gsa_csr_mul_planned
_planned_entry(::GenericSparseMatrixCSC) = :gsa_csc_mul_planned

function _gsa_mul!(C::CuVecOrMat{T}, A, B, α::Number, β::Number) where {T}
    _A, opA = _opA(A)
    P, ldb, opB = _opB(B)
    # checks in the order of the generated methods (src/matrix_csr/matrix_csr.jl:160-190)
    size(A, 2) == size(B, 1) || throw(DimensionMismatch(
        "second dimension of A, $(size(A, 2)), does not match the first dimension of B, $(size(B, 1))"))
    size(A, 1) == size(C, 1) || throw(DimensionMismatch(
        "first dimension of A, $(size(A, 1)), does not match the first dimension of C, $(size(C, 1))"))
    size(B, 2) == size(C, 2) || throw(DimensionMismatch(
        "second dimension of B, $(size(B, 2)), does not match the second dimension of C, $(size(C, 2))"))
    promote_type(eltype(A), eltype(B), typeof(α), typeof(β)) <: T || throw(ArgumentError(
        "element types of A, B, α, and β must be promotable to the element type of C"))
    Ti = eltype(_ptrs(_A)[1])
    p0, p1 = _ptrs(_A)
    a, b = Ref{T}(T(α)), Ref{T}(T(β))
    k = size(C, 2)
    ldc = C isa CuVector ? max(length(C), 1) : max(stride(C, 2), size(C, 1), 1)
    stream = CUDA.stream()
    if _A isa GenericSparseMatrixCOO  # the COO kernel, or the CSR kernels for sorted rows
        st = ccall((:gsa_coo_mul_planned, libgsa), Cint,
            (CUstream, Cint, Cint, Int64, Int64, Int64, CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Cint, Cint,
             Int64, CuPtr{T}, Int64, Cint, CuPtr{T}, Int64, Ref{T}, Ref{T}, Ptr{Cvoid}, Ptr{Cvoid},
             Csize_t),
            stream, gsa_dtype(T), gsa_itype(Ti), _A.m, _A.n, length(_A.nzval), p0, p1, _A.nzval,
            Cint(1), opA, k, P, ldb, opB, C, ldc, a, b, _plan(_A), C_NULL, Csize_t(0))
    else
        # the structure's plan; NULL workspace: libgsa takes it from the stream-ordered pool
        plan = _plan(_A)
        st = ccall((_planned_entry(_A), libgsa), Cint,
            (CUstream, Cint, Cint, Int64, Int64, Int64, CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Cint, Cint,
             Int64, CuPtr{T}, Int64, Cint, CuPtr{T}, Int64, Ref{T}, Ref{T}, Ptr{Cvoid}, Ptr{Cvoid},
             Csize_t),
            stream, gsa_dtype(T), gsa_itype(Ti), _A.m, _A.n, length(_A.nzval), p0, p1, _A.nzval,
            Cint(1), opA, k, P, ldb, opB, C, ldc, a, b, plan, C_NULL, Csize_t(0))
    end
    gsa_check(st)
    return C  # asynchronous, like the package's kernels
end

const GSAReal = Union{Float32, Float64, Int32, Int64}
const GSAComplex = Union{ComplexF32, ComplexF64}

# The package generates one method per wrapper of A and of B (trans_adj_wrappers,
# src/core.jl:102-113: plain, Transpose of a real, Transpose of a complex, Adjoint).  The
# methods here follow the same split, so each one is a strict subtype of the package method it
# replaces (CuArray storage, one element type, the same element-type bound) and more specific
# in every argument: no method ambiguity (the package runs Aqua's check, test/runtests.jl:106-111).
# (type expression, element-type bound) of each wrapper of X:
_wrappers(X) = ((X, :GSAValue), (:(Transpose{T, <:$X}), :GSAReal),
                (:(Transpose{T, <:$X}), :GSAComplex), (:(Adjoint{T, <:$X}), :GSAValue))
# the bound two wrappers share, or nothing when their bounds exclude each other
_bound(a, b) = a === :GSAValue ? b : (b === :GSAValue || a === b ? a : nothing)

for Fmt in (:CSRCu, :CSCCu, :COOCu)
    for (SA, TA) in _wrappers(:($Fmt{T, Ti})), (SB, TB) in _wrappers(:(CuVecOrMat{T}))
        Tb = _bound(TA, TB)
        Tb === nothing && continue
        @eval function LinearAlgebra.mul!(C::CuVecOrMat{T}, A::$SA, B::$SB, α::Number,
                                          β::Number) where {T <: $Tb, Ti <: GSAIndex}
            return _gsa_mul!(C, A, B, α, β)
        end
    end
end

# Three-argument dot (src/matrix_csr/matrix_csr.jl:213-277, src/matrix_csc/matrix_csc.jl:219,
# src/matrix_coo/matrix_coo.jl:227): the scalar comes back to the host.
_dot_entry(::GenericSparseMatrixCSR) = :gsa_csr_dot
_dot_entry(::GenericSparseMatrixCSC) = :gsa_csc_dot

function _gsa_dot(x::CuVector{T}, A, y::CuVector{T}) where {T}
    _A, opA = _opA(A)
    size(A, 1) == length(x) || throw(DimensionMismatch(
        "first dimension of A, $(size(A, 1)), does not match the length of x, $(length(x))"))
    size(A, 2) == length(y) || throw(DimensionMismatch(
        "second dimension of A, $(size(A, 2)), does not match the length of y, $(length(y))"))
    Ti = eltype(_ptrs(_A)[1])
    p0, p1 = _ptrs(_A)
    r = Ref{T}(zero(T))
    if _A isa GenericSparseMatrixCOO
        st = ccall((:gsa_coo_dot, libgsa), Cint,
            (CUstream, Cint, Cint, Int64, Int64, Int64, CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Cint, Cint,
             CuPtr{T}, CuPtr{T}, Ref{T}, Ptr{Cvoid}, Ptr{Cvoid}, Csize_t),
            CUDA.stream(), gsa_dtype(T), gsa_itype(Ti), _A.m, _A.n, length(_A.nzval), p0, p1,
            _A.nzval, Cint(1), opA, x, y, r, _plan(_A), C_NULL, Csize_t(0))
    else
        st = ccall((_dot_entry(_A), libgsa), Cint,
            (CUstream, Cint, Cint, Int64, Int64, Int64, CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Cint, Cint,
             CuPtr{T}, CuPtr{T}, Ref{T}, Ptr{Cvoid}, Ptr{Cvoid}, Csize_t),
            CUDA.stream(), gsa_dtype(T), gsa_itype(Ti), _A.m, _A.n, length(_A.nzval), p0, p1,
            _A.nzval, Cint(1), opA, x, y, r, _plan(_A), C_NULL, Csize_t(0))
    end
    gsa_check(st)
    return r[]
end

for Fmt in (:CSRCu, :CSCCu, :COOCu)
    for (SA, TA) in _wrappers(:($Fmt{T, Ti}))  # one method per package method, as for mul!
        @eval LinearAlgebra.dot(x::CuVector{T}, A::$SA, y::CuVector{T}) where {T <: $TA, Ti <: GSAIndex} =
            _gsa_dot(x, A, y)
    end
end

# Batched products: many mul!(C_i, A_i, B_i, α_i, β_i) of one element and index type in
# one grouped launch, replayed from a CUDA graph (gsa_batch_*).  Not a method of the
# reference; an addition for callers with thousands of small products.
struct GsaGroupItem  # 144 bytes, field order of gsa_group_item
    rowptr::CuPtr{Cvoid}; colval::CuPtr{Cvoid}; nzval::CuPtr{Cvoid}; B::CuPtr{Cvoid}; C::CuPtr{Cvoid}
    m::Int64; n::Int64; nnz::Int64; ldb::Int64; ldc::Int64; k::Int32; b_rowmajor::Int32
    first_tile::Int64
    bin_order::Ptr{Cvoid}; bin_warps::Int64
    alpha::NTuple{16, UInt8}; beta::NTuple{16, UInt8}
end

_bytes16(v::T) where {T} = ntuple(i -> i <= sizeof(T) ? reinterpret(NTuple{sizeof(T), UInt8}, v)[i] : 0x00, 16)

mutable struct GroupedMul{T, Ti}
    handle::Ptr{Cvoid}
    keep::Vector{Any}  # the operands stay alive while the batch does
end

function GroupedMul(products::AbstractVector) # [(C, A::CSRCu, B::CuVecOrMat, α, β), ...]
    T = eltype(products[1][1]); Ti = eltype(products[1][2].rowptr)
    items = GsaGroupItem[]
    for (C, A, B, α, β) in products
        ldb = B isa CuVector ? max(length(B), 1) : max(stride(B, 2), size(B, 1), 1)
        ldc = C isa CuVector ? max(length(C), 1) : max(stride(C, 2), size(C, 1), 1)
        view, warps = Ref{Ptr{Cvoid}}(C_NULL), Ref{Int64}(0)
        if T === ComplexF64  # FP64-bound: walk the plan's bin order
            gsa_check(ccall((:gsa_plan_bin_order, libgsa), Cint, (Ptr{Cvoid}, Ref{Ptr{Cvoid}}, Ref{Int64}),
                            _plan(A), view, warps))
        end
        push!(items, GsaGroupItem(pointer(A.rowptr), pointer(A.colval), pointer(A.nzval), pointer(B),
                                  pointer(C), size(A, 1), size(A, 2), length(A.nzval), ldb, ldc,
                                  Int32(size(C, 2)), Int32(0), 0, view[], warps[],
                                  _bytes16(T(α)), _bytes16(T(β))))
    end
    h = Ref{Ptr{Cvoid}}(C_NULL)
    gsa_check(ccall((:gsa_batch_create, libgsa), Cint,
        (CUstream, Cint, Cint, Cint, Ptr{GsaGroupItem}, Int64, Cint, Cint, Ref{Ptr{Cvoid}}),
        CUDA.stream(), gsa_dtype(T), gsa_itype(Ti), Cint(1), items, length(items), Cint(0), Cint(0), h))
    g = GroupedMul{T, Ti}(h[], Any[products])
    finalizer(g -> ccall((:gsa_batch_destroy, libgsa), Cint, (Ptr{Cvoid},), g.handle), g)
    return g
end

# mode 0: one grouped launch, 1: replay of its captured CUDA graph, 2: one mul! per product
run!(g::GroupedMul; mode::Integer = 1) =
    gsa_check(ccall((:gsa_batch_run, libgsa), Cint, (Ptr{Cvoid}, CUstream, Cint), g.handle,
                    CUDA.stream(), Cint(mode)))

# COO -> CSR / CSC (src/conversions/conversions.jl:171-212, 282-323)
for (Out, entry, colmajor) in ((:GenericSparseMatrixCSR, :gsa_coo_to_csr, 0),
                               (:GenericSparseMatrixCSC, :gsa_coo_to_csc, 1))
    @eval function GenericSparseArrays.$Out(A::COOCu{T, Ti}) where {T <: GSAValue, Ti <: GSAIndex}
        m, n = size(A)
        nz = length(A.nzval)
        major = $colmajor == 1 ? n : m
        ptr = CuVector{Ti}(undef, major + 1)
        idx = CuVector{Ti}(undef, nz)
        val = CuVector{T}(undef, nz)
        st = ccall(($(QuoteNode(entry)), libgsa), Cint,
            (CUstream, Cint, Cint, Int64, Int64, Int64, CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Cint,
             CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Ptr{Cvoid}, Csize_t),
            CUDA.stream(), gsa_dtype(T), gsa_itype(Ti), m, n, nz, A.rowind, A.colind, A.nzval,
            Cint(1), ptr, idx, val, C_NULL, Csize_t(0))
        gsa_check(st)
        return $Out(m, n, ptr, idx, val)
    end
end

# CSR / CSC -> COO (src/conversions/conversions.jl:153-169, 264-280)
for (In, entry) in ((:CSRCu, :gsa_csr_to_coo), (:CSCCu, :gsa_csc_to_coo))
    @eval function GenericSparseArrays.GenericSparseMatrixCOO(A::$In{T, Ti}) where {T <: GSAValue, Ti <: GSAIndex}
        m, n = size(A)
        nz = length(A.nzval)
        p0, p1 = _ptrs(A)
        r = CuVector{Ti}(undef, nz)
        c = CuVector{Ti}(undef, nz)
        v = CuVector{T}(undef, nz)
        st = ccall(($(QuoteNode(entry)), libgsa), Cint,
            (CUstream, Cint, Cint, Int64, Int64, Int64, CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Cint,
             CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}),
            CUDA.stream(), gsa_dtype(T), gsa_itype(Ti), m, n, nz, p0, p1, A.nzval, Cint(1), r, c, v)
        gsa_check(st)
        return GenericSparseMatrixCOO(m, n, r, c, v)
    end
end

# Sparse x sparse (src/matrix_csr/matrix_csr.jl:498-556, src/matrix_csc/matrix_csc.jl:500-560).
# The reference's COO and transposed methods convert their operands and call these.
for (Fmt, fmt) in ((:CSRCu, 0), (:CSCCu, 1))
    @eval function Base.:(*)(A::$Fmt{T, Ti}, B::$Fmt{T, Ti}) where {T <: GSAValue, Ti <: GSAIndex}
        size(A, 2) == size(B, 1) || throw(DimensionMismatch(
            "second dimension of A, $(size(A, 2)), does not match first dimension of B, $(size(B, 1))"))
        m, k, n = size(A, 1), size(A, 2), size(B, 2)
        pa, ia = _ptrs(A)
        pb, ib = _ptrs(B)
        ptr = CuVector{Ti}(undef, ($fmt == 0 ? m : n) + 1)
        nnz_c = Ref{Int64}(0)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        gsa_check(ccall((:gsa_spgemm_create, libgsa), Cint,
            (CUstream, Cint, Cint, Cint, Int64, Int64, Int64, CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Int64,
             CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Int64, Cint, CuPtr{Ti}, Ref{Int64}, Ref{Ptr{Cvoid}}),
            CUDA.stream(), Cint($fmt), gsa_dtype(T), gsa_itype(Ti), m, k, n, pa, ia, A.nzval,
            length(A.nzval), pb, ib, B.nzval, length(B.nzval), Cint(1), ptr, nnz_c, h))
        idx = CuVector{Ti}(undef, nnz_c[])
        val = CuVector{T}(undef, nnz_c[])
        try
            gsa_check(ccall((:gsa_spgemm_compute, libgsa), Cint, (CUstream, Ptr{Cvoid}, CuPtr{Ti}, CuPtr{T}),
                            CUDA.stream(), h[], idx, val))
        finally
            ccall((:gsa_spgemm_destroy, libgsa), Cint, (Ptr{Cvoid},), h[])
        end
        return $(Fmt === :CSRCu ? :GenericSparseMatrixCSR : :GenericSparseMatrixCSC)(m, n, ptr, idx, val)
    end
end

# COO sums (src/matrix_coo/matrix_coo.jl:300-385 A + B, :387-458 A + λI), dropzeros included:
# one sort of the sources where they lie, in-order run sums, zero sums dropped.
function _coo_sum(m, n, A::COOCu{T, Ti}, opa, B, opb, ndiag, λ::T) where {T, Ti}
    na = length(A.nzval)
    nb = B === nothing ? 0 : length(B.nzval)
    total = na + nb + ndiag
    ws = CuVector{UInt8}(undef, ccall((:gsa_coo_sum_workspace_size, libgsa), Csize_t,
                                      (Cint, Int64, Int64, Int64), gsa_dtype(T), m, n, total))
    kept = Ref{Int64}(0)
    nul = CU_NULL
    gsa_check(ccall((:gsa_coo_sum_count, libgsa), Cint,
        (CUstream, Cint, Cint, Int64, Int64, Int64, CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Cint, Int64,
         CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Cint, Int64, Ref{T}, Cint, CuPtr{UInt8}, Csize_t, Ref{Int64}),
        CUDA.stream(), gsa_dtype(T), gsa_itype(Ti), m, n, na, A.rowind, A.colind, A.nzval, opa, nb,
        B === nothing ? nul : B.rowind, B === nothing ? nul : B.colind, B === nothing ? nul : B.nzval,
        opb, ndiag, Ref(λ), Cint(1), ws, length(ws), kept))
    r = CuVector{Ti}(undef, kept[]); c = CuVector{Ti}(undef, kept[]); v = CuVector{T}(undef, kept[])
    gsa_check(ccall((:gsa_coo_sum_copy, libgsa), Cint,
        (CUstream, Cint, Cint, Int64, Int64, Int64, Int64, Cint, CuPtr{UInt8}, CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}),
        CUDA.stream(), gsa_dtype(T), gsa_itype(Ti), m, n, total, kept[], Cint(1), ws, r, c, v))
    return GenericSparseMatrixCOO(m, n, r, c, v)
end

function Base.:+(A::COOCu{T, Ti}, B::COOCu{T, Ti}) where {T <: GSAValue, Ti <: GSAIndex}
    size(A) == size(B) || throw(DimensionMismatch(
        "dimensions must match: A has dims $(size(A)), B has dims $(size(B))"))
    return _coo_sum(size(A)..., A, Cint(0), B, Cint(0), 0, zero(T))
end

# Any J whose λ promotes to the matrix's element type (I, -I, 2.0I on a Float64 matrix ...):
# the reference's result type is promote_type(Tv, typeof(λ)) (src/matrix_coo/matrix_coo.jl:399);
# when that is wider than T, the package's own method runs.
function Base.:+(A::COOCu{T, Ti}, J::UniformScaling{S}) where {T <: GSAValue, Ti <: GSAIndex, S}
    promote_type(T, S) === T ||
        return invoke(Base.:+, Tuple{GenericSparseMatrixCOO, UniformScaling}, A, J)
    m, n = size(A)
    m == n || throw(DimensionMismatch("Matrix must be square to add UniformScaling."))
    iszero(J.λ) && return copy(A)
    return _coo_sum(m, n, A, Cint(0), nothing, Cint(0), n, T(J.λ))
end

# CSR + CSR, CSC + CSC (src/matrix_csr/matrix_csr.jl:290-356, then dropzeros) and A + λI
# (:358-402): the reference's per-row walks, counted, scanned and written on the GPU.
function _compressed_sum(A::Union{CSRCu{T, Ti}, CSCCu{T, Ti}}, B, λ) where {T, Ti}
    csr = A isa GenericSparseMatrixCSR
    outer = csr ? size(A, 1) : size(A, 2)
    pa, ia = _ptrs(A)
    pb, ib = B === nothing ? (CU_NULL, CU_NULL) : _ptrs(B)
    ws = CuVector{UInt8}(undef, ccall((:gsa_compressed_add_workspace_size, libgsa), Csize_t, (Int64,), outer))
    ptr = CuVector{Ti}(undef, outer + 1)
    cnt = Ref{Int64}(0)
    gsa_check(ccall((:gsa_compressed_add_count, libgsa), Cint,
        (CUstream, Cint, Int64, CuPtr{Ti}, CuPtr{Ti}, CuPtr{Ti}, CuPtr{Ti}, Cint, CuPtr{UInt8}, Csize_t, CuPtr{Ti},
         Ref{Int64}), CUDA.stream(), gsa_itype(Ti), outer, pa, ia, pb, ib, Cint(1), ws, length(ws), ptr, cnt))
    idx = CuVector{Ti}(undef, cnt[]); val = CuVector{T}(undef, cnt[])
    gsa_check(ccall((:gsa_compressed_add_copy, libgsa), Cint,
        (CUstream, Cint, Cint, Int64, CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Cint,
         Ptr{T}, Cint, CuPtr{UInt8}, CuPtr{Ti}, CuPtr{T}),
        CUDA.stream(), gsa_dtype(T), gsa_itype(Ti), outer, pa, ia, A.nzval, pb, ib,
        B === nothing ? CU_NULL : B.nzval, Cint(0), λ === nothing ? C_NULL : Ref(T(λ)), Cint(1), ws, idx, val))
    C = (csr ? GenericSparseMatrixCSR : GenericSparseMatrixCSC)(size(A)..., ptr, idx, val)
    return B === nothing ? C : dropzeros(C)
end

for (Fmt, Parent) in ((:CSRCu, :GenericSparseMatrixCSR), (:CSCCu, :GenericSparseMatrixCSC))
    @eval function Base.:+(A::$Fmt{T, Ti}, B::$Fmt{T, Ti}) where {T <: GSAValue, Ti <: GSAIndex}
        size(A) == size(B) || throw(DimensionMismatch(
            "dimensions must match: A has dims $(size(A)), B has dims $(size(B))"))
        return _compressed_sum(A, B, nothing)
    end
    # as for COO: J's λ must promote to T (src/matrix_csr/matrix_csr.jl:358-402), else the
    # package's own method
    @eval function Base.:+(A::$Fmt{T, Ti}, J::UniformScaling{S}) where {T <: GSAValue, Ti <: GSAIndex, S}
        promote_type(T, S) === T || return invoke(Base.:+, Tuple{$Parent, UniformScaling}, A, J)
        m, n = size(A)
        m == n || throw(DimensionMismatch("Matrix must be square to add UniformScaling."))
        iszero(J.λ) && return copy(A)
        return _compressed_sum(A, nothing, T(J.λ))
    end
end

# dropzeros (src/matrix_csr/matrix_csr.jl:649-745 and the CSC / COO methods): flags, one scan,
# a compaction; the count comes back to the host so the outputs can be allocated.
_fmt(::GenericSparseMatrixCSR) = Cint(0)
_fmt(::GenericSparseMatrixCSC) = Cint(1)
_fmt(::GenericSparseMatrixCOO) = Cint(2)
_parts(A::GenericSparseMatrixCSR) = (A.rowptr, A.colval, size(A, 1))
_parts(A::GenericSparseMatrixCSC) = (A.colptr, A.rowval, size(A, 2))
_parts(A::GenericSparseMatrixCOO) = (A.rowind, A.colind, 0)

# one method per format, each a subtype of the package's method for that format
for Fmt in (:CSRCu, :CSCCu, :COOCu)
    @eval SparseArrays.dropzeros(A::$Fmt{T, Ti}) where {T <: GSAValue, Ti <: GSAIndex} = _gsa_dropzeros(A)
end

function _gsa_dropzeros(A::Union{CSRCu{T, Ti}, CSCCu{T, Ti}, COOCu{T, Ti}}) where {T, Ti}
    nz = length(A.nzval)
    p0, p1, outer = _parts(A)
    ws = CuVector{UInt8}(undef, ccall((:gsa_dropzeros_workspace_size, libgsa), Csize_t, (Int64,), nz))
    kept = Ref{Int64}(0)
    gsa_check(ccall((:gsa_dropzeros_count, libgsa), Cint, (CUstream, Cint, Int64, CuPtr{T}, CuPtr{UInt8}, Csize_t,
                    Ref{Int64}), CUDA.stream(), gsa_dtype(T), nz, A.nzval, ws, length(ws), kept))
    o0 = CuVector{Ti}(undef, A isa GenericSparseMatrixCOO ? kept[] : outer + 1)
    o1 = CuVector{Ti}(undef, kept[]); ov = CuVector{T}(undef, kept[])
    gsa_check(ccall((:gsa_dropzeros_copy, libgsa), Cint,
        (CUstream, Cint, Cint, Cint, Int64, Int64, CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Cint, CuPtr{UInt8}, CuPtr{Ti},
         CuPtr{Ti}, CuPtr{T}), CUDA.stream(), _fmt(A), gsa_dtype(T), gsa_itype(Ti), outer, nz, p0, p1, A.nzval,
        Cint(1), ws, o0, o1, ov))
    return typeof(A).name.wrapper(size(A)..., o0, o1, ov)
end

# A + B for a dense B (src/core.jl:66-88): C = copy(B), then every stored entry added.
function Base.:+(A::Union{CSRCu{T, Ti}, CSCCu{T, Ti}, COOCu{T, Ti}}, B::CuMatrix{T}) where {T <: GSAValue, Ti <: GSAIndex}
    size(A) == size(B) || throw(DimensionMismatch(
        "dimensions must match: A has dims $(size(A)), B has dims $(size(B))"))
    C = copy(B)
    p0, p1, _ = _parts(A)
    gsa_check(ccall((:gsa_add_to_dense, libgsa), Cint,
        (CUstream, Cint, Cint, Cint, Int64, Int64, Int64, CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Cint, CuPtr{T}, Int64),
        CUDA.stream(), _fmt(A), gsa_dtype(T), gsa_itype(Ti), size(A)..., length(A.nzval), p0, p1, A.nzval, Cint(1),
        C, max(stride(C, 2), 1)))
    return C
end

end # module
