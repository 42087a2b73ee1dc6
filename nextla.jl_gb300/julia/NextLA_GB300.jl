"""
    NextLA_GB300

Julia binding of `libnextla_gb300.so`, the sm_103a implementation of NextLA.jl's
recursive triangular solve / multiply.  It keeps the reference's entry point
`unified_rectrxm!(side, uplo, transpose, alpha, func, A, B)` (src/rectrxm.jl:43-76)
for `CuArray`s (and strided views / `Transpose` wrappers of them) and reaches the
CUDA kernels through `ccall` on the C ABI declared in include/nextla_gb300.h.

Two forms are provided:
  * `unified_rectrxm!` drives the whole recursion inside the library (one
    `ccall` per call, `nla_trxm`);
  * `unified_rectrxm_julia!` runs the recursion here, like the reference's
    `unified_rec` (src/rectrxm.jl:101-198), with one `ccall` per base case
    (`nla_diag_block`) and per update (`nla_gemm_update`).
Both enqueue on `CUDA.stream()` and return without synchronising, as the
reference's kernel launches do.
"""
module NextLA_GB300

using CUDA
using LinearAlgebra

export unified_rectrxm!, unified_rectrxm_julia!, unified_rectrxm_mixed!, unified_rectrxm_mixed_host!, trsm, trmm,
       getrf2_trsm!

const libnla = get(ENV, "NEXTLA_GB300_LIB", joinpath(@__DIR__, "..", "libnextla_gb300.so"))

const NLA_F16 = Cint(0)
const NLA_F32 = Cint(1)
const NLA_F64 = Cint(2)
const NLA_C32 = Cint(3)
const NLA_C64 = Cint(4)

dtype_code(::Type{Float16}) = NLA_F16
dtype_code(::Type{Float32}) = NLA_F32
dtype_code(::Type{Float64}) = NLA_F64
dtype_code(::Type{ComplexF32}) = NLA_C32
dtype_code(::Type{ComplexF64}) = NLA_C64

function check(rc::Cint)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:nla_last_error, libnla), Cstring, ()))
    (rc == -1 || rc == -2) && throw(ArgumentError(msg))
    error("libnextla_gb300 status $rc: $msg")
end

# (device pointer, leading dimension, transposed) of a column-major operand.
operand(A::CuArray{T,2}) where {T} = (pointer(A), max(stride(A, 2), 1), false)
function operand(A::SubArray{T,2,<:CuArray{T}}) where {T}
    stride(A, 1) == 1 || throw(ArgumentError("views must have unit stride along the first dimension"))
    return (pointer(A), max(stride(A, 2), 1), false)
end
function operand(A::Union{Transpose,Adjoint})
    p, ld, t = operand(parent(A))
    return (p, ld, !t)
end

stream_handle() = CUDA.stream().handle

"""
    unified_rectrxm!(side, uplo, transpose, alpha, func, A, B) -> B

Drop-in for NextLA.unified_rectrxm! on CuArrays of Float16/32/64: solves
op(A) X = alpha B ('S') or forms B := alpha op(A) B ('M') (or the right-side
forms) in place in B.
"""
function unified_rectrxm!(side::Char, uplo::Char, transpose::Char, alpha::Number, func::Char,
                          A::AbstractMatrix{T}, B::AbstractMatrix{T}) where {T<:Union{Float16,Float32,Float64}}
    n = size(A, 1)
    m = side == 'L' ? size(B, 2) : size(B, 1)
    pA, lda, tA = operand(A)
    pB, ldb, tB = operand(B)
    tB && throw(ArgumentError("B must be column-major"))
    tr, up = transpose, uplo
    if tA  # A arrived as a Transpose wrapper: fold it into the flags
        tr = transpose in ('T', 'C') ? 'N' : 'T'
        up = uplo == 'L' ? 'U' : 'L'
    end
    check(ccall((:nla_trxm, libnla), Cint,
                (Cchar, Cchar, Cchar, Cdouble, Cchar, Cint, Int64, Int64, CuPtr{Cvoid}, Int64, CuPtr{Cvoid}, Int64,
                 Ptr{Cvoid}),
                side, up, tr, Float64(alpha), func, dtype_code(T), n, m, pA, lda, pB, ldb, stream_handle()))
    return B
end

"""
    unified_rectrxm!(side, uplo, transpose, alpha, func, A, B) -> B   (ComplexF32, ComplexF64)

The same for complex CuArrays (`nla_trxm_complex`): the reference's
unified_rec takes only real element types (src/rectrxm.jl:101), though its
base-case docstrings list complex ones (src/trsm.jl:180-183).  transpose 'C'
applies the Adjoint; alpha may be complex.  A plain (not Transpose or
Adjoint) A is expected.
"""
function unified_rectrxm!(side::Char, uplo::Char, transpose::Char, alpha::Number, func::Char,
                          A::AbstractMatrix{T}, B::AbstractMatrix{T}) where {T<:Union{ComplexF32,ComplexF64}}
    n = size(A, 1)
    m = side == 'L' ? size(B, 2) : size(B, 1)
    pA, lda, tA = operand(A)
    pB, ldb, tB = operand(B)
    (tA || tB) && throw(ArgumentError("pass A and B as plain column-major arrays and use `transpose`"))
    a = ComplexF64(alpha)
    check(ccall((:nla_trxm_complex, libnla), Cint,
                (Cchar, Cchar, Cchar, Cdouble, Cdouble, Cchar, Cint, Int64, Int64, CuPtr{Cvoid}, Int64, CuPtr{Cvoid},
                 Int64, Ptr{Cvoid}),
                side, uplo, transpose, real(a), imag(a), func, dtype_code(T), n, m, pA, lda, pB, ldb,
                stream_handle()))
    return B
end

"""
    trsm(side, uplo, transa, diag, A, B, alpha=one(eltype(A))) -> B
    trmm(side, uplo, transa, diag, A, B, alpha=one(eltype(A))) -> B

The reference's wrappers (src/trsm.jl:186-204, src/trmm.jl:430-448) with the
same arguments, run through the recursion (`nla_trxm_diag`): transa is applied
and diag 'U' takes the diagonal of A as ones (the reference accepts both but
calls one base-case kernel with op(A) = A and the stored diagonal).
"""
function trxm_diag!(func::Char, side::Char, uplo::Char, transa::Char, diag::Char,
                    A::AbstractMatrix{T}, B::AbstractMatrix{T}, alpha) where {T<:Union{Float16,Float32,Float64}}
    n = size(A, 1)
    m = side == 'L' ? size(B, 2) : size(B, 1)
    pA, lda, tA = operand(A)
    pB, ldb, tB = operand(B)
    tB && throw(ArgumentError("B must be column-major"))
    tr, up = transa, uplo
    if tA
        tr = transa in ('T', 'C') ? 'N' : 'T'
        up = uplo == 'L' ? 'U' : 'L'
    end
    check(ccall((:nla_trxm_diag, libnla), Cint,
                (Cchar, Cchar, Cchar, Cchar, Cdouble, Cchar, Cint, Int64, Int64, CuPtr{Cvoid}, Int64, CuPtr{Cvoid},
                 Int64, Ptr{Cvoid}),
                side, up, tr, diag, Float64(alpha), func, dtype_code(T), n, m, pA, lda, pB, ldb, stream_handle()))
    return B
end
trsm(side, uplo, transa, diag, A, B, alpha=one(eltype(A))) = trxm_diag!('S', side, uplo, transa, diag, A, B, alpha)
trmm(side, uplo, transa, diag, A, B, alpha=one(eltype(A))) = trxm_diag!('M', side, uplo, transa, diag, A, B, alpha)

# --- the reference's recursion driven from Julia ------------------------------

function diag_block!(func, side, uplo, A, B::AbstractMatrix{T}) where {T}
    n = size(A, 1)
    m = side == 'L' ? size(B, 2) : size(B, 1)
    pA, lda, tA = operand(A)
    pB, ldb, _ = operand(B)
    check(ccall((:nla_diag_block, libnla), Cint,
                (Cchar, Cchar, Cchar, Cint, Cint, Int64, Int64, CuPtr{Cvoid}, Int64, CuPtr{Cvoid}, Int64, Ptr{Cvoid}),
                func, side, uplo, Cint(tA), dtype_code(T), n, m, pA, lda, pB, ldb, stream_handle()))
end

# matmul!(output, input1, input2, ..., alpha) of src/matmul.jl:5-66
function matmul!(output::AbstractMatrix{T}, input1, input2, alpha) where {T}
    N, M = size(output)
    R = size(input1, 2)
    p1, ld1, t1 = operand(input1)
    p2, ld2, t2 = operand(input2)
    po, ldo, _ = operand(output)
    check(ccall((:nla_gemm_update, libnla), Cint,
                (Cint, Cint, Cint, Int64, Int64, Int64, Cdouble, CuPtr{Cvoid}, Int64, CuPtr{Cvoid}, Int64, CuPtr{Cvoid},
                 Int64, Ptr{Cvoid}),
                dtype_code(T), Cint(t1), Cint(t2), N, R, M, Float64(alpha), p1, ld1, p2, ld2, po, ldo, stream_handle()))
end

GEMM_ADD!(A, B, C) = matmul!(C, A, B, 1.0)   # src/matmul.jl:69-74
GEMM_SUB!(A, B, C) = matmul!(A, B, C, -1.0)  # src/matmul.jl:76-81

function rec!(func, side, uplo, A, n, B, threshold)
    if n <= threshold
        diag_block!(func, side, uplo, A, B)
        return B
    end
    mid = ispow2(n) ? div(n, 2) : prevpow(2, n)
    A11 = view(A, 1:mid, 1:mid); A22 = view(A, mid+1:n, mid+1:n)
    A21 = view(A, mid+1:n, 1:mid); A12 = view(A, 1:mid, mid+1:n)
    B1, B2 = side == 'L' ? (view(B, 1:mid, :), view(B, mid+1:n, :)) : (view(B, :, 1:mid), view(B, :, mid+1:n))
    if (side == 'L' && uplo == 'L' && func == 'S') || (side == 'R' && uplo == 'U' && func == 'S') ||
       (side == 'L' && uplo == 'U' && func == 'M') || (side == 'R' && uplo == 'L' && func == 'M')
        rec!(func, side, uplo, A11, mid, B1, threshold)
        side == 'L' ? (func == 'S' ? GEMM_SUB!(B2, A21, B1) : GEMM_ADD!(A12, B2, B1)) :
                      (func == 'S' ? GEMM_SUB!(B2, B1, A12) : GEMM_ADD!(B2, A21, B1))
        rec!(func, side, uplo, A22, n - mid, B2, threshold)
    else
        rec!(func, side, uplo, A22, n - mid, B2, threshold)
        side == 'L' ? (func == 'S' ? GEMM_SUB!(B1, A12, B2) : GEMM_ADD!(A21, B1, B2)) :
                      (func == 'S' ? GEMM_SUB!(B1, B2, A21) : GEMM_ADD!(B1, A12, B2))
        rec!(func, side, uplo, A11, mid, B1, threshold)
    end
    return B
end

function scale!(B::AbstractMatrix{T}, alpha) where {T}
    pB, ldb, _ = operand(B)
    check(ccall((:nla_scale, libnla), Cint, (Cint, Int64, Int64, Cdouble, CuPtr{Cvoid}, Int64, Ptr{Cvoid}),
                dtype_code(T), size(B, 1), size(B, 2), Float64(alpha), pB, ldb, stream_handle()))
end

"""
    unified_rectrxm_julia!(side, uplo, transpose, alpha, func, A, B) -> B

The reference's host recursion (thresholds 256 / 16) in Julia, one `ccall`
per base case and per update.
"""
function unified_rectrxm_julia!(side::Char, uplo::Char, transpose::Char, alpha::Number, func::Char,
                                A::AbstractMatrix{T}, B::AbstractMatrix{T}) where {T<:Union{Float16,Float32,Float64}}
    threshold = 16
    n = size(A, 1)
    if transpose == 'T' || transpose == 'C'
        A = Transpose(A)
        uplo = uplo == 'L' ? 'U' : 'L'
    end
    if func == 'S'
        threshold = 256
        scale!(B, alpha)
    end
    rec!(func, side, uplo, A, n, B, threshold)
    func == 'M' && scale!(B, alpha)
    return B
end

# --- mixed-precision form ------------------------------------------------------

struct MixedOpts
    lowp::Cint
    split_terms::Cint
    sweeps::Cint
    residual::Cint
    cutoff::Int64
    corr_out::Ptr{Cdouble}
end

"""
    unified_rectrxm_mixed!(side, uplo, transpose, alpha, func, A, B; lowp=:bf16, split_terms=3, sweeps=2)

FP64 answer for Float64 CuArrays with the updates on the tensor cores
(`nla_trxm_mixed`).
"""
function unified_rectrxm_mixed!(side::Char, uplo::Char, transpose::Char, alpha::Number, func::Char,
                                A::CuMatrix{Float64}, B::CuMatrix{Float64};
                                lowp::Symbol=:bf16, split_terms::Integer=3, sweeps::Integer=2,
                                residual::Symbol=:split, cutoff::Integer=0)
    opts = Ref(MixedOpts(lowp == :bf16 ? 0 : 1, split_terms, sweeps, residual == :split ? 1 : 0, cutoff, C_NULL))
    n = size(A, 1)
    m = side == 'L' ? size(B, 2) : size(B, 1)
    check(ccall((:nla_trxm_mixed, libnla), Cint,
                (Cchar, Cchar, Cchar, Cdouble, Cchar, Int64, Int64, CuPtr{Cdouble}, Int64, CuPtr{Cdouble}, Int64,
                 Ref{MixedOpts}, Ptr{Cvoid}),
                side, uplo, transpose, Float64(alpha), func, n, m, pointer(A), stride(A, 2), pointer(B), stride(B, 2),
                opts, stream_handle()))
    return B
end

"""
    unified_rectrxm_mixed_host!(side, uplo, transpose, alpha, func, A, B; split_terms=7, sweeps=0)

The mixed form on host `Matrix{Float64}` arrays (`nla_trxm_mixed_host`): the
copies of A's triangle and B in and of the result out overlap the solve, and
the result overwrites `B`. Pin `A` and `B` (`CUDA.Mem.pin`) for the overlap.
Returns once `B` holds the result.
"""
function unified_rectrxm_mixed_host!(side::Char, uplo::Char, transpose::Char, alpha::Number, func::Char,
                                     A::Matrix{Float64}, B::Matrix{Float64};
                                     lowp::Symbol=:bf16, split_terms::Integer=7, sweeps::Integer=0,
                                     residual::Symbol=:split, cutoff::Integer=0, host_levels::Integer=0)
    opts = Ref(MixedOpts(lowp == :bf16 ? 0 : 1, split_terms, sweeps, residual == :split ? 1 : 0, cutoff, C_NULL))
    n = size(A, 1)
    m = side == 'L' ? size(B, 2) : size(B, 1)
    dA = CuMatrix{Float64}(undef, size(A))
    dB = CuMatrix{Float64}(undef, size(B))
    check(ccall((:nla_trxm_mixed_host, libnla), Cint,
                (Cchar, Cchar, Cchar, Cdouble, Cchar, Int64, Int64, Ptr{Cdouble}, Int64, Ptr{Cdouble}, Int64,
                 Ptr{Cdouble}, Int64, CuPtr{Cdouble}, Int64, CuPtr{Cdouble}, Int64, Ref{MixedOpts}, Cint, Ptr{Cvoid}),
                side, uplo, transpose, Float64(alpha), func, n, m, pointer(A), max(stride(A, 2), 1), pointer(B),
                max(stride(B, 2), 1), pointer(B), max(stride(B, 2), 1), pointer(dA), max(stride(dA, 2), 1),
                pointer(dB), max(stride(dB, 2), 1), opts, host_levels, stream_handle()))
    CUDA.synchronize()
    return B
end

"""
    trxm_mixed_diag!(func, side, uplo, transa, diag, A, B, alpha)

Float64 trsm/trmm with exact tensor-core updates (`nla_trxm_mixed_diag`):
diag 'U' takes A's diagonal as ones and never reads it.
"""
function trxm_mixed_diag!(func::Char, side::Char, uplo::Char, transa::Char, diag::Char,
                          A::AbstractMatrix{Float64}, B::AbstractMatrix{Float64}, alpha)
    n = size(A, 1)
    m = side == 'L' ? size(B, 2) : size(B, 1)
    pA, lda, tA = operand(A)
    pB, ldb, tB = operand(B)
    tB && throw(ArgumentError("B must be column-major"))
    tr, up = transa, uplo
    if tA
        tr = transa in ('T', 'C') ? 'N' : 'T'
        up = uplo == 'L' ? 'U' : 'L'
    end
    opts = Ref(MixedOpts(0, 7, 0, 1, 0, C_NULL))
    check(ccall((:nla_trxm_mixed_diag, libnla), Cint,
                (Cchar, Cchar, Cchar, Cchar, Cdouble, Cchar, Int64, Int64, CuPtr{Cvoid}, Int64, CuPtr{Cvoid}, Int64,
                 Ref{MixedOpts}, Ptr{Cvoid}),
                side, up, tr, diag, Float64(alpha), func, n, m, pA, lda, pB, ldb, opts, stream_handle()))
    return B
end

"""
    getrf2_trsm!(A, n1; mixed=false)

The triangular solve of the recursive LU (getrf2!, src/lu.jl:277) on the GPU:
A[1:n1, n1+1:end] := L11 \ A[1:n1, n1+1:end] with L11 the unit lower triangle
of A[1:n1, 1:n1], on views of the one CuMatrix.  `mixed=true` (Float64) uses
the exact tensor-core updates.
"""
function getrf2_trsm!(A::CuMatrix{T}, n1::Integer; mixed::Bool=false) where {T}
    (n1 <= 0 || n1 >= size(A, 2)) && return A
    L11 = view(A, 1:n1, 1:n1)
    A12 = view(A, 1:n1, n1+1:size(A, 2))
    if mixed
        trxm_mixed_diag!('S', 'L', 'L', 'N', 'U', L11, A12, one(T))
    else
        trsm('L', 'L', 'N', 'U', L11, A12, one(T))
    end
    return A
end

end # module
