"""Host-side mirror of NextLA.jl's recursive triangular solve / multiply.

The reference's entry point is the Julia function
``unified_rectrxm!(side, uplo, transpose, alpha, func, A, B)``
(src/rectrxm.jl:43-76) with the recursion ``unified_rec`` (src/rectrxm.jl:101-198),
the base cases ``LeftLowerTRSM!`` ... ``RightUpperTRMM!`` (src/trsm.jl:128-150,
src/trmm.jl:332-389) and the updates ``GEMM_ADD!`` / ``GEMM_SUB!``
(src/matmul.jl:69-81).  This module keeps those names (``!`` becomes ``_``),
argument orders and meanings, and drives the same recursion on CUDA tensors;
every base case and every update is one call through the C ABI into the
sm_103a kernels of ``libnextla_gb300.so``.

Matrices are 2-D CUDA tensors holding column-major data, as a Julia ``CuArray``
does: a column-major n x m matrix is a tensor of shape (n, m) with strides
(1, ld).  Slicing gives the same strided views as Julia's ``view``, and ``.T``
gives the ``Transpose`` wrapper.  Work is enqueued on torch's current stream and
is asynchronous, like the reference's kernel launches.

Differences from the reference, by design:
  * unknown characters raise ``ValueError`` instead of falling through to a
    default branch (src/rectrxm.jl:104-124);
  * Float16 updates accumulate in Float32 (src/matmul.jl:50-55 accumulates in
    Float16).
"""

from __future__ import annotations

from . import _lib

_DTYPE_CODES = None


def _dtype_code(t) -> int:
    global _DTYPE_CODES
    if _DTYPE_CODES is None:
        import torch

        _DTYPE_CODES = {torch.float16: _lib.NLA_F16, torch.float32: _lib.NLA_F32, torch.float64: _lib.NLA_F64,
                        torch.complex64: _lib.NLA_C32, torch.complex128: _lib.NLA_C64}
    try:
        return _DTYPE_CODES[t.dtype]
    except KeyError:
        raise ValueError("element type must be Float16, Float32, Float64, ComplexF32 or ComplexF64, got %s"
                         % t.dtype) from None


def _is_complex(t) -> bool:
    return t.dtype.is_complex


def _mat(X):
    """(pointer, leading dimension, transposed) of a 2-D strided view.  A
    complex view with torch's conjugate bit set (``A.T.conj()``, Julia's
    Adjoint) adds 2 to the transposed flag: the library then reads the
    conjugate of every element."""
    if X.dim() != 2:
        raise ValueError("expected a matrix, got a tensor of shape %s" % (tuple(X.shape),))
    if not X.is_cuda:
        raise ValueError("expected a CUDA tensor (the reference's CuArray), got one on %s" % X.device)
    r, c = X.shape
    s0, s1 = X.stride()
    cj = 2 if X.is_conj() else 0
    if s0 == 1 or r <= 1:
        ld = s1 if c > 1 else max(r, 1)
        if ld >= max(r, 1):
            return X.data_ptr(), ld, 0 | cj
    if s1 == 1 or c <= 1:
        ld = s0 if r > 1 else max(c, 1)
        if ld >= max(c, 1):
            return X.data_ptr(), ld, 1 | cj
    raise ValueError("matrix views need a unit stride in one dimension (strides %s)" % ((s0, s1),))


def _stream(X) -> int:
    import torch

    return torch.cuda.current_stream(X.device).cuda_stream


def _check_flags(side, uplo, transpose, func):
    if side not in ("L", "R"):
        raise ValueError("side must be 'L' or 'R', got %r" % (side,))
    if uplo not in ("L", "U"):
        raise ValueError("uplo must be 'L' or 'U', got %r" % (uplo,))
    if transpose not in ("N", "T", "C"):
        raise ValueError("transpose must be 'N', 'T' or 'C', got %r" % (transpose,))
    if func not in ("S", "M"):
        raise ValueError("func must be 'S' or 'M', got %r" % (func,))


def _check_operands(A, B, side):
    if A.dtype != B.dtype:
        raise ValueError("A and B must have the same element type (%s vs %s)" % (A.dtype, B.dtype))
    if A.device != B.device:
        raise ValueError("A and B must be on the same device")
    n = A.shape[0]
    if len(A.shape) != 2 or A.shape[1] != n:
        raise ValueError("A must be square, got %s" % (tuple(A.shape),))
    if len(B.shape) != 2 or (side == "L" and B.shape[0] != n) or (side == "R" and B.shape[1] != n):
        raise ValueError("B of shape %s does not conform with A of size %d for side %r" % (tuple(B.shape), n, side))


# ---------------------------------------------------------------------------
# Base cases (src/trsm.jl:128-150, src/trmm.jl:332-389).
# ---------------------------------------------------------------------------

def _diag_block(func, side, uplo, A, B):
    a, lda, ta = _mat(A)
    b, ldb, tb = _mat(B)
    if tb:
        raise ValueError("B must be a column-major view")
    n = A.shape[0]
    m = B.shape[1] if side == "L" else B.shape[0]
    L = _lib.load()
    _lib.check(L.nla_diag_block(_lib.ch(func), _lib.ch(side), _lib.ch(uplo), ta, _dtype_code(B), n, m, a, lda, b,
                                ldb, _stream(B)))
    return B


def LeftLowerTRSM_(A, B):
    """Solve L X = B in place for a lower-triangular diagonal block (src/trsm.jl:128-132)."""
    return _diag_block("S", "L", "L", A, B)


def LeftUpperTRSM_(A, B):
    """Solve U X = B in place (src/trsm.jl:134-138)."""
    return _diag_block("S", "L", "U", A, B)


def RightLowerTRSM_(A, B):
    """Solve X L = B in place (src/trsm.jl:140-144)."""
    return _diag_block("S", "R", "L", A, B)


def RightUpperTRSM_(A, B):
    """Solve X U = B in place (src/trsm.jl:146-150)."""
    return _diag_block("S", "R", "U", A, B)


def LeftLowerTRMM_(A, B):
    """B := L B in place (src/trmm.jl:332-338)."""
    return _diag_block("M", "L", "L", A, B)


def LeftUpperTRMM_(A, B):
    """B := U B in place (src/trmm.jl:350-355)."""
    return _diag_block("M", "L", "U", A, B)


def RightLowerTRMM_(A, B):
    """B := B L in place (src/trmm.jl:367-372)."""
    return _diag_block("M", "R", "L", A, B)


def RightUpperTRMM_(A, B):
    """B := B U in place (src/trmm.jl:384-389)."""
    return _diag_block("M", "R", "U", A, B)


# ---------------------------------------------------------------------------
# Off-diagonal updates (src/matmul.jl:69-81).
# ---------------------------------------------------------------------------

def matmul_(output, input1, input2, alpha=1.0):
    """output += alpha * input1 * input2 (the matmul! kernel, src/matmul.jl:5-66).
    Transposed inputs are passed as transposed views (the reference passes
    ``Transpose`` wrappers and leaves matmul!'s transA/transB at 'N')."""
    o, ldo, to = _mat(output)
    if to:
        raise ValueError("output must be a column-major view")
    a, ld1, t1 = _mat(input1)
    b, ld2, t2 = _mat(input2)
    N, M = output.shape
    R = input1.shape[1]
    if input1.shape[0] != N or input2.shape != (R, M):
        raise ValueError("matmul_: shapes %s * %s do not conform with %s" % (tuple(input1.shape),
                                                                             tuple(input2.shape),
                                                                             tuple(output.shape)))
    L = _lib.load()
    _lib.check(L.nla_gemm_update(_dtype_code(output), t1, t2, N, R, M, float(alpha), a, ld1, b, ld2, o, ldo,
                                 _stream(output)))
    return output


def GEMM_ADD_(A, B, C):
    """C += A * B (src/matmul.jl:69-74)."""
    return matmul_(C, A, B, 1.0)


def GEMM_SUB_(A, B, C):
    """A -= B * C (src/matmul.jl:76-81)."""
    return matmul_(A, B, C, -1.0)


def scale_(B, alpha):
    """B .= alpha .* B (src/rectrxm.jl:64,72), Float64 (ComplexF64) product
    rounded to B's type."""
    b, ldb, tb = _mat(B)
    if tb:
        raise ValueError("B must be a column-major view")
    L = _lib.load()
    if _is_complex(B):
        a = complex(alpha)
        _lib.check(L.nla_scale_complex(_dtype_code(B), B.shape[0], B.shape[1], a.real, a.imag, b, ldb, _stream(B)))
    else:
        _lib.check(L.nla_scale(_dtype_code(B), B.shape[0], B.shape[1], float(alpha), b, ldb, _stream(B)))
    return B


# ---------------------------------------------------------------------------
# Recursion (src/rectrxm.jl:101-198) and entry point (src/rectrxm.jl:43-76).
# ---------------------------------------------------------------------------

def split_point(n: int) -> int:
    """n/2 when log2(n) is an integer, else the largest power of two below n
    (src/rectrxm.jl:129-133)."""
    if n & (n - 1) == 0:
        return n // 2
    return 1 << (n.bit_length() - 1)


def unified_rec(func, side, uplo, A, n, B, threshold=256):
    """unified_rec (src/rectrxm.jl:101-198) on tensor views."""
    if n <= threshold:
        if func == "S":
            if side == "L" and uplo == "L":
                LeftLowerTRSM_(A, B)
            elif side == "L" and uplo == "U":
                LeftUpperTRSM_(A, B)
            elif side == "R" and uplo == "L":
                RightLowerTRSM_(A, B)
            else:
                RightUpperTRSM_(A, B)
        else:
            if side == "L" and uplo == "L":
                LeftLowerTRMM_(A, B)
            elif side == "L" and uplo == "U":
                LeftUpperTRMM_(A, B)
            elif side == "R" and uplo == "L":
                RightLowerTRMM_(A, B)
            else:
                RightUpperTRMM_(A, B)
        return B

    mid = split_point(n)
    A11 = A[:mid, :mid]
    A22 = A[mid:n, mid:n]
    A21 = A[mid:n, :mid]
    A12 = A[:mid, mid:n]
    if side == "L":
        B1, B2 = B[:mid, :], B[mid:n, :]
    else:
        B1, B2 = B[:, :mid], B[:, mid:n]

    if ((side == "L" and uplo == "L" and func == "S") or (side == "R" and uplo == "U" and func == "S")
            or (side == "L" and uplo == "U" and func == "M") or (side == "R" and uplo == "L" and func == "M")):
        unified_rec(func, side, uplo, A11, mid, B1, threshold)
        if side == "L":
            if func == "S":
                GEMM_SUB_(B2, A21, B1)
            else:
                GEMM_ADD_(A12, B2, B1)
        else:
            if func == "S":
                GEMM_SUB_(B2, B1, A12)
            else:
                GEMM_ADD_(B2, A21, B1)
        unified_rec(func, side, uplo, A22, n - mid, B2, threshold)
    else:
        unified_rec(func, side, uplo, A22, n - mid, B2, threshold)
        if side == "L":
            if func == "S":
                GEMM_SUB_(B1, A12, B2)
            else:
                GEMM_ADD_(A21, B1, B2)
        else:
            if func == "S":
                GEMM_SUB_(B1, B2, A21)
            else:
                GEMM_ADD_(B1, A12, B2)
        unified_rec(func, side, uplo, A11, mid, B1, threshold)
    return B


def _trxm_diag(func, side, uplo, transa, diag, A, B, alpha, mixed=False):
    _check_flags(side, uplo, transa, func)
    if diag not in ("N", "U"):
        raise ValueError("diag must be 'N' or 'U', got %r" % (diag,))
    _check_operands(A, B, side)
    n = A.shape[0]
    a, lda, ta = _mat(A)
    b, ldb, tb = _mat(B)
    if tb:
        raise ValueError("B must be a column-major view")
    tr, up = transa, uplo
    if ta:  # A is a transposed view of its parent: fold that into the flags
        tr = "N" if transa in ("T", "C") else "T"
        up = "U" if uplo == "L" else "L"
    m = B.shape[1] if side == "L" else B.shape[0]
    if mixed:
        import ctypes

        if _dtype_code(B) != _lib.NLA_F64:
            raise ValueError("the mixed form takes Float64 operands")
        opts = _lib.MixedOpts(_lib.NLA_LOWP_BF16, 7, 0, _lib.NLA_RESIDUAL_SPLIT, 0, None)
        _lib.check(_lib.load().nla_trxm_mixed_diag(_lib.ch(side), _lib.ch(up), _lib.ch(tr), _lib.ch(diag),
                                                   float(alpha), _lib.ch(func), n, m, a, lda, b, ldb,
                                                   ctypes.byref(opts), _stream(B)))
        return B
    _lib.check(_lib.load().nla_trxm_diag(_lib.ch(side), _lib.ch(up), _lib.ch(tr), _lib.ch(diag), float(alpha),
                                         _lib.ch(func), _dtype_code(B), n, m, a, lda, b, ldb, _stream(B)))
    return B


def trsm(side, uplo, transa, diag, A, B, alpha=1.0, *, mixed=False):
    """trsm(side, uplo, transa, diag, A, B, alpha) (src/trsm.jl:186-204):
    solves op(A) X = alpha B (side 'L') or X op(A) = alpha B ('R') in place in
    B and returns B.  The reference scales B and calls one base-case kernel,
    ignoring transa and diag (so it is limited to n <= 1024 and op(A) = A);
    here the call runs the whole recursion (nla_trxm_diag), honours transa
    and applies diag 'U' (unit diagonal, never read).  With ``mixed=True``
    (Float64 only) the updates run on the tensor cores with exact 7-slice
    products (nla_trxm_mixed_diag)."""
    return _trxm_diag("S", side, uplo, transa, diag, A, B, alpha, mixed)


def trmm(side, uplo, transa, diag, A, B, alpha=1.0, *, mixed=False):
    """trmm(side, uplo, transa, diag, A, B, alpha) (src/trmm.jl:430-448):
    B := alpha op(A) B (side 'L') or alpha B op(A) ('R'), in place, through
    the recursion; transa and diag 'U' are applied (the reference ignores
    both).  ``mixed`` as for trsm."""
    return _trxm_diag("M", side, uplo, transa, diag, A, B, alpha, mixed)


# ---------------------------------------------------------------------------
# The package's own callers of a triangular solve / multiply, on the GPU path.
# ---------------------------------------------------------------------------

def getrf2_trsm_(A, n1, *, mixed=False):
    """The triangular solve of the recursive LU, getrf2! (src/lu.jl:277):
    A[1:n1, n1+1:end] := L11^-1 A[1:n1, n1+1:end], with L11 the unit lower
    triangle of A[1:n1, 1:n1] (BLAS.trsm!('L', 'L', 'N', 'U', 1, ...)).  Both
    operands are views of the one device array A; the diagonal of A[1:n1,
    1:n1] (which holds U's) is never read.  ``mixed=True`` (Float64) runs
    the exact tensor-core form.  Returns A."""
    n1 = int(n1)
    if n1 <= 0 or n1 >= A.shape[1]:
        return A
    trsm("L", "L", "N", "U", A[:n1, :n1], A[:n1, n1:], 1.0, mixed=mixed)
    return A


def lauum_offdiag_trmm_(uplo, A, i, b, *, mixed=False):
    """The off-diagonal update of the blocked LAUUM (compute_upper!,
    src/lauum.jl:110; compute_lower!, src/lauum.jl:162) on the TRMM path,
    for the diagonal block at 0-based offset i of size b:
      uplo 'U': A[0:i, i:i+b] := A[0:i, i:i+b] * U^T,  U = triu(A[i:i+b, i:i+b]);
      uplo 'L': A[i:i+b, 0:i] := L^T * A[i:i+b, 0:i],  L = tril(A[i:i+b, i:i+b]).
    The reference forms these with a generic product of the whole block (the
    same result when the block's other triangle is zero, as LAUUM's input
    has it); here only the triangle is read.  ``mixed`` as for
    getrf2_trsm_.  Returns A."""
    if uplo not in ("U", "L"):
        raise ValueError("uplo must be 'U' or 'L', got %r" % (uplo,))
    i, b = int(i), int(b)
    if i <= 0 or b <= 0:
        return A
    blk = A[i:i + b, i:i + b]
    if uplo == "U":
        trmm("R", "U", "T", "N", blk, A[:i, i:i + b], 1.0, mixed=mixed)
    else:
        trmm("L", "L", "T", "N", blk, A[i:i + b, :i], 1.0, mixed=mixed)
    return A


def unified_rectrxm_(side, uplo, transpose, alpha, func, A, B, *, native=False, thresholds=None):
    """unified_rectrxm!(side, uplo, transpose, alpha, func, A, B) (src/rectrxm.jl:43-76).

    Solves op(A) X = alpha B (func 'S', side 'L'), X op(A) = alpha B ('S', 'R'),
    or forms B := alpha op(A) B ('M', 'L') / alpha B op(A) ('M', 'R'), in place
    in B, and returns B.  A is n x n; only its ``uplo`` triangle is read.

    By default the recursion runs here, as the reference's Julia host code
    does, with the reference's thresholds (256 for solves, 16 for multiplies,
    src/rectrxm.jl:52,63) unless ``thresholds=(s, m)`` is given.  With
    ``native=True`` the whole recursion runs inside the library (nla_trxm),
    with its own tuned cut-offs unless ``thresholds`` is given.
    """
    _check_flags(side, uplo, transpose, func)
    _check_operands(A, B, side)
    cplx = _is_complex(B)
    if B.is_conj():
        raise ValueError("B must not be a conjugate view (resolve it with B.resolve_conj())")
    n = A.shape[0]
    if native:
        a, lda, ta = _mat(A)
        b, ldb, tb = _mat(B)
        if tb:
            raise ValueError("B must be a column-major view")
        if ta & 2:
            raise ValueError("pass A without torch's conjugate bit and use transpose='C'")
        tr, up = transpose, uplo
        if ta:  # A is a transposed view of its parent: fold that into the flags
            if cplx and transpose == "C":
                raise ValueError("a transposed view of a complex A with transpose='C' is a conjugate without "
                                 "transpose, which unified_rectrxm! cannot express; pass the parent")
            tr = "N" if transpose in ("T", "C") else "T"
            up = "U" if uplo == "L" else "L"
        m = B.shape[1] if side == "L" else B.shape[0]
        L = _lib.load()
        if cplx and complex(alpha).imag != 0.0:
            if thresholds is not None:
                raise ValueError("thresholds are not supported with a complex alpha")
            a_ = complex(alpha)
            _lib.check(L.nla_trxm_complex(_lib.ch(side), _lib.ch(up), _lib.ch(tr), a_.real, a_.imag, _lib.ch(func),
                                          _dtype_code(B), n, m, a, lda, b, ldb, _stream(B)))
            return B
        cs, cm = thresholds if thresholds is not None else (0, 0)
        _lib.check(L.nla_trxm_ex(_lib.ch(side), _lib.ch(up), _lib.ch(tr), float(complex(alpha).real),
                                 _lib.ch(func), _dtype_code(B), n, m, a, lda, b, ldb, int(cs), int(cm), _stream(B)))
        return B

    threshold = 16 if thresholds is None else int(thresholds[1])
    if transpose in ("T", "C"):
        # Transpose(A), or Adjoint(A): for complex data the conjugate view,
        # which the base cases and updates read through torch's conjugate bit.
        A = A.T.conj() if (cplx and transpose == "C") else A.T
        uplo = "U" if uplo == "L" else "L"
    if func == "S":
        threshold = 256 if thresholds is None else int(thresholds[0])
        scale_(B, alpha)
    unified_rec(func, side, uplo, A, n, B, threshold)
    if func == "M":
        scale_(B, alpha)
    return B


# ---------------------------------------------------------------------------
# Mixed-precision form (no counterpart in the reference): FP64 answers with
# the off-diagonal updates on the tcgen05 tensor cores.
# ---------------------------------------------------------------------------

_LOWP = {"bf16": _lib.NLA_LOWP_BF16, "f16": _lib.NLA_LOWP_F16}


def matmul_mixed_(output, input1, input2, alpha=1.0, *, lowp="bf16", split_terms=3):
    """output += alpha * input1 * input2 for Float64 tensors, formed on the
    tensor cores from ``split_terms`` BF16/FP16 slices of each operand."""
    o, ldo, to = _mat(output)
    if to:
        raise ValueError("output must be a column-major view")
    a, ld1, t1 = _mat(input1)
    b, ld2, t2 = _mat(input2)
    N, M = output.shape
    R = input1.shape[1]
    if input1.shape[0] != N or tuple(input2.shape) != (R, M):
        raise ValueError("matmul_mixed_: shapes do not conform")
    for X in (output, input1, input2):
        if _dtype_code(X) != _lib.NLA_F64:
            raise ValueError("the mixed form takes Float64 operands")
    L = _lib.load()
    _lib.check(L.nla_gemm_update_mixed(t1, t2, N, R, M, float(alpha), a, ld1, b, ld2, o, ldo, _LOWP[lowp],
                                       int(split_terms), _stream(output)))
    return output


_RESIDUAL = {"split": _lib.NLA_RESIDUAL_SPLIT, "fp64": _lib.NLA_RESIDUAL_FP64, "dd": _lib.NLA_RESIDUAL_DD}


def residual_(side, uplo, transpose, alpha, A, X, B, R, *, residual="split"):
    """R = alpha*B - op(A) X (side 'L') or alpha*B - X op(A) (side 'R') for
    Float64 tensors, FP64-accurate (``residual`` 'split': tensor cores with
    exact slice products; 'fp64': the FP64 pipe; 'dd': double-double on the
    FP64 pipe, rounded once, for measuring backward errors)."""
    _check_flags(side, uplo, transpose, "M")
    a, lda, ta = _mat(A)
    if ta:
        raise ValueError("pass A untransposed and use `transpose`")
    x, ldx, tx = _mat(X)
    b, ldb, tb = _mat(B)
    r, ldr, tr = _mat(R)
    if tx or tb or tr:
        raise ValueError("X, B and R must be column-major views")
    n = A.shape[0]
    m = X.shape[1] if side == "L" else X.shape[0]
    L = _lib.load()
    _lib.check(L.nla_trxm_residual(_lib.ch(side), _lib.ch(uplo), _lib.ch(transpose), float(alpha), n, m, a, lda, x,
                                   ldx, b, ldb, r, ldr, _RESIDUAL[residual], _stream(R)))
    return R


def unified_rectrxm_mixed_(side, uplo, transpose, alpha, func, A, B, *, lowp="bf16", split_terms=3, sweeps=2,
                           cutoff=0, corrections=False, residual="split"):
    """Mixed-precision unified_rectrxm! for Float64 A and B (in place in B).

    Updates run on the tensor cores from ``split_terms`` slices (``lowp`` 'bf16'
    or 'f16'); diagonal blocks of size ``cutoff`` (0: library default) run in
    FP64; solves add ``sweeps`` FP64-residual refinement sweeps.  With
    ``corrections=True`` returns (B, [max|D|/max|X| per sweep])."""
    import ctypes

    _check_flags(side, uplo, transpose, func)
    _check_operands(A, B, side)
    if _dtype_code(B) != _lib.NLA_F64:
        raise ValueError("the mixed form takes Float64 operands")
    a, lda, ta = _mat(A)
    b, ldb, tb = _mat(B)
    if tb:
        raise ValueError("B must be a column-major view")
    tr, up = transpose, uplo
    if ta:
        tr = "N" if transpose in ("T", "C") else "T"
        up = "U" if uplo == "L" else "L"
    n = A.shape[0]
    m = B.shape[1] if side == "L" else B.shape[0]
    corr = (ctypes.c_double * max(int(sweeps), 1))()
    opts = _lib.MixedOpts(_LOWP[lowp], int(split_terms), int(sweeps), _RESIDUAL[residual], int(cutoff),
                          ctypes.cast(corr, ctypes.POINTER(ctypes.c_double)) if corrections else None)
    L = _lib.load()
    _lib.check(L.nla_trxm_mixed(_lib.ch(side), _lib.ch(up), _lib.ch(tr), float(alpha), _lib.ch(func), n, m, a, lda,
                                b, ldb, ctypes.byref(opts), _stream(B)))
    if corrections:
        return B, [corr[i] for i in range(int(sweeps))] if func == "S" else []
    return B


def device_status(X=None):
    """Synchronise the stream and raise if a bounded device-side wait gave up."""
    L = _lib.load()
    _lib.check(L.nla_device_status(_stream(X) if X is not None else None))


# ---------------------------------------------------------------------------
# Host-buffer forms: CuArray(A), CuArray(B), unified_rectrxm!, copyto! as one
# call, with the copies pipelined against the recursion.
# ---------------------------------------------------------------------------

def _host_mat(X, name):
    """(pointer, leading dimension) of a column-major 2-D CPU tensor view."""
    if X.dim() != 2 or X.is_cuda:
        raise ValueError("%s must be a 2-D CPU tensor" % name)
    r, c = X.shape
    s0, s1 = X.stride()
    if (s0 == 1 or r <= 1) and (c <= 1 or s1 >= max(r, 1)):
        return X.data_ptr(), (s1 if c > 1 else max(r, 1))
    raise ValueError("%s must be a column-major view (strides %s)" % (name, (s0, s1)))


def _host_call(side, uplo, transpose, func, A, B, X, A_dev, B_dev, dtype):
    import torch

    _check_flags(side, uplo, transpose, func)
    if A.dtype != dtype or B.dtype != dtype:
        raise ValueError("A and B must be %s" % dtype)
    n = A.shape[0]
    if tuple(A.shape) != (n, n):
        raise ValueError("A must be square, got %s" % (tuple(A.shape),))
    if (side == "L" and B.shape[0] != n) or (side == "R" and B.shape[1] != n):
        raise ValueError("B of shape %s does not conform with A of size %d for side %r" % (tuple(B.shape), n, side))
    X = B if X is None else X
    if tuple(X.shape) != tuple(B.shape) or X.dtype != dtype:
        raise ValueError("X must have B's shape and element type")
    dev = A_dev.device if A_dev is not None else (B_dev.device if B_dev is not None else torch.device("cuda"))
    if A_dev is None:
        A_dev = torch.empty_strided((n, n), (1, max(n, 1)), dtype=dtype, device=dev)
    if B_dev is None:
        B_dev = torch.empty_strided(tuple(B.shape), (1, max(B.shape[0], 1)), dtype=dtype, device=dev)
    a, lda = _host_mat(A, "A")
    b, ldb = _host_mat(B, "B")
    x, ldx = _host_mat(X, "X")
    ad, ldad, tad = _mat(A_dev)
    bd, ldbd, tbd = _mat(B_dev)
    if tad or tbd or tuple(A_dev.shape) != (n, n) or tuple(B_dev.shape) != tuple(B.shape):
        raise ValueError("A_dev and B_dev must be column-major device arrays of A's and B's shapes")
    m = B.shape[1] if side == "L" else B.shape[0]
    return n, m, (a, lda, b, ldb, x, ldx, ad, ldad, bd, ldbd), X, torch.cuda.current_stream(dev)


def unified_rectrxm_host_(side, uplo, transpose, alpha, func, A, B, *, X=None, A_dev=None, B_dev=None,
                          host_levels=0, synchronize=True):
    """unified_rectrxm! (src/rectrxm.jl:43-76) on host (CPU) tensors A and B,
    column-major and preferably pinned: the result goes to X (default: B, in
    place).  A_dev / B_dev are optional device arrays of A's and B's shapes
    (allocated when not given).  The copies in and out are pipelined with the
    native recursion over its top ``host_levels`` levels (0: library
    default).  With ``synchronize`` the call returns once X holds the result."""
    n, m, ptrs, X, stream = _host_call(side, uplo, transpose, func, A, B, X, A_dev, B_dev, A.dtype)
    code = _dtype_code(A)
    a, lda, b, ldb, x, ldx, ad, ldad, bd, ldbd = ptrs
    L = _lib.load()
    _lib.check(L.nla_trxm_host(_lib.ch(side), _lib.ch(uplo), _lib.ch(transpose), float(alpha), _lib.ch(func), code,
                               n, m, a, lda, b, ldb, x, ldx, ad, ldad, bd, ldbd, int(host_levels),
                               stream.cuda_stream))
    if synchronize:
        stream.synchronize()
    return X


def unified_rectrxm_mixed_host_(side, uplo, transpose, alpha, func, A, B, *, X=None, A_dev=None, B_dev=None,
                                lowp="bf16", split_terms=7, sweeps=0, cutoff=0, residual="split", host_levels=0,
                                synchronize=True):
    """The mixed-precision unified_rectrxm! on Float64 host tensors (see
    ``unified_rectrxm_host_`` for the buffers and ``unified_rectrxm_mixed_``
    for the options; here the defaults are the exact 7-slice updates without
    refinement)."""
    import ctypes

    import torch

    n, m, ptrs, X, stream = _host_call(side, uplo, transpose, func, A, B, X, A_dev, B_dev, torch.float64)
    a, lda, b, ldb, x, ldx, ad, ldad, bd, ldbd = ptrs
    opts = _lib.MixedOpts(_LOWP[lowp], int(split_terms), int(sweeps), _RESIDUAL[residual], int(cutoff), None)
    L = _lib.load()
    _lib.check(L.nla_trxm_mixed_host(_lib.ch(side), _lib.ch(uplo), _lib.ch(transpose), float(alpha), _lib.ch(func),
                                     n, m, a, lda, b, ldb, x, ldx, ad, ldad, bd, ldbd, ctypes.byref(opts),
                                     int(host_levels), stream.cuda_stream))
    if synchronize:
        stream.synchronize()
    return X
