"""CPU oracle for NextLA.jl's `unified_rectrxm!` (src/rectrxm.jl:43-198).

TEST INFRASTRUCTURE ONLY.  This module is the parity checker: only the tests,
the smoke check and the CPU-baseline leg of the benchmark import it.  The
product library never calls it.

It wraps the C restatement in ``rectrxm_oracle.c`` (built into
``oracle/_build/liboracle_rectrxm.so`` by :func:`build`) and adds the
independent checks the reference's own tests use: BLAS trsm/trmm
(test/unified_rectrxm.jl:36-40) through scipy, and the error metrics.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle_rectrxm.so")

DTYPES = {np.dtype(np.float16): 0, np.dtype(np.float32): 1, np.dtype(np.float64): 2}

_lib = None
_lock = threading.Lock()


def build(force: bool = False) -> str:
    """Compile the C oracle with gcc (no FMA contraction, so x86 and Arm agree)."""
    src = os.path.join(HERE, "rectrxm_oracle.c")
    hdrs = [os.path.join(HERE, "rectrxm_oracle_impl.h"), os.path.join(HERE, "rectrxm_oracle_cplx.h")]
    if not force and os.path.exists(LIB_PATH):
        newest = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in hdrs])
        if os.path.getmtime(LIB_PATH) >= newest:
            return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-o", tmp, src, "-lpthread", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            path = build()
            L = ctypes.CDLL(path)
            i64, d, c, i32, p = ctypes.c_int64, ctypes.c_double, ctypes.c_char, ctypes.c_int, ctypes.c_void_p
            L.oracle_rectrxm.argtypes = [c, c, c, d, c, i32, i64, i64, p, i64, p, i64, i64, i64, i32]
            L.oracle_rectrxm.restype = i32
            L.oracle_matmul.argtypes = [i32, i64, i64, i64, d, p, i64, p, i64, i32, p, i64, i32]
            L.oracle_matmul.restype = i32
            L.oracle_leaf.argtypes = [c, c, c, i32, i64, i64, p, i64, i32, p, i64]
            L.oracle_leaf.restype = i32
            L.oracle_rectrxm_cplx.argtypes = [c, c, c, d, d, c, i32, i64, i64, p, i64, p, i64, i64, i64, i32]
            L.oracle_rectrxm_cplx.restype = i32
            L.oracle_split_point.argtypes = [i64]
            L.oracle_split_point.restype = i64
            _lib = L
        return _lib


def _as_f64_fortran(x: np.ndarray) -> np.ndarray:
    return np.asfortranarray(np.asarray(x, dtype=np.float64))


def _ptr(x: np.ndarray):
    return ctypes.c_void_p(x.ctypes.data)


def _ch(s: str):
    return ctypes.c_char(s.encode())


def rectrxm(side, uplo, trans, alpha, func, A, B, *, dtype=None, thresholds=(256, 16), nthreads=1):
    """Return unified_rectrxm!(side, uplo, trans, alpha, func, A, B) as computed
    by the reference algorithm; B is not modified.  ``dtype`` defaults to B's
    element type; the result is returned in that type."""
    dt = np.dtype(dtype if dtype is not None else B.dtype)
    code = DTYPES[dt]
    Af = _as_f64_fortran(np.asarray(A).astype(dt))
    Bf = _as_f64_fortran(np.asarray(B).astype(dt)).copy(order="F")
    n = Af.shape[0]
    if Af.shape != (n, n):
        raise ValueError("A must be square")
    m = Bf.shape[1] if side == "L" else Bf.shape[0]
    if (side == "L" and Bf.shape[0] != n) or (side == "R" and Bf.shape[1] != n):
        raise ValueError("B does not conform with A")
    rc = lib().oracle_rectrxm(_ch(side), _ch(uplo), _ch(trans), float(alpha), _ch(func), code, n, m, _ptr(Af),
                              max(n, 1), _ptr(Bf), max(Bf.shape[0], 1), int(thresholds[0]), int(thresholds[1]),
                              int(nthreads))
    if rc != 0:
        raise ValueError("oracle_rectrxm rejected its arguments")
    return Bf.astype(dt)


def rectrxm_complex(side, uplo, trans, alpha, func, A, B, *, dtype=None, thresholds=(256, 16), nthreads=1):
    """unified_rectrxm! on complex A and B (ComplexF32 or ComplexF64, from
    ``dtype`` or B's type) with complex alpha; trans 'C' takes the Adjoint.
    Returns the result in that type; B is not modified."""
    dt = np.dtype(dtype if dtype is not None else B.dtype)
    code = {np.dtype(np.complex64): 3, np.dtype(np.complex128): 4}[dt]
    Af = np.asfortranarray(np.asarray(A).astype(dt).astype(np.complex128))
    Bf = np.asfortranarray(np.asarray(B).astype(dt).astype(np.complex128)).copy(order="F")
    n = Af.shape[0]
    m = Bf.shape[1] if side == "L" else Bf.shape[0]
    if Af.shape != (n, n) or (side == "L" and Bf.shape[0] != n) or (side == "R" and Bf.shape[1] != n):
        raise ValueError("A must be square and B must conform with it")
    al = complex(alpha)
    rc = lib().oracle_rectrxm_cplx(_ch(side), _ch(uplo), _ch(trans), al.real, al.imag, _ch(func), code, n, m,
                                   _ptr(Af), max(n, 1), _ptr(Bf), max(Bf.shape[0], 1), int(thresholds[0]),
                                   int(thresholds[1]), int(nthreads))
    if rc != 0:
        raise ValueError("oracle_rectrxm_cplx rejected its arguments")
    return Bf.astype(dt)


def matmul(out, in1, in2, alpha, *, t1=False, t2=False, dtype=None):
    """out + alpha * op(in1) @ op(in2) with the reference's 32-wide partial sums."""
    dt = np.dtype(dtype if dtype is not None else out.dtype)
    o = _as_f64_fortran(np.asarray(out).astype(dt)).copy(order="F")
    a = _as_f64_fortran(np.asarray(in1).astype(dt))
    b = _as_f64_fortran(np.asarray(in2).astype(dt))
    N, M = o.shape
    R = a.shape[0] if t1 else a.shape[1]
    rc = lib().oracle_matmul(DTYPES[dt], N, R, M, float(alpha), _ptr(o), max(N, 1), _ptr(a), max(a.shape[0], 1),
                             int(t1), _ptr(b), max(b.shape[0], 1), int(t2))
    if rc != 0:
        raise ValueError("oracle_matmul rejected its arguments")
    return o.astype(dt)


def leaf(func, side, uplo, A, B, *, tA=False, dtype=None):
    """One base-case kernel call (LeftLowerTRSM! ... RightUpperTRMM!)."""
    dt = np.dtype(dtype if dtype is not None else B.dtype)
    a = _as_f64_fortran(np.asarray(A).astype(dt))
    b = _as_f64_fortran(np.asarray(B).astype(dt)).copy(order="F")
    n = a.shape[0]
    m = b.shape[1] if side == "L" else b.shape[0]
    rc = lib().oracle_leaf(_ch(func), _ch(side), _ch(uplo), DTYPES[dt], n, m, _ptr(a), max(n, 1), int(tA), _ptr(b),
                           max(b.shape[0], 1))
    if rc != 0:
        raise ValueError("oracle_leaf rejected its arguments")
    return b.astype(dt)


def split_point(n: int) -> int:
    return int(lib().oracle_split_point(int(n)))


# --------------------------------------------------------------------------
# Independent checks used by the reference's tests and by the error tables.
# --------------------------------------------------------------------------

def blas_rectrxm(side, uplo, trans, alpha, func, A, B):
    """BLAS trsm!/trmm! with diag='N', as in test/unified_rectrxm.jl:36-40,
    computed in float64 (float32 BLAS for float32 inputs)."""
    from scipy.linalg import blas

    dt = np.dtype(B.dtype)
    pre = {np.dtype(np.float32): "s", np.dtype(np.complex64): "c", np.dtype(np.complex128): "z"}.get(dt, "d")
    work = {"s": np.float32, "c": np.complex64, "z": np.complex128, "d": np.float64}[pre]
    a = np.asfortranarray(np.asarray(A, dtype=work))
    b = np.asfortranarray(np.asarray(B, dtype=work))
    ta = {"N": 0, "T": 1, "C": 2}[trans]
    fn = getattr(blas, pre + ("trsm" if func == "S" else "trmm"))
    return fn(alpha, a, b, side=int(side == "R"), lower=int(uplo == "L"), trans_a=ta, diag=0)


def op_matrix(A, uplo, trans):
    """op(tri(A)) as a dense float64 matrix (only the named triangle of A)."""
    T = np.tril(A) if uplo == "L" else np.triu(A)
    T = np.asarray(T, dtype=np.float64)
    return T.T if trans in ("T", "C") else T


def rel_err(X, Xref) -> float:
    wide = np.complex128 if (np.iscomplexobj(X) or np.iscomplexobj(Xref)) else np.float64
    X = np.asarray(X, dtype=wide)
    Xref = np.asarray(Xref, dtype=wide)
    den = np.linalg.norm(Xref)
    return float(np.linalg.norm(X - Xref) / (den if den > 0 else 1.0))


def backward_error(side, uplo, trans, alpha, A, X, B, unit_roundoff=2.0 ** -53) -> float:
    """||op(A) X - alpha B||_inf / (||op(A)||_inf ||X||_inf n u) for a solve
    (side 'L'); the right-side analogue uses X op(A).  Evaluated in float64
    with a compensated product (np.longdouble where it is wider)."""
    opA = op_matrix(A, uplo, trans)
    n = opA.shape[0]
    wide = np.longdouble if np.finfo(np.longdouble).nmant > 52 else np.float64
    Aw = opA.astype(wide)
    Xw = np.asarray(X, dtype=wide)
    Bw = np.asarray(B, dtype=wide)
    R = (Aw @ Xw if side == "L" else Xw @ Aw) - wide(alpha) * Bw
    r = float(np.max(np.sum(np.abs(R), axis=1)))
    na = float(np.max(np.sum(np.abs(opA), axis=1)))
    nx = float(np.max(np.sum(np.abs(np.asarray(X, dtype=np.float64)), axis=1)))
    den = na * nx * n * unit_roundoff
    return r / den if den > 0 else 0.0
