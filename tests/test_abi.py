"""The C-ABI library loads without a GPU, exports every symbol the header
declares, and rejects bad arguments before touching the device."""

import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        names += re.findall(r"NLA_API\s+[\w\s\*]+?\b(nla_\w+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = _declared_symbols()
    for required in ["nla_trxm", "nla_trxm_ex", "nla_diag_block", "nla_gemm_update", "nla_scale", "nla_last_error",
                     "nla_version"]:
        assert required in names


def test_library_exports_every_declared_symbol(lib, pkg):
    from nextla_gb300 import _lib

    for name in _declared_symbols():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, "no ctypes signature for %s" % name


def test_version(lib):
    assert lib.nla_version() >= 100


def _ch(c):
    return ctypes.c_char(c.encode())


@pytest.mark.parametrize("bad", [("X", "L", "N", "S"), ("L", "x", "N", "S"), ("L", "L", "Q", "S"),
                                 ("L", "L", "N", "Z")])
def test_bad_flags_rejected(lib, bad):
    side, uplo, trans, func = bad
    rc = lib.nla_trxm(_ch(side), _ch(uplo), _ch(trans), 1.0, _ch(func), 2, 4, 4, None, 4, None, 4, None)
    assert rc == -1
    assert lib.nla_last_error().decode()


def test_bad_sizes_rejected(lib):
    assert lib.nla_trxm(_ch("L"), _ch("L"), _ch("N"), 1.0, _ch("S"), 2, -1, 4, None, 4, None, 4, None) == -1
    # leading dimension smaller than the row count
    assert lib.nla_trxm(_ch("L"), _ch("L"), _ch("N"), 1.0, _ch("S"), 2, 8, 4, ctypes.c_void_p(16), 4,
                        ctypes.c_void_p(16), 8, None) == -1
    # null pointer with a non-empty matrix
    assert lib.nla_trxm(_ch("L"), _ch("L"), _ch("N"), 1.0, _ch("S"), 2, 8, 4, None, 8, None, 8, None) == -1
    # unknown dtype
    assert lib.nla_trxm(_ch("L"), _ch("L"), _ch("N"), 1.0, _ch("S"), 7, 8, 4, None, 8, None, 8, None) == -2
    # diagonal block larger than the 1024-entry limit of the base case
    assert lib.nla_diag_block(_ch("S"), _ch("L"), _ch("L"), 0, 2, 2048, 1, ctypes.c_void_p(16), 2048,
                              ctypes.c_void_p(16), 2048, None) == -1


def test_empty_problems_are_no_ops(lib):
    # n = 0 or m = 0: nothing to do, no device work, success
    assert lib.nla_trxm(_ch("L"), _ch("L"), _ch("N"), 2.0, _ch("S"), 2, 0, 5, None, 1, None, 1, None) == 0
    assert lib.nla_trxm(_ch("R"), _ch("U"), _ch("T"), 2.0, _ch("M"), 1, 6, 0, ctypes.c_void_p(16), 6, None, 1,
                        None) == 0
    assert lib.nla_gemm_update(2, 0, 0, 0, 5, 3, 1.0, None, 1, ctypes.c_void_p(16), 5, None, 1, None) == 0


def test_python_mirror_rejects_bad_flags(pkg):
    import torch

    A = torch.zeros(2, 2)
    with pytest.raises(ValueError):
        pkg.unified_rectrxm_("Q", "L", "N", 1.0, "S", A, A)
    with pytest.raises(ValueError):
        pkg.unified_rectrxm_("L", "L", "N", 1.0, "X", A, A)


def test_trxm_diag_rejects_bad_diag(lib):
    """nla_trxm_diag validates diag before any device work."""
    import ctypes

    rc = lib.nla_trxm_diag(b"L", b"L", b"N", b"X", 1.0, b"S", 2, 4, 4, ctypes.c_void_p(16), 4,
                           ctypes.c_void_p(16), 4, None)
    assert rc == -1


def test_host_entries_reject_bad_arguments(lib):
    """The host-buffer entry points check flags and buffers before any device
    work: a bad flag, a missing result buffer or a short leading dimension is
    NLA_ERR_ARG."""
    import ctypes

    p = ctypes.c_void_p(16)
    # bad side
    assert lib.nla_trxm_host(b"X", b"L", b"N", 1.0, b"S", 2, 4, 4, p, 4, p, 4, p, 4, p, 4, p, 4, 0, None) == -1
    # no X_host
    assert lib.nla_trxm_host(b"L", b"L", b"N", 1.0, b"S", 2, 4, 4, p, 4, p, 4, None, 4, p, 4, p, 4, 0, None) == -1
    # A_dev leading dimension below n
    assert lib.nla_trxm_host(b"L", b"L", b"N", 1.0, b"S", 2, 4, 4, p, 4, p, 4, p, 4, p, 3, p, 4, 0, None) == -1
    assert lib.nla_trxm_mixed_host(b"L", b"L", b"Q", 1.0, b"S", 4, 4, p, 4, p, 4, p, 4, p, 4, p, 4, None, 0,
                                   None) == -1
    assert lib.nla_trxm_mixed_host(b"L", b"L", b"N", 1.0, b"S", 4, 4, p, 4, p, 4, p, 4, p, 4, None, 4, None, 0,
                                   None) == -1
    assert b"B_dev" in lib.nla_last_error()


def test_trxm_mixed_diag_rejects_bad_diag(lib):
    """nla_trxm_mixed_diag validates diag before any device work."""
    import ctypes

    rc = lib.nla_trxm_mixed_diag(b"L", b"L", b"N", b"Q", 1.0, b"S", 4, 4, ctypes.c_void_p(16), 4,
                                 ctypes.c_void_p(16), 4, None, None)
    assert rc == -1
    assert b"diag" in lib.nla_last_error()
