"""Host-side logic of the batched form, checked on the CPU: size buckets, the
seeded uneven workload, and the tuner's JSON cache."""

import json

import numpy as np
import pytest


def test_bucket_of_boundaries(pkg):
    from nextla_gb300 import batched

    assert batched.bucket_of(16) == 0 and batched.bucket_of(31) == 0
    assert batched.bucket_of(32) == 1 and batched.bucket_of(63) == 1
    assert batched.bucket_of(64) == 2
    assert batched.bucket_of(511) == 4
    assert batched.bucket_of(512) == 5 and batched.bucket_of(1024) == 5


def test_uneven_sizes_are_seeded_and_in_range(pkg):
    from nextla_gb300 import batched

    n, m = batched.uneven_sizes(count=10000, seed=7)
    n2, m2 = batched.uneven_sizes(count=10000, seed=7)
    assert np.array_equal(n, n2) and np.array_equal(m, m2)
    assert n.min() >= 16 and n.max() <= 1024 and m.min() >= 1 and m.max() <= 128
    # log-uniform orders: about half the systems below sqrt(16 * 1024) = 128
    assert 0.45 < np.mean(n < 128) < 0.55
    flops = float((n.astype(float) ** 2 * m).sum())
    assert 6e10 < flops < 1e11  # about 8e10 (10^4 x E[n^2] x E[m])


def test_tuner_cache_roundtrip(pkg, tmp_path, monkeypatch):
    import torch

    from nextla_gb300 import tune

    path = tmp_path / "tune.json"
    monkeypatch.setenv("NLA_TUNE_CACHE", str(path))
    monkeypatch.setattr(torch.cuda, "get_device_name", lambda device=None: "Test GPU")
    assert tune.lookup(torch.float64) is None
    cut, cols = [16, 16, 32, 64, 64, 64], [32, 64, 64, 64, 32, 64]
    path.write_text(json.dumps({"Test GPU": {"f64": {str(b): {"cutoff": c, "cols": w}
                                                     for b, (c, w) in enumerate(zip(cut, cols))}}}))
    assert tune.lookup(torch.float64) == (cut, cols)
    assert tune.lookup(torch.float32) is None
    path.write_text(json.dumps({"Test GPU": {"f64": {"0": 8}}}))  # an older cache layout
    assert tune.lookup(torch.float64) is None
    path.write_text("not json")
    assert tune.lookup(torch.float64) is None


def test_batch_plan_rejects_without_gpu_work(pkg, lib):
    """Descriptor validation happens on the host before any device call."""
    import ctypes

    from nextla_gb300 import _lib

    plan = ctypes.c_void_p()
    bad = (_lib.BatchDesc * 1)(_lib.BatchDesc(2048, 4, 0, 2048, 0, 2048))  # n > 1024
    assert lib.nla_batch_plan_create(ctypes.byref(plan), 2, b"L", b"N", 1, bad, None) == -1
    bad = (_lib.BatchDesc * 1)(_lib.BatchDesc(64, 4, 0, 32, 0, 64))  # lda < n
    assert lib.nla_batch_plan_create(ctypes.byref(plan), 2, b"L", b"N", 1, bad, None) == -1
    cw = (ctypes.c_int * 6)(32, 32, 32, 32, 32, 7)
    good = (_lib.BatchDesc * 1)(_lib.BatchDesc(64, 4, 0, 64, 0, 64))
    assert lib.nla_batch_plan_create(ctypes.byref(plan), 2, b"L", b"N", 1, good, cw) == -1
    assert lib.nla_batch_plan_create(ctypes.byref(plan), 2, b"X", b"N", 1, good, None) == -1
    t = _lib.BatchTuning()
    for b in range(6):
        t.cutoff[b], t.cols[b] = 32, 64
    t.cutoff[3] = 48  # not a leaf order the kernel has
    assert lib.nla_batch_plan_create_tuned(ctypes.byref(plan), 2, b"L", b"N", 1, good, ctypes.byref(t)) == -1
