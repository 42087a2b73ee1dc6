"""Persistent batched solver against the oracle and against the one-launch-
per-system loop, on uneven seeded batches (sizes log-uniform in [16, 1024],
1..128 right-hand sides).  Tolerances as for single systems: Float64 1e-13
relative (vs the oracle; the batched kernel folds alpha into the load),
Float32 1e-5.  Graph replay, persistent launch and the loop must agree bit
for bit with each other where the arithmetic is the same (graph vs
persistent), and within tolerance with the loop."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _system(A_pool, B_pool, s):
    n, m, a_off, lda, b_off, ldb = s
    A = A_pool[a_off:a_off + n * n].reshape(n, n).T.detach().cpu().numpy().astype(np.float64)
    B = B_pool[b_off:b_off + n * m].reshape(m, n).T.detach().cpu().numpy().astype(np.float64)
    return A, B


@pytest.mark.parametrize("dtype_name,tol", [("float64", 1e-13), ("float32", 1e-5)])
@pytest.mark.parametrize("uplo,trans", [("L", "N"), ("U", "N"), ("L", "T"), ("U", "T")])
def test_batched_matches_oracle(pkg, oracle, cuda, dtype_name, tol, uplo, trans):
    import torch

    from nextla_gb300 import batched

    dtype = getattr(torch, dtype_name)
    n, m = batched.uneven_sizes(count=300, seed=11)
    A, B0, systems = batched.make_batch(n, m, dtype, cuda, seed=11, uplo=uplo)
    plan = batched.BatchPlan(dtype, uplo, trans, systems)
    B = B0.clone()
    plan.solve(0.5, A, B, mode="graph")
    torch.cuda.synchronize()
    rng = np.random.default_rng(0)
    for i in rng.choice(len(systems), 12, replace=False):
        Ai, Bi = _system(A, B0, systems[i])
        np_dt = np.float64 if dtype == torch.float64 else np.float32
        ref = oracle.rectrxm("L", uplo, trans, 0.5, "S", Ai.astype(np_dt), Bi.astype(np_dt))
        _, Xi = _system(A, B, systems[i])
        assert oracle.rel_err(Xi, ref) < tol, (i, systems[i][:2])
    plan.close()


def test_batched_modes_agree(pkg, cuda):
    import torch

    from nextla_gb300 import batched

    n, m = batched.uneven_sizes(count=500, seed=3)
    A, B0, systems = batched.make_batch(n, m, torch.float64, cuda, seed=3)
    plan = batched.BatchPlan(torch.float64, "L", "N", systems)
    outs = {}
    for mode in ("graph", "persistent", "loop"):
        B = B0.clone()
        plan.solve(1.0, A, B, mode=mode)
        plan.solve(1.0, A, B0.clone(), mode=mode)  # a second call reuses the captured graph
        torch.cuda.synchronize()
        outs[mode] = B
    assert torch.equal(outs["graph"], outs["persistent"])
    rel = float(torch.linalg.norm(outs["graph"] - outs["loop"]) / torch.linalg.norm(outs["loop"]))
    assert rel < 1e-13
    items, grid, flops = plan.info()
    assert items >= len(systems) and grid >= 1 and flops > 0
    plan.close()


def test_batched_rejects_bad_descriptors(pkg, cuda):
    import torch

    from nextla_gb300 import _lib, batched

    with pytest.raises(_lib.NLAArgumentError):
        batched.BatchPlan(torch.float64, "L", "N", [(2048, 4, 0, 2048, 0, 2048)])
    with pytest.raises(_lib.NLAArgumentError):
        batched.BatchPlan(torch.float64, "L", "N", [(64, 4, 0, 32, 0, 64)])
    with pytest.raises(_lib.NLAArgumentError):
        batched.BatchPlan(torch.float64, "L", "N", [(64, 4, 0, 64, 0, 64)], cols_per_item=[7] * 6)
    with pytest.raises(_lib.NLAArgumentError):
        batched.BatchPlan(torch.float64, "L", "N", [(64, 4, 0, 64, 0, 64)], cutoff=[128] * 6)


def test_tuner_writes_cache(pkg, cuda, tmp_path, monkeypatch):
    import json

    import torch

    from nextla_gb300 import tune

    monkeypatch.setenv("NLA_TUNE_CACHE", str(tmp_path / "tune.json"))
    (cut, cols), timings = tune.tune(torch.float32, cuda, systems_per_bucket=24, reps=1)
    assert len(cut) == 6 and all(c in tune.CUTOFFS for c in cut)
    assert len(cols) == 6 and all(w in tune.COLS for w in cols)
    assert all(len(timings[b]) == len(tune.candidates(torch.float32)) for b in range(6))
    data = json.load(open(tmp_path / "tune.json"))
    assert tune.lookup(torch.float32, cuda) == (cut, cols)
    assert torch.cuda.get_device_name(cuda) in data


def test_batched_mixed_refinement_converges(pkg, cuda):
    """Float32 solves refined with Float64 residuals (nla_batch_solve_mixed):
    with no sweep the batch carries Float32-level error; each sweep shrinks it
    and two sweeps reach the plain Float64 answer to Float64 accuracy.  Systems
    span every size bucket, both transposes and a partial last item."""
    import torch

    from nextla_gb300 import batched

    rng = np.random.default_rng(21)
    n = rng.integers(1, 700, 60)
    n[:6] = [1, 16, 31, 64, 513, 1024]
    m = rng.integers(1, 70, 60)
    for trans in "NT":
        A, B0, systems = batched.make_batch(n, m, torch.float64, cuda, seed=5)
        plan = batched.BatchPlan(torch.float64, "L", trans, systems)
        X = B0.clone()
        plan.solve(0.5, A, X, mode="persistent")
        ref = float(torch.linalg.norm(X))
        errs = []
        for sweeps in (0, 1, 2):
            Y = B0.clone()
            plan.solve_mixed(0.5, A, Y, sweeps=sweeps)
            torch.cuda.synchronize()
            errs.append(float(torch.linalg.norm(Y - X)) / ref)
        plan.close()
        assert 1e-9 < errs[0] < 1e-5, (trans, errs)
        assert errs[1] < errs[0] * 1e-3, (trans, errs)
        assert errs[2] < 1e-14, (trans, errs)


@pytest.mark.parametrize("uplo,trans", [("L", "N"), ("U", "T"), ("L", "T")])
def test_batched_mixed_tensor_core_residual(pkg, oracle, cuda, uplo, trans):
    """The tensor-core residual (exact BF16 slice products) refines as well as
    the FP64-pipe residual: after two sweeps both are within 1e-14 of the plain
    Float64 batch, and sampled systems match the oracle at the Float64
    tolerance.  Systems span every size bucket, partial tiles of rows and of
    right-hand sides, and more than 64 right-hand sides."""
    import torch

    from nextla_gb300 import batched

    rng = np.random.default_rng(23)
    n = rng.integers(1, 1025, 48)
    n[:8] = [1, 7, 16, 129, 200, 513, 1000, 1024]
    m = rng.integers(1, 129, 48)
    m[:4] = [1, 64, 65, 128]
    A, B0, systems = batched.make_batch(n, m, torch.float64, cuda, seed=9, uplo=uplo)
    plan = batched.BatchPlan(torch.float64, uplo, trans, systems)
    X = B0.clone()
    plan.solve(0.75, A, X, mode="persistent")
    ref = float(torch.linalg.norm(X))
    out = {}
    for res in ("split", "fp64"):
        Y = B0.clone()
        plan.solve_mixed(0.75, A, Y, sweeps=2, residual=res)
        pkg.device_status(Y)
        out[res] = Y
        assert float(torch.linalg.norm(Y - X)) / ref < 1e-14, res
    plan.close()
    for i in range(8):
        Ai, Bi = _system(A, B0, systems[i])
        want = oracle.rectrxm("L", uplo, trans, 0.75, "S", Ai, Bi)
        _, Xi = _system(A, out["split"], systems[i])
        assert oracle.rel_err(Xi, want) < 1e-13, (i, systems[i][:2])
