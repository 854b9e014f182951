"""CUDA-graph replay of the generic CG loop, and the batched solver's schedule autotuner, on the GPU.

* The multi-launch CG loop (a general operator program, here a Kronecker operator with a Sum
  preconditioner) gives the same iterate bit for bit whether each block of check_every steps is
  replayed from one captured graph or launched kernel by kernel, and stops at exactly max_iters.
* schedule="tuned" measures the candidates once, keeps the winner in the JSON cache, reads it on the
  next call without measuring, and returns what the explicit winning schedule returns (to 1e-6, the
  solution tolerance: the grid schedule accumulates with FP64 atomics, so its last bits may vary).
"""
import json

import pytest
import torch

import cola_gb300 as cola
from cola_gb300 import tuning
from cola_gb300.linalg.batched import solve_batched
from cola_gb300.workloads import diffusion_family_2d

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")


def _kron_problem(dtype):
    g = torch.Generator().manual_seed(4)
    fs = []
    for m in (24, 20):
        M = torch.randn(m, m, generator=g, dtype=torch.float64)
        fs.append((M @ M.T / m + torch.eye(m, dtype=torch.float64)).to(dtype).to(DEV))
    K = cola.ops.Kronecker(*[cola.ops.Dense(f) for f in fs])
    A = cola.PSD(K + 0.5 * cola.ops.I_like(K))
    d = torch.ones(480, dtype=dtype, device=DEV)
    P = cola.ops.Diagonal(0.5 * d) + cola.ops.Diagonal(0.25 * d)  # a general operator program
    B = torch.randn(480, 3, generator=g, dtype=torch.float64).to(dtype).to(DEV)
    return A, P, B


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_generic_cg_graph_replay_is_bit_identical(dtype):
    A, P, B = _kron_problem(dtype)
    x1, i1 = cola.linalg.cg(A, B, P=P, tol=1e-10, max_iters=400, graph=True)
    x0, i0 = cola.linalg.cg(A, B, P=P, tol=1e-10, max_iters=400, graph=False)
    assert i1["graph"] and not i0["graph"] and not i1["fused"]
    assert i1["iterations"] == i0["iterations"]
    assert torch.equal(x1, x0)
    assert float((A @ x1 - B).norm() / B.norm()) < 1e-6


def test_generic_cg_graph_stops_at_max_iters():
    A, P, B = _kron_problem(torch.float64)
    for mi in (33, 48, 50):  # not, and exactly, a multiple of the 16-step block
        x1, i1 = cola.linalg.cg(A, B, P=P, tol=0.0, max_iters=mi, graph=True)
        x0, i0 = cola.linalg.cg(A, B, P=P, tol=0.0, max_iters=mi, graph=False)
        assert i1["iterations"] == i0["iterations"] == mi + 1
        assert torch.equal(x1, x0)


def test_tuned_schedule_is_cached_and_matches_the_explicit_schedule(tmp_path, monkeypatch):
    monkeypatch.setenv("COLA_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(tuning, "_mem", None)
    fam, B, _, _ = diffusion_family_2d(range(9000, 9010), m=64, device=DEV)
    X1, i1 = solve_batched(fam, B, precond="jacobi", tol=1e-8, schedule="tuned")
    data = json.loads((tmp_path / "tune.json").read_text())
    assert len(data) == 1
    rec = next(iter(data.values()))
    assert rec["schedule"] in tuning.CANDIDATES and len(rec["us_per_step_system"]) >= 2
    assert i1["schedule"] == rec["schedule"]

    def boom(*a, **k):
        raise AssertionError("tuned again although the key is cached")
    monkeypatch.setattr(tuning, "probe_measure", lambda *a, **k: boom)
    X2, i2 = solve_batched(fam, B, precond="jacobi", tol=1e-8, schedule="tuned")
    X3, i3 = solve_batched(fam, B, precond="jacobi", tol=1e-8, schedule=rec["schedule"])
    rel = lambda a, b: float((a - b).norm() / b.norm())  # noqa: E731
    assert rel(X1, X3) < 1e-6 and rel(X2, X3) < 1e-6
    assert bool((i3["status"] == 1).all())
