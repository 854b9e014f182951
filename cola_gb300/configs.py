"""Runners for the benchmark configurations besides the headline family (used by ``bench.py --config``).

Each returns a dict with the throughput, the accuracy against an FP64 reference computed on the GPU,
and the iteration counts.  Inputs are the seeded synthetic stand-ins of ``cola_gb300.workloads``.
"""
from __future__ import annotations

import math
import time

import torch

from . import ops as O
from .annotations import PSD
from .linalg import CG
from .linalg.batched import BatchedCSR, solve_batched, solve_dense_batched
from .linalg.inverse import cg
from .linalg.prng import randn
from .linalg.unary import stochastic_lanczos_quad
from .workloads import dense_spd, diffusion_3d, kron_rbf, rbf_systems


def _timed(fn, steps=2, warmup=1):
    for _ in range(warmup):
        out = fn()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(steps):
        out = fn()
    b.record(st)
    torch.cuda.synchronize()
    return out, a.elapsed_time(b) / 1e3 / steps


def c1_dense(steps=3, warmup=2):
    """solve(PSD(Dense(A)), b, CG(tol=1e-6, max_iters=2000)), n = 2048 FP32, log-uniform spectrum [1e-2, 1e2]."""
    A, b, lam = dense_spd(2048, seed=0, dtype=torch.float32, device="cuda")
    op = PSD(O.Dense(A))
    (x, info), t = _timed(lambda: cg(op, b, tol=1e-6, max_iters=2000), steps, warmup)
    A64, b64 = A.double(), b.double()
    xs = torch.linalg.solve(A64, b64)
    relres = float((b64 - A64 @ x.double()).norm() / b64.norm())
    return {"config": "dense-2048-cg", "solves_per_s": 1 / t, "ms_per_solve": 1e3 * t, "cg_steps": info["iterations"] - 1,
            "fused": info["fused"], "true_relres": relres,
            "err_vs_fp64_solve": float((x.double() - xs).norm() / xs.norm())}


def c2_diffusion3d(nrhs=32, m=128, steps=1, warmup=1):
    """7-point 128^3 diffusion + 1e-3 I, 32 right-hand sides, each to a 1e-8 FP64 true residual."""
    ip, ix, v = diffusion_3d(m=m, device="cuda")
    fam = BatchedCSR(ip, ix, v[None, :], shared=True)
    B = torch.randn(nrhs, fam.n, device="cuda", dtype=torch.float64, generator=torch.Generator("cuda").manual_seed(2))
    out = {"config": f"diffusion3d-{m}^3-{nrhs}rhs", "n": fam.n, "nnz": int(ix.numel())}
    for prec in ("jacobi", "none"):
        (X, info), t = _timed(lambda: solve_batched(fam, B, precond=prec, tol=1e-8), steps, warmup)
        out[prec] = {"rhs_per_s": nrhs / t, "s_per_call": t, "mean_iters": float(info["iterations"].double().mean()),
                     "max_true_relres": float(info["relres"].max())}
    return out


def c3a_rbf_batch(num=256, steps=1, warmup=1, tol=1e-6, max_iters=2000):
    """256 dense RBF systems K + s^2 I of uneven sizes (500..8000), one persistent launch."""
    mats, rhs, meta = rbf_systems(num=num, device="cuda")
    (res, t) = _timed(lambda: solve_dense_batched(mats, rhs, tol=tol, max_iters=max_iters), steps, warmup)
    sols, iters, status = res
    worst = 0.0
    for A, b, x in list(zip(mats, rhs, sols))[:8]:
        r = (b.double() - A.double() @ x.double()).norm() / b.double().norm()
        worst = max(worst, float(r))
    bytes_sweep = sum(n * n * 4 for n, _, _ in meta)
    return {"config": f"rbf-uneven-{num}", "systems_per_s": num / t, "s_per_call": t,
            "mean_iters": float(iters.double().mean()), "max_iters": int(iters.max()),
            "converged": int((status == 1).sum()), "true_relres_first8_max": worst,
            "matrix_bytes_per_sweep": bytes_sweep}


def c3b_kron_slq(probes=64, steps=100, reps=1, warmup=1):
    """logdet(Kronecker(K1, K2, K3) + 0.01 I), 64^3 = 262,144, 64 Rademacher probes, 100 Lanczos steps."""
    Ks, ells = kron_rbf(seed=4, device="cuda")
    K = O.Kronecker(*[O.Dense(k) for k in Ks])
    op = PSD(K + 0.01 * O.I_like(K))
    n = op.shape[0]
    Z = torch.sign(randn(n, probes, dtype=torch.float32, key=5)).to("cuda")
    est, t = _timed(lambda: stochastic_lanczos_quad(op, torch.log, max_iters=steps, tol=0.0, probes=Z), reps, warmup)
    lam = torch.ones(1, dtype=torch.float64, device="cuda")
    for k in Ks:
        lam = torch.kron(lam, torch.linalg.eigvalsh(k.double()))
    exact = float(torch.log(lam + 0.01).sum())
    return {"config": "kron-rbf-64^3-slq", "logdets_per_s": 1 / t, "s_per_logdet": t, "estimate": float(est),
            "exact": exact, "rel_err": abs(float(est) - exact) / abs(exact)}


def c5_lanczos_topk(k=64, steps=256, num_points=1 << 20):
    """64 largest eigenpairs of Sum(Kronecker(A1, A2), L): A1, A2 1024 x 1024 SPD (log-uniform spectrum in
    [1e-2, 1e1]), L the Laplacian of a random geometric graph on 2^20 points (radius 0.002); 256-step
    Lanczos with full reorthogonalisation, FP64 tridiagonal eigensolve.  Accuracy: the same Lanczos run on
    the FP64 operator (same start vector) and the Ritz residuals |A v - lambda v| / |lambda|."""
    from .annotations import SelfAdjoint
    from .linalg import Lanczos, eig
    from .workloads import rgg_laplacian
    A1, _, _ = dense_spd(1024, seed=6, lo=1e-2, hi=1e1, dtype=torch.float32, device="cuda")
    A2, _, _ = dense_spd(1024, seed=61, lo=1e-2, hi=1e1, dtype=torch.float32, device="cuda")
    ip, ix, v = rgg_laplacian(num_points, 0.002, seed=7, device="cuda")
    n = num_points

    def build(dt):
        L = O.Sparse.from_csr(ip, ix, v.to(dt), (n, n))
        return SelfAdjoint(O.Kronecker(O.Dense(A1.to(dt)), O.Dense(A2.to(dt))) + L)
    op32 = build(torch.float32)
    start = randn(n, dtype=torch.float32, key=42)
    (vals, vecs), t = _timed(lambda: eig(op32, k, "LM", Lanczos(start_vector=start, max_iters=steps, tol=1e-12)), 1, 1)
    op64 = build(torch.float64)
    vals64, _ = eig(op64, k, "LM", Lanczos(start_vector=start.double(), max_iters=steps, tol=1e-12))
    AV = op32 @ vecs
    res = (AV - vecs * vals[None, :]).norm(dim=0) / vals.abs()
    return {"config": "kron1024x1024+rgg-lanczos-top64", "n": n, "nnz_L": int(ix.numel()), "s_per_eigsolve": t,
            "eigsolves_per_s": 1 / t, "max_rel_eig_err_vs_fp64_lanczos":
                float(((vals.double() - vals64) / vals64).abs().max()),
            "ritz_rel_residual_top8_max": float(res[-8:].max()), "ritz_rel_residual_top64_median": float(res.median()),
            "lambda_max": float(vals[-1])}


RUNNERS = {"c1": c1_dense, "c2": c2_diffusion3d, "c3a": c3a_rbf_batch, "c3b": c3b_kron_slq, "c5": c5_lanczos_topk}
