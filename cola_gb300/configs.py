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
from .linalg.prng import PRNGKey, randn
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


def _fp64_pcg_oracle(ip, ix, v, B, tol=1e-12, max_iters=20000):
    """FP64 Jacobi-preconditioned CG on the GPU in plain torch tensor ops (torch's sparse CSR product), all
    right-hand sides together with per-column scalars: the FP64 oracle of the shared-matrix solves."""
    n = ip.numel() - 1
    A = torch.sparse_csr_tensor(ip.long(), ix.long(), v.double(), (n, n))
    rows = torch.repeat_interleave(torch.arange(n, device=ip.device), (ip[1:] - ip[:-1]).long())
    dg = torch.zeros(n, dtype=torch.float64, device=ip.device)
    dg.index_add_(0, rows, torch.where(rows == ix.long(), v.double(), torch.zeros_like(v, dtype=torch.float64)))
    dinv = (1.0 / dg)[:, None]
    Bt = B.T.contiguous().double()
    X = torch.zeros_like(Bt)
    R = Bt.clone()
    Z = dinv * R
    P = Z.clone()
    rz = (R * Z).sum(0)
    bn = Bt.norm(dim=0)
    it = 0
    for it in range(1, max_iters + 1):
        AP = A @ P
        al = rz / (P * AP).sum(0)
        X += al * P
        R -= al * AP
        if it % 25 == 0 and bool(((R.norm(dim=0) / bn) < tol).all()):
            break
        Z = dinv * R
        rz2 = (R * Z).sum(0)
        P = Z + (rz2 / rz) * P
        rz = rz2
    return X.T.contiguous(), it


def c2_diffusion3d(nrhs=32, m=128, steps=1, warmup=1):
    """7-point 128^3 diffusion + 1e-3 I, 32 right-hand sides, each to a 1e-8 FP64 true residual: the lockstep
    block schedule (matrix read once per step for all 32) and one cluster per right-hand side, FP32
    against BF16 inner matvecs (FP64 residual replacement in all), with and without Jacobi; solution
    error against an FP64 CG oracle run in plain torch ops."""
    ip, ix, v = diffusion_3d(m=m, device="cuda")
    fam = BatchedCSR(ip, ix, v[None, :], shared=True)
    B = torch.randn(nrhs, fam.n, device="cuda", dtype=torch.float64, generator=torch.Generator("cuda").manual_seed(2))
    X64, it64 = _fp64_pcg_oracle(ip, ix, v, B)
    out = {"config": f"diffusion3d-{m}^3-{nrhs}rhs", "n": fam.n, "nnz": int(ix.numel()),
           "fp64_oracle": f"Jacobi-PCG in torch FP64 ops to relres 1e-12 ({it64} steps)"}
    for prec in ("jacobi", "none"):
        for mv, sched in (("fp32", "block"), ("fp32", "cluster16"), ("bf16", "cluster16")):
            (X, info), t = _timed(lambda: solve_batched(fam, B, precond=prec, tol=1e-8, matvec=mv, schedule=sched),
                                  steps, warmup)
            err = ((X - X64).norm(dim=1) / X64.norm(dim=1)).max()
            out[f"{prec}_{mv}_{sched}"] = {"rhs_per_s": nrhs / t, "s_per_call": t,
                                   "mean_iters": float(info["iterations"].double().mean()),
                                   "max_true_relres": float(info["relres"].max()),
                                   "max_sol_err_vs_fp64": float(err), "schedule": info["schedule"]}
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
    # every CG step of system s reads its n_s^2 FP32 matrix once (the vectors add O(n_s) per step)
    streamed = sum(n * n * 4 * int(k) for (n, _, _), k in zip(meta, iters.tolist()))
    out = {"config": f"rbf-uneven-{num}", "systems_per_s": num / t, "s_per_call": t,
           "mean_iters": float(iters.double().mean()), "max_iters": int(iters.max()),
           "converged": int((status == 1).sum()), "true_relres_first8_max": worst,
           "matrix_bytes_per_sweep": bytes_sweep,
           "roofline": {"bound": "hbm", "matrix_bytes_streamed": streamed, "achieved_gbs": streamed / t / 1e9}}
    # with FP64 residual refinement (no counterpart in the reference): every system to 1e-8, checked
    # with an FP64 residual on all of them
    (res2, t2) = _timed(lambda: solve_dense_batched(mats, rhs, tol=1e-8, max_iters=max_iters, refine=True),
                        steps, warmup)
    sols2, iters2, status2 = res2
    worst2 = 0.0
    for A, b, x in zip(mats, rhs, sols2):
        r = (b.double() - A.double() @ x.double()).norm() / b.double().norm()
        worst2 = max(worst2, float(r))
    out["refined_to_1e-8"] = {"systems_per_s": num / t2, "s_per_call": t2, "converged": int((status2 == 1).sum()),
                              "max_true_relres_all_fp64": worst2,
                              "mean_inner_iters": float(iters2.double().mean())}
    return out


def c3b_kron_slq(probes=64, steps=100, reps=1, warmup=1):
    """logdet(Kronecker(K1, K2, K3) + 0.01 I), 64^3 = 262,144, 64 Rademacher probes, 100 Lanczos steps.
    The Kronecker contractions run on the tensor cores (three-product BF16 split, the default for
    contractions this large) and, for comparison, on the FP32 SIMT path.  Accuracy: the exact FP64
    log-determinant from the three 64 x 64 eigendecompositions."""
    Ks, ells = kron_rbf(seed=4, device="cpu")
    Z = torch.sign(randn(64 ** 3, probes, dtype=torch.float32, key=5)).to("cuda")
    lam = torch.ones(1, dtype=torch.float64)
    for k in Ks:
        lam = torch.kron(lam, torch.linalg.eigvalsh(k.double()))
    exact = float(torch.log(lam + 0.01).sum())
    out = {"config": "kron-rbf-64^3-slq", "exact": exact}
    for prec in ("auto", "fp32"):
        K = O.Kronecker(*[O.Dense(k.cuda()) for k in Ks], precision=prec)
        op = PSD(K + 0.01 * O.I_like(K))
        est, t = _timed(lambda: stochastic_lanczos_quad(op, torch.log, max_iters=steps, tol=0.0, probes=Z), reps,
                        warmup)
        out["tensor_cores_bf16x3" if prec == "auto" else "fp32_simt"] = {
            "logdets_per_s": 1 / t, "s_per_logdet": t, "estimate": float(est),
            "rel_err_vs_exact_fp64": abs(float(est) - exact) / abs(exact)}
    return out


def _arpack_fp64(A1, A2, ip, ix, v, k, tol=1e-8):
    """The FP64 oracle of the Lanczos eigensolve: scipy's ARPACK (eigsh, the k largest) with FP64
    matvecs A1 X A2^T + L x in torch on the GPU -- no kernel of this library involved."""
    import numpy as np
    import scipy.sparse.linalg as spla
    n = ip.numel() - 1
    A1d, A2d = A1.double().cuda(), A2.double().cuda()
    Ld = torch.sparse_csr_tensor(ip.long().cuda(), ix.long().cuda(), v.double().cuda(), (n, n))
    m1, m2 = A1.shape[0], A2.shape[0]

    def mv(x):
        xt = torch.from_numpy(np.ascontiguousarray(x).reshape(-1)).cuda()
        y = (A1d @ xt.reshape(m1, m2) @ A2d.T).reshape(-1) + Ld @ xt
        return y.cpu().numpy()
    t = time.perf_counter()
    w = spla.eigsh(spla.LinearOperator((n, n), matvec=mv, dtype=np.float64), k=k, which="LA", tol=tol,
                   return_eigenvectors=False)
    return np.sort(w), time.perf_counter() - t


def c5_lanczos_topk(k=64, steps=256, num_points=1 << 20):
    """64 largest eigenpairs of Sum(Kronecker(A1, A2), L): A1, A2 1024 x 1024 SPD (log-uniform spectrum in
    [1e-2, 1e1]), L the Laplacian of a random geometric graph on 2^20 points (radius 0.002); 256-step
    Lanczos with full reorthogonalisation, FP64 tridiagonal eigensolve.  Inputs come from CPU random
    generators (the same ones the reference's golden run used).  The Kronecker factors run on the tensor
    cores (three-product BF16 split) and, for comparison, on the FP32 SIMT path.  Accuracy: scipy's ARPACK
    on the FP64 operator (the top 12 Ritz values have converged in 256 steps) and the Ritz residuals
    |A v - lambda v| / |lambda|.  A third arm stores L in reverse Cuthill-McKee order (the same operator)."""
    import numpy as np
    from .annotations import SelfAdjoint
    from .linalg import Lanczos, eig
    from .workloads import rgg_laplacian
    A1, _, _ = dense_spd(1024, seed=6, lo=1e-2, hi=1e1, dtype=torch.float32)
    A2, _, _ = dense_spd(1024, seed=61, lo=1e-2, hi=1e1, dtype=torch.float32)
    ip, ix, v = rgg_laplacian(num_points, 0.002, seed=7, device="cpu")
    n = num_points
    L = O.Sparse.from_csr(ip.cuda(), ix.cuda(), v.cuda(), (n, n))
    start = randn(n, dtype=torch.float32, key=PRNGKey(42)).cuda()  # the reference's default start recipe
    arp, t_arp = _arpack_fp64(A1, A2, ip, ix, v, k)
    out = {"config": "kron1024x1024+rgg-lanczos-top64", "n": n, "nnz_L": int(ix.numel()),
           "fp64_oracle": f"scipy ARPACK eigsh on FP64 torch matvecs ({t_arp:.0f} s)"}
    t0 = time.perf_counter()
    Lr = L.reordered()
    t_reorder = time.perf_counter() - t0
    arms = (("tensor_cores_bf16x3", "auto", L), ("fp32_simt", "fp32", L), ("tensor_cores_bf16x3_rcm_L", "auto", Lr))
    for name, prec, Lx in arms:
        op = SelfAdjoint(O.Kronecker(O.Dense(A1.cuda()), O.Dense(A2.cuda()), precision=prec) + Lx)
        (vals, vecs), t = _timed(lambda: eig(op, k, "LM", Lanczos(start_vector=start, max_iters=steps, tol=1e-12)),
                                 1, 1)
        ours = np.sort(vals.double().cpu().numpy())
        AV = op @ vecs
        res = (AV - vecs * vals[None, :]).norm(dim=0) / vals.abs()
        out[name] = {
            "s_per_eigsolve": t, "eigsolves_per_s": 1 / t,
            "top12_max_rel_err_vs_arpack": float(np.max(np.abs(ours[-12:] - arp[-12:]) / arp[-12:])),
            "top64_max_rel_err_vs_arpack": float(np.max(np.abs(ours - arp) / arp)),
            "ritz_rel_residual_top8_max": float(res[-8:].max()),
            "ritz_rel_residual_top64_median": float(res.median()), "lambda_max": float(vals[-1])}
    # L stored in reverse Cuthill-McKee order (Sparse.reordered, once per operator on the host)
    out["tensor_cores_bf16x3_rcm_L"]["reorder_seconds_once"] = t_reorder
    return out


RUNNERS = {"c1": c1_dense, "c2": c2_diffusion3d, "c3a": c3a_rbf_batch, "c3b": c3b_kron_slq, "c5": c5_lanczos_topk}
