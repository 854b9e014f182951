"""Conjugate gradients restated in numpy (oracle; cola/linalg/inverse/cg.py:39-178 and the
while_loop_winfo bookkeeping of cola/utils/torch_tqdm.py:7-71).  Arithmetic runs in the dtype of
b (float32 reproduces the reference's float32 run up to summation order, float64 is the FP64
oracle)."""
from __future__ import annotations

import numpy as np

SMALL = 1e-40


def safe_div(num, den):
    """do_safe_div (cg.py:173-178)."""
    den = np.where(np.abs(den) < np.asarray(SMALL, dtype=den.dtype), np.asarray(SMALL, dtype=den.dtype), den)
    return num / den


def run_batched_cg(matmat, b, x0, max_iters, tol, precond=None):
    """run_batched_cg (cg.py:94-119) with take_cg_step (:141-154).

    Returns (x, r, k, info) with x and r scaled back by |b| and info = {'iterations', 'errors'}
    as recorded by while_loop_winfo (one error per cond evaluation plus a final one, first two
    dropped)."""
    b = np.asarray(b)
    dt = b.dtype
    norm = lambda v: np.sqrt(np.sum(v * v, axis=0, keepdims=True)).astype(dt)  # noqa: E731
    P = precond if precond is not None else (lambda v: v)
    mult = norm(b)
    bn = safe_div(b, mult)
    x = np.array(x0, dtype=dt, copy=True)
    r = (bn - matmat(x)).astype(dt)                     # initialize (:122-130)
    z = P(r).astype(dt)
    p = z.copy()
    gamma = np.sum(r * z, axis=0, keepdims=True).astype(dt)
    tol_eff = (tol * norm(r) + tol).astype(dt)          # (:101)
    k = 0
    errors = []
    while True:
        errors.append(float(np.mean(norm(r))))
        if not (np.any(norm(r) > tol_eff) and k < max_iters):   # cond_fun (:133-138)
            break
        conv = norm(r) < np.asarray(SMALL, dtype=dt)
        Ap = matmat(p).astype(dt)
        alpha = safe_div(gamma, np.sum(p * Ap, axis=0, keepdims=True).astype(dt))
        alpha = np.where(conv, np.zeros_like(alpha), alpha)
        x = x + alpha * p
        r = r - alpha * Ap
        z = P(r).astype(dt)
        g1 = np.sum(r * z, axis=0, keepdims=True).astype(dt)
        beta = np.where(conv, np.zeros_like(g1), safe_div(g1, gamma))
        gamma = g1
        p = z + beta * p
        k += 1
    errors.append(float(np.mean(norm(r))))
    info = {"iterations": len(errors) - 1, "errors": np.array(errors[2:])}
    return x * mult, r * mult, k, info


def cg_solve(matmat, rhs, x0=None, precond=None, tol=1e-6, max_iters=5000):
    """cg() (cg.py:39-69): vector or matrix right-hand side."""
    rhs = np.asarray(rhs)
    is_vec = rhs.ndim == 1
    B = rhs[:, None] if is_vec else rhs
    X0 = np.zeros_like(B) if x0 is None else (np.asarray(x0)[:, None] if is_vec else np.asarray(x0))
    x, _, k, info = run_batched_cg(matmat, B, X0, max_iters, tol, precond)
    return (x[:, 0] if is_vec else x), k, info


def ir_solve(matvec64, matvec_lo, b, tol=1e-8, inner_tol=1e-4, max_sweeps=20, max_inner=20000, precond=None):
    """FP64 iterative refinement around a low-precision CG (the structure of the batched device
    solver): x += |r| * CG_lo(A, r/|r|), r = b - A x in FP64, until |r|/|b| <= tol."""
    b = np.asarray(b, dtype=np.float64)
    x = np.zeros_like(b)
    r = b.copy()
    bn = np.linalg.norm(b)
    total = 0
    for sweep in range(max_sweeps):
        rn = np.linalg.norm(r)
        if rn / bn <= tol:
            return x, total, sweep, rn / bn
        rhat = (r / rn).astype(np.float32)
        d, k = _plain_pcg(matvec_lo, rhat, inner_tol, max_inner, precond)
        total += k
        x = x + rn * d.astype(np.float64)
        r = b - matvec64(x)
    return x, total, max_sweeps, np.linalg.norm(r) / bn


def _plain_pcg(matvec, b, tol, max_iters, precond):
    P = precond if precond is not None else (lambda v: v)
    x = np.zeros_like(b)
    r = b.copy()
    z = P(r).astype(b.dtype)
    p = z.copy()
    gamma = np.dot(r, z)
    k = 0
    while np.linalg.norm(r) > tol and k < max_iters:
        Ap = matvec(p).astype(b.dtype)
        pap = np.dot(p, Ap)
        if not pap > 0:
            break
        alpha = gamma / pap
        x = x + alpha * p
        r = r - alpha * Ap
        z = P(r).astype(b.dtype)
        g1 = np.dot(r, z)
        p = z + (g1 / gamma) * p
        gamma = g1
        k += 1
    return x, k
