"""The reference's CG loop restated with torch CPU ops -- TEST / BASELINE INFRASTRUCTURE ONLY.

Same operations, in the same order, as cola/linalg/inverse/cg.py:94-178 on the torch backend
(torch.sparse_csr_tensor @ X for Sparse._matmat, operators.py:77-78; norms over axis -2;
do_safe_div; the Diagonal preconditioner d[:, None] * r, operators.py:338-339), including the
per-iteration host read of the mean residual (torch_tqdm.py:42) and of the stop flag
(cg.py:133-138).  bench.py times it on the host cores as the CPU baseline of the reference path.
"""
from __future__ import annotations

import torch

SMALL = 1e-40


def _safe_div(num, den):
    small = torch.tensor(SMALL, dtype=num.dtype)
    return num / torch.where(den.abs() < small, small, den)


def run_batched_cg(matmat, b, x0, max_iters, tol, precond=None):
    P = precond if precond is not None else (lambda v: v)
    mult = torch.linalg.norm(b, dim=-2, keepdim=True)
    bn = _safe_div(b, mult)
    x = x0
    r = bn - matmat(x)
    z = P(r)
    p = z
    gamma = torch.sum(r * z, dim=-2, keepdim=True)
    tol_eff = tol * torch.linalg.norm(r, dim=-2, keepdim=True) + tol
    k = 0
    errors = []
    while True:
        errors.append(torch.linalg.norm(r, dim=-2).mean().item())           # torch_tqdm.py:42
        rs = torch.linalg.norm(r, dim=-2, keepdim=True)
        if not (bool(torch.any(rs > tol_eff)) and k < max_iters):            # cg.py:133-138
            break
        conv = rs < SMALL
        Ap = matmat(p)
        alpha = torch.where(conv, torch.zeros_like(gamma), _safe_div(gamma, torch.sum(p * Ap, dim=-2, keepdim=True)))
        x = x + alpha * p
        r = r - alpha * Ap
        z = P(r)
        g1 = torch.sum(r * z, dim=-2, keepdim=True)
        beta = torch.where(conv, torch.zeros_like(g1), _safe_div(g1, gamma))
        gamma = g1
        p = z + beta * p
        k += 1
    return x * mult, k, errors


def csr_matmat(indptr, indices, values, n):
    A = torch.sparse_csr_tensor(indptr.to(torch.int64), indices.to(torch.int64), values, (n, n))
    return lambda X: A @ X
