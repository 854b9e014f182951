"""Lanczos, Lanczos quadrature and Hutchinson restated in numpy (oracle).

Follows cola/linalg/decompositions/lanczos.py:185-296 (init_lanczos, lanczos_fact,
do_double_gram), cola/linalg/unary/unary.py:46-60 (LanczosUnary._matmat),
cola/linalg/tbd/slq.py:37-52 (slq_fwd) and cola/linalg/trace/diagonal_estimation.py:159-210.
Tridiagonal eigenproblems are solved with numpy.linalg.eigh in float64.
"""
from __future__ import annotations

import numpy as np


def lanczos(matmat, rhs, max_iters, tol):
    """Batched Lanczos with full CGS2 reorthogonalisation.

    rhs: (n, bs).  Returns (alpha (bs, iters-1), beta (bs, iters), Q (bs, n, iters), i_final) where
    alpha/beta are the reference's names: beta = the diagonal of T, alpha = its off-diagonal."""
    rhs = np.asarray(rhs)
    dt = rhs.dtype
    n, bs = rhs.shape
    max_iters = min(max_iters, n)
    diag = np.zeros((bs, max_iters), dtype=dt)
    subdiag = np.zeros((bs, max_iters + 1), dtype=dt)
    V = np.zeros((bs, n, max_iters + 2), dtype=dt)
    V[:, :, 1] = (rhs / np.linalg.norm(rhs, axis=0, keepdims=True)).T    # init_lanczos (:275-284)
    i = 1
    while True:
        is_large = (subdiag[:, i - 1] > tol * subdiag[:, 1]) | (i <= 1)  # cond_fun (:263-268)
        if not (i <= max_iters and np.any(is_large)):
            break
        V[:, :, i] = V[:, :, i] / np.linalg.norm(V[:, :, i], axis=-1, keepdims=True)
        w = matmat(V[:, :, i].T).T.astype(dt)                              # (bs, n)
        diag[:, i - 1] = np.sum(w * V[:, :, i], axis=-1)
        w = w - (diag[:, [i - 1]] * V[:, :, i] + subdiag[:, [i - 1]] * V[:, :, i - 1])
        for _ in range(2):                                                 # do_double_gram (:287-296)
            h = np.einsum("bnj,bn->bj", V, w)
            w = w - np.einsum("bnj,bj->bn", V, h)
        V[:, :, i + 1] = w
        subdiag[:, i] = np.linalg.norm(w, axis=-1)
        i += 1
    iters = i - 1
    alpha = subdiag[:, 1:-1][:, : max(iters - 1, 0)]
    beta = diag[:, :iters]
    Q = V[:, :, 1 : iters + 1]
    return alpha, beta, Q, i


def tridiag_dense(alpha, beta):
    T = np.diag(beta.astype(np.float64))
    if beta.size > 1:
        T += np.diag(alpha.astype(np.float64), -1) + np.diag(alpha.astype(np.float64), 1)
    return T


def lanczos_eigs(matmat, start, max_iters, tol):
    """lanczos_eigs (lanczos.py:34-61) for one start vector: ascending eigenvalues and Ritz vectors."""
    alpha, beta, Q, _ = lanczos(matmat, np.asarray(start)[:, None], max_iters, tol)
    evals, evecs = np.linalg.eigh(tridiag_dense(alpha[0], beta[0]))
    return evals, Q[0] @ evecs


def lanczos_unary_matmat(matmat, f, V, max_iters, tol, eps):
    """LanczosUnary._matmat (unary.py:46-60): f(A) V by Lanczos quadrature; eps = finfo(dtype).eps."""
    V = np.asarray(V)
    alpha, beta, Q, _ = lanczos(matmat, V, max_iters, tol)
    out = np.zeros_like(V, dtype=np.float64)
    norms = np.linalg.norm(V, axis=0)
    for b in range(V.shape[1]):
        ev, P = np.linalg.eigh(tridiag_dense(alpha[b], beta[b]))
        thresh = 10 * eps * np.max(np.abs(ev))
        fe = np.where(np.abs(ev) > thresh, f(np.where(np.abs(ev) > thresh, ev, 1.0)), 0.0)
        out[:, b] = Q[b].astype(np.float64) @ (P @ (fe * P[0, :] * norms[b]))
    return out


def slq_estimate(matmat, f, probes, max_iters, tol, eps):
    """slq_fwd (tbd/slq.py:37-52): n * mean_b sum_j tau_bj^2 f(lambda_bj)."""
    probes = np.asarray(probes)
    n = probes.shape[0]
    alpha, beta, _, _ = lanczos(matmat, probes, max_iters, tol)
    ests = []
    for b in range(probes.shape[1]):
        ev, P = np.linalg.eigh(tridiag_dense(alpha[b], beta[b]))
        const = 10 * eps * np.max(ev)
        fv = np.where(np.abs(ev) > const, f(np.where(np.abs(ev) > const, ev, 1.0)), 0.0)
        ests.append(n * np.sum(P[0, :] ** 2 * fv))
    return float(np.mean(ests)), np.array(ests)


def hutchinson_diag(apply, n, probe_rounds, bs):
    """hutchinson_diag_estimate body (diagonal_estimation.py:182-210) for k = 0 with the probe
    blocks given: returns the per-entry mean of (A z) * z."""
    s = np.zeros(n)
    for z in probe_rounds:
        s += np.sum(apply(z) * z, axis=-1)
    return s / (len(probe_rounds) * bs)
