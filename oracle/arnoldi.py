"""Arnoldi and GMRES restated in numpy -- TEST INFRASTRUCTURE ONLY (the CPU oracle of the
reference's non-symmetric Krylov path; the package never imports it).

``arnoldi`` follows cola/linalg/decompositions/arnoldi.py:166-201 (driver), 303-324
(``arnoldi_fact``: one modified Gram-Schmidt pass, norm clipped at tol/2, the stop test
``norm > tol * H[1, 0]`` after the first step) and 327-334 (``init_arnoldi``); ``gmres`` follows
cola/linalg/inverse/gmres.py:39-117 (the default branch: the square m x m part of H, normal
equations H^T H + diag(padding) with columns whose largest entry is below 10 tol max|H| padded
and their coefficients zeroed).
"""
from __future__ import annotations

import numpy as np


def arnoldi(A, v0, max_iters, tol):
    """Q (n, m+1), H (m+1, m), iterations (the reference's info['iterations']).  A: (n, n) array."""
    n = A.shape[0]
    max_iters = min(int(max_iters), n)
    Q = np.zeros((n, max_iters + 1), dtype=A.dtype)
    H = np.zeros((max_iters + 1, max_iters), dtype=A.dtype)
    norm = np.linalg.norm(v0)
    Q[:, 0] = v0 / norm
    idx = 0
    evals = 0
    while True:
        evals += 1
        is_large = (norm > tol * H[1, 0]) or idx <= 0
        if not (idx < max_iters and is_large):
            break
        w = A @ Q[:, idx]
        h = np.zeros(max_iters + 1, dtype=A.dtype)
        for j in range(idx + 1):
            h[j] = np.dot(Q[:, j], w)
            w = w - h[j] * Q[:, j]
        norm = np.linalg.norm(w)
        w = w / max(norm, tol / 2.0)
        h[idx + 1] = norm
        H[:, idx] = h
        Q[:, idx + 1] = w
        idx += 1
    return Q, H, evals


def gmres(A, b, max_iters, tol, x0=None):
    """Solution of A x = b by the reference's GMRES (x0 = 0 by default).  b: (n,) or (n, k)."""
    is_vector = b.ndim == 1
    B = b[:, None] if is_vector else b
    X0 = np.zeros_like(B) if x0 is None else (x0[:, None] if is_vector else x0)
    out = np.zeros_like(B)
    for c in range(B.shape[1]):
        res = B[:, c] - A @ X0[:, c]
        Q, H, _ = arnoldi(A, res, max_iters, tol)
        Q, H = Q[:, :-1], H[:-1, :]
        beta = np.linalg.norm(res)
        largest = np.abs(H).max(axis=-1)
        thresh = 10 * tol * largest.max()
        pad = np.where(largest < thresh, 1.0, 0.0)
        y = np.linalg.solve(H.T @ H + np.diag(pad), H.T[:, 0]) * beta
        y = np.where(largest < thresh, 0.0, y)
        out[:, c] = X0[:, c] + Q @ y
    return out[:, 0] if is_vector else out
