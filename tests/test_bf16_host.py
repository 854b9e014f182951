"""The BF16 inner-matvec storage (COLAGB_MATVEC_BF16), restated on the host: off-diagonals rounded to
BF16, diagonal d'_i = a_ii - sum_j (bf16(a_ij) - a_ij).  For a weighted-Laplacian-type operator the
perturbation A' - A is a Laplacian of the rounding errors, so |x^T (A' - A) x| <= 2^-9 x^T A x for every
x -- checked here on random vectors and on the extreme eigenvectors, with a plain BF16 rounding of all
entries (diagonal included) as the contrast that breaks the bound."""
import numpy as np
import torch

from cola_gb300.workloads import diffusion_values_2d, grid_pattern_2d


def consistent_bf16(indptr, indices, vals):
    n = len(indptr) - 1
    rows = np.repeat(np.arange(n), np.diff(indptr))
    off = rows != indices
    v16 = vals.copy()
    v16[off] = torch.from_numpy(vals[off]).bfloat16().double().numpy()
    corr = np.zeros(n)
    np.add.at(corr, rows[off], v16[off] - vals[off])
    v16[~off] = vals[~off] - corr[rows[~off]]
    return v16


def dense(indptr, indices, vals, n):
    A = np.zeros((n, n))
    rows = np.repeat(np.arange(n), np.diff(indptr))
    np.add.at(A, (rows, indices), vals)
    return A


def test_consistent_bf16_diagonal_keeps_energy_norm_within_2_pow_minus_9():
    m = 24
    ip, ix, ok = grid_pattern_2d(m)
    g = torch.Generator().manual_seed(0)
    a = torch.exp(2.0 * torch.randn(1, m, m, generator=g, dtype=torch.float64))
    vals = diffusion_values_2d(a, ok)[0].double().numpy()
    ip, ix = ip.numpy(), ix.numpy()
    n = m * m
    A = dense(ip, ix, vals, n)
    A1 = dense(ip, ix, consistent_bf16(ip, ix, vals), n)
    A0 = dense(ip, ix, torch.from_numpy(vals).bfloat16().double().numpy(), n)  # plain rounding
    E1, E0 = A1 - A, A0 - A
    assert np.allclose(A1, A1.T)
    rng = np.random.default_rng(1)
    X = np.concatenate([rng.standard_normal((n, 64)), np.linalg.eigh(A)[1][:, :8]], axis=1)
    ratio1 = np.abs(np.einsum("ij,ij->j", X, E1 @ X)) / np.einsum("ij,ij->j", X, A @ X)
    ratio0 = np.abs(np.einsum("ij,ij->j", X, E0 @ X)) / np.einsum("ij,ij->j", X, A @ X)
    assert ratio1.max() <= 2.0 ** -9
    # plain rounding of the diagonal too is not bounded that way on the smooth (low-energy) modes
    assert ratio0.max() > 2.0 ** -9
    # and the consistent form stays SPD
    assert np.linalg.eigvalsh(A1).min() > 0
