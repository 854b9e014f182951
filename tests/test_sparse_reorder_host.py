"""Sparse.reordered(): the same matrix stored in reverse Cuthill-McKee order (host-side checks)."""
import numpy as np
import torch

import cola_gb300 as cola
from cola_gb300.workloads import rgg_laplacian


def _rgg(n=600, r=0.08, seed=3):
    ip, ix, v = rgg_laplacian(n, r, seed=seed, device="cpu")
    return cola.ops.Sparse.from_csr(ip, ix, v.double(), (n, n))


def test_reordered_is_the_same_matrix_with_a_narrow_band():
    A = _rgg()
    R = A.reordered()
    assert R.perm is not None and sorted(R.perm.tolist()) == list(range(A.shape[0]))
    assert torch.equal(R.to_dense(), A.to_dense())
    # stored matrix = P A P^T, with a much smaller bandwidth than the random numbering
    perm = R.perm.long()
    stored = A.to_dense()[perm][:, perm]
    rows = torch.repeat_interleave(torch.arange(A.shape[0]), (R.indptr[1:] - R.indptr[:-1]).long())
    S = torch.zeros_like(stored)
    S[rows, R.indices.long()] = R.values
    assert torch.equal(S, stored)
    band = lambda ip, ix: int((ix.long() - torch.repeat_interleave(torch.arange(len(ip) - 1), (ip[1:] - ip[:-1]).long())).abs().max())
    assert band(R.indptr, R.indices) < band(A.indptr, A.indices) / 4
    assert R.reordered() is R


def test_reordered_transpose_and_tensor_matmat():
    from cola_gb300.linalg.autodiff import torch_matmat
    A = _rgg(seed=5)
    R = A.reordered()
    X = torch.randn(A.shape[0], 3, dtype=torch.float64, generator=torch.Generator().manual_seed(0))
    assert torch.allclose(torch_matmat(R, X), A.to_dense() @ X, rtol=1e-12, atol=1e-12)
    assert torch.equal(R.T.to_dense(), A.to_dense().T)
