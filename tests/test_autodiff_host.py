"""The differentiable matvec restatement used by the backward passes (CPU, no GPU needed)."""
import pytest
import torch

from cola_gb300 import ops as O
from cola_gb300.linalg.autodiff import operator_tensors, torch_matmat


def _ops():
    g = torch.Generator().manual_seed(0)
    A = torch.randn(6, 6, generator=g, dtype=torch.float64)
    B = torch.randn(3, 3, generator=g, dtype=torch.float64)
    C = torch.randn(2, 2, generator=g, dtype=torch.float64)
    d = torch.rand(6, generator=g, dtype=torch.float64) + 1
    rows = torch.tensor([0, 0, 1, 2, 3, 4, 5, 5, 2])
    cols = torch.tensor([0, 3, 1, 2, 3, 0, 5, 1, 2])
    vals = torch.randn(9, generator=g, dtype=torch.float64)
    S = O.Sparse(vals, rows, cols, (6, 6))
    Sd = torch.zeros(6, 6, dtype=torch.float64).index_put_((rows, cols), vals, accumulate=True)
    Bd = torch.block_diag(B, C, C)
    # (operator, its dense matrix written out independently of the library)
    return [(O.Dense(A), A), (S, Sd), (O.Diagonal(d), torch.diag(d)),
            (O.Dense(A) + 0.5 * O.I_like(O.Dense(A)), A + 0.5 * torch.eye(6, dtype=torch.float64)),
            (O.Product(O.Dense(A), O.Diagonal(d)), A @ torch.diag(d)),
            (O.Kronecker(O.Dense(B), O.Dense(C)), torch.kron(B, C)),
            (O.BlockDiag(O.Dense(B), O.Dense(C), multiplicities=[1, 2]), Bd), (O.Sum(O.Dense(A), S), A + Sd)]


@pytest.mark.parametrize("i", range(8))
def test_torch_matmat_matches_dense(i):
    M, D = _ops()[i]
    X = torch.randn(M.shape[1], 3, generator=torch.Generator().manual_seed(1), dtype=torch.float64)
    torch.testing.assert_close(torch_matmat(M, X), D @ X, rtol=1e-12, atol=1e-12)


def test_vjp_through_the_restatement_matches_dense_autograd():
    A = torch.randn(5, 5, dtype=torch.float64, requires_grad=True)
    d = torch.rand(5, dtype=torch.float64, requires_grad=True)
    M = O.Product(O.Dense(A), O.Diagonal(d))
    assert {id(t) for t in operator_tensors(M)} == {id(A), id(d)}
    X = torch.randn(5, 2, dtype=torch.float64)
    W = torch.randn(5, 2, dtype=torch.float64)
    (torch_matmat(M, X) * W).sum().backward()
    ga, gd = A.grad.clone(), d.grad.clone()
    A.grad = None
    d.grad = None
    ((A @ torch.diag(d)) @ X * W).sum().backward()
    torch.testing.assert_close(ga, A.grad)
    torch.testing.assert_close(gd, d.grad)
