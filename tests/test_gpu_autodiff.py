"""Derivatives through the device CG and SLQ (the reference's cg_bwd / slq_bwd rules) against
torch autograd of dense FP64 solves."""
import pytest
import torch

import cola_gb300 as cola
from cola_gb300 import ops as O
from cola_gb300.annotations import PSD
from cola_gb300.linalg.inverse import cg
from cola_gb300.linalg.unary import stochastic_lanczos_quad

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")


def spd(n, seed, dtype=torch.float64):
    g = torch.Generator().manual_seed(seed)
    Q, _ = torch.linalg.qr(torch.randn(n, n, generator=g, dtype=torch.float64))
    lam = torch.exp(torch.empty(n, dtype=torch.float64).uniform_(0, 3, generator=g))
    return ((Q * lam) @ Q.T).to(dtype).to(DEV)


def test_cg_gradients_dense_matrix_and_rhs():
    n = 48
    A0 = spd(n, 0)
    b0 = torch.randn(n, dtype=torch.float64, device=DEV)
    w = torch.randn(n, dtype=torch.float64, device=DEV)
    A = A0.clone().requires_grad_(True)
    b = b0.clone().requires_grad_(True)
    x, info = cg(PSD(O.Dense(A)), b, tol=1e-12, max_iters=500)
    (x * w).sum().backward()
    A2 = A0.clone().requires_grad_(True)
    b2 = b0.clone().requires_grad_(True)
    (torch.linalg.solve(A2, b2) * w).sum().backward()
    torch.testing.assert_close(b.grad, b2.grad, rtol=1e-8, atol=1e-10)
    torch.testing.assert_close(A.grad, A2.grad, rtol=1e-8, atol=1e-10)
    assert info["iterations"] > 1


def test_cg_gradients_sparse_values_and_diagonal_shift():
    n = 64
    A0 = spd(n, 1)
    A0 = torch.where(A0.abs() > 0.3, A0, torch.zeros_like(A0)) + 5 * torch.eye(n, dtype=torch.float64, device=DEV)
    rows, cols = torch.nonzero(A0, as_tuple=True)
    vals = A0[rows, cols].clone().requires_grad_(True)
    d = torch.full((n,), 0.5, dtype=torch.float64, device=DEV, requires_grad=True)
    op = PSD(O.Sparse(vals, rows, cols, (n, n)) + O.Diagonal(d))
    B = torch.randn(n, 3, dtype=torch.float64, device=DEV)
    W = torch.randn(n, 3, dtype=torch.float64, device=DEV)
    X, _ = cg(op, B, tol=1e-12, max_iters=1000)
    (X * W).sum().backward()
    v2 = A0[rows, cols].clone().requires_grad_(True)
    d2 = torch.full((n,), 0.5, dtype=torch.float64, device=DEV, requires_grad=True)
    M = torch.zeros(n, n, dtype=torch.float64, device=DEV).index_put((rows, cols), v2) + torch.diag(d2)
    (torch.linalg.solve(M, B) * W).sum().backward()
    torch.testing.assert_close(vals.grad, v2.grad, rtol=1e-7, atol=1e-9)
    torch.testing.assert_close(d.grad, d2.grad, rtol=1e-7, atol=1e-9)


def test_slq_logdet_gradient_is_the_probe_estimate_of_a_inverse():
    """d/dA of the SLQ estimate with the reference's rule: (1/N) sum_i (A^-1 z_i) z_i^T with the
    forward's probes z_i (an unbiased estimate of A^-T = d logdet / dA)."""
    n, N = 40, 64
    A0 = spd(n, 2)
    A = A0.clone().requires_grad_(True)
    Z = torch.randn(n, N, dtype=torch.float64, device=DEV, generator=torch.Generator(DEV).manual_seed(3))
    est = stochastic_lanczos_quad(PSD(O.Dense(A)), torch.log, max_iters=n, tol=1e-12, probes=Z)
    est.backward()
    expect = torch.linalg.solve(A0, Z) @ Z.T / N
    # the backward rule solves A^-1 z_i by CG to tol 1e-6 (slq_bwd), so ~1e-6 relative agreement
    torch.testing.assert_close(A.grad, expect, rtol=1e-4, atol=1e-6)
    # the estimate itself agrees with the exact log-determinant to SLQ accuracy
    exact = torch.linalg.slogdet(A0)[1]
    assert abs(float(est) - float(exact)) < 0.1 * abs(float(exact)) + 1.0


def test_no_graph_without_requires_grad():
    A0 = spd(16, 4)
    x, _ = cg(PSD(O.Dense(A0)), torch.ones(16, dtype=torch.float64, device=DEV), tol=1e-10)
    assert not x.requires_grad
