"""The structured matvec's vector-Jacobian products on the device (colagb_matmat_vjp) against torch
autograd of the dense product, and the CG / SLQ backward passes that use them (cg_bwd,
cola/linalg/inverse/cg.py:72-86): Dense, Sparse and Diagonal leaves under Sum and ScalarMul, FP32 and
FP64; a Kronecker tree is refused by the kernel and falls back to the tensor-op restatement."""
import ctypes as C

import pytest
import torch

import cola_gb300 as cola
from cola_gb300 import _capi
from cola_gb300.linalg.autodiff import _vjp_params_device
from cola_gb300.lowering import lower

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")


def _operators(dtype):
    g = torch.Generator().manual_seed(0)
    n = 40
    D = torch.randn(n, n, generator=g, dtype=dtype)
    d = torch.rand(n, generator=g, dtype=dtype) + 1
    rows = torch.arange(n).repeat_interleave(3)
    cols = torch.stack([torch.arange(n), (torch.arange(n) + 1) % n, (torch.arange(n) + 7) % n], 1).reshape(-1)
    vals = torch.randn(3 * n, generator=g, dtype=dtype)
    order = torch.argsort(rows * n + cols)
    S = cola.ops.Sparse(vals[order].to(DEV), rows[order].to(DEV), cols[order].to(DEV), (n, n))
    Dd, dd = cola.ops.Dense(D.to(DEV)), cola.ops.Diagonal(d.to(DEV))
    return Dd + S + dd + 0.5 * cola.ops.I_like(Dd), [Dd.A, S.values, dd.diag], (Dd, S, dd)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_matmat_vjp_kernels_match_autograd(dtype):
    A, tensors, (Dd, S, dd) = _operators(dtype)
    g = torch.Generator().manual_seed(1)
    X = torch.randn(40, 3, generator=g, dtype=dtype).to(DEV)
    G = torch.randn(40, 3, generator=g, dtype=dtype).to(DEV)
    got = _vjp_params_device(A, tensors, X, G)
    assert got is not None
    # reference: autograd of the dense matrix that the operator represents
    Dt = Dd.A.detach().clone().requires_grad_(True)
    vt = S.values.detach().clone().requires_grad_(True)
    dt = dd.diag.detach().clone().requires_grad_(True)
    Sd = torch.zeros(40, 40, dtype=dtype, device=DEV).index_put((S.row_indices, S.col_indices), vt, accumulate=True)
    Y = Dt @ X + Sd @ X + dt[:, None] * X + 0.5 * X
    ref = torch.autograd.grad((G * Y).sum(), [Dt, vt, dt])
    tol = 1e-5 if dtype == torch.float32 else 1e-12
    for a, b in zip(got, ref):
        assert float((a - b).norm() / b.norm()) < tol


def test_matmat_vjp_refuses_kronecker_and_cg_backward_still_works():
    g = torch.Generator().manual_seed(2)
    F1 = torch.randn(6, 6, generator=g, dtype=torch.float64)
    F1 = (F1 @ F1.T + 6 * torch.eye(6, dtype=torch.float64)).to(DEV).requires_grad_(True)
    F2 = (torch.eye(5, dtype=torch.float64) * 2).to(DEV)
    K = cola.ops.Kronecker(cola.ops.Dense(F1), cola.ops.Dense(F2))
    low = lower(K)
    ptrs = (C.c_void_p * len(low.nodes))()
    X = torch.randn(30, 1, dtype=torch.float64, device=DEV)
    st = _capi.load().colagb_matmat_vjp(low.handle, X.data_ptr(), 1, X.data_ptr(), 1, 1, 1.0, ptrs,
                                        _capi.stream_ptr(DEV))
    assert st == _capi.ERR_UNSUPPORTED
    b = torch.randn(30, dtype=torch.float64, device=DEV)
    x, _ = cola.linalg.cg(cola.PSD(K), b, tol=1e-12, max_iters=500)
    x.sum().backward()
    Kd = torch.kron(F1.detach(), F2)
    F1r = F1.detach().clone().requires_grad_(True)
    xr = torch.linalg.solve(torch.kron(F1r, F2), b)
    xr.sum().backward()
    assert float((F1.grad - F1r.grad).norm() / F1r.grad.norm()) < 1e-8
    _ = Kd


def test_cg_backward_through_device_vjp_matches_dense_autograd():
    g = torch.Generator().manual_seed(3)
    n = 50
    M = torch.randn(n, n, generator=g, dtype=torch.float64)
    A0 = (M @ M.T / n + torch.eye(n, dtype=torch.float64)).to(DEV)
    A = A0.clone().requires_grad_(True)
    d = (torch.rand(n, generator=g, dtype=torch.float64) + 1).to(DEV).requires_grad_(True)
    op = cola.PSD(cola.ops.Dense(A) + cola.ops.Diagonal(d))
    b = torch.randn(n, generator=g, dtype=torch.float64).to(DEV)
    x, _ = cola.linalg.cg(op, b, tol=1e-13, max_iters=2000)
    (x * torch.arange(n, device=DEV)).sum().backward()
    Ar = A0.clone().requires_grad_(True)
    dr = d.detach().clone().requires_grad_(True)
    xr = torch.linalg.solve(Ar + torch.diag(dr), b)
    (xr * torch.arange(n, device=DEV)).sum().backward()
    assert float((A.grad - Ar.grad).norm() / Ar.grad.norm()) < 1e-8
    assert float((d.grad - dr.grad).norm() / dr.grad.norm()) < 1e-8
