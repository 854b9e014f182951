"""The learned FSAI factor through the reference's preconditioner hook: CG(P=G^T G) on one operator of
the 512 x 512-style diffusion family (here 128 x 128), cola.linalg.solve(PSD(Sparse), b, CG(P=...))
as the reference would call it (cola/linalg/inverse/cg.py:124, 150).  P applied as a LinearOperator must
give the solution of the batched solver's built-in FSAI path and need fewer CG steps than Jacobi
(P = Diagonal(1 / diag A)) and than no preconditioner."""
import torch
import pytest

import cola_gb300 as cola
from cola_gb300.linalg.batched import solve_batched
from cola_gb300.precond.learned_fsai import learned_preconditioner, preconditioner_for
from cola_gb300.workloads import diffusion_family_2d

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")


def test_learned_factor_as_cg_preconditioner_operator():
    fam, B, _, _ = diffusion_family_2d([5000], m=128, device=DEV)
    n = fam.n
    A = cola.PSD(cola.ops.Sparse.from_csr(fam.indptr, fam.indices, fam.values[0], (n, n)))
    b = B[0].float()
    P = learned_preconditioner(A)
    rows = torch.repeat_interleave(torch.arange(n, device=DEV), (fam.indptr[1:] - fam.indptr[:-1]).long())
    dg = torch.zeros(n, device=DEV).index_add_(0, rows, torch.where(rows == fam.indices.long(), fam.values[0],
                                                                    torch.zeros_like(fam.values[0])))
    its = {}
    sols = {}
    for name, Pop in (("learned", P), ("jacobi", cola.ops.Diagonal(1.0 / dg)), ("none", None)):
        x, info = cola.linalg.cg(A, b, P=Pop, tol=1e-6, max_iters=20000)
        its[name] = info["iterations"]
        sols[name] = x
        r = float((b.double() - torch.sparse_csr_tensor(fam.indptr.long(), fam.indices.long(), fam.values[0].double(),
                                                          (n, n)) @ x.double()).norm() / b.double().norm())
        assert r < 1e-4, (name, r)
    assert its["learned"] < its["jacobi"] < its["none"], its
    # the same factor inside the batched solver, to a tight FP64 residual: the two solutions agree
    Xb, ib = solve_batched(fam, B, precond="fsai", fsai=preconditioner_for(fam), tol=1e-10)
    x64 = Xb[0]
    assert float((sols["learned"].double() - x64).norm() / x64.norm()) < 1e-3
    # solve() with the algorithm object, as the reference's dispatch reaches it (inv.py:66-69)
    xs = cola.linalg.solve(A, b, cola.linalg.CG(tol=1e-6, max_iters=20000, P=P))
    assert torch.equal(xs, sols["learned"])
