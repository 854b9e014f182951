"""solve / inv / cg (cola/linalg/inverse/inv.py, cola/linalg/inverse/cg.py).

``cg`` runs the whole conjugate-gradient loop in libcolagb (colagb_cg_solve): a single persistent
kernel for Dense / Sparse operators (optionally plus c*I) with identity or Diagonal
preconditioning, otherwise the generic device loop over the lowered operator program.  The info
dict carries the reference's keys (torch_tqdm.py:28, 53, 62) plus ``fused``.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import torch

from .. import _capi
from .. import ops as O
from ..annotations import PSD, Unitary
from ..lowering import lower, operator_device
from .algorithms import CG, GMRES, LU, Algorithm, Auto, Cholesky


class IterativeOperatorWInfo(O.LinearOperator):
    """Lazy A^-1 through an iterative algorithm; stores the last call's info (algorithm_base.py:17-30)."""

    def __init__(self, A: O.LinearOperator, alg: Algorithm):
        self.device = A.device
        super().__init__(A.dtype, A.shape)
        self.A = A
        self.alg = alg
        self.info = {}

    def _matmat(self, X):
        Y, self.info = self.alg(self.A, X)
        return Y

    def __str__(self):
        return f"{self.alg}({self.A})"


def cg(A: O.LinearOperator, rhs: torch.Tensor, x0=None, P=None, tol=1e-6, max_iters=5000, pbar=False,
       check_every: int = 16, allow_fused: bool = True, graph: bool = True):
    """Solve A X = B by CG (cg.py:39-69).  Returns (solution, info).

    ``graph``: when the multi-launch loop runs (general operators / preconditioners), replay one
    captured CUDA graph per block of ``check_every`` steps instead of launching every kernel.

    Differentiable in ``rhs`` and in the operator's tensors with the reference's rule (cg_bwd,
    cg.py:72-86): the adjoint is one more CG solve with the same tolerance, iterations and P."""
    from .autodiff import cg_with_grad, wants_grad
    if wants_grad(A, rhs):
        def solve(b, first=[True]):
            use_x0 = x0 if first[0] else None
            first[0] = False
            return _cg_device(A, b.detach(), use_x0, P, tol, max_iters, check_every, allow_fused, graph)
        return cg_with_grad(A, rhs, solve)
    return _cg_device(A, rhs, x0, P, tol, max_iters, check_every, allow_fused, graph)


def _cg_device(A, rhs, x0, P, tol, max_iters, check_every, allow_fused, graph=True):
    low = lower(A)
    dev = operator_device(A, low)
    _capi.require_cuda(rhs)
    lib = _capi.load()
    dt = low.compute_dtype
    is_vector = rhs.dim() == 1
    B = rhs.reshape(-1, 1) if is_vector else rhs
    B = B.to(dt).contiguous()
    n, k = B.shape
    if x0 is None:
        X = torch.zeros_like(B)
    else:
        X = (x0.reshape(-1, 1) if x0.dim() == 1 else x0).to(dt).contiguous().clone()
    plow = None
    if P is not None and not isinstance(P, O.Identity):
        plow = lower(P)
    max_iters = int(max_iters)
    hist = torch.zeros(max_iters + 1, dtype=dt, device=dev)
    prm = _capi.CgParams(tol=float(tol), max_iters=max_iters, check_every=int(check_every),
                         allow_fused=1 if allow_fused else 0, graph=0 if graph else 1, spin_limit=0)
    res = _capi.CgResult()
    nbytes = C.c_size_t()
    _capi.check(lib.colagb_cg_workspace_bytes(low.handle, plow.handle if plow else None, k, C.byref(nbytes)), "cg")
    ws = _capi.workspace(nbytes.value, dev)
    t0 = time.time()
    _capi.check(lib.colagb_cg_solve(low.handle, plow.handle if plow else None, B.data_ptr(), k, X.data_ptr(), k, k,
                                    C.byref(prm), hist.data_ptr(), ws.data_ptr(), nbytes.value, C.byref(res),
                                    _capi.stream_ptr(dev)), "cg")
    elapsed = time.time() - t0
    its = int(res.iterations)
    h = hist[: its + 1].double().cpu().numpy()
    # while_loop_winfo records the error at every cond evaluation plus once more at the end and drops
    # the first two entries (torch_tqdm.py:45-62)
    errors = np.concatenate([h, h[-1:]])[2:]
    info = {"iterations": its + 1, "errors": errors, "iteration_time": elapsed / (its + 1), "fused": bool(res.fused),
            "graph": bool(res.graph)}
    soln = X.reshape(-1) if is_vector else X
    return soln, info


# ---------------------------------------------------------------------------------------------
# inv / solve dispatch (inv.py:24-165)

def solve(A, b, alg: Algorithm = Auto()):
    """A^-1 b (inv.py:24-39)."""
    return inv(A, alg) @ b


def _dense_cholesky_inv(A):
    L = torch.linalg.cholesky(A.to_dense())
    return _DenseSolve(L, A, kind="chol")


def _dense_lu_inv(A):
    return _DenseSolve(A.to_dense(), A, kind="lu")


class _DenseSolve(O.LinearOperator):
    """Small dense inverses for Auto on operators of at most 1e6 entries (inv.py:73-111)."""

    def __init__(self, M, A, kind):
        self.device = A.device
        super().__init__(A.dtype, A.shape)
        self.M, self.kind = M, kind

    def _matmat(self, X):
        if self.kind == "chol":
            return torch.cholesky_solve(X.to(self.M.dtype), self.M)
        return torch.linalg.solve(self.M, X.to(self.M.dtype))


def inv(A: O.LinearOperator, alg: Algorithm = Auto()):
    """Lazy inverse with the reference's dispatch rules (inv.py:43-165)."""
    # structural rules first (they win over the algorithm rules in the reference's dispatch)
    if A.isa(Unitary):
        from ..fns import adjoint
        return Unitary(adjoint(A))
    if isinstance(A, O.Identity):
        return A
    if isinstance(A, O.ScalarMul):
        return O.ScalarMul(1 / A.c, shape=A.shape, dtype=A.dtype, device=A.device)
    if isinstance(A, O.Diagonal):
        return O.Diagonal(1.0 / A.diag)
    if isinstance(A, O.Product) and all(M.shape[-2] == M.shape[-1] for M in A.Ms):
        return O.Product(*reversed([inv(M, alg) for M in A.Ms]))
    if isinstance(A, O.BlockDiag):
        return O.BlockDiag(*[inv(M, alg) for M in A.Ms], multiplicities=A.multiplicities)
    if isinstance(A, O.Kronecker):
        return O.Kronecker(*[inv(M, alg) for M in A.Ms])
    if isinstance(alg, GMRES):
        return IterativeOperatorWInfo(A, alg)
    if isinstance(alg, CG):
        assert A.isa(PSD), "CG only valid for PSD matrices, wrap in cola.PSD if desired"
        return IterativeOperatorWInfo(A, alg)
    if isinstance(alg, Auto):
        small = bool(np.prod(A.shape) <= 1e6)
        if A.isa(PSD):
            return inv(A, Cholesky() if small else CG(**alg.__dict__))
        if small:
            return inv(A, LU())
        return inv(A, GMRES(**alg.__dict__))
    if isinstance(alg, Cholesky):
        assert A.isa(PSD), "Cholesky only valid for PSD matrices, wrap in cola.PSD if desired"
        return _dense_cholesky_inv(A)
    if isinstance(alg, LU):
        return _dense_lu_inv(A)
    raise NotImplementedError(f"inv with {type(alg).__name__} is not implemented")
