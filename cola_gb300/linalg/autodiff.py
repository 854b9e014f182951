"""Reverse-mode derivatives of the iterative solvers (cola/utils/custom_autodiff.py:43-70).

* ``cg``: the adjoint of x = A^-1 b is db = A^-1 dx (one more CG solve on the device, A symmetric)
  and, for the operator's tensors theta, the vector-Jacobian product of theta -> A(theta) x with
  -db (cg_bwd, cola/linalg/inverse/cg.py:72-86).
* ``stochastic_lanczos_quad`` (f = log): d/dtheta ~ (1/N) sum_i vjp(theta -> A(theta) z_i) at
  A^-1 z_i / N with the forward's own probes z_i, the A^-1 z_i from CG with tol 1e-6 and 100
  iterations (slq_bwd, cola/linalg/tbd/slq.py:10-31; like the reference, this rule is that of
  f = log).

The vector-Jacobian products with respect to the operator's tensors run in the library's kernels
(``colagb_matmat_vjp``) for Dense / Sparse / Diagonal leaves under Sum / ScalarMul / Identity; for
Product, Kronecker and BlockDiag trees they go through ``torch_matmat``, a differentiable tensor-op
restatement of the operator tree's matvec, which only runs in backward passes.
"""
from __future__ import annotations

import torch

from .. import ops as O


def operator_tensors(A: O.LinearOperator) -> list:
    """The tensors an operator tree is built from (each once), in a fixed order."""
    out, seen = [], set()

    def add(t):
        if isinstance(t, torch.Tensor) and id(t) not in seen:
            seen.add(id(t))
            out.append(t)

    def walk(M):
        if isinstance(M, O.Dense):
            add(M.A)
        elif isinstance(M, O.Sparse):
            add(M.values)
        elif isinstance(M, O.Diagonal):
            add(M.diag)
        elif isinstance(M, (O.Sum, O.Product, O.Kronecker, O.BlockDiag)):
            for c in M.Ms:
                walk(c)
    walk(A)
    return out


def torch_matmat(A: O.LinearOperator, X: torch.Tensor, sub: dict | None = None) -> torch.Tensor:
    """A @ X with tensor ops, differentiable in the operator's tensors; ``sub`` maps id(tensor) to a
    replacement (the copies that gradients are taken with respect to)."""
    sub = sub or {}

    def t(x):
        return sub.get(id(x), x)

    if isinstance(A, O.Dense):
        return t(A.A).to(X.dtype) @ X
    if isinstance(A, O.Sparse):
        if A.perm is not None:  # stored in a permuted order: the triplets in original coordinates
            rows, cols = A.row_indices.to(torch.int64), A.col_indices.to(torch.int64)
        else:
            rows = torch.repeat_interleave(torch.arange(A.shape[0], device=X.device),
                                           (A.indptr[1:] - A.indptr[:-1]).to(torch.int64))
            cols = A.indices.to(torch.int64)
        contrib = t(A.values).to(X.dtype)[:, None] * X[cols]
        return torch.zeros((A.shape[0], X.shape[1]), dtype=X.dtype, device=X.device).index_add(0, rows, contrib)
    if isinstance(A, O.Diagonal):
        return t(A.diag).to(X.dtype)[:, None] * X
    if isinstance(A, O.ScalarMul):
        return A.c * X
    if isinstance(A, O.Identity):
        return X
    if isinstance(A, O.Sum):
        out = torch_matmat(A.Ms[0], X, sub)
        for M in A.Ms[1:]:
            out = out + torch_matmat(M, X, sub)
        return out
    if isinstance(A, O.Product):
        out = X
        for M in reversed(A.Ms):
            out = torch_matmat(M, out, sub)
        return out
    if isinstance(A, O.Kronecker):
        k = X.shape[1]
        dims = [M.shape[1] for M in A.Ms]
        Y = X.reshape(*dims, k)
        for i, M in enumerate(A.Ms):
            Yi = Y.movedim(i, 0)
            rest = Yi.shape[1:]
            Zi = torch_matmat(M, Yi.reshape(M.shape[1], -1), sub)
            Y = Zi.reshape(M.shape[0], *rest).movedim(0, i)
        return Y.reshape(A.shape[0], k)
    if isinstance(A, O.BlockDiag):
        outs, r0 = [], 0
        k = X.shape[1]
        for M, c in zip(A.Ms, A.multiplicities):
            nb = M.shape[1]
            Xb = X[r0: r0 + c * nb].reshape(c, nb, k).permute(1, 0, 2).reshape(nb, c * k)
            Yb = torch_matmat(M, Xb, sub).reshape(M.shape[0], c, k).permute(1, 0, 2).reshape(c * M.shape[0], k)
            outs.append(Yb)
            r0 += c * nb
        return torch.cat(outs, 0)
    raise NotImplementedError(f"no differentiable matvec for {type(A).__name__}")


def _vjp_params_device(A, tensors, X, dual):
    """The same gradients from the library's VJP kernels (colagb_matmat_vjp: Dense / Sparse / Diagonal
    leaves in the compute type under Sum / ScalarMul / Identity), or None where the tree needs the
    tensor-op restatement."""
    import ctypes as C
    from .. import _capi
    from ..lowering import lower
    try:
        low = lower(A)
    except NotImplementedError:
        return None
    dt = low.compute_dtype
    want = {id(p): p for p in tensors}
    grads = {}
    ptrs = (C.c_void_p * len(low.nodes))()
    for node, t in low.leaf_tensors.items():
        if id(t) in want:
            if t.dtype != dt or not t.is_cuda:
                return None
            if id(t) not in grads:
                grads[id(t)] = torch.zeros(t.shape, dtype=dt, device=t.device)
            ptrs[node] = grads[id(t)].data_ptr()
    Xc = X.detach().to(dt).contiguous()
    Gc = dual.detach().to(dt).contiguous()
    k = Xc.shape[1]
    st = _capi.load().colagb_matmat_vjp(low.handle, Xc.data_ptr(), k, Gc.data_ptr(), k, k, 1.0, ptrs,
                                        _capi.stream_ptr(Xc.device))
    if st == _capi.ERR_UNSUPPORTED:
        return None
    _capi.check(st, "matmat vjp")
    return [grads.get(id(p)) if id(p) in grads else torch.zeros_like(p) for p in tensors]


def _vjp_params(A, tensors, X, dual):
    """Gradients of sum(dual * (A(theta) @ X)) with respect to `tensors`: on the device by the library's
    VJP kernels where the operator tree allows, else through the tensor-op restatement."""
    if not tensors:
        return []
    if X.is_cuda:
        g = _vjp_params_device(A, tensors, X, dual)
        if g is not None:
            return [gi.to(p.dtype) for gi, p in zip(g, tensors)]
    with torch.enable_grad():
        copies = [p.detach().requires_grad_(True) for p in tensors]
        sub = {id(p): c for p, c in zip(tensors, copies)}
        Y = torch_matmat(A, X.detach(), sub)
        g = torch.autograd.grad(Y, copies, grad_outputs=dual.to(Y.dtype), allow_unused=True)
    return [None if gi is None else gi.to(p.dtype) for gi, p in zip(g, tensors)]


class _CGFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, box, b, *tensors):
        x, info = box["solve"](b)
        box["info"] = info
        ctx.box = box
        ctx.save_for_backward(x, *tensors)
        return x

    @staticmethod
    def backward(ctx, gx):
        x, *tensors = ctx.saved_tensors
        box = ctx.box
        db, _ = box["solve"](gx.contiguous())
        need = list(ctx.needs_input_grad[2:])
        grads = [None] * len(tensors)
        if any(need):
            X = x.reshape(x.shape[0], -1)
            D = -db.reshape(X.shape)
            sel = [p for p, nd in zip(tensors, need) if nd]
            g = iter(_vjp_params(box["A"], sel, X, D))
            grads = [next(g) if nd else None for nd in need]
        return (None, db if ctx.needs_input_grad[1] else None, *grads)


def cg_with_grad(A, rhs, solve):
    """x = A^-1 rhs with the CG adjoint rule; `solve(b) -> (x, info)` runs the device CG."""
    box = {"A": A, "solve": solve}
    tensors = operator_tensors(A)
    x = _CGFn.apply(box, rhs, *tensors)
    return x, box["info"]


class _SLQFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, box, *tensors):
        est = box["forward"]()
        ctx.box = box
        ctx.save_for_backward(*tensors)
        return est

    @staticmethod
    def backward(ctx, g):
        tensors = ctx.saved_tensors
        box = ctx.box
        need = list(ctx.needs_input_grad[1:])
        if not any(need):
            return (None, *([None] * len(tensors)))
        Z = box["probes"]
        solves = box["solve"](Z)
        d = (g / Z.shape[1]) * solves
        sel = [p for p, nd in zip(tensors, need) if nd]
        it = iter(_vjp_params(box["A"], sel, Z, d))
        return (None, *[next(it) if nd else None for nd in need])


def slq_with_grad(A, probes, forward, solve):
    """The SLQ estimate with the reference's backward rule (f = log)."""
    box = {"A": A, "probes": probes, "forward": forward, "solve": solve}
    return _SLQFn.apply(box, *operator_tensors(A))


def wants_grad(A, *extra) -> bool:
    if not torch.is_grad_enabled():
        return False
    if any(isinstance(e, torch.Tensor) and e.requires_grad for e in extra):
        return True
    return any(t.requires_grad for t in operator_tensors(A))
