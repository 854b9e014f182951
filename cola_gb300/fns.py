"""Composition sugar (cola/fns.py): lazify, densify, dot, add, mul, kron, transpose, adjoint.

The reference selects these rules by multiple dispatch on operator types (fns.py:63-221); the
same rules are written out here as explicit type tests.
"""
from __future__ import annotations

from numbers import Number

import torch

from . import ops as O
from .annotations import SelfAdjoint


def lazify(A):
    """Array -> Dense; operators pass through (fns.py:33-38)."""
    return A if isinstance(A, O.LinearOperator) else O.Dense(A)


def densify(A):
    return A.to_dense() if isinstance(A, O.LinearOperator) else A


def dot(A, B):
    """Operator product (fns.py:63-90): Identity factors drop out, Products flatten."""
    if isinstance(B, O.Identity):
        return A
    if isinstance(A, O.Identity):
        return B
    a = A.Ms if isinstance(A, O.Product) else (A,)
    b = B.Ms if isinstance(B, O.Product) else (B,)
    return O.Product(*(a + b))


def add(A, B):
    """Operator sum (fns.py:93-115): Sums flatten."""
    A, B = lazify(A), lazify(B)
    a = A.Ms if isinstance(A, O.Sum) else (A,)
    b = B.Ms if isinstance(B, O.Sum) else (B,)
    return O.Sum(*(a + b))


def _is_scalar(c):
    return isinstance(c, Number) or (isinstance(c, torch.Tensor) and c.dim() == 0)


def mul(A, c):
    """Scalar multiple (fns.py:118-137): ScalarMul absorbs scalars, other operators become
    Product(ScalarMul(c), A)."""
    if isinstance(A, O.ScalarMul) and isinstance(c, O.ScalarMul):
        return O.ScalarMul(A.c * c.c, A.shape, A.dtype, A.device)
    if _is_scalar(A) and isinstance(c, O.LinearOperator):
        A, c = c, A
    if not _is_scalar(c):
        raise NotImplementedError("mul expects a scalar")
    c = c.item() if isinstance(c, torch.Tensor) else c
    if isinstance(A, O.ScalarMul):
        return O.ScalarMul(A.c * c, A.shape, A.dtype, A.device)
    S = O.ScalarMul(c, (A.shape[-2], A.shape[-2]), A.dtype, A.device)
    return O.Product(S, A)


def kron(A, B):
    """Kronecker product (fns.py:196-221)."""
    A, B = lazify(A), lazify(B)
    if isinstance(A, O.Diagonal) and isinstance(B, O.Diagonal):
        return O.Diagonal((A.diag[:, None] * B.diag[None, :]).reshape(-1))
    a = A.Ms if isinstance(A, O.Kronecker) else (A,)
    b = B.Ms if isinstance(B, O.Kronecker) else (B,)
    return O.Kronecker(*(a + b))


def transpose(A):
    """Transpose (fns.py:140-168)."""
    if isinstance(A, O.Transpose):
        return A.A
    if isinstance(A, O.Dense):
        return O.Dense(A.A.T.contiguous())
    if isinstance(A, O.Sparse):
        return O.Sparse(A.data, A.col_indices, A.row_indices, shape=(A.shape[1], A.shape[0]))
    if isinstance(A, (O.Diagonal, O.ScalarMul, O.Identity)) or A.isa(SelfAdjoint):
        return A
    return O.Transpose(A)


def adjoint(A):
    """Adjoint; for the real operators of this path it equals the transpose (fns.py:171-193)."""
    return transpose(A)


__all__ = ["lazify", "densify", "dot", "add", "mul", "kron", "transpose", "adjoint"]
