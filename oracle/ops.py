"""Structured matvecs in numpy (oracle; cola/ops/operators.py).  Each returns a matmat callable
X (cols, k) -> (rows, k) plus its shape."""
from __future__ import annotations

from functools import reduce

import numpy as np


class Op:
    def __init__(self, shape, fn):
        self.shape = tuple(shape)
        self.fn = fn

    def __call__(self, X):
        X = np.asarray(X)
        if X.ndim == 1:
            return self.fn(X[:, None])[:, 0]
        return self.fn(X)


def dense_op(A):
    """Dense._matmat (operators.py:26-28)."""
    A = np.asarray(A)
    return Op(A.shape, lambda X: A @ X)


def csr_op(indptr, indices, values, shape):
    """Sparse._matmat (operators.py:77-78), rows summed in index order."""
    indptr, indices, values = map(np.asarray, (indptr, indices, values))

    def fn(X):
        out = np.zeros((shape[0], X.shape[1]), dtype=np.result_type(values, X))
        for i in range(shape[0]):
            b, e = indptr[i], indptr[i + 1]
            if e > b:
                out[i] = values[b:e] @ X[indices[b:e]]
        return out
    return Op(shape, fn)


def diag_op(d):
    """Diagonal._matmat (operators.py:338-339)."""
    d = np.asarray(d)
    return Op((d.size, d.size), lambda X: d[:, None] * X)


def sum_op(*ops):
    """Sum._matmat (operators.py:182-183)."""
    return Op(ops[0].shape, lambda X: reduce(np.add, [o(X) for o in ops]))


def product_op(*ops):
    """Product._matmat (operators.py:153-156): right to left."""
    def fn(X):
        for o in ops[::-1]:
            X = o(X)
        return X
    return Op((ops[0].shape[0], ops[-1].shape[1]), fn)


def kron_op(*ops):
    """Kronecker._matmat (operators.py:216-223): contract each factor along its own axis."""
    rows = int(np.prod([o.shape[0] for o in ops]))
    cols = int(np.prod([o.shape[1] for o in ops]))

    def fn(X):
        ev = X.reshape(*[o.shape[1] for o in ops], -1)
        for i, o in enumerate(ops):
            front = np.moveaxis(ev, i, 0)
            shape = (o.shape[0],) + front.shape[1:]
            out = o(front.reshape(o.shape[1], -1)).reshape(shape)
            ev = np.moveaxis(out, 0, i)
        return ev.reshape(rows, ev.shape[-1])
    return Op((rows, cols), fn)


def blockdiag_op(ops, multiplicities=None):
    """BlockDiag._matmat (operators.py:299-310)."""
    mult = multiplicities or [1] * len(ops)
    rows = sum(o.shape[0] * c for o, c in zip(ops, mult))
    cols = sum(o.shape[1] * c for o, c in zip(ops, mult))

    def fn(X):
        k = X.shape[1]
        i = 0
        ys = []
        for o, c in zip(ops, mult):
            i_end = i + c * o.shape[1]
            elems = o(X[i:i_end].T.reshape(k * c, o.shape[1]).T)
            ys.append(elems.T.reshape(k, c * o.shape[0]).T)
            i = i_end
        return np.concatenate(ys, axis=0)
    return Op((rows, cols), fn)
