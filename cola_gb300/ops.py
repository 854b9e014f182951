"""LinearOperator types of the CoLA API (cola/ops/operator_base.py, cola/ops/operators.py).

Same class names, constructor arguments and composition rules as the reference;
``A @ X`` lowers the operator tree to a libcolagb operator program and runs it
on the GPU (``colagb_matmat``).  There is no CPU execution path: operators may be
built from CPU tensors (construction and shape logic are host code), but applying
one requires CUDA tensors.
"""
from __future__ import annotations

from functools import reduce
from numbers import Number
from typing import Any, Sequence

import torch

from . import _capi

Array = torch.Tensor


def _find_device(objs) -> torch.device | None:
    for o in objs:
        if isinstance(o, torch.Tensor):
            return o.device
        if isinstance(o, LinearOperator):
            return o.device
        if isinstance(o, (list, tuple)):
            d = _find_device(o)
            if d is not None:
                return d
    return None


def _promote(*dtypes):
    return reduce(torch.promote_types, dtypes)


class LinearOperator:
    """Linear operator base class (operator_base.py:16-36).

    Subclasses define ``_matmat``; composite types also lower to an operator program
    (``_lower``) so that the CG / Lanczos kernels can apply them on the device.
    """

    def __init__(self, dtype, shape, matmat=None, annotations=frozenset()):
        self.dtype = dtype
        self.shape = tuple(int(s) for s in shape)
        if matmat is not None:
            self._matmat = matmat
            self._custom_matmat = True
        from .annotations import get_annotations
        self.annotations = set(get_annotations(self)) | set(annotations)
        if not hasattr(self, "device") or self.device is None:
            self.device = torch.device("cpu")

    # ---- protocol -------------------------------------------------------------------------
    def isa(self, annotation) -> bool:
        return any(issubclass(a, annotation) for a in self.annotations)

    def _matmat(self, X: Array) -> Array:
        from .lowering import apply_operator
        return apply_operator(self, X)

    def __matmul__(self, X):
        if isinstance(X, LinearOperator):
            from .fns import dot
            return dot(self, X)
        assert X.shape[0] == self.shape[-1], f"dimension mismatch {self.shape} vs {tuple(X.shape)}"
        if X.dim() == 1:
            return self._matmat(X.reshape(-1, 1)).reshape(-1)
        if X.dim() >= 2:
            return self._matmat(X)
        raise NotImplementedError

    def __rmatmul__(self, X):
        if isinstance(X, LinearOperator):
            from .fns import dot
            return dot(X, self)
        raise NotImplementedError("X @ A is not on the accelerated path (use A.T @ X.T)")

    def to_dense(self) -> Array:
        eye = torch.eye(self.shape[-1], dtype=self.dtype, device=self.device)
        return self @ eye

    def to(self, device, dtype=None):
        raise NotImplementedError("move the underlying tensors and rebuild the operator")

    @property
    def T(self):
        from .fns import transpose
        return transpose(self)

    @property
    def H(self):
        from .fns import adjoint
        return adjoint(self)

    def __add__(self, other):
        if isinstance(other, Number) and other == 0:
            return self
        from .fns import add
        return add(self, other)

    def __radd__(self, other):
        return self.__add__(other)

    def __mul__(self, c):
        from .fns import mul
        return mul(self, c)

    def __rmul__(self, c):
        return self * c

    def __neg__(self):
        return -1 * self

    def __sub__(self, x):
        return self.__add__(-x)

    def __truediv__(self, x):
        return self.__mul__(1 / x)

    def __repr__(self):
        M, N = self.shape
        return "<%dx%d %s with dtype=%s>" % (M, N, self.__class__.__name__, self.dtype)

    def __str__(self):
        return self.__class__.__name__


class Dense(LinearOperator):
    """Dense matrix (operators.py:12-38); row-major storage, float32 / bfloat16 / float64."""

    def __init__(self, A: Array):
        self.A = A
        self.device = A.device
        super().__init__(dtype=A.dtype, shape=A.shape)

    def to_dense(self):
        return self.A


class Sparse(LinearOperator):
    """CSR sparse matrix from COO triplets (operators.py:48-81).

    As in the reference the triplets are sorted by row and duplicate entries are summed
    (scipy's ``coo_array(...).tocsr()``, operators.py:71-75); here the conversion runs with
    tensor ops on the tensors' own device.  Indices are stored as int32.
    """

    def __init__(self, data, row_indices, col_indices, shape):
        self.device = data.device
        super().__init__(dtype=data.dtype, shape=shape)
        n_rows, n_cols = self.shape
        row = row_indices.to(torch.int64)
        col = col_indices.to(torch.int64)
        order = torch.argsort(row, stable=True)
        self.data = data[order]
        self.row_indices = row_indices[order]
        self.col_indices = col_indices[order]
        # sum duplicates, sort columns within rows
        key = row[order] * max(n_cols, 1) + col[order]
        ukey, inv = torch.unique(key, sorted=True, return_inverse=True)
        vals = torch.zeros(ukey.numel(), dtype=torch.float64 if data.dtype != torch.float64 else data.dtype,
                           device=data.device)
        vals.index_add_(0, inv, self.data.to(vals.dtype))
        urow = torch.div(ukey, max(n_cols, 1), rounding_mode="floor")
        ucol = ukey - urow * max(n_cols, 1)
        counts = torch.bincount(urow, minlength=n_rows)
        indptr = torch.zeros(n_rows + 1, dtype=torch.int64, device=data.device)
        indptr[1:] = torch.cumsum(counts, 0)
        self.indptr = indptr.to(torch.int32).contiguous()
        self.indices = ucol.to(torch.int32).contiguous()
        self.values = vals.to(data.dtype).contiguous()
        self.nnz = int(self.values.numel())

    @classmethod
    def from_csr(cls, indptr: Array, indices: Array, values: Array, shape) -> "Sparse":
        """Wrap an existing CSR triple (int32 indices, sorted columns) without conversion."""
        obj = cls.__new__(cls)
        obj.device = values.device
        LinearOperator.__init__(obj, dtype=values.dtype, shape=shape)
        obj.indptr = indptr.to(torch.int32).contiguous()
        obj.indices = indices.to(torch.int32).contiguous()
        obj.values = values.contiguous()
        obj.nnz = int(values.numel())
        counts = obj.indptr[1:] - obj.indptr[:-1]
        obj.row_indices = torch.repeat_interleave(torch.arange(shape[0], device=values.device, dtype=torch.int64),
                                                  counts.to(torch.int64))
        obj.col_indices = obj.indices.to(torch.int64)
        obj.data = obj.values
        return obj

    perm = None  # stored order of a reordered matrix (see reordered)

    def reordered(self, method: str = "rcm") -> "Sparse":
        """The same matrix stored in a bandwidth-reducing order: P A P^T with P from reverse
        Cuthill-McKee on the pattern (symmetrised), computed once on the host with scipy, like the
        reference's own host-side CSR construction (operators.py:64-76).  Products gather x through
        the permutation and write y through it (colagb_op_node.perm), so the operator still means A;
        what changes is locality: on a graph numbered in random order every x gather of the original
        storage is a scattered memory sector, on the reordered one neighbouring rows read neighbouring
        entries.  Square matrices only."""
        if method != "rcm":
            raise ValueError("method must be 'rcm'")
        n, m = self.shape
        if n != m:
            raise ValueError("reordered() needs a square matrix")
        if self.perm is not None:
            return self
        import numpy as np
        import scipy.sparse as sp
        from scipy.sparse.csgraph import reverse_cuthill_mckee
        ip, ix = self.indptr.cpu().numpy(), self.indices.cpu().numpy()
        pattern = sp.csr_matrix((np.ones(ix.size, dtype=np.int8), ix, ip), shape=(n, n))
        perm = torch.as_tensor(reverse_cuthill_mckee(pattern, symmetric_mode=False).astype(np.int64),
                               device=self.device)
        inv = torch.empty_like(perm)
        inv[perm] = torch.arange(n, device=self.device)
        counts = (self.indptr[1:] - self.indptr[:-1]).to(torch.int64)
        old_row = torch.repeat_interleave(torch.arange(n, device=self.device), counts)
        new_row, new_col = inv[old_row], inv[self.indices.to(torch.int64)]
        order = torch.argsort(new_row * n + new_col)
        obj = Sparse.__new__(Sparse)
        obj.device = self.device
        LinearOperator.__init__(obj, dtype=self.dtype, shape=self.shape)
        indptr = torch.zeros(n + 1, dtype=torch.int64, device=self.device)
        indptr[1:] = torch.cumsum(torch.bincount(new_row, minlength=n), 0)
        obj.indptr = indptr.to(torch.int32).contiguous()
        obj.indices = new_col[order].to(torch.int32).contiguous()
        obj.values = self.values[order].contiguous()
        obj.nnz = self.nnz
        obj.perm = perm.to(torch.int32).contiguous()
        # the triplets in the original coordinates, in the stored order (transpose, to_dense)
        obj.row_indices = perm[new_row[order]]
        obj.col_indices = perm[new_col[order]]
        obj.data = obj.values
        return obj

    def to_dense(self):
        D = torch.zeros(self.shape, dtype=self.dtype, device=self.device)
        if self.perm is not None:
            D.index_put_((self.row_indices.to(torch.int64), self.col_indices.to(torch.int64)), self.values,
                         accumulate=True)
            return D
        rows = torch.repeat_interleave(torch.arange(self.shape[0], device=self.device),
                                       (self.indptr[1:] - self.indptr[:-1]).to(torch.int64))
        D.index_put_((rows, self.indices.to(torch.int64)), self.values, accumulate=True)
        return D


class ScalarMul(LinearOperator):
    """c * I (operators.py:84-101)."""

    def __init__(self, c, shape, dtype=None, device=None):
        self.device = device if device is not None else torch.device("cpu")
        super().__init__(dtype=dtype or torch.float32, shape=shape)
        self.c = c.item() if isinstance(c, torch.Tensor) else c

    def __str__(self):
        return f"{self.c}"


class Identity(LinearOperator):
    """Identity (operators.py:104-127)."""

    def __init__(self, shape, dtype):
        self.device = torch.device("cpu")
        super().__init__(dtype=dtype, shape=shape)

    def to(self, device, dtype=None):
        self.device = torch.device(device)
        return self

    def __str__(self):
        return "I"


def I_like(A: LinearOperator) -> Identity:
    """Identity with the shape, dtype and device of A (operators.py:130-136)."""
    op = Identity(dtype=A.dtype, shape=A.shape)
    op.to(A.device)
    return op


def _lazify(M):
    return M if isinstance(M, LinearOperator) else Dense(M)


class Product(LinearOperator):
    """Product of operators, applied right to left (operators.py:139-165)."""

    def __init__(self, *Ms):
        self.Ms = tuple(_lazify(M) for M in Ms)
        devices = [M.device for M in self.Ms]
        assert all(x == devices[0] for x in devices), "There is a device mismatch in Product"
        for M1, M2 in zip(self.Ms[:-1], self.Ms[1:]):
            if M1.shape[-1] != M2.shape[-2]:
                raise ValueError(f"dimension mismatch {M1.shape} vs {M2.shape}")
        self.device = devices[0]
        super().__init__(_promote(*(M.dtype for M in self.Ms)), (self.Ms[0].shape[-2], self.Ms[-1].shape[-1]))

    def __str__(self):
        return "".join(str(M) for M in self.Ms)


class Sum(LinearOperator):
    """Sum of operators (operators.py:168-196)."""

    def __init__(self, *Ms):
        self.Ms = tuple(_lazify(M) for M in Ms)
        devices = [M.device for M in self.Ms]
        assert all(x == devices[0] for x in devices), "There is a device mismatch in Sum"
        shape = self.Ms[0].shape
        for M in self.Ms:
            if M.shape != shape:
                raise ValueError(f"dimension mismatch {M.shape} vs {shape}")
        self.device = devices[0]
        super().__init__(self.Ms[0].dtype, shape)

    def __str__(self):
        return "+".join(str(M) for M in self.Ms)


class Kronecker(LinearOperator):
    """Kronecker product M1 (x) M2 (x) ... (operators.py:199-228).

    ``precision`` (keyword only; FP32 operators) selects the arithmetic of the factor contractions:
    "auto" (default) runs large contractions (>= 2^26 multiply-adds, Dense factors with >= 256
    columns) on the tensor cores with the three-product BF16 split and the rest in FP32; "bf16x3", "bf16" and "fp32" force
    one kind.  FP64 operators always contract in FP64."""

    def __init__(self, *Ms, precision: str = "auto"):
        if precision not in ("auto", "fp32", "bf16", "bf16x3"):
            raise ValueError(f"unknown Kronecker precision {precision!r}")
        self.precision = precision
        self.Ms = tuple(_lazify(M) for M in Ms)
        self.device = _find_device(self.Ms)
        shape = (reduce(lambda a, b: a * b, [M.shape[-2] for M in self.Ms]),
                 reduce(lambda a, b: a * b, [M.shape[-1] for M in self.Ms]))
        super().__init__(_promote(*(M.dtype for M in self.Ms)), shape)

    def to_dense(self):
        Ms = [M.to_dense() for M in self.Ms]
        return reduce(torch.kron, Ms)

    def __str__(self):
        return "⊗".join(str(M) for M in self.Ms)


class BlockDiag(LinearOperator):
    """Block-diagonal operator with block multiplicities (operators.py:278-320)."""

    def __init__(self, *Ms, multiplicities=None):
        self.Ms = tuple(_lazify(M) for M in Ms)
        self.multiplicities = [1 for _ in Ms] if multiplicities is None else list(multiplicities)
        self.device = _find_device(self.Ms)
        shape = (sum(M.shape[-2] * c for M, c in zip(self.Ms, self.multiplicities)),
                 sum(M.shape[-1] * c for M, c in zip(self.Ms, self.multiplicities)))
        super().__init__(_promote(*(M.dtype for M in self.Ms)), shape)

    def to_dense(self):
        blocks = [M.to_dense() for M, c in zip(self.Ms, self.multiplicities) for _ in range(c)]
        return torch.block_diag(*blocks)

    def __str__(self):
        return "⊕".join(str(M) for M in self.Ms)


class Diagonal(LinearOperator):
    """Diagonal operator (operators.py:323-348)."""

    def __init__(self, diag):
        assert len(diag.shape) == 1, f"diagonal is not a vector, it is of shape {diag.shape=}"
        self.diag = diag
        self.device = diag.device
        super().__init__(dtype=diag.dtype, shape=(len(diag),) * 2)

    def to_dense(self):
        return torch.diag(self.diag)


class Tridiagonal(LinearOperator):
    """Tridiagonal operator (operators.py:351-374): lower band alpha, diagonal beta, upper band gamma.

    Used as the container of the Lanczos T; it is built on the host path and applied with tensor ops
    (it never appears inside a CG/Lanczos loop)."""

    def __init__(self, alpha: Array, beta: Array, gamma: Array):
        def as_mat(v):
            return v.reshape(-1, 1) if v.dim() == 1 else v
        self.alpha, self.beta, self.gamma = as_mat(alpha), as_mat(beta), as_mat(gamma)
        self.device = beta.device
        super().__init__(dtype=beta.dtype, shape=(self.beta.shape[0], self.beta.shape[0]))

    def _matmat(self, X):
        out = self.beta * X
        out[:-1] += self.gamma * X[1:]
        out[1:] += self.alpha * X[:-1]
        return out

    def to_dense(self):
        m = self.beta.shape[0]
        T = torch.diag(self.beta[:, 0])
        if m > 1:
            T = T + torch.diag(self.alpha[:, 0], -1) + torch.diag(self.gamma[:, 0], 1)
        return T


class Transpose(LinearOperator):
    """Transpose of an operator (operators.py:382-397); only self-adjoint, Dense, Sparse and
    Diagonal transposes are materialised (see fns.transpose)."""

    def __init__(self, A):
        self.A = A
        self.device = A.device
        super().__init__(dtype=A.dtype, shape=(A.shape[1], A.shape[0]))


__all__ = ["LinearOperator", "Dense", "Sparse", "ScalarMul", "Identity", "I_like", "Product", "Sum", "Kronecker",
           "BlockDiag", "Diagonal", "Tridiagonal", "Transpose", "Array"]
