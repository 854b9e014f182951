"""Lower a LinearOperator tree to a libcolagb operator program (colagb_op_create) and apply it.

Supported node types are the structured operators on the Krylov hot path: Dense, Sparse (CSR),
Diagonal, ScalarMul, Identity, Sum, Product, Kronecker and BlockDiag, in any nesting.  The
handle is cached on the operator; the tensors it points to stay referenced by the operator.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _capi
from . import ops as O

_F64_TYPES = (torch.float64,)
_LEAF_TYPES = (torch.float32, torch.float64, torch.bfloat16)


class Lowered:
    """An operator program handle plus the host arrays that describe it."""

    def __init__(self, op: O.LinearOperator):
        self.nodes: list[_capi.OpNode] = []
        self.leaf_tensors: dict[int, torch.Tensor] = {}  # node index -> the operator tensor it reads
        self._keep: list = []
        self.device: torch.device | None = None
        self.any64 = False
        root = self._lower(op)
        arr = (_capi.OpNode * len(self.nodes))(*self.nodes)
        self._arr = arr
        handle = C.c_void_p()
        lib = _capi.load()
        _capi.check(lib.colagb_op_create(arr, len(self.nodes), root, C.byref(handle)), "operator")
        self.handle = handle
        self.shape = op.shape
        self.compute_dtype = torch.float64 if self.any64 else torch.float32
        self._lib = lib

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self._lib.colagb_op_free(h)
            except Exception:
                pass

    # ---- node construction --------------------------------------------------------------
    def _add(self, **kw) -> int:
        nd = _capi.OpNode()
        for k, v in kw.items():
            setattr(nd, k, v)
        self.nodes.append(nd)
        return len(self.nodes) - 1

    def _dev(self, t: torch.Tensor):
        if self.device is None:
            self.device = t.device
        elif t.device != self.device:
            raise AssertionError(f"device mismatch in operator: {t.device} vs {self.device}")

    def _leaf_dtype(self, t: torch.Tensor) -> int:
        if t.dtype not in _LEAF_TYPES:
            raise NotImplementedError(f"operator storage dtype {t.dtype} is not supported (float32, bfloat16, float64)")
        if t.dtype in _F64_TYPES:
            self.any64 = True
        return _capi.TORCH_TO_CODE[t.dtype]

    def _children(self, kids: list[int]):
        arr = (C.c_int32 * len(kids))(*kids)
        self._keep.append(arr)
        return C.cast(arr, C.POINTER(C.c_int32)), len(kids)

    def _lower(self, op: O.LinearOperator) -> int:
        rows, cols = op.shape
        if getattr(op, "_custom_matmat", False):
            raise NotImplementedError("operators defined by a Python matmat cannot run inside the device Krylov "
                                      "loops; compose Dense/Sparse/Diagonal/Kronecker/Sum/Product/BlockDiag instead")
        if isinstance(op, O.Dense):
            A = op.A
            if A.dim() != 2:
                raise ValueError("Dense expects a 2-D tensor")
            if A.stride(1) != 1 or A.stride(0) < A.shape[1]:
                A = A.contiguous()
            self._keep.append(A)
            self._dev(A)
            self.leaf_tensors[len(self.nodes)] = op.A
            return self._add(kind=_capi.OP_DENSE, dtype=self._leaf_dtype(A), rows=rows, cols=cols, data=A.data_ptr(),
                             ld=A.stride(0) if A.shape[0] > 0 else cols)
        if isinstance(op, O.Sparse):
            self._keep += [op.indptr, op.indices, op.values]
            self._dev(op.values)
            self.leaf_tensors[len(self.nodes)] = op.values
            extra = {}
            if op.perm is not None:
                self._keep.append(op.perm)
                extra["perm"] = op.perm.data_ptr()
            return self._add(kind=_capi.OP_CSR, dtype=self._leaf_dtype(op.values), rows=rows, cols=cols,
                             data=op.values.data_ptr(), indptr=op.indptr.data_ptr(), indices=op.indices.data_ptr(),
                             nnz=op.nnz, **extra)
        if isinstance(op, O.Diagonal):
            d = op.diag.contiguous()
            self._keep.append(d)
            self._dev(d)
            self.leaf_tensors[len(self.nodes)] = op.diag
            return self._add(kind=_capi.OP_DIAG, dtype=self._leaf_dtype(d), rows=rows, cols=cols, data=d.data_ptr())
        if isinstance(op, O.ScalarMul):
            return self._add(kind=_capi.OP_SCALAR, rows=rows, cols=cols, scalar=float(op.c))
        if isinstance(op, O.Identity):
            return self._add(kind=_capi.OP_IDENTITY, rows=rows, cols=cols)
        if isinstance(op, O.Product):
            Ms = op.Ms
            # c * I folds to a scalar node (cola.fns.mul builds Product(ScalarMul(c), I))
            if all(isinstance(M, (O.ScalarMul, O.Identity)) for M in Ms):
                c = 1.0
                for M in Ms:
                    c *= float(M.c) if isinstance(M, O.ScalarMul) else 1.0
                return self._add(kind=_capi.OP_SCALAR, rows=rows, cols=cols, scalar=c)
            kids = [self._lower(M) for M in Ms]
            ptr, nk = self._children(kids)
            return self._add(kind=_capi.OP_PRODUCT, rows=rows, cols=cols, children=ptr, num_children=nk)
        if isinstance(op, O.Sum):
            kids = [self._lower(M) for M in op.Ms]
            ptr, nk = self._children(kids)
            return self._add(kind=_capi.OP_SUM, rows=rows, cols=cols, children=ptr, num_children=nk)
        if isinstance(op, O.Kronecker):
            kids = [self._lower(M) for M in op.Ms]
            ptr, nk = self._children(kids)
            return self._add(kind=_capi.OP_KRON, rows=rows, cols=cols, children=ptr, num_children=nk,
                             precision=_capi.KRON_PRECISION[op.precision])
        if isinstance(op, O.BlockDiag):
            kids = [self._lower(M) for M in op.Ms]
            ptr, nk = self._children(kids)
            mult = (C.c_int64 * nk)(*[int(m) for m in op.multiplicities])
            self._keep.append(mult)
            return self._add(kind=_capi.OP_BLOCKDIAG, rows=rows, cols=cols, children=ptr, num_children=nk,
                             multiplicities=C.cast(mult, C.POINTER(C.c_int64)))
        raise NotImplementedError(f"{type(op).__name__} is not lowered to the device operator program")


def lower(op: O.LinearOperator) -> Lowered:
    low = op.__dict__.get("_lowered")
    if low is None:
        low = Lowered(op)
        op.__dict__["_lowered"] = low
    return low


def operator_device(op: O.LinearOperator, low: Lowered) -> torch.device:
    dev = low.device if low.device is not None else op.device
    if dev is None or dev.type != "cuda":
        raise ValueError("cola_gb300 computes on the GPU: build operators from CUDA tensors "
                         f"(operator lives on {dev}); there is no CPU execution path")
    return dev


def apply_operator(op: O.LinearOperator, X: torch.Tensor, alpha: float = 1.0) -> torch.Tensor:
    """Y = alpha * op @ X on the device (X: (cols, k))."""
    low = lower(op)
    dev = operator_device(op, low)
    if X.device != dev:
        raise ValueError(f"X is on {X.device}, operator on {dev}")
    lib = _capi.load()
    X = X.to(low.compute_dtype).contiguous()
    k = X.shape[1]
    Y = torch.empty((op.shape[0], k), dtype=low.compute_dtype, device=dev)
    nbytes = C.c_size_t()
    _capi.check(lib.colagb_matmat_workspace_bytes(low.handle, k, C.byref(nbytes)), "matmat")
    ws = _capi.workspace(nbytes.value, dev) if nbytes.value else None
    _capi.check(lib.colagb_matmat(low.handle, X.data_ptr(), k, Y.data_ptr(), k, k, alpha, 0.0,
                                  ws.data_ptr() if ws is not None else None, nbytes.value,
                                  _capi.stream_ptr(dev)), "matmat")
    return Y
