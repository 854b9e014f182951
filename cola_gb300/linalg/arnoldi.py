"""Arnoldi and GMRES for non-symmetric operators (cola/linalg/decompositions/arnoldi.py:166-201,
cola/linalg/inverse/gmres.py:39-117).

The Arnoldi loop runs in libcolagb (``colagb_arnoldi``): one device matvec per step of the lowered
operator, two classical Gram-Schmidt passes over the basis slots (the reference makes one modified
pass; both give the same H and Q up to rounding), the reference's tol/2 clip and stop test.
``gmres`` forms the reference's small least-squares step, the normal equations of the square
m x m Hessenberg part with its zero-column padding, on the device in FP64.
"""
from __future__ import annotations

import ctypes as C
import time

import torch

from .. import _capi
from .. import ops as O
from ..annotations import Unitary
from ..lowering import lower, operator_device
from .prng import PRNGKey, randn


def run_arnoldi(A: O.LinearOperator, V0: torch.Tensor, max_iters: int, tol: float, check_every: int = 8):
    """Device Arnoldi from the (n, bs) start block V0: returns (Q (bs, n, m+1), H (bs, m+1, m), steps)."""
    low = lower(A)
    dev = operator_device(A, low)
    lib = _capi.load()
    dt = low.compute_dtype
    V0 = V0.to(device=dev, dtype=dt).contiguous()
    n, bs = V0.shape
    m = min(int(max_iters), n)
    basis = torch.empty((m + 2, n, bs), dtype=dt, device=dev)
    H = torch.empty((bs, m + 1, m), dtype=dt, device=dev)
    steps = C.c_int32()
    prm = _capi.LanczosParams(tol=float(tol), max_iters=m, check_every=int(check_every))
    nbytes = C.c_size_t()
    _capi.check(lib.colagb_arnoldi_workspace_bytes(low.handle, bs, m, C.byref(nbytes)), "arnoldi")
    ws = _capi.workspace(nbytes.value, dev)
    _capi.check(lib.colagb_arnoldi(low.handle, V0.data_ptr(), bs, bs, C.byref(prm), basis.data_ptr(), H.data_ptr(),
                                   C.byref(steps), ws.data_ptr(), nbytes.value, _capi.stream_ptr(dev)), "arnoldi")
    Q = basis[1:].permute(2, 1, 0)  # slot j + 1 -> Q[:, :, j]; (bs, n, m + 1)
    return Q, H, int(steps.value)


def _dense(M):
    D = O.Dense.__new__(O.Dense)
    D.A, D.device, D.dtype, D.shape, D.annotations = M, M.device, M.dtype, tuple(M.shape[-2:]), set()
    return D


def arnoldi(A: O.LinearOperator, start_vector=None, max_iters=100, tol: float = 1e-7, use_householder: bool = False,
            pbar: bool = False, key=None):
    """Arnoldi decomposition A Q_m = Q_{m+1} H (arnoldi.py:166-201); returns (Q, H, info).

    For a 1-D start vector Q is Unitary(Dense(n x (m+1))) and H Dense((m+1) x m); for an (n, bs) block
    both are batched over the start vectors.  ``use_householder`` is not supported on this path."""
    if use_householder:
        raise NotImplementedError("Householder Arnoldi is not on the GPU path (use the default Gram-Schmidt)")
    if start_vector is None:
        key = PRNGKey(42) if key is None else key
        start_vector = randn(A.shape[-1], dtype=A.dtype, key=key)
    is_vector = start_vector.dim() == 1
    V0 = start_vector[:, None] if is_vector else start_vector
    t0 = time.time()
    Q, H, steps = run_arnoldi(A, V0, max_iters, tol)
    info = {"iterations": steps + 1, "iteration_time": (time.time() - t0) / (steps + 1)}
    if is_vector:
        Qd = _dense(Q[0])
        Qd.annotations = {Unitary}
        return Qd, _dense(H[0]), info
    Qd = _dense(Q)
    Qd.annotations = {Unitary}
    return Qd, _dense(H), info


def gmres(A: O.LinearOperator, rhs: torch.Tensor, x0=None, max_iters=100, tol=1e-7, P=None,
          use_householder=False, use_triangular=False, pbar=False):
    """Solves A X = B by the reference's GMRES (gmres.py:39-117); returns (solution, info).

    ``P`` is accepted and, as in the reference's forward pass, not applied."""
    if use_triangular or use_householder:
        raise NotImplementedError("the triangular / Householder GMRES variants are not on the GPU path")
    is_vector = rhs.dim() == 1
    B = rhs[:, None] if is_vector else rhs
    X0 = torch.zeros_like(B) if x0 is None else (x0[:, None] if x0.dim() == 1 else x0)
    X0 = X0.to(B.dtype)
    res = B - (A @ X0 if bool(X0.abs().max() > 0) else torch.zeros_like(B))
    t0 = time.time()
    Q, H, steps = run_arnoldi(A, res, max_iters, tol)
    Q, H = Q[:, :, :-1], H[:, :-1, :]                 # (k, n, m), (k, m, m)
    Hd = H.double()
    beta = torch.linalg.norm(res.double(), dim=-2)   # (k,)
    HT = Hd.transpose(1, 2)
    largest = Hd.abs().amax(-1)                      # (k, m)
    overall = largest.reshape(largest.shape[0], -1).amax(-1)
    thresh = 10 * tol * overall[:, None]
    pad = torch.where(largest < thresh, torch.ones_like(largest), torch.zeros_like(largest))
    y = torch.linalg.solve(HT @ Hd + torch.diag_embed(pad), HT[..., 0, None]).squeeze(-1) * beta[:, None]
    y = torch.where(largest < thresh, torch.zeros_like(y), y)
    pred = (Q.double() @ y[..., None])[..., 0].T    # (n, k)
    soln = (X0.double() + pred).to(B.dtype)
    info = {"iterations": steps + 1, "iteration_time": (time.time() - t0) / (steps + 1)}
    return (soln[:, 0] if is_vector else soln), info
