"""Lanczos, Lanczos eigensolver, eig (cola/linalg/decompositions/lanczos.py:34-61, 185-232,
cola/linalg/eig/eigs.py:76-111) and the tridiagonal eigensolver.

The Lanczos loop (with full CGS2 reorthogonalisation) runs in libcolagb (colagb_lanczos); the
tridiagonal eigenproblems are solved on the GPU (colagb_tridiag_eig_f64 / _f32) where the
reference calls eigh in the operator dtype.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import torch

from .. import _capi
from .. import ops as O
from ..annotations import SelfAdjoint, Unitary
from ..lowering import lower, operator_device
from .algorithms import Algorithm, Auto, Eigh, Lanczos, get_slice
from .prng import PRNGKey, randn


class LanczosResult:
    """Raw device output of one Lanczos run (basis slots, diag, subdiag, final loop index)."""

    def __init__(self, basis, diag, subdiag, i_final, max_iters, elapsed):
        self.basis, self.diag, self.subdiag = basis, diag, subdiag
        self.i_final, self.max_iters, self.elapsed = i_final, max_iters, elapsed

    @property
    def iters(self):
        return self.i_final - 1

    def alpha_beta_q(self):
        """(alpha = subdiag[:, 1:iters], beta = diag[:, :iters], Q slots 1..iters) as in lanczos.py:222-224."""
        it = self.iters
        alpha = self.subdiag[:, 1:-1][:, : max(it - 1, 0)]
        beta = self.diag[:, :it]
        Q = self.basis[1 : it + 1]  # (iters, n, bs)
        return alpha, beta, Q

    def info(self):
        """The reference's info dict (lanczos_fact error function, lanczos.py:256-261)."""
        sub = self.subdiag.double().cpu().numpy()
        errs = []
        for i in range(1, self.i_final + 1):
            rel = sub[:, i - 1] / np.maximum(sub[:, 1], 1e-30) if sub.shape[1] > 1 else np.zeros(sub.shape[0])
            errs.append(float(np.max(rel)) + (1.0 if i <= 1 else 0.0))
        errs.append(errs[-1])
        return {"iterations": self.i_final, "errors": np.array(errs[2:]),
                "iteration_time": self.elapsed / max(self.i_final, 1)}


def run_lanczos(A: O.LinearOperator, V0: torch.Tensor, max_iters: int, tol: float, check_every: int = 8):
    """Run the device Lanczos loop from the (n, bs) start block V0."""
    low = lower(A)
    dev = operator_device(A, low)
    lib = _capi.load()
    dt = low.compute_dtype
    V0 = V0.to(device=dev, dtype=dt).contiguous()
    n, bs = V0.shape
    m = int(max_iters)
    basis = torch.empty((m + 2, n, bs), dtype=dt, device=dev)
    diag = torch.empty((bs, m), dtype=dt, device=dev)
    subdiag = torch.empty((bs, m + 1), dtype=dt, device=dev)
    steps = C.c_int32()
    prm = _capi.LanczosParams(tol=float(tol), max_iters=m, check_every=int(check_every))
    nbytes = C.c_size_t()
    _capi.check(lib.colagb_lanczos_workspace_bytes(low.handle, bs, m, C.byref(nbytes)), "lanczos")
    ws = _capi.workspace(nbytes.value, dev)
    t0 = time.time()
    _capi.check(lib.colagb_lanczos(low.handle, V0.data_ptr(), bs, bs, C.byref(prm), basis.data_ptr(),
                                   diag.data_ptr(), subdiag.data_ptr(), C.byref(steps), ws.data_ptr(), nbytes.value,
                                   _capi.stream_ptr(dev)), "lanczos")
    return LanczosResult(basis, diag, subdiag, int(steps.value), m, time.time() - t0)


def _batched_tridiagonal(alpha, beta):
    """A batch of Tridiagonal operators stored like the reference's vmap(Tridiagonal) result."""
    T = O.Tridiagonal.__new__(O.Tridiagonal)
    T.alpha, T.beta, T.gamma = alpha[..., None], beta[..., None], alpha[..., None]
    T.device = beta.device
    T.dtype = beta.dtype
    T.shape = (beta.shape[-1], beta.shape[-1])
    T.annotations = set()
    return T


def _batched_dense(Q):
    D = O.Dense.__new__(O.Dense)
    D.A, D.device, D.dtype, D.shape, D.annotations = Q, Q.device, Q.dtype, tuple(Q.shape[-2:]), {Unitary}
    return D


def lanczos(A: O.LinearOperator, start_vector=None, max_iters=100, tol=1e-7, pbar=False, key=None):
    """Lanczos decomposition A ~ Q T Q^T (lanczos.py:185-232); returns (Q, T, info).

    For a 1-D start vector Q is Unitary(Dense(n x iters)) and T a Tridiagonal; for an (n, bs)
    block both are batched over the bs start vectors.
    """
    max_iters = min(int(max_iters), A.shape[0])
    if start_vector is None:
        key = PRNGKey(42) if key is None else key
        start_vector = randn(A.shape[0], dtype=A.dtype if A.dtype != torch.bfloat16 else torch.float32, key=key)
    rhs = start_vector[:, None] if start_vector.dim() == 1 else start_vector
    res = run_lanczos(A, rhs.to(A.device) if A.device.type == "cuda" else rhs, max_iters, tol)
    alpha, beta, Q = res.alpha_beta_q()
    info = res.info()
    Qb = Q.permute(2, 1, 0)  # (bs, n, iters) as the reference's V[..., 1:iters+1]
    if start_vector.dim() == 1:
        return Unitary(O.Dense(Qb[0])), O.Tridiagonal(alpha[0], beta[0], alpha[0]), info
    return _batched_dense(Qb), _batched_tridiagonal(alpha, beta), info


def tridiag_eigh(beta: torch.Tensor, alpha: torch.Tensor, want_vectors: bool = True):
    """Eigen-decomposition of symmetric tridiagonals on the GPU, in the precision of the recurrence
    that produced them: FP32 tridiagonals (from FP32 / BF16 operators) are solved in FP32, like the
    reference's eigh of the FP32 T (lanczos.py:57, unary.py:52), everything else in FP64.

    beta: (batch, m) diagonals, alpha: (batch, m-1) off-diagonals.  Returns (evals (batch, m)
    ascending, evecs (batch, m, m) or first-row weights (batch, m), status)."""
    lib = _capi.load()
    dev = beta.device
    _capi.require_cuda(beta)
    bsz, m = beta.shape
    dt = torch.float32 if beta.dtype in (torch.float32, torch.bfloat16, torch.float16) else torch.float64
    a = beta.to(dt).contiguous()
    b = torch.zeros((bsz, m), dtype=dt, device=dev)
    if m > 1:
        b[:, : m - 1] = alpha.to(dt)
    evals = torch.empty((bsz, m), dtype=dt, device=dev)
    first = torch.empty((bsz, m), dtype=dt, device=dev)
    evecs = torch.empty((bsz, m, m), dtype=dt, device=dev) if want_vectors else None
    status = torch.zeros(bsz, dtype=torch.int32, device=dev)
    fn = lib.colagb_tridiag_eig_f32 if dt == torch.float32 else lib.colagb_tridiag_eig_f64
    _capi.check(fn(a.data_ptr(), b.data_ptr(), m, bsz, evals.data_ptr(), first.data_ptr(),
                   evecs.data_ptr() if evecs is not None else None, status.data_ptr(), _capi.stream_ptr(dev)),
                "tridiagonal eigensolver")
    return evals, (evecs if want_vectors else first), status


def ritz_vectors(Q: torch.Tensor, S: torch.Tensor) -> torch.Tensor:
    """Q (iters, n) basis slots times selected eigenvector columns S (iters, k) -> (n, k), via the
    library's dense GEMM (as Dense(S^T) applied to the basis rows)."""
    from ..lowering import apply_operator
    St = O.Dense(S.T.contiguous().to(Q.dtype))
    Vt = apply_operator(St, Q)  # (k, n)
    return Vt.T


def lanczos_eigs(A: O.LinearOperator, start_vector=None, max_iters: int = 100, tol: float = 1e-7,
                 pbar: bool = False, key=None, k_select: slice | None = None):
    """Eigenvalues (ascending) and Ritz vectors from Lanczos (lanczos.py:34-61)."""
    max_iters = min(int(max_iters), A.shape[0])
    if start_vector is None:
        key = PRNGKey(42) if key is None else key
        start_vector = randn(A.shape[0], dtype=A.dtype if A.dtype != torch.bfloat16 else torch.float32, key=key)
    rhs = start_vector[:, None] if start_vector.dim() == 1 else start_vector[:, :1]
    res = run_lanczos(A, rhs.to(A.device), max_iters, tol)
    alpha, beta, Q = res.alpha_beta_q()
    evals, evecs, _ = tridiag_eigh(beta[:1], alpha[:1], want_vectors=True)
    evals, evecs = evals[0], evecs[0]
    sel = k_select if k_select is not None else slice(None)
    idx = torch.arange(evals.shape[0], device=evals.device)[sel]
    V = ritz_vectors(Q[:, :, 0], evecs[:, idx])
    return evals.to(A.dtype), V, res.info(), evals[idx].to(A.dtype)


def eig(A: O.LinearOperator, k: int, which: str = "LM", alg: Algorithm = Auto()):
    """Eigenpairs of A (eigs.py:20-111): Lanczos branch slices the sorted Ritz pairs."""
    if isinstance(alg, Auto):
        SA = A.isa(SelfAdjoint)
        small = bool(np.prod(A.shape) <= 1e6)
        if SA and small:
            alg = Eigh()
        elif SA:
            alg = Lanczos(**alg.__dict__)
        else:
            raise NotImplementedError("eig of non-self-adjoint operators (Arnoldi / Eig) is not on this path")
    if isinstance(alg, Eigh):
        evals, evecs = torch.linalg.eigh(A.to_dense())
        sl = get_slice(k, which)
        return evals[sl], evecs[:, sl]
    if isinstance(alg, Lanczos):
        assert A.isa(SelfAdjoint), "Lanczos only valid for SelfAdjoint, wrap in cola.SelfAdjoint if desired"
        sl = get_slice(k, which)
        _, V, _, sel_vals = lanczos_eigs(A, alg.start_vector, alg.max_iters, alg.tol, alg.pbar, alg.key, k_select=sl)
        return sel_vals, V
    raise NotImplementedError(f"eig with {type(alg).__name__} is not implemented")


def eigmax(A, alg: Algorithm = Auto()):
    es, _ = eig(A, k=1, which="LM", alg=alg)
    return es[0]


def eigmin(A, alg: Algorithm = Auto()):
    es, _ = eig(A, k=1, which="SM", alg=alg)
    return es[0]
