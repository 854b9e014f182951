"""f(A) through Lanczos quadrature, trace / diag estimation and logdet
(cola/linalg/unary/unary.py:37-60, 94-137, 249-262; cola/linalg/trace/diag_trace.py;
cola/linalg/trace/diagonal_estimation.py:108-210; cola/linalg/logdet/logdet.py;
cola/linalg/tbd/slq.py:37-75).
"""
from __future__ import annotations

import math
from functools import reduce
from typing import Callable

import numpy as np
import torch

from .. import ops as O
from ..annotations import PSD, SelfAdjoint
from .algorithms import LU, Algorithm, Auto, Cholesky, Eigh, Exact, Hutch, Lanczos
from .lanczos import run_lanczos, tridiag_eigh
from .prng import PRNGKey, next_key, randn


def _basis_combine(basis: torch.Tensor, coef: torch.Tensor, m: int) -> torch.Tensor:
    """out[:, b] = sum_{j<m} basis[j+1][:, b] * coef[b, j] on the device."""
    import ctypes as C
    from .. import _capi
    lib = _capi.load()
    _, n, bs = basis.shape
    coef = coef.to(basis.dtype).contiguous()
    out = torch.empty((n, bs), dtype=basis.dtype, device=basis.device)
    _capi.check(lib.colagb_basis_combine(basis.data_ptr(), n, bs, m, coef.data_ptr(), coef.shape[1], out.data_ptr(),
                                         _capi.TORCH_TO_CODE[basis.dtype], _capi.stream_ptr(basis.device)),
                "basis combine")
    return out


class LanczosUnary(O.LinearOperator):
    """Lazy f(A) for self-adjoint A: batched Lanczos on the probe block, FP64 eigendecomposition of each
    tridiagonal and the quadrature |z| Q P (f(lambda) * P[0, :]) (unary.py:37-60)."""

    def __init__(self, A: O.LinearOperator, f: Callable, **kwargs):
        self.device = A.device
        super().__init__(A.dtype, A.shape, annotations={SelfAdjoint})
        self.A, self.f = A, f
        self.kwargs = dict(kwargs)
        self.info = {}
        self.last_T = None

    def _quadrature(self, V):
        kw = {k: v for k, v in self.kwargs.items() if k != "start_vector"}
        max_iters = min(int(kw.get("max_iters", 100)), self.A.shape[0])
        res = run_lanczos(self.A, V, max_iters, kw.get("tol", 1e-7))
        self.info.update(res.info())
        alpha, beta, _ = res.alpha_beta_q()
        evals, P, _ = tridiag_eigh(beta, alpha, want_vectors=True)
        self.last_T = (alpha, beta, evals)
        eps = torch.finfo(self.dtype).eps
        thresh = 10 * eps * evals.abs().max(dim=1, keepdim=True).values
        fe = torch.where(evals.abs() > thresh, self.f(evals), torch.zeros_like(evals))
        return res, evals, P, fe

    def _matmat(self, V):
        V = V.to(self.A.device)
        res, evals, P, fe = self._quadrature(V)
        norms = torch.linalg.norm(V.double(), dim=0)  # (bs,)
        w = P[:, 0, :] * norms[:, None]               # (bs, m)
        coef = torch.einsum("bij,bj->bi", P, fe * w)   # (bs, m): P (f(lambda) * P[0,:] |z|)
        return _basis_combine(res.basis, coef.to(res.basis.dtype), res.iters)

    def quadratic_forms(self, V):
        """z_b^T f(A) z_b = |z_b|^2 sum_j P[0, j]^2 f(lambda_j) for every probe column (the SLQ estimate)."""
        V = V.to(self.A.device)
        _, evals, P, fe = self._quadrature(V)
        norms2 = (V.double() ** 2).sum(0)
        return norms2 * (P[:, 0, :] ** 2 * fe).sum(1)


def apply_unary(f: Callable, A: O.LinearOperator, alg: Algorithm = Auto()):
    """f(A) (unary.py:94-137)."""
    if isinstance(alg, Auto):
        psd, small = A.isa(PSD), np.prod(A.shape) <= 1e6
        if psd and small:
            alg = Eigh()
        elif psd:
            alg = Lanczos(**alg.__dict__)
        else:
            raise NotImplementedError("f(A) of non-PSD operators (Eig / Arnoldi) is not on this path")
    if isinstance(alg, Lanczos):
        assert A.isa(SelfAdjoint), "Lanczos only valid for SelfAdjoint, wrap in cola.SelfAdjoint if desired"
        return LanczosUnary(A, f, **alg.__dict__)
    if isinstance(alg, Eigh):
        evals, evecs = torch.linalg.eigh(A.to_dense())
        return O.Dense((evecs * f(evals)[None, :]) @ evecs.T)
    raise NotImplementedError(f"apply_unary with {type(alg).__name__}")


def log(A: O.LinearOperator, alg: Algorithm = Auto()):
    """Matrix logarithm of a PD operator (unary.py:249-262)."""
    if isinstance(A, O.Kronecker):
        raise NotImplementedError("log of a Kronecker product: use logdet, which factorises it")
    return apply_unary(torch.log, A, alg)


def exp(A: O.LinearOperator, alg: Algorithm = Auto()):
    """Matrix exponential of a self-adjoint operator (unary.py:228-246)."""
    return apply_unary(torch.exp, A, alg)


def sqrt(A: O.LinearOperator, alg: Algorithm = Auto()):
    """Matrix square root of a PSD operator (unary.py:265-280); Diagonal / ScalarMul / Identity exactly,
    a Nystrom preconditioner in its own form (preconditioners.py:163-170)."""
    from .preconditioning import NystromPrecondLazy, sqrt as nystrom_sqrt
    if isinstance(A, NystromPrecondLazy):
        return nystrom_sqrt(A)
    if isinstance(A, O.Diagonal):
        return O.Diagonal(torch.sqrt(A.diag))
    if isinstance(A, O.ScalarMul):
        return O.ScalarMul(math.sqrt(A.c), A.shape, A.dtype, A.device)
    if isinstance(A, O.Identity):
        return A
    return apply_unary(torch.sqrt, A, alg)


def pow(A: O.LinearOperator, alpha: float, alg: Algorithm = Auto()):
    """A ** alpha for a PSD operator (unary.py:283-334)."""
    return apply_unary(lambda x: x ** alpha, A, alg)


# ---------------------------------------------------------------------------------------------
# diag / trace

def exact_diag(A: O.LinearOperator, k: int, bs: int):
    """Main diagonal through blocks of identity columns (diagonal_estimation.py:117-128)."""
    if k != 0:
        raise NotImplementedError("only the main diagonal is on this path")
    n = A.shape[0]
    bs = min(100, n)
    out = []
    for i in range(0, n, bs):
        cols = torch.arange(i, min(i + bs, n), device=A.device)
        chunk = torch.zeros((n, cols.numel()), dtype=A.dtype, device=A.device)
        chunk[cols, torch.arange(cols.numel(), device=A.device)] = 1
        out.append(((A @ chunk) * chunk).sum(-1))
    return reduce(torch.add, out)


def hutchinson_diag_estimate(A: O.LinearOperator, k=0, bs=100, tol=3e-2, max_iters=10000, pbar=False, rand="normal",
                             key=None):
    """Stochastic diagonal estimate (diagonal_estimation.py:159-210).  Probes come from the keyed
    host generator exactly as in the reference (100 probes per round, key advanced by sha_hash)."""
    if k != 0:
        raise NotImplementedError("only the main diagonal is on this path")
    n = A.shape[0]
    bs = min(100, n)
    assert tol > 1e-3, "tolerance chosen too high for stochastic diagonal estimation"
    assert rand in ["normal", "rademacher"], "rand must be 'normal' or 'rademacher'"
    key = PRNGKey(42) if key is None else key
    dt = A.dtype if A.dtype != torch.bfloat16 else torch.float32
    diag_sum = torch.zeros(n, dtype=torch.float64, device=A.device)
    diag_sumsq = torch.zeros(n, dtype=torch.float64, device=A.device)
    i = 0
    errs = []

    def err():
        mean = diag_sum / (i * bs)
        stderr = torch.sqrt((diag_sumsq / (i * bs) - mean**2) / (i * bs))
        return float(torch.mean(stderr / torch.maximum(mean.abs(), 0.1 * torch.ones_like(mean))))

    while i == 0 or (i < max_iters and err() > tol):
        key = next_key(key)
        z = randn(n, bs, dtype=dt, key=key)
        if rand == "rademacher":
            z = torch.sign(z)
        z = z.to(A.device)
        est = ((A @ z) * z).double()
        diag_sum += est.sum(-1)
        diag_sumsq += (est**2).sum(-1)
        i += 1
        errs.append(err())
    mean = (diag_sum / (i * bs)).to(dt)
    return mean, {"iterations": i, "errors": np.array(errs)}


def diag(A: O.LinearOperator, k: int = 0, alg: Algorithm = Auto()):
    """Diagonal extraction (diag_trace.py:23-128)."""
    if isinstance(A, O.Dense):
        return torch.diagonal(A.A, k)
    if isinstance(A, O.Diagonal) and k == 0:
        return A.diag
    if isinstance(alg, Auto):
        tol = alg.__dict__.get("tol", 1e-6)
        alg = Exact() if tol < 1 / np.sqrt(10 * np.prod(A.shape)) else Hutch(**alg.__dict__)
    if isinstance(alg, (Exact, Hutch)):
        return alg(A, k)
    raise NotImplementedError(f"diag with {type(alg).__name__}")


def trace(A: O.LinearOperator, alg: Algorithm = Auto()):
    """Trace (diag_trace.py:131-147); Kronecker traces factorise."""
    assert A.shape[0] == A.shape[1], "Can't trace non square matrix"
    if isinstance(A, O.Kronecker):
        return reduce(lambda a, b: a * b, [trace(M, alg) for M in A.Ms])
    return diag(A, 0, alg).sum()


# ---------------------------------------------------------------------------------------------
# logdet

def _prod(xs):
    return reduce(lambda x, y: x * y, xs, 1)


def slogdet(A: O.LinearOperator, log_alg: Algorithm = Auto(), trace_alg: Algorithm = Auto()):
    """(sign, log|det A|) with the reference's structural rules (logdet.py:52-184)."""
    if isinstance(A, O.Identity):
        z = torch.zeros((), dtype=A.dtype)
        return 1.0 + z, z
    if isinstance(A, O.ScalarMul):
        c = torch.as_tensor(A.c, dtype=A.dtype)
        return c / c.abs(), torch.log(c.abs())
    if isinstance(A, O.Diagonal):
        mag = A.diag.abs()
        return torch.prod(A.diag / mag), torch.sum(torch.log(mag))
    if isinstance(A, O.Kronecker):
        signs, logdets = zip(*[slogdet(Ai, log_alg, trace_alg) for Ai in A.Ms])
        sizes = [Ai.shape[-1] for Ai in A.Ms]
        prod = _prod(sizes)
        return (_prod([signs[i] ** (prod / sizes[i]) for i in range(len(sizes))]),
                sum(logdets[i] * prod / sizes[i] for i in range(len(sizes))))
    if isinstance(A, O.BlockDiag):
        signs, logdets = zip(*[slogdet(Ai, log_alg, trace_alg) for Ai in A.Ms])
        return (_prod(s**n for s, n in zip(signs, A.multiplicities)),
                sum(ld * n for ld, n in zip(logdets, A.multiplicities)))
    if isinstance(A, O.Product) and all(M.shape[-2] == M.shape[-1] for M in A.Ms):
        signs, logdets = zip(*[slogdet(Ai, log_alg, trace_alg) for Ai in A.Ms])
        return _prod(signs), sum(logdets)
    if isinstance(log_alg, Auto):
        is_psd, small = A.isa(PSD), np.prod(A.shape) <= 1e6
        if is_psd and small:
            log_alg = Cholesky()
        elif not is_psd and small:
            log_alg = LU()
        elif is_psd:
            log_alg = Lanczos(**log_alg.__dict__)
        else:
            raise NotImplementedError("logdet of large non-PSD operators (Arnoldi) is not on this path")
    if isinstance(log_alg, Cholesky):
        assert A.isa(PSD), "Cholesky only valid for PSD matrices, wrap in cola.PSD if necessary"
        L = torch.linalg.cholesky(A.to_dense())
        ld = 2 * torch.sum(torch.log(torch.diagonal(L).abs()))
        return torch.ones((), dtype=ld.dtype, device=ld.device), ld
    if isinstance(log_alg, LU):
        return torch.linalg.slogdet(A.to_dense())
    if isinstance(log_alg, Lanczos):
        logA = log(A, log_alg)
        tr = trace(logA, trace_alg)
        mag = tr.abs()
        return tr / mag, mag
    raise NotImplementedError(f"slogdet with {type(log_alg).__name__}")


def logdet(A: O.LinearOperator, log_alg: Algorithm = Auto(), trace_alg: Algorithm = Auto()):
    """log|det A| (logdet.py:29-49)."""
    _, ld = slogdet(A, log_alg=log_alg, trace_alg=trace_alg)
    return ld


def stochastic_lanczos_quad(A: O.LinearOperator, fun: Callable, max_iters: int = 100, tol: float = 1e-5, vtol=0.1,
                            pbar: bool = False, key=None, probes: torch.Tensor | None = None):
    """tr f(A) ~ n * mean_b sum_j tau_bj^2 f(lambda_bj) over Gaussian probes (tbd/slq.py:37-75).

    ``probes`` (n, num_samples) may be passed to reuse identical probe vectors.  Differentiable in
    the operator's tensors with the reference's backward rule (that of f = log)."""
    num_samples = max(int(1 / vtol**2), 1)
    n = A.shape[0]
    if probes is None:
        key = PRNGKey(0) if key is None else key
        probes = randn(n, num_samples, dtype=A.dtype, key=key)
    probes = probes.to(A.device)

    def forward():
        res = run_lanczos(A, probes, min(int(max_iters), n), tol)
        alpha, beta, _ = res.alpha_beta_q()
        evals, first, _ = tridiag_eigh(beta, alpha, want_vectors=False)
        eps = torch.finfo(A.dtype).eps
        const = 10 * eps * evals.max(dim=1, keepdim=True).values
        fv = torch.where(evals.abs() > const, fun(evals), torch.zeros_like(evals))
        approx = (first**2 * fv).sum(-1)
        return (n * approx).mean()

    from .autodiff import slq_with_grad, wants_grad
    if wants_grad(A):
        # backward of the reference (slq_bwd, tbd/slq.py:10-31): the rule of f = log, A^-1 z_i by CG
        # with tol 1e-6 and 100 iterations on the forward's own probes
        from .inverse import cg
        return slq_with_grad(A, probes, forward, lambda Z: cg(A, Z, tol=1e-6, max_iters=100)[0])
    return forward()
