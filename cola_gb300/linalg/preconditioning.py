"""The Nystrom preconditioner for ``CG(P=...)`` (cola/linalg/preconditioning/preconditioners.py:88-190).

``NystromPrecond(A, rank)`` approximates A by U diag(Lambda) U^T from the product A @ Omega with a
keyed Gaussian n x rank block (``get_nys_approx``, preconditioners.py:142-153), and is the operator

    P = I + U diag(s) U^T,    s = (min(Lambda) + mu) / (Lambda + mu) - 1

(preconditioners.py:111-124), which maps the approximated eigenvalues of A to min(Lambda) + mu and
leaves the rest of the spectrum alone.  It is built as ``Sum(I, Product(Dense(U), Diagonal(s),
Dense(U^T)))``, so the device CG applies it inside its own operator program.  A @ Omega runs through
the library's matmat; the rank x rank and n x rank factorisations (QR, Cholesky, triangular solve,
SVD) of the construction are torch.linalg calls on the operator's device.

``sqrt`` and ``inverse`` of such an operator (preconditioners.py:163-190) keep U and take the square
root of, or swap, the numerator and denominator of s.
"""
from __future__ import annotations

import torch

from .. import ops as O
from .prng import PRNGKey, randn


def get_nys_approx(A, Omega: torch.Tensor, eps: float):
    """(Lambda, U) with A ~ U diag(Lambda) U^T from A @ Omega (preconditioners.py:142-153): Omega is
    orthonormalised, A Omega shifted by nu = eps |A Omega|_F, and the shifted Nystrom factor
    B = Y C^{-T} (C C^T = Omega^T Y) gives U and Lambda = max(sigma(B)^2 - nu, 0)."""
    Omega, _ = torch.linalg.qr(Omega, mode="reduced")
    Y = A @ Omega
    nu = eps * torch.linalg.norm(Y, ord="fro")
    Y = Y + nu * Omega
    C = torch.linalg.cholesky(Omega.T @ Y)
    B = torch.linalg.solve_triangular(C, Y.T, upper=False).T
    U, sigma, _ = torch.linalg.svd(B, full_matrices=False)
    return torch.clip(sigma ** 2 - nu, min=0.0), U


class NystromPrecondLazy(O.Sum):
    """I + U diag(num / denom - 1) U^T for given U, num, denom (preconditioners.py:126-138)."""

    def __init__(self, dtype, shape, U, subspace_num, subspace_denom):
        self._set_subspace(dtype, shape, U, subspace_num, subspace_denom)

    def _set_subspace(self, dtype, shape, U, subspace_num, subspace_denom):
        self.U = U
        self.subspace_num = subspace_num
        self.subspace_denom = subspace_denom
        scaling = subspace_num / subspace_denom - 1
        self.subspace_scaling = scaling[:, None]
        eye = O.Identity(shape, dtype)
        eye.to(U.device)
        self.__dict__.pop("_lowered", None)  # a rebuilt operator lowers afresh
        super().__init__(eye, O.Product(O.Dense(U), O.Diagonal(scaling.to(U.dtype).contiguous()),
                                        O.Dense(U.T.contiguous())))


class NystromPrecond(NystromPrecondLazy):
    """Nystrom preconditioner of a positive definite operator A (preconditioners.py:88-124).

    rank: the approximation's rank; mu: the regularisation of (A + mu I) x = b the preconditioner is
    made for, scaled by the largest approximated eigenvalue when adjust_mu; eps: the shift of the
    construction; key: the PRNG key of Omega (PRNGKey(42) by default, drawn like the reference's
    CPU draws and moved to A's device)."""

    def __init__(self, A, rank, mu=1e-7, eps=1e-8, adjust_mu=True, key=None):
        key = PRNGKey(42) if key is None else key
        Omega = randn(A.shape[0], rank, dtype=A.dtype, device=A.device, key=key)
        self._create_approx(A=A, Omega=Omega, mu=mu, eps=eps, adjust_mu=adjust_mu)

    def _create_approx(self, A, Omega, mu, eps, adjust_mu):
        self.Lambda, U = get_nys_approx(A=A, Omega=Omega, eps=eps)
        self.adjusted_mu = amu = mu * torch.max(self.Lambda) if adjust_mu else mu
        num = torch.min(self.Lambda) + amu
        self.preconditioned_eigmax = num
        self.preconditioned_eigmin = amu
        self._set_subspace(A.dtype, A.shape, U, num, self.Lambda + amu)


def sqrt(A: NystromPrecondLazy) -> NystromPrecondLazy:
    """P^(1/2) of a Nystrom preconditioner (preconditioners.py:163-170)."""
    return NystromPrecondLazy(A.dtype, A.shape, A.U.clone(), torch.sqrt(torch.as_tensor(A.subspace_num).clone()),
                              torch.sqrt(A.subspace_denom.clone()))


def inverse(A: NystromPrecondLazy) -> NystromPrecondLazy:
    """P^(-1) of a Nystrom preconditioner (preconditioners.py:179-190)."""
    return NystromPrecondLazy(A.dtype, A.shape, A.U.clone(), A.subspace_denom.clone(),
                              torch.as_tensor(A.subspace_num).clone())
