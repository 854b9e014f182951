"""Algorithm objects of the CoLA API (cola/linalg/algorithm_base.py, inverse/cg.py:11-36,
decompositions/decompositions.py:118-144, trace/diagonal_estimation.py:15-84).

Same dataclass fields and defaults as the reference; ``CG`` adds nothing the reference lacks,
the device-specific knobs live in keyword-only extras with defaults that keep the reference's
behaviour.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from types import SimpleNamespace
from typing import Any, Optional

import torch

from ..ops import LinearOperator

PRNGKey = Any


class Algorithm:
    pass


class Auto(SimpleNamespace, Algorithm):
    """Let the dispatch rules pick an algorithm; keyword arguments are forwarded to it."""


@dataclass
class CG(Algorithm):
    """Conjugate gradients (cg.py:11-36): solves A X = B for PSD A, many right-hand sides at once.

    Args:
        tol: stop when every column's residual (of the column-normalised system) is below tol*|r0|+tol.
        max_iters: iteration cap.
        pbar: accepted for compatibility (no progress bar: the loop runs on the device).
        x0: (n,) or (n, k) initial guess.
        P: preconditioner (a LinearOperator approximating A^-1), default identity.
    """
    tol: float = 1e-6
    max_iters: int = 1000
    pbar: bool = False
    x0: Any = None
    P: Optional[LinearOperator] = None

    def __call__(self, A, b):
        from .inverse import cg
        return cg(A, b, **self.__dict__)


@dataclass
class GMRES(Algorithm):
    """Generalised minimal residual for square (non-symmetric) A (gmres.py:11-36)."""
    tol: float = 1e-6
    max_iters: int = 1000
    pbar: bool = False
    x0: Any = None
    P: Optional[LinearOperator] = None

    def __call__(self, A, b):
        from .arnoldi import gmres
        return gmres(A, b, **self.__dict__)


@dataclass
class Arnoldi(Algorithm):
    """Arnoldi decomposition A Q = Q H (decompositions.py:147-174)."""
    start_vector: Any = None
    max_iters: int = 1_000
    tol: float = 1e-6
    pbar: bool = False
    key: Optional[PRNGKey] = None

    def __call__(self, A: LinearOperator):
        from .arnoldi import arnoldi
        return arnoldi(A, **self.__dict__)


@dataclass
class Lanczos(Algorithm):
    """Lanczos decomposition Q^T A Q = T for self-adjoint A (decompositions.py:118-144)."""
    start_vector: Any = None
    max_iters: int = 1_000
    tol: float = 1e-6
    pbar: bool = False
    key: Optional[PRNGKey] = None

    def __call__(self, A: LinearOperator):
        from .lanczos import lanczos
        return lanczos(A, **self.__dict__)


@dataclass
class Exact(Algorithm):
    """Exact diagonal, e_i^T A e_i in blocks of bs columns (diagonal_estimation.py:15-33)."""
    bs: int = 100
    pbar: bool = False

    def __call__(self, A, k):
        from .unary import exact_diag
        return exact_diag(A, k, self.bs)


@dataclass
class Hutch(Algorithm):
    """Hutchinson diagonal / trace estimator (diagonal_estimation.py:36-58)."""
    tol: float = 3e-2
    max_iters: int = 10_000
    bs: int = 100
    rand: str = "normal"
    pbar: bool = False
    key: Optional[PRNGKey] = None

    def __call__(self, A, k):
        from .unary import hutchinson_diag_estimate
        return hutchinson_diag_estimate(A, k, **self.__dict__)[0]


@dataclass
class Cholesky(Algorithm):
    """Dense Cholesky (decompositions.py:29) -- small operators only, not the Krylov path."""


@dataclass
class LU(Algorithm):
    """Dense LU (decompositions.py:44) -- small operators only, not the Krylov path."""


@dataclass
class Eigh(Algorithm):
    """Dense symmetric eigendecomposition -- small operators only."""


def get_slice(num, which):
    """Eigenpair slice of an ascending spectrum (decompositions.py:214-224)."""
    if num == -1:
        raise ValueError(f"Number of eigenvalues {num} must be explicitly specified")
    if which == "SM":
        return slice(0, num, None)
    if which == "LM":
        return slice(-1 if num is None else -num, None, None)
    raise NotImplementedError(f"which={which} is not implemented")
