"""cola.linalg equivalents on the GPU Krylov path."""
from .algorithms import (LU, Algorithm, Arnoldi, Auto, CG, Cholesky, Eigh, Exact, GMRES, Hutch, Lanczos, get_slice)
from .arnoldi import arnoldi, gmres
from .batched import BatchedCSR, solve_batched
from .inverse import IterativeOperatorWInfo, cg, inv, solve
from .lanczos import eig, eigmax, eigmin, lanczos, lanczos_eigs, run_lanczos, tridiag_eigh
from .preconditioning import NystromPrecond, NystromPrecondLazy, get_nys_approx
from .prng import PRNGKey, next_key, randn, sha_hash
from .batched import solve_dense_batched
from .unary import (LanczosUnary, apply_unary, diag, exact_diag, exp, hutchinson_diag_estimate, log, logdet, pow,
                    slogdet, sqrt, stochastic_lanczos_quad, trace)

__all__ = [
    "Algorithm", "Auto", "CG", "GMRES", "Arnoldi", "arnoldi", "gmres", "Lanczos", "Exact", "Hutch", "Cholesky", "LU", "Eigh", "get_slice",
    "IterativeOperatorWInfo", "cg", "inv", "solve", "eig", "eigmax", "eigmin", "lanczos", "lanczos_eigs",
    "run_lanczos", "tridiag_eigh", "PRNGKey", "next_key", "randn", "sha_hash", "LanczosUnary", "apply_unary",
    "diag", "exact_diag", "hutchinson_diag_estimate", "log", "logdet", "slogdet", "stochastic_lanczos_quad",
    "trace", "BatchedCSR", "solve_batched", "solve_dense_batched", "exp", "sqrt", "pow",
    "NystromPrecond", "NystromPrecondLazy", "get_nys_approx",
]
