"""cola_gb300 -- CoLA's iterative Krylov hot path (CG, Lanczos, SLQ and the structured matvecs they
call) as hand-written sm_103a CUDA behind the CoLA operator / linalg API.

    import cola_gb300 as cola
    A = cola.PSD(cola.ops.Sparse(data, rows, cols, shape))        # CUDA tensors
    x = cola.linalg.solve(A, b, cola.linalg.CG(tol=1e-6, max_iters=2000))

All compute runs in libcolagb.so (built in-tree by ``cola_gb300._build.build()``); there is no
CPU execution path.
"""
from . import annotations, fns, linalg, ops
from .annotations import PSD, Hermitian, SelfAdjoint, Stiefel, Unitary
from .fns import add, densify, dot, kron, lazify, mul, transpose
from .linalg import CG, Auto, Exact, Hutch, Lanczos, eig, inv, logdet, slogdet, solve, trace
from .ops import (BlockDiag, Dense, Diagonal, I_like, Identity, Kronecker, LinearOperator, Product, ScalarMul, Sparse,
                  Sum, Tridiagonal)

__version__ = "0.1.0"

__all__ = [
    "ops", "linalg", "fns", "annotations", "PSD", "SelfAdjoint", "Hermitian", "Unitary", "Stiefel", "lazify",
    "densify", "dot", "add", "mul", "kron", "transpose", "CG", "Lanczos", "Auto", "Exact", "Hutch", "solve", "inv",
    "eig", "logdet", "slogdet", "trace", "LinearOperator", "Dense", "Sparse", "Diagonal", "Kronecker", "Sum",
    "Product", "BlockDiag", "ScalarMul", "Identity", "I_like", "Tridiagonal",
]
