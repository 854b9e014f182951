"""CPU oracle for the Krylov hot path -- TEST INFRASTRUCTURE ONLY.

A plain numpy restatement of the reference algorithms (CoLA's run_batched_cg, lanczos_fact,
LanczosUnary, slq_fwd, hutchinson_diag_estimate and the structured matvecs).  It is imported by
tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker / the CPU
reference timing, never by the cola_gb300 package.

Parity pinning: every function here is checked against golden vectors produced by running the
reference itself (tests/golden/make_golden.py imports the reference's source tree through test-only
stand-ins for its two missing dependencies) and against the reference test suite's known-answer cases.
"""
from .cg import run_batched_cg, cg_solve  # noqa: F401
from .lanczos import lanczos, lanczos_eigs, lanczos_unary_matmat, slq_estimate, hutchinson_diag  # noqa: F401
from .ops import dense_op, csr_op, diag_op, kron_op, sum_op, product_op, blockdiag_op  # noqa: F401
