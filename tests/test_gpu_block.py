"""The batched solver's block schedule (COLAGB_SCHED_BLOCK): the right-hand sides of one matrix advance
in lockstep as the columns of an (n, k) block, like the reference's multi-column CG (cg.py:94-154).
Each column must reach the FP64 true residual on its own, and give the solution the one-cluster-per-
right-hand-side schedule gives (within 1e-6 relative), for padded widths (k not a power of two), more
columns than one launch takes (k > 128), zero right-hand sides and both preconditioners."""
import pytest
import torch

from cola_gb300.linalg.batched import BatchedCSR, solve_batched
from cola_gb300.workloads import diffusion_3d

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")


def _family(m, seed=1):
    ip, ix, v = diffusion_3d(m=m, seed=seed, shift=1e-3, device=DEV)
    return BatchedCSR(ip, ix, v[None, :], shared=True), (ip, ix, v)


def _relres(csr, B, X):
    ip, ix, v = csr
    n = ip.numel() - 1
    A = torch.sparse_csr_tensor(ip.long(), ix.long(), v.double(), (n, n))
    R = B.T - A @ X.T
    return R.norm(dim=0) / B.norm(dim=1).clamp_min(1e-300)


@pytest.mark.parametrize("prec", ["jacobi", "none"])
@pytest.mark.parametrize("k", [5, 32])
def test_block_schedule_matches_cluster_schedule(prec, k):
    fam, csr = _family(24)
    B = torch.randn(k, fam.n, device=DEV, dtype=torch.float64, generator=torch.Generator("cuda").manual_seed(k))
    Xb, ib = solve_batched(fam, B, precond=prec, tol=1e-9)
    assert ib["schedule"] == "block"
    Xc, ic = solve_batched(fam, B, precond=prec, tol=1e-9, schedule="cluster16")
    assert bool((ib["status"] == 1).all()) and float(ib["relres"].max()) <= 1e-9
    assert float(_relres(csr, B, Xb).max()) <= 1.01e-9
    assert float((Xb - Xc).norm() / Xc.norm()) < 1e-6
    # lockstep columns take about as many steps as independent ones
    kb, kc = ib["iterations"].double(), ic["iterations"].double()
    assert float((kb / kc).max()) < 1.3 and float((kb / kc).min()) > 0.7, (kb.tolist(), kc.tolist())


def test_block_schedule_many_columns_and_zero_rhs():
    fam, csr = _family(12)
    k = 130  # two launches: 128 + 2 columns
    B = torch.randn(k, fam.n, device=DEV, dtype=torch.float64, generator=torch.Generator("cuda").manual_seed(3))
    B[7].zero_()
    X, info = solve_batched(fam, B, precond="jacobi", tol=1e-10, schedule="block")
    assert bool((info["status"] == 1).all())
    assert torch.all(X[7] == 0)
    rr = _relres(csr, B, X)
    rr[7] = 0
    assert float(rr.max()) <= 1.01e-10


def test_block_schedule_refuses_what_it_cannot_run():
    fam, _ = _family(12)
    B = torch.randn(4, fam.n, device=DEV, dtype=torch.float64)
    with pytest.raises(NotImplementedError, match="block schedule"):
        solve_batched(fam, B, precond="jacobi", schedule="block", matvec="bf16")
    own = BatchedCSR(fam.indptr, fam.indices, fam.values.expand(4, -1).contiguous())
    with pytest.raises(NotImplementedError, match="block schedule"):
        solve_batched(own, B, precond="jacobi", schedule="block")
