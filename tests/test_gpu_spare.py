"""The on-chip schedule's companion CTAs (one 512-thread CTA per SM the clusters leave free, vectors in
global memory): same algorithm, stop rule and outputs as the clusters.  spare="only" runs every system
on them; spare="off" on the clusters alone; "auto" mixes the two on batches larger than the tail
reserve (about ten systems per resident cluster)."""
import numpy as np
import pytest
import torch

import cola_gb300 as cola

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")


def rel(a, b):
    a, b = a.detach().double().cpu().numpy(), b.detach().double().cpu().numpy()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _fsai(fam):
    from cola_gb300.precond.learned_fsai import g_values
    return g_values(fam, None)


def _true_relres(fam, B, X, idx):
    out = []
    for s in idx:
        v = fam.values[s if fam.values.shape[0] > 1 else 0].double()
        A = torch.sparse_csr_tensor(fam.indptr.long(), fam.indices.long(), v, (fam.n, fam.n))
        r = B[s].double() - (A @ X[s].double().unsqueeze(1)).squeeze(1)
        out.append(float(r.norm() / B[s].double().norm()))
    return max(out)


@pytest.mark.parametrize("m,S", [(32, 5), (64, 3), (512, 2)])
@pytest.mark.parametrize("precond", ["none", "jacobi", "fsai"])
def test_companion_ctas_match_clusters(precond, m, S):
    from cola_gb300.workloads import diffusion_family_2d
    if m == 512 and precond == "none":
        pytest.skip("plain CG on 512 x 512 takes ~10,000 steps on one SM")
    fam, B, _, _ = diffusion_family_2d(range(70, 70 + S), m=m, device=DEV)
    kw = dict(precond=precond, tol=1e-8, schedule="onchip", fsai=_fsai(fam) if precond == "fsai" else None)
    X1, i1 = cola.linalg.solve_batched(fam, B, spare="only", **kw)
    X2, i2 = cola.linalg.solve_batched(fam, B, spare="off", **kw)
    assert i1["schedule"] == "onchip"
    assert i1["companion_systems"] == S and i2["companion_systems"] == 0
    assert torch.all(i1["status"] == 1) and torch.all(i2["status"] == 1), (i1["status"], i2["status"])
    assert float(i1["relres"].max()) <= 1e-8
    assert _true_relres(fam, B, X1, range(S)) <= 1.01e-8
    k1, k2 = i1["iterations"].double(), i2["iterations"].double()
    assert float(((k1 - k2).abs() - (0.15 * k2 + 3)).max()) <= 0, (k1.tolist(), k2.tolist())
    assert rel(X1, X2) < 1e-6


def test_companion_ctas_limits_and_nan():
    from cola_gb300.workloads import diffusion_family_2d
    fam, B, _, _ = diffusion_family_2d(range(60, 63), m=32, device=DEV)
    X, info = cola.linalg.solve_batched(fam, B, precond="jacobi", tol=1e-8, schedule="onchip", spare="only")
    # the step cap: MAX_ITERS with the FP64-refined iterate returned
    X2, i2 = cola.linalg.solve_batched(fam, B, precond="none", tol=1e-12, max_inner_iters=20, schedule="onchip",
                                       spare="only")
    assert torch.all(i2["status"] == 2) and torch.all(i2["iterations"] == 20) and bool(torch.isfinite(X2).all())
    # a NaN right-hand side is reported for that system only
    B3 = B.clone()
    B3[1, 5] = float("nan")
    X3, i3 = cola.linalg.solve_batched(fam, B3, precond="jacobi", tol=1e-8, schedule="onchip", spare="only")
    assert i3["status"].tolist() == [1, 4, 1]
    assert rel(X3[0], X[0]) < 1e-6 and rel(X3[2], X[2]) < 1e-6
    # restart mode
    X4, i4 = cola.linalg.solve_batched(fam, B, precond="jacobi", tol=1e-8, mode="restart", schedule="onchip",
                                       spare="only")
    assert torch.all(i4["status"] == 1)
    assert _true_relres(fam, B, X4, range(3)) <= 1.01e-8


def test_auto_mixes_clusters_and_companions_on_a_large_batch():
    """256 systems of the 512 x 512 family with the closed-form FSAI factor: the clusters and the
    companion CTAs share the batch; every system meets the FP64 stop rule (checked independently on a
    sample) and the step counts match the clusters-only run's to a few per cent on average."""
    from cola_gb300.workloads import diffusion_family_2d
    fam, B, _, _ = diffusion_family_2d(range(200, 456), m=512, device=DEV)
    kw = dict(precond="fsai", tol=1e-8, schedule="onchip", fsai=_fsai(fam))
    X1, i1 = cola.linalg.solve_batched(fam, B, spare="auto", **kw)
    X2, i2 = cola.linalg.solve_batched(fam, B, spare="off", **kw)
    assert torch.all(i1["status"] == 1) and torch.all(i2["status"] == 1)
    # the companions take a share, the clusters keep the tail (28 systems per resident cluster; 7 clusters
    # of 16 CTAs at this size on a 152-SM GB300)
    from cola_gb300.linalg.batched import onchip_schedule_info
    nc = onchip_schedule_info(fam.n, 512)["clusters_in_flight"]
    assert 0 < i1["companion_systems"] <= max(0, 256 - 28 * nc) and i2["companion_systems"] == 0, \
        (i1["companion_systems"], nc)
    assert float(i1["relres"].max()) <= 1e-8
    assert _true_relres(fam, B, X1, range(0, 256, 29)) <= 1.01e-8
    m1, m2 = float(i1["iterations"].double().mean()), float(i2["iterations"].double().mean())
    assert abs(m1 - m2) <= 0.05 * m2, (m1, m2)
    assert rel(X1, X2) < 1e-6
