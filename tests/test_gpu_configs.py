"""Parity with the reference at the benchmark configurations' full sizes.

The fixtures tests/golden/cfg_*.npz were recorded by running the reference CoLA itself on the same
seeded inputs (tests/golden/make_golden_configs.py); the inputs are regenerated here with CPU random
generators and checked against the checksums stored with each case before anything is compared.
Tolerances are the ones the benchmark specification states: solutions 1e-6 relative (FP64 /
refined results), eigenvalues 1e-5 relative, log-determinants within the SLQ standard error of the
same 64 probes; FP32 CG runs compare iteration counts and true residuals with the reference's FP32
run.  Where the reference's own FP32 result is measurably off the FP64 oracle, the test says by how
much and holds this implementation to the oracle.
"""
from pathlib import Path

import numpy as np
import pytest
import torch

import cola_gb300 as cola
from cola_gb300 import workloads as W
from cola_gb300.linalg.prng import randn as keyed_randn

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")
GOLD = Path(__file__).resolve().parent / "golden"


def fixture(name):
    return np.load(GOLD / f"cfg_{name}.npz")


def probe_vectors(n, count=4, seed=99):
    return np.sign(np.random.default_rng(seed).standard_normal((count, n)))


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_c1_dense_2048_cg_matches_reference():
    g = fixture("c1")
    A, b, _ = W.dense_spd(2048, seed=0, lo=1e-2, hi=1e2, dtype=torch.float32)
    assert rel(probe_vectors(2048) @ A.double().numpy(), g["a_proj"]) < 1e-12  # same inputs
    op = cola.PSD(cola.ops.Dense(A.to(DEV)))
    # FP32, the reference's stop rule: iteration count within 5 %, true residual within 1.5x
    x, info = cola.linalg.cg(op, b.to(DEV), tol=1e-6, max_iters=2000)
    A64, b64 = A.double(), b.double()
    relres = float((b64 - A64 @ x.cpu().double()).norm() / b64.norm())
    it = info["iterations"]  # counted like the reference's info["iterations"]
    assert abs(it - int(g["iterations32"])) <= 0.05 * int(g["iterations32"]), (it, int(g["iterations32"]))
    assert relres <= 1.5 * float(g["relres32"]), (relres, float(g["relres32"]))
    # FP64: the solution within 1e-6 of the reference's FP64 solution
    op64 = cola.PSD(cola.ops.Dense(A64.to(DEV)))
    x64, _ = cola.linalg.cg(op64, b64.to(DEV), tol=1e-13, max_iters=20000)
    assert rel(x64.cpu().numpy(), g["x64"]) < 1e-6


def test_c3a_uneven_rbf_first8_match_reference():
    """One persistent launch over the first 8 systems of the uneven RBF batch, against the reference's
    one-call-per-system FP32 CG(tol=1e-6, max_iters=2000): the ill-conditioned systems stagnate at the
    same true-residual level in both."""
    g = fixture("c3a")
    mats, rhs, meta = W.rbf_systems(num=8, seed=3, device="cpu")
    assert [m[0] for m in meta] == list(g["n"])
    sols, iters, status = cola.linalg.solve_dense_batched([A.to(DEV) for A in mats], [b.to(DEV) for b in rhs],
                                                          tol=1e-6, max_iters=2000)
    for s, (A, b, x) in enumerate(zip(mats, rhs, sols)):
        r = float((b.double() - A.double() @ x.cpu().double()).norm() / b.double().norm())
        r_ref = float(g["relres"][s])
        # same order of magnitude of the final true residual (FP32 drift dominates both)
        assert r <= 3.0 * r_ref + 1e-6 and r >= r_ref / 30.0, (s, r, r_ref)
        if r_ref < 1e-3:  # well-conditioned systems: the same number of steps within 10 %
            assert abs(int(iters[s]) - int(g["iterations"][s])) <= 0.1 * int(g["iterations"][s]) + 2, \
                (s, int(iters[s]), int(g["iterations"][s]))


def test_c3a_refined_systems_reach_the_true_residual():
    """With FP64 refinement (which the reference does not have) the same 8 systems, including the ones
    FP32 CG stagnates on, reach a true relative residual of 1e-8 checked in FP64."""
    mats, rhs, meta = W.rbf_systems(num=8, seed=3, device="cpu")
    sols, iters, status = cola.linalg.solve_dense_batched([A.to(DEV) for A in mats], [b.to(DEV) for b in rhs],
                                                          tol=1e-8, max_iters=2000, refine=True)
    assert bool((status == 1).all()), status.tolist()
    for A, b, x in zip(mats, rhs, sols):
        r = float((b.double() - A.double() @ x.cpu().double()).norm() / b.double().norm())
        assert r <= 1.01e-8, r


def test_c3b_kron_slq_against_reference_and_exact_logdet():
    """Identical probes, FP32.  In FP32 the operator's own rounding (about eps * |A| = 5e-4 absolute) is
    not small against its smallest eigenvalues (0.01), so two FP32 runs of the same recurrence resolve
    the bottom of the spectrum differently: the reference's tridiagonals reach a smallest Ritz value of
    0.01085, these 0.0102, and the per-probe quadratures differ by ~2 %.  The test holds the estimate to
    the exact FP64 log-determinant and requires it to be no farther from it than the reference's
    estimate is; the FP64 test below compares with the reference probe by probe."""
    g = fixture("c3b")
    Ks, ells = W.kron_rbf(seed=4, m=64, factors=3, device="cpu", dtype=torch.float32)
    n = 64 ** 3
    Z = torch.sign(keyed_randn(n, 64, dtype=torch.float32, key=5))
    assert rel(probe_vectors(n) @ Z.double().numpy(), g["z_proj"]) < 1e-12
    K = cola.ops.Kronecker(*[cola.ops.Dense(k.to(DEV)) for k in Ks])
    op = cola.PSD(K + 0.01 * cola.ops.I_like(K))
    F = cola.linalg.LanczosUnary(op, torch.log, max_iters=100, tol=0.0)
    quad = F.quadratic_forms(Z.to(DEV)).cpu().numpy()
    est, ref_est, exact = quad.mean(), float(g["estimate"]), float(g["exact"])
    print(f"c3b: estimate {est:.6e}, reference {ref_est:.6e} (stderr {float(g['stderr']):.1f}), exact FP64 "
          f"{exact:.6e}; rel vs exact {abs(est - exact) / abs(exact):.2e} (reference {abs(ref_est - exact) / abs(exact):.2e})")
    assert abs(est - exact) <= abs(ref_est - exact)
    assert abs(est - exact) / abs(exact) < 5e-3


def test_c3b_kron_slq_fp64_matches_reference_probe_by_probe():
    """The same SLQ in FP64 on the first 16 probes: the reference's and this implementation's quadratic
    forms z^T log(A) z agree probe by probe, and the estimates lie within the SLQ standard error of the
    same probes (the stated tolerance)."""
    g = fixture("c3b64")
    Ks, ells = W.kron_rbf(seed=4, m=64, factors=3, device="cpu", dtype=torch.float32)
    n = 64 ** 3
    Z = torch.sign(keyed_randn(n, 64, dtype=torch.float32, key=5))[:, :16].double()
    K = cola.ops.Kronecker(*[cola.ops.Dense(k.double().to(DEV)) for k in Ks])
    op = cola.PSD(K + 0.01 * cola.ops.I_like(K))
    quad = cola.linalg.LanczosUnary(op, torch.log, max_iters=100, tol=0.0).quadratic_forms(Z.to(DEV)).cpu().numpy()
    ref = g["quad"]
    worst = float(np.max(np.abs(quad - ref) / np.abs(ref)))
    print(f"c3b fp64: max per-probe rel diff {worst:.2e}, estimate {quad.mean():.8e} vs {float(g['estimate']):.8e}")
    assert worst < 1e-6
    stderr = float(np.std(ref) / np.sqrt(ref.size))
    assert abs(quad.mean() - float(g["estimate"])) < stderr


def test_c4_instance_refined_solution_matches_reference_fp64():
    g = fixture("c4")
    fam, B, _, _ = W.diffusion_family_2d([5000], m=512, device="cpu")
    v = fam.values[0].double().numpy()
    assert rel(probe_vectors(v.size) @ v, g["values_proj"]) < 1e-6  # same inputs up to FP32 rounding
    famd = cola.linalg.BatchedCSR(fam.indptr.to(DEV), fam.indices.to(DEV), fam.values.to(DEV))
    for prec in ("jacobi", "none"):
        X, info = cola.linalg.solve_batched(famd, B.to(DEV), precond=prec, tol=1e-11)
        assert int(info["status"][0]) == 1
        x = X[0].cpu().numpy()
        assert rel(x[::16], g["x_sub"]) < 1e-6, (prec, rel(x[::16], g["x_sub"]))
        assert rel(probe_vectors(x.size) @ x, g["x_proj"]) < 1e-6


@pytest.mark.parametrize("precision", ["auto", "fp32"])
def test_c5_lanczos_top64_matches_reference_and_arpack(precision):
    """The reference's own FP32 Lanczos sits ~1.3e-5 (relative) above the FP64 ARPACK eigenvalues on
    this operator, on every converged Ritz value; so the comparison with the reference allows 1e-5 beyond
    that offset, and the converged values are held to the FP64 oracle directly.  "auto" runs the
    Kronecker factors on the tensor cores (three-product BF16 split), "fp32" on the FP32 SIMT path."""
    g = fixture("c5")
    A1, _, _ = W.dense_spd(1024, seed=6, lo=1e-2, hi=1e1, dtype=torch.float32)
    A2, _, _ = W.dense_spd(1024, seed=61, lo=1e-2, hi=1e1, dtype=torch.float32)
    ip, ix, v = W.rgg_laplacian(1 << 20, 0.002, seed=7, device="cpu")
    n = 1 << 20
    assert int(ix.numel()) == int(g["l_nnz"])
    assert rel(probe_vectors(1024) @ A1.double().numpy(), g["a1_proj"]) < 1e-12
    start = keyed_randn(n, dtype=torch.float32, key=cola.linalg.PRNGKey(42))
    # torch's CPU normal generator agrees across host architectures to FP32 rounding, not bit for bit
    assert rel(probe_vectors(n) @ start.double().numpy(), g["start_proj"]) < 1e-6
    L = cola.ops.Sparse.from_csr(ip.to(DEV), ix.to(DEV), v.to(DEV), (n, n))
    K = cola.ops.Kronecker(cola.ops.Dense(A1.to(DEV)), cola.ops.Dense(A2.to(DEV)), precision=precision)
    op = cola.SelfAdjoint(K + L)
    vals, _ = cola.linalg.eig(op, 64, "LM", cola.linalg.Lanczos(start_vector=start.to(DEV), max_iters=256, tol=1e-12))
    ours = np.sort(vals.double().cpu().numpy())
    ref = np.sort(np.asarray(g["ref_evals"], dtype=np.float64))
    arp = np.sort(g["arpack_evals"])
    conv = slice(52, 64)  # the top 12 Ritz values have converged (reference and ARPACK agree to ~1e-5)
    ref_offset = float(np.max(np.abs(ref[conv] - arp[conv]) / arp[conv]))
    vs_ref = np.abs(ours - ref) / np.abs(ref)
    vs_arp = np.abs(ours[conv] - arp[conv]) / arp[conv]
    print(f"c5 {precision}: max rel vs reference {vs_ref.max():.2e} (reference vs ARPACK {ref_offset:.2e}), "
          f"converged vs ARPACK {vs_arp.max():.2e}")
    assert vs_ref.max() < 1e-5 + ref_offset
    assert vs_arp.max() < 1e-5
