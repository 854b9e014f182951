"""CUDA path (through the C ABI) against the oracle, the golden vectors recorded from the reference,
and FP64 references.  Tolerances are stated per test."""
import numpy as np
import pytest
import torch

import oracle
import cola_gb300 as cola
from cola_gb300.linalg import CG, Hutch, Lanczos
from cola_gb300 import ops as O
from cola_gb300.linalg.prng import PRNGKey, next_key, randn

pytestmark = pytest.mark.gpu
DEV = "cuda"


def rel(a, b):
    a = a.detach().double().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a, dtype=np.float64)
    b = b.detach().double().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def T(x, dtype=None):
    t = torch.as_tensor(np.asarray(x))
    return t.to(DEV, dtype=dtype) if dtype else t.to(DEV)


def csr(rows, cols, vals, n, dtype):
    return cola.ops.Sparse(T(vals, dtype), T(rows), T(cols), (n, n))


# ---------------------------------------------------------------------------------------------
# structured matvecs

@pytest.mark.parametrize("dtype,tol", [(torch.float32, 1e-5), (torch.float64, 1e-12), (torch.bfloat16, 1e-2)])
@pytest.mark.parametrize("k", [1, 3, 17, 70])
def test_dense_matmat(dtype, tol, k):
    g = torch.Generator().manual_seed(k)
    A = torch.randn(131, 97, generator=g)
    X = torch.randn(97, k, generator=g)
    op = cola.ops.Dense(A.to(DEV, dtype))
    cdt = torch.float64 if dtype == torch.float64 else torch.float32
    Y = op @ X.to(DEV, cdt)
    ref = A.to(dtype).double() @ X.to(cdt).double()
    assert rel(Y, ref) < tol


@pytest.mark.parametrize("k", [1, 2, 5, 33, 64])
@pytest.mark.parametrize("dtype,tol", [(torch.float32, 1e-5), (torch.float64, 1e-12)])
def test_csr_matmat(k, dtype, tol):
    from cola_gb300.workloads import diffusion_3d
    ip, ix, v = diffusion_3d(m=9, device=DEV)
    n = 9**3
    counts = (ip[1:] - ip[:-1]).long()
    rows = torch.repeat_interleave(torch.arange(n, device=DEV), counts)
    op = cola.ops.Sparse(v.to(dtype), rows, ix.long(), (n, n))
    X = torch.randn(n, k, device=DEV, dtype=dtype)
    dense = torch.zeros(n, n, dtype=torch.float64, device=DEV)
    dense[rows, ix.long()] = v.double()
    assert rel(op @ X, dense @ X.double()) < tol


def _irregular_csr(n, seed, long_rows=(), long_len=300):
    """Row lengths 0..20 (with empty rows), a few rows of long_len entries, unsorted-in-space columns."""
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 21, n)
    lens[rng.random(n) < 0.1] = 0
    for r in long_rows:
        lens[r] = long_len
    ip = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    ix = np.concatenate([np.sort(rng.choice(n, size=int(c), replace=False)) for c in lens]).astype(np.int32)
    v = rng.standard_normal(int(ip[-1]))
    return ip, ix, v


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64, torch.bfloat16])
@pytest.mark.parametrize("misalign", [False, True])
def test_csr_spmv_irregular_rows(dtype, misalign):
    """Single-column CSR products on ragged rows: empty rows, 32-row groups whose nonzeros overflow the
    streaming kernel's buffer (rows of 300), a row count that is not a multiple of 32, and index /
    value arrays that are not 16-byte aligned (the scalar-load variant)."""
    n = 2000 + 17
    ip, ix, v = _irregular_csr(n, seed=11, long_rows=(5, 6, 7, 40, 1999))
    cdt = torch.float64 if dtype == torch.float64 else torch.float32
    vals = torch.as_tensor(v).to(dtype)
    idx = torch.as_tensor(ix)
    if misalign:  # same data one element into a larger buffer
        vals = torch.cat([vals[:1], vals])[1:]
        idx = torch.cat([idx[:1], idx])[1:]
    op = cola.ops.Sparse.from_csr(torch.as_tensor(ip).to(DEV), idx.to(DEV), vals.to(DEV), (n, n))
    x = torch.randn(n, device=DEV, dtype=cdt)
    dense = torch.zeros(n, n, dtype=torch.float64)
    rows = np.repeat(np.arange(n), np.diff(ip))
    dense[torch.as_tensor(rows), torch.as_tensor(ix).long()] = vals.double()
    ref = dense.to(DEV) @ x.double()
    y = op @ x
    assert y.dtype == cdt
    tol = 1e-12 if dtype == torch.float64 else 1e-5
    assert rel(y, ref) < tol
    # Sum of two leaves: the second product accumulates into the first (beta = 1)
    y2 = (op + op) @ x
    assert rel(y2, 2 * ref) < tol


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64, torch.bfloat16])
@pytest.mark.parametrize("k", [1, 3])
def test_reordered_sparse_products(dtype, k):
    """A Sparse stored in reverse Cuthill-McKee order (gather x through the permutation, write y
    through it) gives the original matrix's products, alone, in a Sum (accumulating into y) and batched
    through a Kronecker factor's column blocks."""
    from cola_gb300.workloads import rgg_laplacian
    n = 4096
    ip, ix, v = rgg_laplacian(n, 0.03, seed=11, device="cpu")
    A = cola.ops.Sparse.from_csr(ip.to(DEV), ix.to(DEV), v.to(DEV, dtype), (n, n))
    R = A.reordered()
    cdt = torch.float64 if dtype == torch.float64 else torch.float32
    X = torch.randn(n, k, device=DEV, dtype=cdt)
    ref = A @ X
    tol = 1e-12 if dtype == torch.float64 else 1e-6
    assert rel(R @ X, ref) < tol
    D = cola.ops.Diagonal(torch.linspace(1, 2, n, device=DEV, dtype=cdt))
    assert rel((R + D) @ X, ref + D @ X) < tol


def test_reordered_sparse_in_lanczos_and_cg():
    """Lanczos on Kronecker + reordered graph Laplacian gives the original operator's Ritz values, and
    CG on a reordered SPD matrix the original's solution (the fused single-operator path does not take
    permuted leaves: the generic loop runs)."""
    from cola_gb300.workloads import dense_spd, rgg_laplacian
    m = 64
    n = m * m
    ip, ix, v = rgg_laplacian(n, 0.05, seed=12, device="cpu")
    L = cola.ops.Sparse.from_csr(ip.to(DEV), ix.to(DEV), v.to(DEV, torch.float64), (n, n))
    A1, _, _ = dense_spd(m, seed=1, lo=1e-1, hi=1e1, dtype=torch.float64)
    K = cola.ops.Kronecker(cola.ops.Dense(A1.to(DEV)), cola.ops.Dense(A1.to(DEV)))
    start = torch.randn(n, dtype=torch.float64, generator=torch.Generator().manual_seed(3)).to(DEV)
    alg = Lanczos(start_vector=start, max_iters=60, tol=1e-12)
    v0, _ = cola.eig(cola.SelfAdjoint(K + L), 5, "LM", alg)
    v1, _ = cola.eig(cola.SelfAdjoint(K + L.reordered()), 5, "LM", alg)
    assert rel(v1, v0) < 1e-9  # each row's entries are summed in the new column order
    Lr = L.reordered()
    S = cola.PSD(Lr + cola.ops.I_like(Lr))
    b = torch.randn(n, dtype=torch.float64, device=DEV)
    x, info = cola.linalg.cg(S, b, tol=1e-10, max_iters=5000)
    Ad = L.to_dense() + torch.eye(n, device=DEV, dtype=torch.float64)
    assert float((b - Ad @ x).norm() / b.norm()) < 1e-9


def test_sparse_known_answer(golden):
    g = golden("ops_sparse_known")
    S = cola.ops.Sparse(T(g["data"]), T(g["rows"]), T(g["cols"]), (3, 4))
    y = S @ T(g["x"])
    np.testing.assert_allclose(y.cpu().numpy(), g["y"], rtol=1e-6)


def test_sparse_duplicates_and_unsorted():
    """Duplicate COO entries are summed and columns sorted, with values kept aligned."""
    data = T([1.0, 2.0, 3.0, 4.0, 5.0], torch.float32)
    rows = T([1, 0, 1, 0, 1])
    cols = T([2, 1, 0, 1, 2])
    S = cola.ops.Sparse(data, rows, cols, (2, 3))
    D = torch.zeros(2, 3)
    for d, r, c in zip([1.0, 2, 3, 4, 5], [1, 0, 1, 0, 1], [2, 1, 0, 1, 2]):
        D[r, c] += d
    X = torch.randn(3, 2)
    assert rel(S @ X.to(DEV), D @ X) < 1e-6


def test_composites_golden(golden):
    g = golden("ops_kron")
    K = cola.ops.Kronecker(cola.ops.Dense(T(g["A1"])), cola.ops.Dense(T(g["A2"])))
    assert rel(K @ T(g["X"]), g["Y"]) < 1e-12
    g = golden("ops_blockdiag")
    BD = cola.ops.BlockDiag(cola.ops.Dense(T(g["B1"])), cola.ops.Dense(T(g["B2"])), multiplicities=[2, 3])
    assert rel(BD @ T(g["X"]), g["Y"]) < 1e-12
    g = golden("ops_sum_product")
    D = cola.ops.Dense(T(g["D"]))
    S = D + cola.ops.Diagonal(T(g["d"])) + 0.5 * cola.ops.I_like(D)
    assert rel(S @ T(g["X"]), g["Ysum"]) < 1e-12
    P = D @ cola.ops.Dense(T(g["D"].T.copy()))
    assert rel(P @ T(g["X"]), g["Yprod"]) < 1e-12


def test_kron_three_factors_and_strided():
    rng = np.random.default_rng(3)
    Ms = [rng.standard_normal((s, s)) for s in (4, 3, 5)]
    K = cola.ops.Kronecker(*[cola.ops.Dense(T(M)) for M in Ms])
    X = rng.standard_normal((60, 7))
    ref = np.kron(np.kron(Ms[0], Ms[1]), Ms[2]) @ X
    assert rel(K @ T(X), ref) < 1e-12
    # non-contiguous X (leading dimension > k) goes through the executor's copy path
    Xw = T(rng.standard_normal((60, 9)))[:, :7]
    assert rel(K @ Xw, np.kron(np.kron(Ms[0], Ms[1]), Ms[2]) @ Xw.cpu().numpy()) < 1e-12
    # nested: Kronecker of a Sum and a Diagonal
    A = cola.ops.Dense(T(Ms[0])) + 2.0 * cola.ops.I_like(cola.ops.Dense(T(Ms[0])))
    d = rng.standard_normal(3)
    K2 = cola.ops.Kronecker(A, cola.ops.Diagonal(T(d)))
    X2 = rng.standard_normal((12, 4))
    assert rel(K2 @ T(X2), np.kron(Ms[0] + 2 * np.eye(4), np.diag(d)) @ X2) < 1e-12


# ---------------------------------------------------------------------------------------------
# CG

@pytest.mark.parametrize("fused", [True, False])
def test_cg_dense_f64_golden(golden, fused):
    g = golden("cg_dense_f64")
    op = cola.PSD(cola.ops.Dense(T(g["A"])))
    x, info = cola.linalg.inverse.cg(op, T(g["b"]), tol=float(g["tol"]), max_iters=int(g["max_iters"]),
                                     allow_fused=fused)
    assert info["fused"] == fused
    assert rel(x, g["x"]) < 1e-9
    assert abs(info["iterations"] - int(g["iterations"])) <= 0.03 * int(g["iterations"]) + 2
    np.testing.assert_allclose(info["errors"][:10], g["errors"][:10], rtol=1e-10)


@pytest.mark.parametrize("fused", [True, False])
def test_cg_dense_f32_golden(golden, fused):
    g = golden("cg_dense_f32")
    A = cola.PSD(cola.ops.Dense(T(g["A"])))
    Ainv = cola.inv(A, CG(tol=float(g["tol"]), max_iters=int(g["max_iters"])))
    x = Ainv @ T(g["b"]) if fused else cola.linalg.inverse.cg(A, T(g["b"]), tol=float(g["tol"]),
                                                              max_iters=int(g["max_iters"]), allow_fused=False)[0]
    # float32: iteration count within 5 % of the reference's, solution within 2e-3 of the reference's
    if fused:
        assert abs(Ainv.info["iterations"] - int(g["iterations"])) <= 0.05 * int(g["iterations"]) + 1
    assert rel(x, g["x"]) < 2e-3
    xs = np.linalg.solve(g["A"].astype(np.float64), g["b"].astype(np.float64))
    assert rel(x, xs) < 1.5 * rel(g["x"], xs) + 1e-4


@pytest.mark.parametrize("fused", [True, False])
def test_cg_multi_rhs_jacobi_x0(golden, fused):
    g = golden("cg_multi_jacobi_x0")
    P = cola.ops.Diagonal(T(g["dinv"]))
    x, info = cola.linalg.inverse.cg(cola.PSD(cola.ops.Dense(T(g["A"]))), T(g["B"]), x0=T(g["X0"]), P=P,
                                     tol=float(g["tol"]), max_iters=int(g["max_iters"]), allow_fused=fused)
    assert info["fused"] == fused
    assert abs(info["iterations"] - int(g["iterations"])) <= 1
    assert rel(x, g["x"]) < 1e-9


@pytest.mark.parametrize("tag", ["f32", "f64"])
@pytest.mark.parametrize("fused", [True, False])
def test_cg_sparse_golden(golden, tag, fused):
    g = golden(f"cg_sparse_{tag}")
    n = g["B"].shape[0]
    dt = torch.float32 if tag == "f32" else torch.float64
    op = cola.PSD(csr(g["rows"], g["cols"], g["vals"], n, dt))
    x, info = cola.linalg.inverse.cg(op, T(g["B"], dt), tol=float(g["tol"]), max_iters=int(g["max_iters"]),
                                     allow_fused=fused)
    assert info["fused"] == fused
    if tag == "f64":
        assert abs(info["iterations"] - int(g["iterations"])) <= 1
        assert rel(x, g["x"]) < 1e-9
    else:
        assert abs(info["iterations"] - int(g["iterations"])) <= 2
        assert rel(x, g["x"]) < 1e-4


def test_cg_repeated_eig(golden):
    g = golden("cg_repeated_eig")
    x, info = cola.linalg.inverse.cg(cola.PSD(cola.ops.Dense(T(g["A"]))), T(g["rhs"]), tol=1e-11, max_iters=100)
    assert info["iterations"] - 1 < 7
    assert rel(x, g["x"]) < 1e-4


def test_cg_general_preconditioner_and_shift():
    """Generic path: Sum(Sparse, c I) operator with a Product preconditioner, against the oracle."""
    from cola_gb300.workloads import grid_pattern_2d, diffusion_values_2d
    m = 12
    ip, ix, ok = grid_pattern_2d(m, DEV)
    a = torch.exp(torch.randn(1, m, m, device=DEV, dtype=torch.float64))
    v = diffusion_values_2d(a, ok)[0].double()
    n = m * m
    S = cola.ops.Sparse.from_csr(ip, ix, v, (n, n))
    Aop = cola.PSD(S + 0.3 * cola.ops.I_like(S))
    dg = torch.zeros(n, dtype=torch.float64, device=DEV)
    rows = torch.repeat_interleave(torch.arange(n, device=DEV), (ip[1:] - ip[:-1]).long())
    dg.index_add_(0, rows, torch.where(rows == ix.long(), v, torch.zeros_like(v)))
    dinv = 1.0 / (dg + 0.3)
    P = cola.ops.Diagonal(dinv.sqrt()) @ cola.ops.Diagonal(dinv.sqrt())
    B = torch.randn(n, 2, device=DEV, dtype=torch.float64)
    x, info = cola.linalg.inverse.cg(Aop, B, P=P, tol=1e-10, max_iters=400)
    assert not info["fused"]
    Ad = torch.zeros(n, n, dtype=torch.float64, device=DEV)
    Ad[rows, ix.long()] = v
    Ad += 0.3 * torch.eye(n, device=DEV, dtype=torch.float64)
    xo, ko, info_o = oracle.cg_solve(oracle.dense_op(Ad.cpu().numpy()), B.cpu().numpy(),
                                     precond=lambda r: dinv.cpu().numpy()[:, None] * r, tol=1e-10, max_iters=400)
    assert rel(x, xo) < 1e-8
    assert abs(info["iterations"] - info_o["iterations"]) <= 1
    # the fused kernel on the same shifted operator with Jacobi agrees
    x2, info2 = cola.linalg.inverse.cg(Aop, B, P=cola.ops.Diagonal(dinv), tol=1e-10, max_iters=400)
    assert info2["fused"] and rel(x2, xo) < 1e-8


@pytest.mark.parametrize("tag", ["f32", "f64"])
def test_nystrom_preconditioner_matches_reference(golden, tag):
    """NystromPrecond on the device operator path against the reference's own NystromPrecond (its
    test matrices, rank 5): Lambda, the dense P (mu = 0 and the defaults), sqrt and inverse, and CG
    with P (run_batched_cg, tol 1e-8)."""
    from cola_gb300.linalg import NystromPrecond, sqrt
    from cola_gb300.linalg.preconditioning import inverse
    g = golden(f"nystrom_{tag}")
    f64 = tag == "f64"
    tol = 1e-9 if f64 else 2e-5
    A = cola.ops.Dense(T(g["A"]))
    P = NystromPrecond(A, rank=int(g["rank"]), mu=0, eps=float(g["eps"]))
    assert rel(P.Lambda, g["Lambda"]) < tol
    assert rel(P.to_dense(), g["P"]) < tol
    assert rel(NystromPrecond(A, rank=int(g["rank"])).to_dense(), g["P_default"]) < tol
    assert rel(sqrt(P).to_dense(), g["P_sqrt"]) < tol
    assert rel(inverse(P).to_dense(), g["P_inv"]) < tol
    assert abs(float(P.preconditioned_eigmax) - float(g["eigmax"])) < tol
    x, info = cola.linalg.inverse.cg(A, T(g["rhs"]), P=P, tol=1e-8, max_iters=100)
    assert not info["fused"]
    assert rel(x, g["x"]) < (1e-9 if f64 else 1e-5)
    assert abs(int(info["iterations"]) - int(g["k"])) <= (1 if f64 else 3)


def test_cg_edge_cases():
    A = cola.PSD(cola.ops.Dense(torch.tensor([[2.0]], device=DEV)))
    x, info = cola.linalg.inverse.cg(A, torch.tensor([4.0], device=DEV), tol=1e-8)
    assert abs(x.item() - 2.0) < 1e-6
    # max_iters = 0 returns x0 scaled back, zero steps
    B = torch.ones(3, device=DEV)
    A3 = cola.PSD(cola.ops.Diagonal(torch.tensor([1.0, 2.0, 4.0], device=DEV)))
    x, info = cola.linalg.inverse.cg(A3, B, tol=1e-8, max_iters=0)
    assert info["iterations"] == 1 and torch.all(x == 0)
    # a zero right-hand side stays zero (safe division)
    x, info = cola.linalg.inverse.cg(A3, torch.zeros(3, device=DEV), tol=1e-8, max_iters=10)
    assert torch.all(x == 0)
    with pytest.raises(AssertionError):
        cola.inv(cola.ops.Dense(torch.eye(3, device=DEV)), CG())


# ---------------------------------------------------------------------------------------------
# Lanczos, eig, SLQ

def test_lanczos_batched_golden(golden):
    g = golden("lanczos_batched")
    Q, Tm, info = cola.linalg.lanczos(cola.ops.Dense(T(g["A"])), T(g["V0"]), max_iters=int(g["max_iters"]),
                                      tol=float(g["tol"]))
    assert info["iterations"] == int(g["iterations"])
    assert rel(Tm.beta[:, :, 0], g["beta"]) < 1e-10
    assert rel(Tm.alpha[:, :, 0], g["alpha"]) < 1e-10
    assert rel(Q.A, g["Q"]) < 1e-9


@pytest.mark.parametrize("case", ["early", "three", "two"])
def test_lanczos_known_answers(golden, case):
    g = golden(f"lanczos_case_{case}")
    Q, Tm, info = cola.linalg.lanczos(cola.ops.Dense(T(g["A"], torch.float32)), T(g["rhs"], torch.float32),
                                      max_iters=3, tol=1e-7)
    assert info["iterations"] - 1 == int(g["iterations"]) - 1
    np.testing.assert_allclose(Tm.beta[:, :, 0].cpu().numpy(), g["beta"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(Tm.alpha[:, :, 0].cpu().numpy(), g["alpha"], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("m", [120, 450])
def test_lanczos_fp32_long_run_orthogonality(m):
    """Single-vector FP32 Lanczos over hundreds of steps (the 128-bit warp-per-slot projection and the
    float4 subtraction of every CGS2 pass): the basis stays orthonormal to FP32 accuracy and the five
    isolated top Ritz values equal the FP64 run's."""
    from cola_gb300.workloads import diffusion_family_2d
    fam, _, _, _ = diffusion_family_2d([3], m=128, device=DEV)
    n = fam.n
    ip, ix, v = fam.indptr, fam.indices, fam.values[0]
    start = torch.randn(n, 1, generator=torch.Generator().manual_seed(1), dtype=torch.float64)
    from cola_gb300.linalg.lanczos import run_lanczos
    Qs, ev = {}, {}
    spikes = torch.zeros(n, dtype=torch.float64)
    spikes[torch.randperm(n, generator=torch.Generator().manual_seed(2))[:5]] = torch.tensor(
        [300., 250, 200, 150, 100], dtype=torch.float64)
    for dt in (torch.float32, torch.float64):
        A = cola.ops.Sparse.from_csr(ip, ix, v.to(dt), (n, n)) + cola.ops.Diagonal(spikes.to(DEV, dt))
        r = run_lanczos(A, start.to(DEV, dt), m, 1e-12)
        alpha, beta, Q = r.alpha_beta_q()  # alpha (1, k-1), beta (1, k), Q (k, n, 1)
        Qs[dt] = Q[:, :, 0].double()
        T = np.diag(beta[0].double().cpu().numpy())
        if alpha.shape[1] > 0:
            off = alpha[0].double().cpu().numpy()
            T += np.diag(off, 1) + np.diag(off, -1)
        ev[dt] = np.sort(np.linalg.eigvalsh(T))[-5:]
    Q32 = Qs[torch.float32]
    G = Q32 @ Q32.T
    assert float((G - torch.eye(G.shape[0], device=DEV, dtype=torch.float64)).abs().max()) < 1e-4
    assert np.max(np.abs(ev[torch.float32] - ev[torch.float64]) / np.abs(ev[torch.float64])) < 1e-5


def test_eig_lanczos_golden(golden):
    g = golden("eig_lanczos")
    op = cola.SelfAdjoint(cola.ops.Dense(T(g["A"])))
    vals, vecs = cola.eig(op, 5, "LM", Lanczos(max_iters=40, tol=1e-10))
    # eigenvalues within 1e-5 relative of the reference's (here far tighter: FP64 throughout)
    assert rel(vals, g["evals"]) < 1e-9
    V = vecs.cpu().numpy()
    s = np.sign(np.sum(V * g["evecs"], axis=0))
    assert rel(V * s, g["evecs"]) < 1e-7


def test_lanczos_unary_golden(golden):
    g = golden("lanczos_unary_log")
    F = cola.linalg.LanczosUnary(cola.PSD(cola.ops.Dense(T(g["A"]))), torch.log, max_iters=int(g["max_iters"]),
                                 tol=float(g["tol"]))
    Y = F @ T(g["Z"])
    assert rel(Y, g["Y"]) < 1e-8


def test_logdet_slq_dense_golden(golden):
    g = golden("logdet_slq_dense")
    op = cola.PSD(cola.ops.Dense(T(g["A"])))
    ld = cola.logdet(op, Lanczos(max_iters=int(g["max_iters"]), tol=float(g["tol"])),
                     Hutch(max_iters=int(g["hutch_iters"]), key=PRNGKey(42)))
    # identical probes: agreement far inside the SLQ standard error
    assert abs(float(ld) - float(g["logdet"])) < 1e-7


def test_logdet_kron_slq_golden(golden):
    g = golden("logdet_kron_slq")
    K = cola.ops.Kronecker(*[cola.ops.Dense(T(g[k])) for k in ("K1", "K2", "K3")])
    op = cola.PSD(K + 0.01 * cola.ops.I_like(K))
    ld = cola.logdet(op, Lanczos(max_iters=40, tol=1e-10), Hutch(max_iters=3, rand="rademacher", key=PRNGKey(7)))
    assert abs(float(ld) - float(g["logdet"])) < 1e-6


@pytest.mark.parametrize("name", ["sqrt", "exp", "pow"])
def test_unary_family_against_eigh(name):
    """f(A) v by Lanczos quadrature (full Krylov space: exact up to rounding) vs a dense FP64 eigh."""
    rng = np.random.default_rng(7)
    Q, _ = np.linalg.qr(rng.standard_normal((40, 40)))
    lam = np.exp(rng.uniform(np.log(0.2), np.log(3.0), 40))
    A = (Q * lam) @ Q.T
    op = cola.PSD(cola.ops.Dense(T(A)))
    f = {"sqrt": (lambda: cola.linalg.sqrt(op, Lanczos(max_iters=40, tol=1e-13)), np.sqrt),
         "exp": (lambda: cola.linalg.exp(op, Lanczos(max_iters=40, tol=1e-13)), np.exp),
         "pow": (lambda: cola.linalg.pow(op, 0.3, Lanczos(max_iters=40, tol=1e-13)), lambda x: x ** 0.3)}[name]
    F = f[0]()
    V = rng.standard_normal((40, 3))
    ref = (Q * f[1](lam)) @ Q.T @ V
    assert rel(F @ T(V), ref) < 1e-8


def test_slq_tbd_golden(golden):
    g = golden("slq_tbd")
    est = cola.linalg.stochastic_lanczos_quad(cola.ops.Dense(T(g["A"])), torch.log, max_iters=30, tol=1e-7,
                                              probes=T(g["probes"]))
    assert abs(float(est) - float(g["estimate"])) < 1e-8


@pytest.mark.parametrize("m", [1, 2, 3, 31, 32, 33, 100, 257])
def test_tridiag_eigh(m):
    rng = np.random.default_rng(m)
    bsz = 4
    a = rng.standard_normal((bsz, m))
    b = rng.standard_normal((bsz, max(m - 1, 0)))
    ev, P, status = cola.linalg.tridiag_eigh(T(a), T(b), want_vectors=True)
    ev2, first, _ = cola.linalg.tridiag_eigh(T(a), T(b), want_vectors=False)
    assert int(status.sum()) == 0
    for i in range(bsz):
        Tm = np.diag(a[i]) + (np.diag(b[i], -1) + np.diag(b[i], 1) if m > 1 else 0)
        w, V = np.linalg.eigh(Tm)
        np.testing.assert_allclose(ev[i].cpu().numpy(), w, rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(ev2[i].cpu().numpy(), w, rtol=1e-10, atol=1e-12)
        Pm = P[i].cpu().numpy()
        np.testing.assert_allclose(Tm @ Pm, Pm * w[None, :], atol=1e-9)
        np.testing.assert_allclose(np.abs(first[i].cpu().numpy()), np.abs(V[0]), atol=1e-9)


@pytest.mark.parametrize("m", [1, 2, 33, 100, 256])
def test_tridiag_eigh_fp32(m):
    """FP32 tridiagonals (from FP32 recurrences) are solved in FP32, as the reference's eigh of the FP32
    T: eigenvalues within a few FP32 ulps of the norm, eigenvectors orthonormal and satisfying
    T P = P diag(w) to FP32 accuracy."""
    rng = np.random.default_rng(100 + m)
    bsz = 3
    a = rng.standard_normal((bsz, m)).astype(np.float32)
    b = rng.standard_normal((bsz, max(m - 1, 0))).astype(np.float32)
    ev, P, status = cola.linalg.tridiag_eigh(T(a, torch.float32), T(b, torch.float32), want_vectors=True)
    ev2, first, _ = cola.linalg.tridiag_eigh(T(a, torch.float32), T(b, torch.float32), want_vectors=False)
    assert ev.dtype == torch.float32 and P.dtype == torch.float32
    assert int(status.sum()) == 0
    for i in range(bsz):
        Tm = np.diag(a[i].astype(np.float64))
        if m > 1:
            Tm += np.diag(b[i].astype(np.float64), -1) + np.diag(b[i].astype(np.float64), 1)
        w, V = np.linalg.eigh(Tm)
        nrm = max(np.abs(w).max(), 1e-30)
        assert np.abs(ev[i].cpu().numpy() - w).max() <= 64 * 1.2e-7 * nrm
        assert np.abs(ev2[i].cpu().numpy() - w).max() <= 64 * 1.2e-7 * nrm
        Pm = P[i].cpu().double().numpy()
        # orthogonality and residual to O(m eps) of FP32, as for any backward-stable QL
        assert np.abs(Pm.T @ Pm - np.eye(m)).max() < 8 * m * 1.2e-7 + 1e-6
        assert np.abs(Tm @ Pm - Pm * w[None, :]).max() < (8 * m * 1.2e-7 + 1e-6) * nrm


@pytest.mark.parametrize("dtype,scale", [(torch.float32, 1e25), (torch.float32, 1e-25), (torch.float64, 1e200),
                                         (torch.float64, 1e-200)])
def test_tridiag_eigh_scaled(dtype, scale):
    """Entries far from 1 (whose squares would overflow or underflow) give the scaled eigenvalues: each
    matrix is scaled by a power of two before the sweeps."""
    rng = np.random.default_rng(7)
    a = rng.standard_normal((2, 40))
    b = rng.standard_normal((2, 39))
    ev, _, st = cola.linalg.tridiag_eigh(T(a * scale, dtype), T(b * scale, dtype), want_vectors=False)
    ev1, _, _ = cola.linalg.tridiag_eigh(T(a, dtype), T(b, dtype), want_vectors=False)
    assert int(st.sum()) == 0
    got = ev.double().cpu().numpy() / scale
    ref = ev1.double().cpu().numpy()
    tol = 1e-5 if dtype == torch.float32 else 1e-12
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()


# ---------------------------------------------------------------------------------------------
# batched systems on a shared pattern, FP64 iterative refinement

@pytest.mark.parametrize("schedule", ["grid", "cluster8", "cluster16", "onchip"])
@pytest.mark.parametrize("precond", ["none", "jacobi"])
def test_batched_ir_small_family(precond, schedule):
    from cola_gb300.workloads import diffusion_family_2d
    fam, B, _, _ = diffusion_family_2d(range(7), m=24, device=DEV)
    B[3].zero_()  # a zero right-hand side converges at once with x = 0
    X, info = cola.linalg.solve_batched(fam, B, precond=precond, tol=1e-8, schedule=schedule)
    assert torch.all(info["status"] == 1), info["status"]
    assert float(info["relres"].max()) <= 1e-8
    R = B - fam.matvec(X)
    rr = R.norm(dim=1) / B.norm(dim=1).clamp_min(1e-300)
    rr[3] = 0
    assert float(rr.max()) <= 1.01e-8
    assert torch.all(X[3] == 0)
    n = fam.n
    for s in (0, 6):
        A = torch.sparse_csr_tensor(fam.indptr.long(), fam.indices.long(), fam.values[s].double(), (n, n)).to_dense()
        xs = torch.linalg.solve(A, B[s])
        assert rel(X[s], xs) < 1e-6


@pytest.mark.parametrize("mode", ["reliable", "restart"])
def test_batched_modes_converge_and_agree(mode):
    from cola_gb300.workloads import diffusion_family_2d
    fam, B, _, _ = diffusion_family_2d(range(20, 25), m=32, device=DEV)
    X, info = cola.linalg.solve_batched(fam, B, precond="jacobi", tol=1e-8, mode=mode)
    assert torch.all(info["status"] == 1) and float(info["relres"].max()) <= 1e-8
    R = B - fam.matvec(X)
    assert float((R.norm(dim=1) / B.norm(dim=1)).max()) <= 1.01e-8
    # reliable updates keep the Krylov recurrence: close to the step count of an FP64 Jacobi-CG
    n = fam.n
    A = torch.sparse_csr_tensor(fam.indptr.long(), fam.indices.long(), fam.values[0].double(), (n, n)).to_dense()
    A64 = A.cpu().numpy()
    dinv = 1.0 / np.diag(A64)
    xo, ko, info_o = oracle.cg_solve(oracle.dense_op(A64), B[0].cpu().numpy(), precond=lambda r: dinv * r, tol=5e-9,
                                     max_iters=5000)
    if mode == "reliable":
        assert int(info["iterations"][0]) <= 1.15 * ko + 5, (int(info["iterations"][0]), ko)


def test_batched_fsai_fallback_and_edge_inputs():
    from cola_gb300.linalg.batched import FsaiPattern
    from cola_gb300.workloads import diffusion_family_2d
    fam, B, _, _ = diffusion_family_2d(range(30, 33), m=16, device=DEV)
    pat = FsaiPattern(fam.indptr, fam.indices)
    # a deliberately poor G (identity on the pattern's diagonal only): still SPD, judged by FP64 residuals
    gv = torch.zeros((3, pat.g_nnz), device=DEV)
    rows = torch.repeat_interleave(torch.arange(fam.n, device=DEV), (pat.g_indptr[1:] - pat.g_indptr[:-1]).long())
    gv[:, rows == pat.g_indices.long()] = 1.0
    X, info = cola.linalg.solve_batched(fam, B, precond="fsai", fsai=(pat, gv), tol=1e-8)
    assert torch.all((info["status"] == 1) | (info["status"] == 5))
    assert float(info["relres"].max()) <= 1e-8
    with pytest.raises(ValueError):
        cola.linalg.solve_batched(fam, B[:, :-1], precond="jacobi")
    with pytest.raises(ValueError):
        cola.linalg.solve_batched(fam, B, precond="fsai")


def test_batched_shared_values_many_rhs():
    """One 3-D 7-point operator, many right-hand sides as independent systems (values stored once)."""
    from cola_gb300.linalg.batched import BatchedCSR
    from cola_gb300.workloads import diffusion_3d
    ip, ix, v = diffusion_3d(m=12, device=DEV)
    fam = BatchedCSR(ip, ix, v[None, :], shared=True)
    B = torch.randn(6, fam.n, device=DEV, dtype=torch.float64)
    X, info = cola.linalg.solve_batched(fam, B, precond="jacobi", tol=1e-8)
    assert torch.all(info["status"] == 1)
    R = B - fam.matvec(X)
    assert float((R.norm(dim=1) / B.norm(dim=1)).max()) <= 1.01e-8


def _closed_form_fsai(fam):
    from cola_gb300.precond.learned_fsai import g_values
    return g_values(fam, None)


@pytest.mark.parametrize("m,S", [(32, 5), (30, 3), (256, 2)])
@pytest.mark.parametrize("precond", ["none", "jacobi", "fsai"])
def test_onchip_schedule_matches_cluster_schedule(precond, m, S):
    """On-chip vectors + diagonal storage against the CSR cluster schedule: same algorithm, same stop
    rule; both reach the FP64 tolerance and take about the same number of CG steps (their reductions
    sum in different orders, and over ~1000 FP32 steps that moves the count by up to ~10%)."""
    from cola_gb300.workloads import diffusion_family_2d
    fam, B, _, _ = diffusion_family_2d(range(40, 40 + S), m=m, device=DEV)
    kw = dict(precond=precond, tol=1e-8, fsai=_closed_form_fsai(fam) if precond == "fsai" else None)
    X1, i1 = cola.linalg.solve_batched(fam, B, schedule="onchip", **kw)
    X2, i2 = cola.linalg.solve_batched(fam, B, schedule="cluster8", **kw)
    assert torch.all(i1["status"] == 1) and torch.all(i2["status"] == 1), (i1["status"], i2["status"])
    R = B - fam.matvec(X1)
    assert float((R.norm(dim=1) / B.norm(dim=1)).max()) <= 1.01e-8
    assert float(i1["relres"].max()) <= 1e-8
    k1, k2 = i1["iterations"].double(), i2["iterations"].double()
    assert float(((k1 - k2).abs() - (0.15 * k2 + 3)).max()) <= 0, (k1.tolist(), k2.tolist())
    assert rel(X1, X2) < 1e-6


@pytest.mark.parametrize("schedule", ["onchip", "cluster8", "grid"])
def test_batched_no_wait_gives_the_same_solutions(schedule):
    """wait=False returns once the solve is enqueued; in stream order the outputs are those of the
    waiting call (same kernel, same inputs: bit-identical where the reductions have a fixed order),
    and the replacement count is None
    (on-chip, cluster) or still reported (grid, which always waits)."""
    from cola_gb300.workloads import diffusion_family_2d
    fam, B, _, _ = diffusion_family_2d(range(60, 63), m=32, device=DEV)
    X1, i1 = cola.linalg.solve_batched(fam, B, precond="jacobi", schedule=schedule)
    X2, i2 = cola.linalg.solve_batched(fam, B, precond="jacobi", schedule=schedule, wait=False)
    torch.cuda.synchronize()
    if schedule == "grid":  # its block sums meet in FP64 atomics: the order, and the last bits, vary
        assert rel(X1, X2) < 1e-6
    else:
        assert torch.equal(X1, X2) and torch.equal(i1["iterations"], i2["iterations"])
    assert i1["sweeps"] is not None and i1["sweeps"] >= 1
    assert (i2["sweeps"] is None) == (schedule != "grid")


def test_onchip_three_d_shared_values_and_unsupported_patterns():
    from cola_gb300.linalg.batched import BatchedCSR
    from cola_gb300.workloads import diffusion_3d, rgg_laplacian
    ip, ix, v = diffusion_3d(m=12, device=DEV)  # 7 diagonals, offsets up to 144
    fam = BatchedCSR(ip, ix, v[None, :], shared=True)
    B = torch.randn(5, fam.n, device=DEV, dtype=torch.float64, generator=torch.Generator(DEV).manual_seed(3))
    X, info = cola.linalg.solve_batched(fam, B, precond="jacobi", tol=1e-8, schedule="onchip")
    assert torch.all(info["status"] == 1)
    R = B - fam.matvec(X)
    assert float((R.norm(dim=1) / B.norm(dim=1)).max()) <= 1.01e-8
    # an unstructured pattern (random geometric graph Laplacian + I): not diagonal-structured
    ip, ix, v = rgg_laplacian(400, 0.12, seed=1, device=DEV)
    rows = torch.repeat_interleave(torch.arange(400, device=DEV), (ip[1:] - ip[:-1]).long())
    v = v + 0.5 * (rows == ix.long()).float()
    fam = BatchedCSR(ip, ix, torch.stack([v, 2 * v]))
    B = torch.randn(2, 400, device=DEV, dtype=torch.float64)
    with pytest.raises(NotImplementedError):
        cola.linalg.solve_batched(fam, B, precond="jacobi", tol=1e-8, schedule="onchip")
    X, info = cola.linalg.solve_batched(fam, B, precond="jacobi", tol=1e-8)  # auto: cluster schedule
    assert torch.all(info["status"] == 1)
    R = B - fam.matvec(X)
    assert float((R.norm(dim=1) / B.norm(dim=1)).max()) <= 1.01e-8


@pytest.mark.parametrize("precond", ["none", "jacobi"])
def test_onchip_halo_as_long_as_a_strip(precond):
    """3-D 7-point operator on 32^3 cells: the halo (m^2 = 1024 rows) is exactly one strip of a CTA
    (R = 4096 rows in strips of 1024), the longest halo the on-chip strip layout takes.  Same
    solutions as the CSR cluster schedule."""
    from cola_gb300.linalg.batched import BatchedCSR, onchip_schedule_info
    from cola_gb300.workloads import diffusion_3d
    ip, ix, v = diffusion_3d(m=32, device=DEV)
    fam = BatchedCSR(ip, ix, v[None, :], shared=True)
    geo = onchip_schedule_info(fam.n, 32 * 32)
    assert geo["cluster_size"] == 8 and geo["rows_per_cta"] == 4096 and geo["clusters_in_flight"] > 0
    B = torch.randn(3, fam.n, device=DEV, dtype=torch.float64, generator=torch.Generator(DEV).manual_seed(9))
    X1, i1 = cola.linalg.solve_batched(fam, B, precond=precond, tol=1e-8, schedule="onchip")
    X2, i2 = cola.linalg.solve_batched(fam, B, precond=precond, tol=1e-8, schedule="cluster8")
    assert i1["schedule"] == "onchip"
    assert torch.all(i1["status"] == 1) and torch.all(i2["status"] == 1)
    R = B - fam.matvec(X1)
    assert float((R.norm(dim=1) / B.norm(dim=1)).max()) <= 1.01e-8
    assert rel(X1, X2) < 1e-6
    k1, k2 = i1["iterations"].double(), i2["iterations"].double()
    assert float(((k1 - k2).abs() - (0.15 * k2 + 3)).max()) <= 0, (k1.tolist(), k2.tolist())


def test_dense_batched_uneven_matches_per_system_reference_loop():
    """Uneven dense systems in one launch; each equals a separate reference CG call (oracle, float32)."""
    from cola_gb300.linalg.batched import solve_dense_batched
    rng = np.random.default_rng(5)
    mats, rhs, np_mats = [], [], []
    for n in (37, 64, 129, 250, 5, 1):
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        lam = np.exp(rng.uniform(np.log(0.1), np.log(10.0), n))
        A = ((Q * lam) @ Q.T).astype(np.float32)
        b = rng.standard_normal(n).astype(np.float32)
        np_mats.append((A, b))
        mats.append(T(A))
        rhs.append(T(b))
    sols, iters, status = solve_dense_batched(mats, rhs, tol=1e-6, max_iters=500)
    for (A, b), x, k in zip(np_mats, sols, iters.tolist()):
        xo, ko, info = oracle.cg_solve(oracle.dense_op(A), b, tol=1e-6, max_iters=500)
        assert abs(k - ko) <= 0.05 * ko + 2, (k, ko)
        xs = np.linalg.solve(A.astype(np.float64), b.astype(np.float64))
        assert rel(x, xs) < 1e-4
    assert torch.all(status == 1)


def test_dense_batched_quad_loads_every_row_alignment():
    """Sizes whose rows start at every offset within a 16-byte quad and are long enough for the
    unrolled 128-bit loop (n >= 512), next to tiny ones; each system against the oracle's CG and an
    FP64 solve."""
    from cola_gb300.linalg.batched import solve_dense_batched
    rng = np.random.default_rng(11)
    mats, rhs, np_mats = [], [], []
    for n in (515, 3, 1026, 2051, 7, 1, 2):
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        lam = np.exp(rng.uniform(np.log(0.5), np.log(5.0), n))
        A = ((Q * lam) @ Q.T).astype(np.float32)
        b = rng.standard_normal(n).astype(np.float32)
        np_mats.append((A, b))
        mats.append(T(A))
        rhs.append(T(b))
    sols, iters, status = solve_dense_batched(mats, rhs, tol=1e-6, max_iters=400)
    for (A, b), x, k in zip(np_mats, sols, iters.tolist()):
        xo, ko, info = oracle.cg_solve(oracle.dense_op(A), b, tol=1e-6, max_iters=400)
        assert abs(k - ko) <= 0.05 * ko + 2, (A.shape[0], k, ko)
        xs = np.linalg.solve(A.astype(np.float64), b.astype(np.float64))
        assert rel(x, xs) < 1e-4, A.shape[0]
    assert torch.all(status == 1)


def test_batched_ir_matches_oracle_iteration_structure():
    """The device restarted-refinement loop and the oracle's restatement need comparable inner iterations."""
    from cola_gb300.workloads import diffusion_family_2d
    fam, B, _, _ = diffusion_family_2d([11], m=20, device=DEV)
    X, info = cola.linalg.solve_batched(fam, B, precond="none", tol=1e-8, inner_tol=1e-4, mode="restart")
    n = fam.n
    A = torch.sparse_csr_tensor(fam.indptr.long(), fam.indices.long(), fam.values[0].double(), (n, n)).to_dense()
    A64 = A.cpu().numpy()
    A32 = A64.astype(np.float32)
    x, total, sweeps, rr = oracle.cg.ir_solve(lambda v: A64 @ v, lambda v: A32 @ v, B[0].cpu().numpy(), tol=1e-8,
                                              inner_tol=1e-4)
    assert rr <= 1e-8
    assert abs(int(info["iterations"][0]) - total) <= 0.15 * total + 5
    assert rel(X[0], x) < 1e-6


# ---------------------------------------------------------------------------------------------
# non-symmetric operators: Arnoldi and GMRES against the reference's golden outputs

def test_arnoldi_matches_reference(golden):
    from cola_gb300.linalg.arnoldi import arnoldi
    g = golden("arnoldi_dense")
    A = T(g["A"])
    Q, H, info = arnoldi(O.Dense(A), start_vector=T(g["v0"]), max_iters=int(g["max_iters"]), tol=float(g["tol"]))
    Qd, Hd = Q.to_dense().cpu().numpy(), H.to_dense().cpu().numpy()
    assert info["iterations"] == int(g["iterations"])
    # the reference's single modified Gram-Schmidt pass keeps its basis orthogonal to ~1e-6 here;
    # two classical passes keep it to ~1e-15, so the late entries agree to the reference's accuracy
    np.testing.assert_allclose(Hd[:, :3], g["H"][:, :3], rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(Hd, g["H"], rtol=0, atol=1e-5)
    np.testing.assert_allclose(Qd, g["Q"], rtol=0, atol=1e-5)
    np.testing.assert_allclose(g["A"] @ Qd[:, :-1], Qd @ Hd, rtol=0, atol=1e-10)
    assert np.abs(Qd.T @ Qd - np.eye(Qd.shape[1])).max() < 1e-12


@pytest.mark.parametrize("tag", ["full", "short"])
def test_gmres_matches_reference(golden, tag):
    from cola_gb300.linalg.arnoldi import gmres
    g = golden(f"gmres_dense_{tag}")
    x, info = gmres(O.Dense(T(g["A"])), T(g["b"]), max_iters=int(g["max_iters"]), tol=float(g["tol"]))
    assert rel(x, g["x"]) < 1e-8
    assert info["iterations"] == int(g["iterations"]) or tag == "full"


def test_gmres_multi_rhs_f32_and_dispatch(golden):
    g = golden("gmres_dense_multi_f32")
    op = O.Dense(T(g["A"]))
    X = cola.linalg.inv(op, cola.linalg.GMRES(max_iters=int(g["max_iters"]), tol=float(g["tol"]))) @ T(g["B"])
    assert rel(X, g["x"]) < 1e-4
    # Auto on a large operator without the PSD annotation dispatches to GMRES (inv.py:72-95)
    n = 4096
    main = torch.full((n,), 4.0, device=DEV)
    up = torch.full((n - 1,), -1.5, device=DEV)
    lo = torch.full((n - 1,), -0.5, device=DEV)
    rows = torch.cat([torch.arange(n), torch.arange(n - 1), torch.arange(1, n)]).to(DEV)
    cols = torch.cat([torch.arange(n), torch.arange(1, n), torch.arange(n - 1)]).to(DEV)
    S = O.Sparse(torch.cat([main, up, lo]), rows, cols, (n, n))
    b = torch.randn(n, device=DEV)
    x = cola.linalg.inv(S, cola.linalg.Auto(max_iters=60, tol=1e-7)) @ b
    r = b - S @ x
    assert float(r.norm() / b.norm()) < 1e-5


def test_onchip_limits_restart_nan_and_geometry():
    from cola_gb300.linalg.batched import onchip_schedule_info
    from cola_gb300.workloads import diffusion_family_2d
    fam, B, _, _ = diffusion_family_2d(range(60, 63), m=32, device=DEV)
    # restart mode (classic refinement) on the on-chip schedule
    X, info = cola.linalg.solve_batched(fam, B, precond="jacobi", tol=1e-8, mode="restart", schedule="onchip")
    assert info["schedule"] == "onchip" and torch.all(info["status"] == 1)
    R = B - fam.matvec(X)
    assert float((R.norm(dim=1) / B.norm(dim=1)).max()) <= 1.01e-8
    # the step cap: MAX_ITERS (2) with the FP64-refined iterate returned
    X2, i2 = cola.linalg.solve_batched(fam, B, precond="none", tol=1e-12, max_inner_iters=20, schedule="onchip")
    assert torch.all(i2["status"] == 2) and torch.all(i2["iterations"] == 20) and bool(torch.isfinite(X2).all())
    assert float(i2["relres"].max()) < 1.0
    # a NaN right-hand side is reported for that system only
    B3 = B.clone()
    B3[1, 5] = float("nan")
    X3, i3 = cola.linalg.solve_batched(fam, B3, precond="jacobi", tol=1e-8, schedule="onchip")
    assert i3["status"].tolist() == [1, 4, 1]
    assert rel(X3[0], X[0]) < 1e-6 and rel(X3[2], X[2]) < 1e-6
    # geometry of the schedule for the 512 x 512 family
    g = onchip_schedule_info(512 * 512, 512)
    assert g["cluster_size"] == 16 and g["rows_per_cta"] == 16384 and g["clusters_in_flight"] >= 1
    assert onchip_schedule_info(2 ** 22, 4)["cluster_size"] == 0  # too large to hold on chip
