"""Generate the golden vectors under tests/golden/ by running the reference CoLA itself.

Run in a container that holds the reference source (it is not needed anywhere else):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py <path of the reference source tree>

The reference needs `plum` and `optree`, which this image lacks; the test-only stand-ins in
tests/golden/_shims provide the API surface CoLA uses.  Every case stores its inputs and the
reference's outputs in one .npz file; tests compare the oracle and the CUDA path against them.
"""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
if len(sys.argv) < 2 or not (Path(sys.argv[1]) / "cola").is_dir():
    sys.exit("usage: make_golden.py <path of the reference source tree (the directory holding cola/)>")
REF = Path(sys.argv[1])
sys.path[:0] = [str(HERE / "_shims"), str(REF)]

import torch  # noqa: E402

torch.set_num_threads(4)
import cola  # noqa: E402
from cola.linalg.decompositions.lanczos import lanczos  # noqa: E402
from cola.linalg.inverse.cg import run_batched_cg  # noqa: E402
from cola.linalg.unary.unary import LanczosUnary  # noqa: E402
from cola.backends import torch_fns  # noqa: E402


def save(name, **arrays):
    out = {k: (v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(v)) for k, v in arrays.items()}
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(f"wrote {name}.npz ({', '.join(out)})")


def spd_from_spectrum(n, lo, hi, seed, dtype):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    lam = np.exp(rng.uniform(np.log(lo), np.log(hi), n))
    return ((Q * lam) @ Q.T).astype(dtype), lam


def diffusion_2d(m, seed, dtype):
    """5-point finite-volume variable-coefficient diffusion on an m x m grid (Dirichlet), CSR."""
    rng = np.random.default_rng(seed)
    a = np.exp(rng.standard_normal((m, m)))
    rows, cols, vals = [], [], []
    idx = lambda i, j: i * m + j  # noqa: E731
    for i in range(m):
        for j in range(m):
            d = 0.0
            for di, dj in ((-1, 0), (1, 0), (0, -1), (0, 1)):
                ii, jj = i + di, j + dj
                if 0 <= ii < m and 0 <= jj < m:
                    t = 2 * a[i, j] * a[ii, jj] / (a[i, j] + a[ii, jj])
                    rows.append(idx(i, j)); cols.append(idx(ii, jj)); vals.append(-t)
                else:
                    t = 2 * a[i, j]
                d += t
            rows.append(idx(i, j)); cols.append(idx(i, j)); vals.append(d)
    rows, cols, vals = np.array(rows), np.array(cols), np.array(vals, dtype=dtype)
    # the reference's Sparse pairs row-argsorted values with scipy's column-sorted CSR indices
    # (operators.py:65-76), which is only consistent when triplets arrive sorted by (row, col)
    order = np.lexsort((cols, rows))
    return rows[order], cols[order], vals[order]


def case_cg_dense():
    for dt, tol in ((np.float32, 1e-6), (np.float64, 1e-10)):
        A, _ = spd_from_spectrum(64, 1e-2, 1e2, 0, dt)
        b = np.random.default_rng(1).standard_normal(64).astype(dt)
        op = cola.PSD(cola.ops.Dense(torch.from_numpy(A)))
        Ainv = cola.linalg.inv(op, cola.linalg.CG(tol=tol, max_iters=500))
        x = Ainv @ torch.from_numpy(b)
        tag = "f32" if dt == np.float32 else "f64"
        save(f"cg_dense_{tag}", A=A, b=b, tol=tol, max_iters=500, x=x, iterations=Ainv.info["iterations"],
             errors=Ainv.info["errors"])


def case_cg_multi_jacobi_x0():
    A, _ = spd_from_spectrum(48, 1e-1, 1e2, 2, np.float64)
    A = A + np.diag(np.linspace(1, 50, 48))
    rng = np.random.default_rng(3)
    B = rng.standard_normal((48, 3))
    X0 = 0.1 * rng.standard_normal((48, 3))
    P = cola.ops.Diagonal(torch.from_numpy(1.0 / np.diag(A)))
    x, info = cola.linalg.CG(tol=1e-9, max_iters=300, x0=torch.from_numpy(X0), P=P)(
        cola.PSD(cola.ops.Dense(torch.from_numpy(A))), torch.from_numpy(B))
    save("cg_multi_jacobi_x0", A=A, B=B, X0=X0, dinv=1.0 / np.diag(A), tol=1e-9, max_iters=300, x=x,
         iterations=info["iterations"], errors=info["errors"])


def case_cg_sparse():
    for dt, tol in ((np.float32, 1e-6), (np.float64, 1e-10)):
        r, c, v = diffusion_2d(12, 4, dt)
        n = 144
        B = np.random.default_rng(5).standard_normal((n, 2)).astype(dt)
        # The reference's Sparse pairs values permuted by an unstable row argsort with scipy's
        # column-sorted CSR indices (operators.py:65-76), so its matrix is generally not the one
        # given; the reference CG is therefore recorded on Dense of the same matrix.
        Ad = np.zeros((n, n), dtype=dt)
        np.add.at(Ad, (r, c), v)
        op = cola.PSD(cola.ops.Dense(torch.from_numpy(Ad)))
        x, info = cola.linalg.CG(tol=tol, max_iters=600)(op, torch.from_numpy(B))
        tag = "f32" if dt == np.float32 else "f64"
        save(f"cg_sparse_{tag}", rows=r, cols=c, vals=v, B=B, tol=tol, max_iters=600, x=x,
             iterations=info["iterations"], errors=info["errors"])


def case_cg_repeated_eig():
    from cola.utils.utils_for_tests import generate_pd_from_diag
    diag = np.array([1.0] * 10 + [0.5] * 10 + [0.25] * 10, dtype=np.float32)
    A = np.array(generate_pd_from_diag(diag, dtype=diag.dtype), dtype=np.float32)
    rhs = np.ones((30, 1), dtype=np.float32)
    x, _, k, _ = run_batched_cg(cola.ops.Dense(torch.from_numpy(A)), torch.from_numpy(rhs),
                                torch.zeros(30, 1), 100, 1e-11, cola.ops.I_like(cola.ops.Dense(torch.from_numpy(A))),
                                pbar=False)
    save("cg_repeated_eig", A=A, rhs=rhs, x=x, k=int(k))


def case_lanczos():
    A, _ = spd_from_spectrum(50, 1e-1, 1e1, 6, np.float64)
    V0 = np.random.default_rng(7).standard_normal((50, 3))
    Q, T, info = lanczos(cola.ops.Dense(torch.from_numpy(A)), torch.from_numpy(V0), max_iters=20, tol=1e-7)
    save("lanczos_batched", A=A, V0=V0, max_iters=20, tol=1e-7, alpha=T.alpha[:, :, 0], beta=T.beta[:, :, 0],
         Q=Q.to_dense(), iterations=info["iterations"])
    # known-answer tridiagonals of the reference suite (tests/algorithms/test_lanczos.py:268-300)
    cases = {
        "early": (np.diag([4.0, 2.0, 1.0]), np.array([[1.0, 0.0, 0.0]]).T),
        "three": (np.array([[7.0, 0, 1.0], [0, 1.0, 0.1], [1.0, 0.1, 3.0]]), np.array([[0.0, 1.0, 0.0]]).T),
        "two": (np.array([[1.0, 0.1, 0.0], [0.1, 2.0, 0.1], [0.0, 0.1, 4.0]]), np.array([[1.0, 0.0, 0.0]]).T),
    }
    for name, (M, rhs) in cases.items():
        Q, T, info = lanczos(cola.ops.Dense(torch.from_numpy(M).float()), torch.from_numpy(rhs).float(),
                             max_iters=3, tol=1e-7)
        save(f"lanczos_case_{name}", A=M, rhs=rhs, alpha=T.alpha[:, :, 0], beta=T.beta[:, :, 0],
             iterations=info["iterations"])


def case_eig():
    A, lam = spd_from_spectrum(40, 1e-1, 1e1, 8, np.float64)
    op = cola.SelfAdjoint(cola.ops.Dense(torch.from_numpy(A)))
    vals, vecs = cola.linalg.eig(op, 5, "LM", cola.linalg.Lanczos(max_iters=40, tol=1e-10))
    start = torch_fns.randn(40, dtype=torch.float64, device=None, key=torch_fns.PRNGKey(42))
    save("eig_lanczos", A=A, lam=np.sort(lam), start=start, evals=vals, evecs=vecs.to_dense())


def case_lanczos_unary():
    A, lam = spd_from_spectrum(60, 1e-1, 1e1, 9, np.float64)
    Z = torch.sign(torch_fns.randn(60, 4, dtype=torch.float64, device=None, key=torch_fns.PRNGKey(11)))
    op = cola.PSD(cola.ops.Dense(torch.from_numpy(A)))
    F = LanczosUnary(op, torch.log, max_iters=25, tol=1e-7)
    Y = F @ Z
    save("lanczos_unary_log", A=A, Z=Z, Y=Y, max_iters=25, tol=1e-7, logdet=np.sum(np.log(lam)))


def case_logdet_slq():
    A, lam = spd_from_spectrum(60, 1e-1, 1e1, 10, np.float64)
    op = cola.PSD(cola.ops.Dense(torch.from_numpy(A)))
    ld = cola.linalg.logdet(op, cola.linalg.Lanczos(max_iters=30, tol=1e-6),
                            cola.linalg.Hutch(max_iters=2, key=torch_fns.PRNGKey(42)))
    save("logdet_slq_dense", A=A, logdet=ld, exact=np.sum(np.log(lam)), max_iters=30, tol=1e-6, hutch_iters=2)


def case_kron_slq():
    rng = np.random.default_rng(12)

    def rbf(m, ell):
        x = np.linspace(0, 1, m)
        return np.exp(-((x[:, None] - x[None, :]) ** 2) / (2 * ell**2))
    Ks = [rbf(4, 0.3), rbf(5, 0.2), rbf(3, 0.5)]
    K = cola.ops.Kronecker(*[cola.ops.Dense(torch.from_numpy(k)) for k in Ks])
    op = cola.PSD(K + 0.01 * cola.ops.I_like(K))
    ld = cola.linalg.logdet(op, cola.linalg.Lanczos(max_iters=40, tol=1e-10),
                            cola.linalg.Hutch(max_iters=3, rand="rademacher", key=torch_fns.PRNGKey(7)))
    lam = np.ones(1)
    for k in Ks:
        lam = np.kron(lam, np.linalg.eigvalsh(k))
    save("logdet_kron_slq", K1=Ks[0], K2=Ks[1], K3=Ks[2], logdet=ld, exact=np.sum(np.log(lam + 0.01)))
    _ = rng


def case_slq_tbd():
    spec = importlib.util.spec_from_file_location("cola_tbd_slq", REF / "cola/linalg/tbd/slq.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["cola_tbd_slq"] = mod  # cola.utils.export looks the module up by name
    spec.loader.exec_module(mod)
    A, lam = spd_from_spectrum(30, 1e-1, 1e1, 13, np.float64)
    key = torch_fns.PRNGKey(3)
    est = mod.stochastic_lanczos_quad(cola.ops.Dense(torch.from_numpy(A)), torch.log, max_iters=30, tol=1e-7,
                                      vtol=1 / np.sqrt(20), key=key)
    probes = torch_fns.randn(30, 20, dtype=torch.float64, device=None, key=key)
    save("slq_tbd", A=A, probes=probes, estimate=est, exact=np.sum(np.log(lam)))


def case_ops():
    # Sparse known answer (tests/test_operators.py:171-203)
    data = torch.tensor([4.0, 5.0, 6.0, 1.0, 2.0, 3.0])
    ri = torch.tensor([2, 2, 2, 0, 0, 1])
    ci = torch.tensor([0, 1, 2, 1, 3, 3])
    S = cola.ops.Sparse(data, ri, ci, shape=(3, 4))
    x1 = torch.tensor([1.0, 0.0, -1.0, 1.0])
    save("ops_sparse_known", data=data, rows=ri, cols=ci, x=x1, y=S @ x1)
    rng = np.random.default_rng(14)
    A1, A2 = rng.standard_normal((2, 3)), rng.standard_normal((4, 2))
    X = rng.standard_normal((6, 2))
    K = cola.ops.Kronecker(cola.ops.Dense(torch.from_numpy(A1)), cola.ops.Dense(torch.from_numpy(A2)))
    save("ops_kron", A1=A1, A2=A2, X=X, Y=K @ torch.from_numpy(X))
    B1, B2 = rng.standard_normal((3, 3)), rng.standard_normal((2, 2))
    Xb = rng.standard_normal((3 * 2 + 2 * 3, 2))
    BD = cola.ops.BlockDiag(cola.ops.Dense(torch.from_numpy(B1)), cola.ops.Dense(torch.from_numpy(B2)),
                            multiplicities=[2, 3])
    save("ops_blockdiag", B1=B1, B2=B2, X=Xb, Y=BD @ torch.from_numpy(Xb))
    D, d = rng.standard_normal((5, 5)), rng.standard_normal(5)
    Xs = rng.standard_normal((5, 3))
    Dop = cola.ops.Dense(torch.from_numpy(D))
    SumOp = Dop + cola.ops.Diagonal(torch.from_numpy(d)) + 0.5 * cola.ops.I_like(Dop)
    ProdOp = Dop @ cola.ops.Dense(torch.from_numpy(D.T.copy()))
    save("ops_sum_product", D=D, d=d, X=Xs, Ysum=SumOp @ torch.from_numpy(Xs), Yprod=ProdOp @ torch.from_numpy(Xs))


def case_arnoldi_gmres():
    """Non-symmetric operators: Arnoldi (arnoldi.py:166-201, 303-334) and GMRES (gmres.py:39-117)."""
    from cola.linalg.decompositions.arnoldi import arnoldi
    from cola.linalg.inverse.gmres import gmres
    rng = np.random.default_rng(7)
    n = 40
    A = 3 * np.eye(n) + 0.5 * rng.standard_normal((n, n)) / np.sqrt(n)
    b = rng.standard_normal(n)
    At, bt = torch.from_numpy(A), torch.from_numpy(b)
    Q, H, info = arnoldi(cola.ops.Dense(At), start_vector=bt, max_iters=12, tol=1e-12)
    save("arnoldi_dense", A=A, v0=b, max_iters=12, tol=1e-12, Q=Q.to_dense(), H=H.to_dense(),
         iterations=info["iterations"])
    for tag, m in (("full", 30), ("short", 8)):
        x, info = gmres(cola.ops.Dense(At), bt, max_iters=m, tol=1e-10)
        save(f"gmres_dense_{tag}", A=A, b=b, max_iters=m, tol=1e-10, x=x, iterations=info["iterations"])
    # two right-hand sides at once, float32
    B = rng.standard_normal((n, 2)).astype(np.float32)
    X, info = gmres(cola.ops.Dense(At.float()), torch.from_numpy(B), max_iters=25, tol=1e-6)
    save("gmres_dense_multi_f32", A=A.astype(np.float32), B=B, max_iters=25, tol=1e-6, x=X, iterations=info["iterations"])


def case_nystrom():
    """The reference's Nystrom preconditioner (preconditioners.py:88-190) on its own test matrices
    (tests/algorithms/test_cg.py: spectrum 1 - x^0.75 on 25 points, rank 5, mu 0), its sqrt and
    inverse, and run_batched_cg with it as P."""
    from cola.linalg.preconditioning.preconditioners import NystromPrecond, inverse as nys_inverse, sqrt as nys_sqrt
    from cola.utils.utils_for_tests import generate_pd_from_diag, generate_spectrum
    diag = generate_spectrum(coeff=0.75, scale=1.0, size=25, dtype=np.float32)
    A32 = np.array(generate_pd_from_diag(diag, dtype=diag.dtype, seed=21), dtype=np.float32)
    for dt in (np.float32, np.float64):
        A = A32.astype(dt)
        At = torch.from_numpy(A)
        P = NystromPrecond(cola.ops.Dense(At), rank=5, mu=0, eps=1e-8)
        Pdef = NystromPrecond(cola.ops.Dense(At), rank=5)  # mu = 1e-7, adjust_mu = True
        rhs = np.ones((25, 5), dtype=dt)
        x, _, k, _ = run_batched_cg(cola.ops.Dense(At), torch.from_numpy(rhs), torch.zeros(25, 5, dtype=At.dtype), 100,
                                    1e-8, P, pbar=False)
        tag = "f32" if dt == np.float32 else "f64"
        save(f"nystrom_{tag}", A=A, rank=5, eps=1e-8, Lambda=P.Lambda, P=P.to_dense(), P_default=Pdef.to_dense(),
             P_sqrt=nys_sqrt(P).to_dense(), P_inv=nys_inverse(P).to_dense(), rhs=rhs, x=x, k=int(k),
             eigmax=P.preconditioned_eigmax, eigmin=P.preconditioned_eigmin)


if __name__ == "__main__":
    import os
    cases = [case_cg_dense, case_cg_multi_jacobi_x0, case_cg_sparse, case_cg_repeated_eig, case_lanczos, case_eig,
             case_lanczos_unary, case_logdet_slq, case_kron_slq, case_slq_tbd, case_ops, case_arnoldi_gmres,
             case_nystrom]
    only = [x for x in os.environ.get("GOLDEN_ONLY", "").split(",") if x]
    for fn in cases:
        if not only or fn.__name__ in only:
            fn()
