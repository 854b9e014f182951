"""Golden data at the benchmark configurations' full sizes, recorded from the reference CoLA itself.

Run in a container that holds the reference source (it is not needed anywhere else):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden_configs.py <reference source tree> [case ...]

Cases (each writes tests/golden/cfg_<case>.npz):
  c1   solve(PSD(Dense(A)), b, CG(tol=1e-6, max_iters=2000)) on the 2048 dense system, FP32, plus the same
       solve in FP64 to tol 1e-13 (cg.py:94-119)
  c3a  the first 8 uneven RBF systems K + s^2 I, one reference FP32 CG(tol=1e-6, max_iters=2000) each
  c3b  LanczosUnary(Kron(K1, K2, K3) + 0.01 I, log, max_iters=100) @ Z with the 64 Rademacher probes
       (unary.py:46-60), FP32; the per-probe quadratic forms z^T log(A) z
  c3b64  the same in FP64 on the first 16 of those probes (in FP32 the operator's rounding, about
       eps * |A| = 5e-4, is not small against its smallest eigenvalues, 0.01)
  c4   one 512 x 512 diffusion instance, CG(P=Diagonal(1/diag A)) in FP64 to tol 1e-12 (cg.py:124, 150)
  c5   eig(SelfAdjoint(Kron(A1, A2) + L), 64, "LM", Lanczos(max_iters=256)) with the host start vector,
       FP32 (eigs.py:106-111), and scipy's ARPACK eigsh on the FP64 operator as the FP64 oracle

Inputs come from the seeded generators of cola_gb300.workloads and cola_gb300.linalg.prng with CPU
random generators, so a GPU test regenerates the same inputs on any machine; every case stores
checksums of its inputs so that a test can confirm it.  Large outputs are stored as samples (every
16th entry) plus norms and projections, to keep the files small.
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
if len(sys.argv) < 2 or not (Path(sys.argv[1]) / "cola").is_dir():
    sys.exit("usage: make_golden_configs.py <path of the reference source tree (the directory holding cola/)> [case ...]")
REF = Path(sys.argv[1])
sys.path[:0] = [str(HERE / "_shims"), str(REF), str(ROOT)]

import torch  # noqa: E402

torch.set_num_threads(8)
import cola  # noqa: E402
from cola.backends import torch_fns  # noqa: E402
from cola.linalg.decompositions.lanczos import lanczos  # noqa: E402
from cola.linalg.unary.unary import LanczosUnary  # noqa: E402

from cola_gb300 import workloads as W  # noqa: E402  (seeded input generators only)
from cola_gb300.linalg.prng import randn as keyed_randn  # noqa: E402


def save(name, **arrays):
    out = {k: (v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(v)) for k, v in arrays.items()}
    np.savez_compressed(HERE / f"cfg_{name}.npz", **out)
    print(f"wrote cfg_{name}.npz ({', '.join(out)})", flush=True)


def probe_vectors(n, count=4, seed=99):
    """Fixed +-1 projection vectors (numpy generator) for checksums of long vectors."""
    return np.sign(np.random.default_rng(seed).standard_normal((count, n)))


def case_c1():
    A, b, _ = W.dense_spd(2048, seed=0, lo=1e-2, hi=1e2, dtype=torch.float32)
    t0 = time.perf_counter()
    Ainv = cola.linalg.inv(cola.PSD(cola.ops.Dense(A)), cola.linalg.CG(tol=1e-6, max_iters=2000))
    x32 = Ainv @ b
    t32 = time.perf_counter() - t0
    it32 = int(Ainv.info["iterations"])
    A64, b64 = A.double(), b.double()
    Ainv64 = cola.linalg.inv(cola.PSD(cola.ops.Dense(A64)), cola.linalg.CG(tol=1e-13, max_iters=20000))
    x64 = Ainv64 @ b64
    relres32 = float((b64 - A64 @ x32.double()).norm() / b64.norm())
    relres64 = float((b64 - A64 @ x64).norm() / b64.norm())
    P = probe_vectors(2048)
    save("c1", x32=x32, iterations32=it32, relres32=relres32, seconds32=t32, x64=x64,
         iterations64=int(Ainv64.info["iterations"]), relres64=relres64, b=b,
         a_proj=P @ A64.numpy(), a_sum=float(A64.sum()))


def case_c3a():
    mats, rhs, meta = W.rbf_systems(num=8, seed=3, device="cpu")
    xs, its, rel, ns = [], [], [], []
    for A, b in zip(mats, rhs):
        Ainv = cola.linalg.inv(cola.PSD(cola.ops.Dense(A)), cola.linalg.CG(tol=1e-6, max_iters=2000))
        x = Ainv @ b
        its.append(int(Ainv.info["iterations"]))
        rel.append(float((b.double() - A.double() @ x.double()).norm() / b.double().norm()))
        ns.append(A.shape[0])
        xs.append(x.double().numpy()[::16])
        print(f"  c3a system n={A.shape[0]} iters={its[-1]} relres={rel[-1]:.2e}", flush=True)
    save("c3a", n=np.array(ns), iterations=np.array(its), relres=np.array(rel),
         x_sub=np.concatenate(xs), s2=np.array([m[2] for m in meta]), ell=np.array([m[1] for m in meta]))


def c3b_inputs():
    Ks, ells = W.kron_rbf(seed=4, m=64, factors=3, device="cpu", dtype=torch.float32)
    n = 64 ** 3
    Z = torch.sign(keyed_randn(n, 64, dtype=torch.float32, key=5))
    return Ks, ells, Z


def case_c3b():
    Ks, ells, Z = c3b_inputs()
    K = cola.ops.Kronecker(*[cola.ops.Dense(k) for k in Ks])
    op = cola.PSD(K + 0.01 * cola.ops.I_like(K))
    t0 = time.perf_counter()
    # the tridiagonals of the same run, for diagnosing the quadrature (lanczos.py:185-232)
    _, T, _ = lanczos(op, Z, max_iters=100, tol=0.0)
    T_dense = torch.vmap(T.__class__.to_dense)(T)
    F = LanczosUnary(op, torch.log, max_iters=100, tol=0.0)
    Y = F @ Z
    secs = time.perf_counter() - t0
    quad = (Z.double() * Y.double()).sum(0)  # z_j^T log(A) z_j
    lam = np.ones(1)
    for k in Ks:
        lam = np.kron(lam, np.linalg.eigvalsh(k.double().numpy()))
    exact = float(np.sum(np.log(lam + 0.01)))
    save("c3b", quad=quad, estimate=float(quad.mean()), stderr=float(quad.std() / np.sqrt(64)), exact=exact,
         ells=np.array(ells), z_sum=float(Z.double().sum()), z_proj=probe_vectors(Z.shape[0]) @ Z.double().numpy(),
         seconds=secs, T_diag=torch.diagonal(T_dense, 0, -2, -1).float(),
         T_off=torch.diagonal(T_dense, 1, -2, -1).float())


def case_c3b64():
    Ks, ells, Z = c3b_inputs()
    Z = Z[:, :16].double()
    K = cola.ops.Kronecker(*[cola.ops.Dense(k.double()) for k in Ks])
    op = cola.PSD(K + 0.01 * cola.ops.I_like(K))
    t0 = time.perf_counter()
    Y = LanczosUnary(op, torch.log, max_iters=100, tol=0.0) @ Z
    secs = time.perf_counter() - t0
    quad = (Z * Y).sum(0)
    save("c3b64", quad=quad, estimate=float(quad.mean()), seconds=secs)


def case_c4():
    fam, B, _, params = W.diffusion_family_2d([5000], m=512, device="cpu")
    n = fam.n
    ip, ix = fam.indptr.long(), fam.indices.long()
    rows = torch.repeat_interleave(torch.arange(n), ip[1:] - ip[:-1])
    v = fam.values[0].double()
    dg = torch.zeros(n, dtype=torch.float64)
    dg.index_add_(0, rows, torch.where(rows == ix, v, torch.zeros_like(v)))
    A = cola.PSD(cola.ops.Sparse(v, rows, ix, (n, n)))  # triplets in (row, col) order
    b = B[0].double()
    t0 = time.perf_counter()
    Ainv = cola.linalg.inv(A, cola.linalg.CG(tol=1e-12, max_iters=100000, P=cola.ops.Diagonal(1.0 / dg)))
    x = Ainv @ b
    secs = time.perf_counter() - t0
    Acsr = torch.sparse_csr_tensor(ip, ix, v, (n, n))
    relres = float((b - Acsr @ x).norm() / b.norm())
    P = probe_vectors(n)
    save("c4", x_sub=x[::16], x_norm=float(x.norm()), x_proj=P @ x.numpy(), iterations=int(Ainv.info["iterations"]),
         relres=relres, seconds=secs, values_sum=float(v.sum()), values_proj=probe_vectors(v.numel()) @ v.numpy(),
         b_sum=float(b.sum()), ell_var=np.array(params[0]))


def c5_inputs():
    A1, _, _ = W.dense_spd(1024, seed=6, lo=1e-2, hi=1e1, dtype=torch.float32)
    A2, _, _ = W.dense_spd(1024, seed=61, lo=1e-2, hi=1e1, dtype=torch.float32)
    ip, ix, v = W.rgg_laplacian(1 << 20, 0.002, seed=7, device="cpu")
    return A1, A2, ip, ix, v


def case_c5():
    A1, A2, ip, ix, v = c5_inputs()
    n = 1 << 20
    rows = torch.repeat_interleave(torch.arange(n), (ip[1:] - ip[:-1]).long())
    L = cola.ops.Sparse(v, rows, ix.long(), (n, n))
    op = cola.SelfAdjoint(cola.ops.Kronecker(cola.ops.Dense(A1), cola.ops.Dense(A2)) + L)
    start = torch_fns.randn(n, dtype=torch.float32, device=None, key=torch_fns.PRNGKey(42))
    t0 = time.perf_counter()
    vals, _ = cola.linalg.eig(op, 64, "LM", cola.linalg.Lanczos(start_vector=start, max_iters=256, tol=1e-12))
    secs = time.perf_counter() - t0
    print(f"  c5 reference Lanczos {secs:.1f} s", flush=True)
    # FP64 oracle: ARPACK on the FP64 operator
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    A1d, A2d = A1.double().numpy(), A2.double().numpy()
    Ld = sp.csr_matrix((v.double().numpy(), ix.numpy(), ip.numpy()), shape=(n, n))

    def mv(x):
        X = x.reshape(1024, 1024)
        return (A1d @ X @ A2d.T).reshape(-1) + Ld @ x
    t1 = time.perf_counter()
    w = spla.eigsh(spla.LinearOperator((n, n), matvec=mv, dtype=np.float64), k=64, which="LA", tol=1e-12,
                   return_eigenvectors=False)
    t_arpack = time.perf_counter() - t1
    print(f"  c5 ARPACK {t_arpack:.1f} s", flush=True)
    save("c5", ref_evals=vals, arpack_evals=np.sort(w), seconds_ref=secs, seconds_arpack=t_arpack,
         start_sum=float(start.double().sum()), start_proj=probe_vectors(n) @ start.double().numpy(),
         l_nnz=int(ix.numel()), l_sum_abs=float(v.double().abs().sum()),
         a1_proj=probe_vectors(1024) @ A1.double().numpy(), a2_proj=probe_vectors(1024) @ A2.double().numpy())


if __name__ == "__main__":
    cases = {"c1": case_c1, "c3a": case_c3a, "c3b": case_c3b, "c3b64": case_c3b64, "c4": case_c4, "c5": case_c5}
    for name in (sys.argv[2:] or list(cases)):
        t = time.perf_counter()
        cases[name]()
        print(f"{name}: {time.perf_counter() - t:.1f} s", flush=True)
