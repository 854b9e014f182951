"""One run of a benchmark configuration's Krylov kernel, for profiling (launch lists, ncu captures).

    python -m cola_gb300.cases_krylov c5 [--scale 0.25] [--repeat 1] [--precision auto|fp32]
    python -m cola_gb300.cases_krylov c3b [--probes 64]
    python -m cola_gb300.cases_krylov c1
    python -m cola_gb300.cases_krylov c2 [--scale 0.5] [--schedule block|cluster16] [--matvec fp32|bf16]
    python -m cola_gb300.cases_krylov c3a [--systems 16] [--steps 20]

c5: 256-step Lanczos top-64 of Kronecker(A1, A2) + L (random-geometric-graph Laplacian); --scale < 1
shrinks the factors and the graph (n = (1024 s)^2 rows) so that a capture stays small.  c3b: the
Kronecker SLQ log-determinant with 64 probes and 100 steps.  c1: the 2048 dense CG solve.  Prints one
JSON line per run with its wall time (CUDA-synchronised).  c2: the 7-point diffusion solve of 32
right-hand sides to a 1e-8 FP64 residual with Jacobi (grid side 128 s).  c3a: the first --systems
of the 256 uneven dense RBF systems, FP32 CG to 1e-6 in one persistent launch, at most --steps steps
(0: 2000).
"""
from __future__ import annotations

import argparse
import json
import time

import torch


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("config", choices=["c1", "c2", "c3a", "c3b", "c5"])
    ap.add_argument("--schedule", default="auto")
    ap.add_argument("--matvec", default="fp32", choices=["fp32", "bf16"])
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--precision", default="auto", choices=["auto", "fp32", "bf16", "bf16x3"])
    ap.add_argument("--probes", type=int, default=64)
    ap.add_argument("--steps", type=int, default=0, help="Lanczos / SLQ steps (0: the configuration's)")
    ap.add_argument("--reorder", action="store_true", help="c5: store L in reverse Cuthill-McKee order")
    ap.add_argument("--systems", type=int, default=256, help="c3a: how many of the 256 systems")
    args = ap.parse_args(argv)

    import cola_gb300 as cola
    from cola_gb300 import workloads as W
    from cola_gb300.linalg.prng import PRNGKey, randn

    dev = torch.device("cuda")
    if args.config == "c5":
        m = max(64, int(1024 * args.scale) // 16 * 16)
        A1, _, _ = W.dense_spd(m, seed=6, lo=1e-2, hi=1e1, dtype=torch.float32)
        A2, _, _ = W.dense_spd(m, seed=61, lo=1e-2, hi=1e1, dtype=torch.float32)
        n = m * m
        ip, ix, v = W.rgg_laplacian(n, 0.002 / args.scale, seed=7, device="cpu")
        L = cola.ops.Sparse.from_csr(ip.to(dev), ix.to(dev), v.to(dev), (n, n))
        if args.reorder:
            L = L.reordered()
        op = cola.SelfAdjoint(cola.ops.Kronecker(cola.ops.Dense(A1.to(dev)), cola.ops.Dense(A2.to(dev)),
                                                 precision=args.precision) + L)
        start = randn(n, dtype=torch.float32, key=PRNGKey(42)).to(dev)
        steps = args.steps or 256

        def run():
            return cola.linalg.eig(op, 64, "LM", cola.linalg.Lanczos(start_vector=start, max_iters=steps, tol=1e-12))
    elif args.config == "c3b":
        Ks, _ = W.kron_rbf(seed=4, device="cpu")
        K = cola.ops.Kronecker(*[cola.ops.Dense(k.to(dev)) for k in Ks], precision=args.precision)
        op = cola.PSD(K + 0.01 * cola.ops.I_like(K))
        Z = torch.sign(randn(64 ** 3, args.probes, dtype=torch.float32, key=5)).to(dev)
        steps = args.steps or 100

        def run():
            return cola.linalg.stochastic_lanczos_quad(op, torch.log, max_iters=steps, tol=0.0, probes=Z)
    elif args.config == "c3a":
        from cola_gb300.linalg.batched import solve_dense_batched
        mats, rhs, _ = W.rbf_systems(num=args.systems, device=dev)
        steps = args.steps or 2000

        def run():
            return solve_dense_batched(mats, rhs, tol=1e-6, max_iters=steps)
    elif args.config == "c2":
        from cola_gb300.linalg.batched import BatchedCSR, solve_batched
        m = max(8, int(128 * args.scale))
        ip, ix, v = W.diffusion_3d(m=m, device=dev)
        fam = BatchedCSR(ip, ix, v[None, :], shared=True)
        B = torch.randn(32, fam.n, device=dev, dtype=torch.float64, generator=torch.Generator("cuda").manual_seed(2))

        def run():
            return solve_batched(fam, B, precond="jacobi", tol=1e-8, schedule=args.schedule, matvec=args.matvec)
    else:
        A, b, _ = W.dense_spd(2048, seed=0, lo=1e-2, hi=1e2, dtype=torch.float32)
        op = cola.PSD(cola.ops.Dense(A.to(dev)))
        bd = b.to(dev)

        def run():
            return cola.linalg.cg(op, bd, tol=1e-6, max_iters=2000)
    for rep in range(args.repeat):
        torch.cuda.synchronize()
        t = time.perf_counter()
        run()
        torch.cuda.synchronize()
        print(json.dumps({"config": args.config, "repeat": rep, "scale": args.scale, "precision": args.precision,
                          "seconds": time.perf_counter() - t}), flush=True)


if __name__ == "__main__":
    main()
