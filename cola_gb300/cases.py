"""One batched solve of the 2-D diffusion family, for profiling and latency measurements.

    python -m cola_gb300.cases --systems 8 --m 512 --precond jacobi --schedule onchip --repeat 2 [--spare off]

Runs ``--repeat`` identical solves (the first one also pays for workspace allocation) and prints one
JSON line per solve: wall time, solves/s, mean / max CG steps, FP64 relative residual, and the time
per CG step of the slowest system (the per-iteration latency of one system when ``--systems`` does
not exceed the clusters in flight).  ``--precond learned`` builds the trained network's factor in
every repeat (timed apart, ``build_seconds``); ``--build-only`` runs just that build.
"""
from __future__ import annotations

import argparse
import json
import time

import torch


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--systems", type=int, default=8)
    ap.add_argument("--m", type=int, default=512, help="grid side: systems are m^2 x m^2")
    ap.add_argument("--precond", default="jacobi", choices=["none", "jacobi", "fsai", "learned"])
    ap.add_argument("--build-only", action="store_true", help="learned / fsai: only build the factor")
    ap.add_argument("--schedule", default="auto", choices=["auto", "grid", "cluster8", "cluster16", "onchip"])
    ap.add_argument("--repeat", type=int, default=2)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--spare", default="off", choices=["auto", "off", "only"],
                    help="on-chip schedule: the companion CTAs on the SMs the clusters leave free")
    args = ap.parse_args(argv)

    import cola_gb300 as cola
    from cola_gb300.linalg.batched import onchip_schedule_info
    from cola_gb300.workloads import diffusion_family_2d

    fam, B, _, _ = diffusion_family_2d(range(args.systems), m=args.m, device="cuda")
    net = pat = None
    if args.precond in ("fsai", "learned"):
        from cola_gb300.linalg.batched import FsaiPattern
        from cola_gb300.precond import learned_fsai
        pat = FsaiPattern(fam.indptr, fam.indices)
        if args.precond == "learned":
            net = learned_fsai.FsaiNet.load(learned_fsai.WEIGHTS, device="cuda")
    print(json.dumps({"onchip": onchip_schedule_info(fam.n, args.m)}), flush=True)
    for rep in range(args.repeat):
        fsai, tb = None, 0.0
        if pat is not None:
            torch.cuda.synchronize()
            tb = time.perf_counter()
            fsai = learned_fsai.g_values(fam, net, pat)
            torch.cuda.synchronize()
            tb = time.perf_counter() - tb
            if args.build_only:
                print(json.dumps({"repeat": rep, "precond": args.precond, "systems": args.systems, "n": fam.n,
                                  "build_seconds": tb}), flush=True)
                continue
        torch.cuda.synchronize()
        t = time.perf_counter()
        X, info = cola.linalg.solve_batched(fam, B, precond="fsai" if pat is not None else args.precond,
                                            tol=args.tol, fsai=fsai, schedule=args.schedule, spare=args.spare)
        torch.cuda.synchronize()
        t = time.perf_counter() - t
        it = info["iterations"].double()
        print(json.dumps({"repeat": rep, "schedule": args.schedule, "spare": args.spare, "precond": args.precond,
                          "systems": args.systems,
                          "n": fam.n, "seconds": t, "build_seconds": tb, "solves_per_s": args.systems / t,
                          "mean_iters": float(it.mean()), "max_iters": int(it.max()),
                          "us_per_step_slowest": 1e6 * t / max(1, int(it.max())),
                          "max_relres": float(info["relres"].max()),
                          "all_converged": bool((info["status"] == 1).all())}), flush=True)


if __name__ == "__main__":
    main()
