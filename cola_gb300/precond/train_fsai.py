"""Train the learned FSAI network on the 512 x 512 variable-diffusion family and evaluate it.

    python -m cola_gb300.precond.train_fsai [--train 2048] [--epochs 8] [--out path]

Training data: instances with seeds 1000.. (held apart from the validation seeds 4000.. and the
benchmark's test seeds 5000..); for each instance a pair (r, e) with r ~ N(0, 1) and e = A^-1 r
solved by this project's batched CG (Jacobi-PCG, FP64 refinement to 1e-7).  The network, loss,
backward and Adam all run in libcolagb kernels.
"""
from __future__ import annotations

import argparse
import json
import time

import torch

from ..linalg.batched import BatchedCSR, solve_batched
from ..workloads import diffusion_family_2d
from . import learned_fsai as L


def make_pairs(seeds, m, device, chunk=256, k_steps=150):
    """Residual / error pairs from this project's CG: x* solves A x = b (FP64-refined), x_k is the
    closed-form-FSAI PCG iterate after k_steps; the pair is (r_k = b - A x_k, e_k = x* - x_k), the part
    of the error that preconditioned CG has not removed yet."""
    sts, rs, es = [], [], []
    for c0 in range(0, len(seeds), chunk):
        fam, B, _, _ = diffusion_family_2d(seeds[c0: c0 + chunk], m=m, device=device)
        pat, g0 = L.g_values(fam, None)
        X, _ = solve_batched(fam, B, precond="fsai", fsai=(pat, g0), tol=1e-9)
        Xk, _ = solve_batched(fam, B, precond="fsai", fsai=(pat, g0), tol=1e-9, max_inner_iters=k_steps,
                              fallback=False)
        E = X - Xk
        R = B - fam.matvec(Xk)
        # plus a white-noise error per instance, so that the loss also sees the high-frequency part of
        # the spectrum (a factor tuned only on smooth errors could inflate the largest eigenvalues)
        W = torch.randn_like(E)
        RW = fam.matvec(W)
        st = L.stencil(fam, m)
        for e_, r_ in ((E, R), (W, RW)):
            nrm = torch.sqrt((e_ * r_).sum(dim=1, keepdim=True)).clamp_min(1e-300)  # |e|_A
            sts.append(st)
            rs.append((r_ / nrm).float().view(-1, m, m))
            es.append((e_ / nrm).float().view(-1, m, m))
        del fam, B, X, Xk, E, R, W, RW
    return torch.cat(sts), torch.cat(rs), torch.cat(es)


def evaluate(net, seeds, m, device, inner_tol=1e-4):
    fam, B, _, _ = diffusion_family_2d(seeds, m=m, device=device)
    out = {}
    for name in ["plain", "jacobi", "fsai_closed_form", "learned"]:
        kw = dict(tol=1e-8, inner_tol=inner_tol)
        if name == "plain":
            kw["precond"] = "none"
        elif name == "jacobi":
            kw["precond"] = "jacobi"
        else:
            pat, gv = L.g_values(fam, net if name == "learned" else None)
            kw.update(precond="fsai", fsai=(pat, gv), fallback=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        X, info = solve_batched(fam, B, **kw)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out[name] = {"mean_iters": float(info["iterations"].double().mean()),
                     "max_relres": float(info["relres"].max()), "seconds": dt,
                     "solves_per_s": fam.num_systems / dt,
                     "fallbacks": int((info["status"] == 5).sum())}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=2048)
    ap.add_argument("--val", type=int, default=32)
    ap.add_argument("--m", type=int, default=512)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--out", default=str(L.WEIGHTS))
    ap.add_argument("--report", default="")
    args = ap.parse_args()
    dev = torch.device("cuda")
    t0 = time.perf_counter()
    st, r, e = make_pairs(list(range(1000, 1000 + args.train)), args.m, dev)
    t_data = time.perf_counter() - t0
    net = L.FsaiNet(dev, seed=0)
    val_seeds = list(range(4000, 4000 + args.val))
    before = evaluate(net, val_seeds, args.m, dev)
    t1 = time.perf_counter()
    hist = L.train(net, st, r, e, epochs=args.epochs, batch=args.batch, lr=args.lr)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    torch.save(net.state_dict(), args.out)
    after = evaluate(net, val_seeds, args.m, dev)
    rep = {"train_instances": args.train, "epochs": args.epochs, "loss_history": hist, "data_seconds": t_data,
           "train_seconds": t_train, "validation_before": before, "validation_after": after}
    print(json.dumps(rep, indent=1))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(rep, f, indent=1)


if __name__ == "__main__":
    main()
