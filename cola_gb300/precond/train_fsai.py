"""Train the learned FSAI network on the 512 x 512 variable-diffusion family and evaluate it.

    python -m cola_gb300.precond.train_fsai [--train 2048] [--epochs 8] [--out path]

Training data: instances with seeds 1000.. (held apart from the validation seeds 4000.. and the
benchmark's test seeds 5000..); for each instance the error that closed-form-FSAI PCG has left after
150 steps (the smooth, slowly converging bottom of the spectrum) and a white-noise error (the top),
each with its residual.  Default loss: mean log Rayleigh quotient of P A on the white-noise errors
minus that on the smooth errors, a scale-free proxy of log cond(P A).  The network, loss, backward
and Adam all run in libcolagb kernels.  After every epoch the validation instances are
solved with the current factor; the weights with the fewest mean PCG iterations are kept (the
untrained network, which reproduces closed-form FSAI, is the first candidate).
"""
from __future__ import annotations

import argparse
import json
import math
import time

import torch

from ..linalg.batched import BatchedCSR, solve_batched
from ..workloads import diffusion_family_2d
from . import learned_fsai as L


def make_pairs(seeds, m, device, chunk=256, k_steps=150, white=True, net=None):
    """Residual / error pairs from this project's CG: x* solves A x = b (FP64-refined), x_k is the
    PCG iterate after k_steps with the factor of `net` (closed form when None); the pair is
    (r_k = b - A x_k, e_k = x* - x_k), the part
    of the error that preconditioned CG has not removed yet (kind 0, the bottom of the spectrum).
    With `white`, also a white-noise error and its residual per instance (kind 1, the top)."""
    sts, rs, es, kinds = [], [], [], []
    for c0 in range(0, len(seeds), chunk):
        fam, B, _, _ = diffusion_family_2d(seeds[c0: c0 + chunk], m=m, device=device)
        pat, g0 = L.g_values(fam, net)
        X, _ = solve_batched(fam, B, precond="fsai", fsai=(pat, g0), tol=1e-9)
        Xk, _ = solve_batched(fam, B, precond="fsai", fsai=(pat, g0), tol=1e-9, max_inner_iters=k_steps,
                              fallback=False)
        E = X - Xk
        R = B - fam.matvec(Xk)
        # optionally a white-noise error per instance as well (the high-frequency part of the
        # spectrum; the row normalisation diag(G A G^T) = 1 already bounds the largest eigenvalues)
        pairs = [(E, R)]
        if white:
            W = torch.randn_like(E)
            pairs.append((W, fam.matvec(W)))
        st = L.stencil(fam, m)
        for kd, (e_, r_) in enumerate(pairs):
            nrm = torch.sqrt((e_ * r_).sum(dim=1, keepdim=True)).clamp_min(1e-300)  # |e|_A
            sts.append(st)
            rs.append((r_ / nrm).float().view(-1, m, m))
            es.append((e_ / nrm).float().view(-1, m, m))
            kinds.append(torch.full((st.shape[0],), kd, dtype=torch.int64, device=device))
        del fam, B, X, Xk, E, R, pairs
    return torch.cat(sts), torch.cat(rs), torch.cat(es), torch.cat(kinds)


def evaluate(net, seeds, m, device, inner_tol=0.1, only=("plain", "jacobi", "fsai_closed_form", "learned")):
    fam, B, _, _ = diffusion_family_2d(seeds, m=m, device=device)
    out = {}
    for name in only:
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


def set_constant_output(net, o1, o2):
    """Network weights whose output is the constant (0, o1, o2) in every cell: zero last-layer
    weights, biases o.  The factor is then closed-form FSAI with its N and W entries scaled by
    (1 + tanh o1), (1 + tanh o2) and every row renormalised."""
    W, b = net.layer(len(L.LAYERS) - 1)
    W.zero_()
    b.copy_(torch.tensor([0.0, o1, o2], device=b.device))


def set_feature_map(net, theta):
    """Network weights computing, per cell, o1 = theta[0] + sum_k theta[1+k] h_k and
    o2 = theta[13] + sum_k theta[14+k] h_k over h = (ReLU(f), ReLU(-f)) of the six local features f:
    layer 1 splits each feature into its two signs (center taps +-1), layer 2 passes the 12
    channels through, layer 3 combines them.  A piecewise-linear map of each cell's coefficients to
    the over-relaxation of its two off-diagonals."""
    net.params.zero_()
    W1, _ = net.layer(0)
    W2, _ = net.layer(1)
    W3, b3 = net.layer(2)
    for k in range(6):
        W1[k, k, 1, 1] = 1.0
        W1[6 + k, k, 1, 1] = -1.0
    for c in range(12):
        W2[c, c, 1, 1] = 1.0
    th = torch.as_tensor(theta, dtype=torch.float32, device=net.params.device)
    b3[1], b3[2] = th[0], th[13]
    W3[1, :12, 1, 1] = th[1:13]
    W3[2, :12, 1, 1] = th[14:26]


def search_features(net, seeds, m, device, wn, wv, sweeps=3, log=print):
    """Coordinate search of the 26 parameters of set_feature_map on the mean PCG iteration count of
    the given instances, from the global over-relaxation (wn, wv); a move is kept when it saves more
    than 0.2 % of the iterations.  Returns (theta, mean iterations, evaluations)."""
    fam, B, _, _ = diffusion_family_2d(seeds, m=m, device=device)
    evals = [0]

    def cost(th):
        set_feature_map(net, th)
        pat, gv = L.g_values(fam, net)
        _, info = solve_batched(fam, B, precond="fsai", fsai=(pat, gv), tol=1e-8, fallback=True)
        evals[0] += 1
        ok = bool(((info["status"] == 1) | (info["status"] == 5)).all())
        return float(info["iterations"].double().mean()) if ok else float("inf")

    theta = [0.0] * 26
    theta[0], theta[13] = math.atanh(wn), math.atanh(wv)
    best = cost(theta)
    log(f"features search: start {best:.1f}")
    steps = [0.5] + [0.5] * 4 + [0.5] * 4 + [0.2] * 4  # bias, |ratio| features, log-contrast features
    for sw in range(sweeps):
        for d0 in (0, 13):
            for j in range(13):
                q = d0 + j
                step = steps[j] / (2 ** sw)
                for sgn in (1, -1):
                    trial = list(theta)
                    trial[q] += sgn * step
                    c = cost(trial)
                    if c < best * 0.998:
                        theta, best = trial, c
                        log(f"features search: sweep {sw} param {q} -> {theta[q]:+.3f}: {best:.1f}")
                        break
    return theta, best, evals[0]


def search(net, seeds, m, device, log=print):
    """Direct search for the over-relaxation (w_N, w_W) = (tanh o1, tanh o2) of the FSAI off-diagonals
    that minimises the mean PCG iteration count on the given training instances: a coarse grid, then
    compass steps with halving.  Returns (w_N, w_W, mean iterations, evaluations)."""
    fam, B, _, _ = diffusion_family_2d(seeds, m=m, device=device)
    cache = {}

    def cost(wn, wv):
        key = (round(wn, 4), round(wv, 4))
        if key not in cache:
            set_constant_output(net, math.atanh(wn), math.atanh(wv))
            pat, gv = L.g_values(fam, net)
            _, info = solve_batched(fam, B, precond="fsai", fsai=(pat, gv), tol=1e-8, fallback=True)
            ok = bool(((info["status"] == 1) | (info["status"] == 5)).all())
            cache[key] = float(info["iterations"].double().mean()) if ok else float("inf")
            log(f"search: w_N {wn:+.3f} w_W {wv:+.3f} -> {cache[key]:.1f} mean iterations")
        return cache[key]

    grid = [-0.25, 0.0, 0.25, 0.5, 0.75, 0.9]
    best = min(((cost(a, b), a, b) for a in grid for b in grid))
    step = 0.125
    while step >= 0.015:
        moved = False
        for da, db in ((step, 0), (-step, 0), (0, step), (0, -step)):
            a, b = best[1] + da, best[2] + db
            if -0.95 < a < 0.97 and -0.95 < b < 0.97:
                c = cost(a, b)
                if c < best[0]:
                    best, moved = (c, a, b), True
        if not moved:
            step /= 2
    return best[1], best[2], best[0], len(cache)


def instance_headroom(net, seeds, m, device, wns, wvs, log=print):
    """Per-instance optimum of the global over-relaxation: every (w_N, w_W) of the grid on every instance
    (PCG iterations to 1e-8).  Returns the iteration table (combos x instances), the best single combo
    and the mean over instances of each instance's own best -- the most any factor that picks one
    over-relaxation per operator (which is all a network of these features can do better than the
    constant) could gain."""
    fam, B, _, _ = diffusion_family_2d(seeds, m=m, device=device)
    combos, table = [], []
    for wn in wns:
        for wv in wvs:
            set_constant_output(net, math.atanh(wn), math.atanh(wv))
            pat, gv = L.g_values(fam, net)
            _, info = solve_batched(fam, B, precond="fsai", fsai=(pat, gv), tol=1e-8, fallback=True)
            combos.append((wn, wv))
            table.append(info["iterations"].double())
            log(f"headroom: w_N {wn:.3f} w_W {wv:.3f} -> {float(table[-1].mean()):.1f}")
    T = torch.stack(table)  # (combos, instances)
    mean = T.mean(dim=1)
    g = int(mean.argmin())
    per = T.min(dim=0)
    return {"combos": combos, "global_best": combos[g], "global_best_mean_iters": float(mean[g]),
            "per_instance_best_mean_iters": float(per.values.mean()),
            "per_instance_best_combo": [combos[int(i)] for i in per.indices],
            "headroom_fraction": float(1 - per.values.mean() / mean[g])}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=2048)
    ap.add_argument("--val", type=int, default=32)
    ap.add_argument("--m", type=int, default=512)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-4)
    ap.add_argument("--out", default=str(L.WEIGHTS))
    ap.add_argument("--report", default="")
    ap.add_argument("--search", action="store_true",
                    help="fit the off-diagonal over-relaxation by direct search on PCG iterations "
                         "(instances 1000 .. 1000 + --search-systems) instead of gradient training")
    ap.add_argument("--search-systems", type=int, default=64)
    ap.add_argument("--headroom", action="store_true",
                    help="measure how much an over-relaxation chosen per operator could save over the global "
                         "fit: a grid around it on --search-systems training instances (report only)")
    ap.add_argument("--features", action="store_true",
                    help="after the global search, fit a per-cell over-relaxation, piecewise linear in the "
                         "local coefficient features (coordinate search on PCG iterations)")
    ap.add_argument("--refresh", type=int, default=1,
                    help="regenerate the smooth errors with the current network every this many epochs "
                         "(0: never); the slowest modes of the current factor are what the loss must see")
    ap.add_argument("--loss", default="spectral", choices=["spectral", "pair"],
                    help="spectral: log Rayleigh quotient on white-noise errors minus on smooth errors "
                         "(a log-condition proxy); pair: |P r - e|_A^2 / |e|_A^2 on the smooth errors")
    args = ap.parse_args()
    dev = torch.device("cuda")
    if args.headroom:
        net = L.FsaiNet(dev, seed=0)
        seeds = list(range(1000, 1000 + args.search_systems))
        rep = instance_headroom(net, seeds, args.m, dev, wns=[0.80, 0.85, 0.90, 0.95],
                                wvs=[0.675, 0.725, 0.775, 0.825, 0.875])
        rep["instances"] = args.search_systems
        print(json.dumps({k: v for k, v in rep.items() if k != "per_instance_best_combo"}, indent=1))
        if args.report:
            with open(args.report, "w") as f:
                json.dump(rep, f, indent=1)
        return
    if args.search:
        net = L.FsaiNet(dev, seed=0)
        val_seeds = list(range(4000, 4000 + args.val))
        before = evaluate(net, val_seeds, args.m, dev)
        t0 = time.perf_counter()
        seeds = list(range(1000, 1000 + args.search_systems))
        wn, wv, it, nev = search(net, seeds, args.m, dev)
        set_constant_output(net, math.atanh(wn), math.atanh(wv))
        rep = {"method": "direct search of the off-diagonal over-relaxation on PCG iterations",
               "train_instances": args.search_systems, "w_N": wn, "w_W": wv, "train_mean_iters": it,
               "evaluations": nev}
        if args.features:
            glob = evaluate(net, val_seeds, args.m, dev, only=("learned",))["learned"]["mean_iters"]
            theta, it2, nev2 = search_features(net, seeds, args.m, dev, wn, wv)
            set_feature_map(net, theta)
            feat = evaluate(net, val_seeds, args.m, dev, only=("learned",))["learned"]["mean_iters"]
            rep.update(method="direct search: global over-relaxation, then a per-cell map of local features",
                       theta=theta, train_mean_iters_features=it2, evaluations_features=nev2,
                       validation_global_mean_iters=glob, validation_features_mean_iters=feat)
            if feat >= glob:  # the per-cell map did not generalise: keep the global fit
                set_constant_output(net, math.atanh(wn), math.atanh(wv))
                rep["kept"] = "global"
            else:
                rep["kept"] = "features"
        t_search = time.perf_counter() - t0
        torch.save(net.state_dict(), args.out)
        after = evaluate(net, val_seeds, args.m, dev)
        rep.update(search_seconds=t_search, validation_before=before, validation_after=after)
        print(json.dumps(rep, indent=1))
        if args.report:
            with open(args.report, "w") as f:
                json.dump(rep, f, indent=1)
        return
    t0 = time.perf_counter()
    st, r, e, kind = make_pairs(list(range(1000, 1000 + args.train)), args.m, dev, white=args.loss == "spectral")
    if args.lr <= 0:
        raise SystemExit("--lr must be positive")
    t_data = time.perf_counter() - t0
    net = L.FsaiNet(dev, seed=0)
    val_seeds = list(range(4000, 4000 + args.val))
    before = evaluate(net, val_seeds, args.m, dev)
    best = {"epoch": -1, "mean_iters": before["learned"]["mean_iters"], "params": net.params.clone()}
    epochs_log = []

    def on_epoch(ep, loss):
        it = evaluate(net, val_seeds, args.m, dev, only=("learned",))["learned"]["mean_iters"]
        epochs_log.append({"epoch": ep, "loss": loss, "val_mean_iters": it})
        print(f"epoch {ep}: validation mean PCG iterations {it:.1f} (best {best['mean_iters']:.1f})", flush=True)
        if it < best["mean_iters"]:
            best.update(epoch=ep, mean_iters=it, params=net.params.clone())

    t1 = time.perf_counter()
    state, hist = {}, []
    train_seeds = list(range(1000, 1000 + args.train))
    for ep in range(args.epochs):
        if ep > 0 and args.refresh and ep % args.refresh == 0:
            del st, r, e, kind
            st, r, e, kind = make_pairs(train_seeds, args.m, dev, white=args.loss == "spectral", net=net)
        hist += L.train(net, st, r, e, epochs=1, batch=args.batch, lr=args.lr, seed=ep,
                        on_epoch=lambda _, loss: on_epoch(ep, loss), kind=kind if args.loss == "spectral" else None,
                        state=state)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    net.params.copy_(best["params"])
    torch.save(net.state_dict(), args.out)
    after = evaluate(net, val_seeds, args.m, dev)
    rep = {"train_instances": args.train, "epochs": args.epochs, "loss": args.loss, "lr": args.lr,
           "loss_history": hist, "data_seconds": t_data,
           "train_seconds": t_train, "epochs_log": epochs_log, "kept_epoch": best["epoch"],
           "validation_before": before, "validation_after": after}
    print(json.dumps(rep, indent=1))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(rep, f, indent=1)


if __name__ == "__main__":
    main()
