"""Benchmark: CG solves/sec to a 1e-8 true relative residual on the 512 x 512 variable-diffusion family.

Workload (one step): the 256 held-out instances of the 2-D variable-coefficient diffusion family
(5-point CSR, n = 262,144, Matern-3/2 log-coefficient fields, seeds 5000-5255, b ~ N(0,1)), all
solved in one batched call to |b - A x| / |b| <= 1e-8 measured in FP64.  The headline method is
FP32 preconditioned CG inside FP64 iterative refinement with the learned FSAI preconditioner
(Jacobi fallback); plain CG and Jacobi-PCG run through the same kernel for comparison.  Every timed
step includes the build of the step's preconditioner (the network's inference and the assembly of
G for all 256 operators); the network's weights and the pattern of G, which depend only on the
mesh, are loaded once before timing.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--method M]

--impl reference times the reference's CG loop (restated with the same torch CPU ops, float64,
Jacobi preconditioner, tol giving the same 1e-8 residual) on the host cores over a bounded sample.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np
import torch

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "CG solves/sec to 1e-8 rel. residual: learned mixed-prec PCG vs plain CG, 1 GB300"
UNIT = "solves/s"
WORKLOAD = "diffusion2d-512x512-family-test256"
TEST_SEEDS0 = 5000
SYSTEMS = 256
M = 512


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v: float, world: int) -> float:
    if world == 1:
        return v
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard_seeds(rank: int, systems: int) -> range:
    """Instance seeds of one rank: ranks solve disjoint sets of `systems` instances (weak scaling)."""
    return range(TEST_SEEDS0 + rank * systems, TEST_SEEDS0 + (rank + 1) * systems)


def diagonal_counts(fam):
    """Diagonals of the family's pattern and of the FSAI operator G^T G on its lower pattern."""
    ip = fam.indptr.cpu().long()
    rows = torch.repeat_interleave(torch.arange(fam.n), ip[1:] - ip[:-1])
    off = torch.unique(fam.indices.cpu().long() - rows)
    low = off[off <= 0]
    moff = torch.unique((low[None, :] - low[:, None]).flatten())
    return int(off.numel()), int(moff.numel())


def bytes_per_system_iter(n, nnz, method, schedule="cluster8", nd=5, nm=7):
    """Algorithmic memory bytes of one FP32 PCG step of one system.

    On-chip schedule: the Krylov vectors stay in the cluster's shared memory, so a step moves only
    the matrix diagonals (nd n 4 bytes; Jacobi adds 1/diag, n 4; FSAI adds the nm bfloat16
    diagonals of M = G^T G, nm n 2).  Other schedules: the CSR values (the batch shares one pattern, read from L2) + 6
    vector streams (p read, x r/w, r r/w, p write) + the preconditioner (Jacobi: the diagonal; FSAI:
    G and G^T values and the intermediate t written and read)."""
    if schedule == "onchip":
        b = nd * n * 4
        if method == "jacobi":
            b += n * 4
        elif method in ("learned", "fsai"):
            b += nm * n * 2  # M = G^T G in bfloat16
        return b
    b = nnz * 4 + 6 * n * 4
    if method == "jacobi":
        b += n * 4
    elif method in ("learned", "fsai"):
        g_nnz = (nnz + n) // 2
        b += 2 * g_nnz * 4 + 2 * n * 4
    return b


def bytes_per_replacement(n, nnz):
    """One FP64 residual replacement: x += d (x r/w, d r/w) and r = b - A x (values, x and b read, r write)."""
    return nnz * 4 + 24 * n + 20 * n


def preconditioner_builder(method, fam, dev):
    """The per-family preconditioner build, run inside every timed step: `build(family)` returns the
    (pattern, G values) of the FSAI factor from the trained network ("learned": stencil extraction,
    features, three convolutions, assembly) or in closed form ("fsai": stencil, assembly), None for
    the other methods.  What depends only on the mesh -- the network's weights and the pattern of G --
    is loaded / analysed once, here."""
    from cola_gb300.linalg.batched import FsaiPattern
    from cola_gb300.precond import learned_fsai
    if method not in ("learned", "fsai"):
        return lambda f: None
    net = None
    if method == "learned":
        if not learned_fsai.WEIGHTS.exists():
            raise FileNotFoundError(f"trained weights {learned_fsai.WEIGHTS} not found")
        net = learned_fsai.FsaiNet.load(learned_fsai.WEIGHTS, device=dev)
    pat = FsaiPattern(fam.indptr, fam.indices)
    return lambda f: learned_fsai.g_values(f, net, pat)


# this library's kernels per batch of 64 systems in a preconditioner build (learned_fsai.g_values):
# the stencil extraction and the fused build (network + assembly, or the closed form)
BUILD_LAUNCHES_PER_64 = {"learned": 2, "fsai": 2}


PRECOND = {"plain": "none", "jacobi": "jacobi", "learned": "fsai", "fsai": "fsai"}
# DRAM bytes (read + write) of one on-chip solve launch per system, from one ncu capture of
# k_onchip_pcg on 7 systems of this workload (FSAI, ~1056 steps each): 210.8 MB + 145.8 MB.  DRAM
# traffic is per system (reading its CSR values and right-hand side, writing its diagonals and x):
# the diagonals of the systems in flight are re-read from L2 at every step.
ONCHIP_DRAM_BYTES_PER_SYSTEM = 356.6e6 / 7
KERNEL_OF = {"onchip": "k_onchip_pcg", "cluster8": "k_cluster_pcg", "cluster16": "k_cluster_pcg",
             "grid": "k_batched_ir"}


def launches_per_solve(schedule, method, systems, spare="off"):
    """This library's kernels per timed step: the preconditioner build, then per chunk of <= 1024
    systems the on-chip schedule runs the pattern analysis (bitmap + collect, for A and, with FSAI,
    for G) and the solve kernel (plus the companion kernel with spare="auto"); the other schedules
    one solve kernel."""
    chunks = (systems + 1023) // 1024
    build = BUILD_LAUNCHES_PER_64.get(method, 0) * ((systems + 63) // 64)
    if schedule == "onchip":
        return build + chunks * (1 + 2 * (2 if PRECOND[method] == "fsai" else 1) + (1 if spare == "auto" else 0))
    return build + chunks


def companion_roofline(systems, mean_steps, n, nd, nm, solve_s, hbm_peak):
    """The on-chip schedule's companion CTAs (one per SM the clusters leave free) stream each system
    they solve from global memory: per CG step and row the matrix (nd FP32 + nm bfloat16 diagonals)
    and 48 B of FP32 vector traffic (A p: p read, A p written; r update: r r/w, A p read; M r: r read,
    z written; p / d update: z read, p r/w, d r/w).  `systems` is what they solved in the waited
    last warm-up step of the same batch (the split between the two kernels varies a little run to run)."""
    if systems is None:
        return None
    per_row = nd * 4 + nm * 2 + 48
    nbytes = systems * mean_steps * per_row * n
    return {"systems_per_step": systems, "bytes_per_row_step": per_row, "dram_bytes_est": nbytes,
            "dram_gbs_est": nbytes / solve_s / 1e9, "dram_frac_est": nbytes / solve_s / 1e9 / hbm_peak,
            "note": "the companions' DRAM traffic is not in `traffic` (an ncu capture of the clusters alone)"}


def read_bandwidth(dev, nbytes: int, reps=(2, 12), tries: int = 3) -> float:
    """Read bandwidth in GB/s of this library's streaming probe over an nbytes buffer: the time of
    reps[1] - reps[0] extra passes (CUDA events on the launching stream, best of `tries`).  A buffer
    that fits in L2 gives the L2 -> SM read bandwidth."""
    import ctypes as C
    from cola_gb300 import _capi
    lib = _capi.load()
    buf = torch.ones(nbytes // 4, dtype=torch.float32, device=dev)
    sink = torch.zeros(1, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)

    def timed(r):
        best = float("inf")
        for _ in range(tries):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            _capi.check(lib.colagb_read_bandwidth_probe(C.c_void_p(buf.data_ptr()), buf.numel() * 4, r,
                                                        C.c_void_p(sink.data_ptr()), C.c_void_p(st.cuda_stream)),
                        "read probe")
            b.record(st)
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(b) / 1e3)
        return best

    timed(reps[0])  # warm: the buffer is now resident in L2 if it fits
    t0, t1 = timed(reps[0]), timed(reps[1])
    return nbytes * (reps[1] - reps[0]) / max(t1 - t0, 1e-9) / 1e9


def independent_quality(fam, B, X, sample: int = 8, tol64: float = 1e-13, max_iters: int = 40000):
    """Checks of a batched solve that share no code with the solver: for `sample` systems spread over
    the batch, the FP64 true relative residual |b - A x| / |b| with torch's sparse CSR product, and the
    relative error of x against an FP64 Jacobi-preconditioned CG run to relres tol64 in plain torch
    tensor ops (all sampled systems advanced together, one set of CG scalars per system)."""
    S, n = X.shape
    idx = sorted({int(round(i * (S - 1) / max(sample - 1, 1))) for i in range(min(sample, S))})
    ip, ix = fam.indptr.long(), fam.indices.long()
    nnz = ix.numel()
    k = len(idx)
    vals = fam.values[idx].double()
    # block-diagonal CSR of the sampled systems
    bip = torch.cat([ip[:-1] + j * nnz for j in range(k)] + [torch.tensor([k * nnz], device=ip.device)])
    bix = torch.cat([ix + j * n for j in range(k)])
    Ab = torch.sparse_csr_tensor(bip, bix, vals.reshape(-1), (k * n, k * n))

    def mv(v):  # (k, n) -> (k, n)
        return (Ab @ v.reshape(-1, 1)).reshape(k, n)

    b = B[idx].double()
    x = X[idx].double()
    relres = ((b - mv(x)).norm(dim=1) / b.norm(dim=1))
    rows = torch.repeat_interleave(torch.arange(n, device=ip.device), ip[1:] - ip[:-1])
    dg = torch.zeros(k, n, dtype=torch.float64, device=ip.device)
    dg.index_add_(1, rows, torch.where((rows == ix)[None, :], vals, torch.zeros_like(vals)))
    dinv = 1.0 / dg
    x64 = torch.zeros_like(b)
    r = b.clone()
    z = dinv * r
    p = z.clone()
    rz = (r * z).sum(1)
    bn = b.norm(dim=1)
    it = 0
    for it in range(1, max_iters + 1):
        ap = mv(p)
        al = rz / (p * ap).sum(1)
        x64 += al[:, None] * p
        r -= al[:, None] * ap
        if it % 50 == 0 and bool(((r.norm(dim=1) / bn) < tol64).all()):
            break
        z = dinv * r
        rz2 = (r * z).sum(1)
        p = z + (rz2 / rz)[:, None] * p
        rz = rz2
    relres64 = ((b - mv(x64)).norm(dim=1) / bn)
    err = ((x - x64).norm(dim=1) / x64.norm(dim=1))
    return {"sampled_systems": idx, "max_true_relres_indep": float(relres.max()),
            "max_sol_err_vs_fp64": float(err.max()),
            "fp64_oracle": f"Jacobi-PCG in torch FP64 tensor ops, {it} steps, max relres "
                           f"{float(relres64.max()):.1e}"}


def run_ours(args, world, rank, local):
    import cola_gb300 as cola
    from cola_gb300 import _capi
    from cola_gb300.linalg.batched import solve_batched
    from cola_gb300.workloads import diffusion_family_2d

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _capi.load()
    fam, B, coeff, _ = diffusion_family_2d(shard_seeds(rank, args.systems), m=args.m, device=dev)
    n, nnz = fam.n, fam.indices.numel()
    method = args.method
    try:
        build = preconditioner_builder(method, fam, dev)
    except FileNotFoundError as e:  # trained weights missing: say so and time Jacobi-PCG
        print(f"# learned preconditioner unavailable ({e}); timing jacobi", file=sys.stderr)
        method = "jacobi"
        build = preconditioner_builder(method, fam, dev)
    prec = PRECOND[method]
    kw = dict(precond=prec, tol=1e-8, inner_tol=args.inner_tol, mode=args.mode, schedule=args.schedule,
              spare=args.spare)
    st = torch.cuda.current_stream(dev)

    side = torch.cuda.Stream(dev)  # the next step's preconditioner build

    def build_on_side(f, after=None):
        """f's preconditioner, built on the side stream (after event `after`); (fsai, ready event)."""
        with torch.cuda.stream(side):
            if after is not None:
                side.wait_event(after)
            fs = build(f)
            ready = torch.cuda.Event()
            ready.record(side)
        return fs, ready

    def run_steps(k, marks=None, wait_last=False):
        """k steps on the resident family.  Step i's solve runs on the main stream; step i + 1's
        preconditioner is built on the side stream meanwhile, on the SMs that the solve's persistent
        clusters leave free (112 of the 152 hold the on-chip schedule).  Each step still builds its
        own preconditioner: the first build is inside the run, the others overlap a solve."""
        start = torch.cuda.Event()
        start.record(st)
        fs, ready = build_on_side(fam, start)
        infos = []
        X = None
        for i in range(k):
            st.wait_event(ready)
            if marks:
                marks[i][0].record(st)
            X, info = solve_batched(fam, B, fsai=fs, wait=wait_last and i == k - 1, **kw)
            if marks:
                marks[i][1].record(st)
            if fs is not None:
                fs[1].record_stream(st)  # G values allocated on the side stream, read by this solve
            infos.append(info)
            if i + 1 < k:
                fs, ready = build_on_side(fam)
        return X, infos

    X, infos = run_steps(max(1, args.warmup), wait_last=True)
    sweeps_max = infos[-1]["sweeps"]  # the timed steps solve the same systems
    companion_systems = infos[-1].get("companion_systems")
    torch.cuda.synchronize()
    b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    b0.record(st)
    build(fam)
    b1.record(st)
    torch.cuda.synchronize()
    build_ms = b0.elapsed_time(b1)  # one build alone, for the report
    barrier(world)
    marks = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(args.steps)]
    e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        torch.cuda.nvtx.range_push("timed")  # lets a profiler capture exactly the timed steps
        e_start.record(st)
        X, infos = run_steps(args.steps, marks)
        e_end.record(st)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        wall = time.perf_counter() - t0
    barrier(world)
    t_dev = e_start.elapsed_time(e_end) / 1e3
    t_solve = sum(m0.elapsed_time(m1) for m0, m1 in marks) / 1e3  # the solve calls alone
    t_max = max_over_ranks(t_dev, world)
    iters_total = sum(int(inf["iterations"].sum().item()) for inf in infos)
    info = infos[-1]
    relres_max = max(float(inf["relres"].max().item()) for inf in infos)
    status_ok = all(bool(torch.all((inf["status"] == 1) | (inf["status"] == 5)).item()) for inf in infos)
    value = world * args.systems * args.steps / t_max

    # end to end through the public API from pinned host buffers: every step copies its family's
    # values and right-hand sides in (H2D), builds the preconditioner, solves and copies the solutions
    # out (D2H).  The copies run on two copy streams and the build on the side stream, all overlapping
    # the neighbouring steps' solves (double-buffered device inputs), the way a stream of families
    # would be fed.
    vals_h = fam.values.cpu().pin_memory()
    B_h = B.cpu().pin_memory()
    X_h = [torch.empty_like(B_h).pin_memory() for _ in range(2)]
    e2e_steps = max(1, args.steps)
    from cola_gb300.linalg.batched import BatchedCSR
    h2d_s, d2h_s = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    vals_buf = [torch.empty_like(fam.values) for _ in range(2)]
    B_buf = [torch.empty_like(B) for _ in range(2)]
    free = [torch.cuda.Event() for _ in range(2)]   # input buffer k no longer read by its solve
    for k in range(2):
        free[k].record(st)

    def e2e_run(nsteps, marks=None):
        start = torch.cuda.Event()
        start.record(st)

        def copy_in(i):  # step i's H2D, then its preconditioner build on the side stream
            k = i % 2
            with torch.cuda.stream(h2d_s):
                h2d_s.wait_event(start)
                h2d_s.wait_event(free[k])
                vals_buf[k].copy_(vals_h, non_blocking=True)
                B_buf[k].copy_(B_h, non_blocking=True)
                arrived = torch.cuda.Event()
                arrived.record(h2d_s)
            fam_d = BatchedCSR(fam.indptr, fam.indices, vals_buf[k])
            fs, ready = build_on_side(fam_d, arrived)
            return fam_d, fs, ready

        nxt = copy_in(0)
        for i in range(nsteps):
            k = i % 2
            fam_d, fs, ready = nxt
            st.wait_event(ready)
            if marks:
                marks[i][0].record(st)
            Xd, _ = solve_batched(fam_d, B_buf[k], fsai=fs, wait=False, **kw)
            free[k].record(st)
            if fs is not None:
                fs[1].record_stream(st)
            if marks:
                marks[i][1].record(st)
            with torch.cuda.stream(d2h_s):
                d2h_s.wait_event(free[k])
                X_h[k].copy_(Xd, non_blocking=True)
            Xd.record_stream(d2h_s)
            if i + 1 < nsteps:
                nxt = copy_in(i + 1)  # copies and build of the next step overlap this solve
        st.wait_stream(d2h_s)

    e2e_run(1)  # untimed: the device buffers of this path come from the allocator's cache afterwards
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    marks = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(e2e_steps)]
    e0.record(st)
    e2e_run(e2e_steps, marks)
    e1.record(st)
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(e0.elapsed_time(e1) / 1e3, world)
    solve_ms = sum(m[0].elapsed_time(m[1]) for m in marks)
    e2e = {"value": world * args.systems * e2e_steps / t_e2e, "unit": UNIT,
           "h2d_bytes_per_step": vals_h.numel() * 4 + B_h.numel() * 8, "d2h_bytes_per_step": X_h[0].numel() * 8,
           "ms_per_step": 1e3 * t_e2e / e2e_steps, "steps": e2e_steps,
           "copies": "H2D and D2H on two copy streams, overlapping the neighbouring steps' solves; each "
                     "step's preconditioner build on a third stream after its H2D",
           "split_ms": {"first_h2d_and_build": e0.elapsed_time(marks[0][0]),
                        "solve_per_step": solve_ms / e2e_steps, "last_d2h": marks[-1][1].elapsed_time(e1)}}

    hbm_peak, hbm_kind = peaks()
    # CG steps only: the FP64 residual replacements (about 1 % of the traffic) are left out, so the
    # achieved figure is a lower bound
    sched_ran = info.get("schedule", args.schedule)
    nd, nm = diagonal_counts(fam)
    alg_bytes_step = (iters_total / args.steps) * bytes_per_system_iter(n, nnz, method, sched_ran, nd, nm)
    # over the solve call (pattern analysis + k_onchip_pcg); the preconditioner build is timed apart
    solve_s = t_solve / args.steps
    achieved = alg_bytes_step / solve_s / 1e9
    # The on-chip kernel re-reads its diagonals from L2 at every step (the systems in flight fit in
    # L2): its roofline denominator is the L2 -> SM read bandwidth, measured here on a buffer of the
    # same size as that working set; the HBM figures are reported beside it.
    onchip = sched_ran == "onchip"
    l2_gbs = read_bandwidth(dev, 64 << 20)
    dram = ONCHIP_DRAM_BYTES_PER_SYSTEM * args.systems if onchip else None
    roof = {"bound": "l2" if onchip else "hbm", "achieved": achieved,
            "peak": l2_gbs if onchip else hbm_peak, "unit": "GB/s",
            "frac": achieved / (l2_gbs if onchip else hbm_peak),
            "peak_kind": ("measured in this run: L2 -> SM read stream over a 64 MB L2-resident buffer "
                          "(colagb_read_bandwidth_probe)") if onchip else hbm_kind,
            "traffic": dram,
            "traffic_note": "ncu DRAM bytes of a 7-system capture scaled by systems" if onchip else None,
            "l2_read_gbs": l2_gbs,
            "hbm": {"peak": hbm_peak, "peak_kind": hbm_kind,
                    "dram_gbs": dram / solve_s / 1e9 if dram is not None else None,
                    "dram_frac": dram / solve_s / 1e9 / hbm_peak if dram is not None else None,
                    "alg_gbs_over_hbm_peak": achieved / hbm_peak},
            "binding": ("per-SM L1/shared-memory data path and step latency: the matrix diagonals stream from "
                        "L2 (ncu: 96 % L2 hit rate, DRAM 0.3 % busy), the Krylov vectors live in shared "
                        "memory, each step ends in cluster-wide reductions") if onchip else
                       "HBM streaming of the CSR values and Krylov vectors",
            "kernel": KERNEL_OF.get(sched_ran, "k_cluster_pcg"), "schedule": sched_ran,
            "alg_bytes_per_launch": alg_bytes_step,
            "companions": companion_roofline(companion_systems, iters_total / args.steps / args.systems,
                                             n, nd, nm, solve_s, hbm_peak) if onchip else None,
            "solve_ms_per_step": 1e3 * solve_s,
            "build_ms_alone": build_ms,
            "build_overlap": "step i + 1's build runs beside step i's solve on a second stream"}
    quality = {"max_true_relres_fp64": relres_max, "all_converged": status_ok,
               "mean_inner_iters_per_system": iters_total / args.steps / args.systems,
               "max_fp64_replacements": sweeps_max}
    quality.update(independent_quality(fam, B, X))
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32-inner/f64-refinement", "data": "synthetic",
        "config": {"workload": WORKLOAD, "systems_per_gpu": args.systems, "grid": f"{args.m}x{args.m}", "n": n,
                   "nnz": nnz, "method": method, "tol": 1e-8, "refinement": args.mode, "inner_tol": args.inner_tol,
                   "schedule": sched_ran, "spare_sms": args.spare,
                   "l2": "inputs larger than L2 (CSR values + right-hand sides > 1.5 GB per step)",
                   "parallelism": f"replicas{world}"},
        "quality": quality,
        "e2e": e2e,
        "roofline": roof,
        "gpu_launches": args.steps * launches_per_solve(sched_ran, method, args.systems, args.spare),
        "wall_s_timed": wall,
    }
    clk_s = clk.summary()
    if clk_s:
        out["clocks"] = clk_s
    if args.compare and args.compare != "none" and rank == 0:
        cmp = {}
        for mth in args.compare.split(","):
            if mth == method:
                continue
            try:
                build2 = preconditioner_builder(mth, fam, dev)
            except FileNotFoundError:
                continue
            kw2 = dict(precond=PRECOND[mth], tol=1e-8, inner_tol=args.inner_tol, mode=args.mode,
                       schedule=args.schedule)
            solve_batched(fam, B, fsai=build2(fam), **kw2)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            _, inf2 = solve_batched(fam, B, fsai=build2(fam), **kw2)
            b.record(st)
            torch.cuda.synchronize()
            t2 = a.elapsed_time(b) / 1e3
            cmp[mth] = {"value": args.systems / t2, "unit": UNIT,
                        "mean_inner_iters_per_system": float(inf2["iterations"].double().mean().item()),
                        "max_true_relres_fp64": float(inf2["relres"].max().item())}
        out["compare"] = cmp
        if "plain" in cmp:
            out["speedup_vs_plain_cg"] = value / world / cmp["plain"]["value"]
    if rank == 0 and args.cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args, fam, B, sample_s=args.cpu_seconds)
    return out


def reference_package():
    """The unmodified reference package (`cola`), installed by pip into baseline/_ref, or None.

    Its two dependencies that no wheel here provides (plum, optree) come from the test-only stand-ins
    under tests/golden/_shims; where tqdm is absent (it is only used for progress bars, which stay
    off), a silent stand-in module is registered.  The reference's own code runs unchanged."""
    ref = ROOT / "baseline" / "_ref"
    if not (ref / "cola").is_dir():
        return None
    for pth in (str(ref), str(ROOT / "tests" / "golden" / "_shims")):
        if pth not in sys.path:
            sys.path.insert(0, pth)
    import importlib.util

    def _have(name):
        if name in sys.modules:  # includes the stand-in below, registered by an earlier call
            return True
        try:
            return importlib.util.find_spec(name) is not None
        except (ImportError, ValueError):
            return False
    if not _have("tqdm"):
        import types

        class _Bar:
            def __init__(self, *a, **k):
                pass

            def update(self, *a, **k):
                pass

            def set_description(self, *a, **k):
                pass

            def close(self):
                pass
        mod, auto = types.ModuleType("tqdm"), types.ModuleType("tqdm.auto")
        mod.tqdm = auto.tqdm = _Bar
        mod.auto = auto
        sys.modules["tqdm"], sys.modules["tqdm.auto"] = mod, auto
    import cola
    return cola


def _jacobi_inputs(fam, B, s):
    indptr, indices = fam.indptr.cpu().long(), fam.indices.cpu().long()
    n = fam.n
    vals = fam.values[s].double().cpu()
    rows = torch.repeat_interleave(torch.arange(n), indptr[1:] - indptr[:-1])
    dg = torch.zeros(n, dtype=torch.float64)
    dg.index_add_(0, rows, torch.where(rows == indices, vals, torch.zeros_like(vals)))
    return indptr, indices, rows, vals, dg, B[s].double().cpu()


def cpu_baseline(args, fam, B, sample_s=15.0):
    """The reference's Jacobi-preconditioned CG on the host cores (all threads, float64), over a bounded
    sample of the same instances: cola.linalg.solve(PSD(Sparse), b, CG(tol=5e-9, P=Diagonal(1/diag)))
    of the installed reference package (kind "reference"); without it, the repo's restatement of the
    reference CG loop with the same torch CPU ops (kind "port")."""
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    cola_ref = reference_package()
    n = fam.n
    done, t_used, iters, worst = 0, 0.0, [], 0.0
    s = 0
    op_kind = "Sparse"
    while t_used < sample_s and s < fam.num_systems:
        indptr, indices, rows, vals, dg, b = _jacobi_inputs(fam, B, s)
        Acsr = torch.sparse_csr_tensor(indptr, indices, vals, (n, n))
        if cola_ref is not None:
            # the reference's own operator and algorithm objects; building the CSR (host scipy) is set-up.
            # Its Sparse pairs row-argsorted values with scipy's column-sorted indices through an
            # unstable argsort (operators.py:64-76): where that reorders the (row-sorted) triplets, the
            # operator is not the given matrix, and the same CSR product (Sparse._matmat, operators.py:77-78)
            # is wrapped in the reference's LinearOperator base class instead.
            A0 = cola_ref.ops.Sparse(vals, rows, indices, (n, n))
            probe = torch.randn(n, dtype=torch.float64, generator=torch.Generator().manual_seed(s))
            if not torch.allclose(A0 @ probe, Acsr @ probe, rtol=1e-12, atol=0.0):
                op_kind = "LinearOperator(CSR @ X) (the reference's Sparse reordered the values on this host)"

                class _CSR(cola_ref.ops.LinearOperator):
                    def __init__(self, M):
                        super().__init__(dtype=M.dtype, shape=M.shape)
                        self.M = M

                    def _matmat(self, X):
                        return self.M @ X
                A0 = _CSR(Acsr)
            A = cola_ref.PSD(A0)
            P = cola_ref.ops.Diagonal(1.0 / dg)
            alg = cola_ref.linalg.CG(tol=5e-9, max_iters=100000, P=P)
            t0 = time.perf_counter()
            Ainv = cola_ref.linalg.inv(A, alg)
            x = Ainv @ b
            t_used += time.perf_counter() - t0
            iters.append(int(Ainv.info["iterations"]) if hasattr(Ainv, "info") and "iterations" in Ainv.info else -1)
        else:
            from oracle.torch_ref import csr_matmat, run_batched_cg
            mm = csr_matmat(indptr.int(), indices.int(), vals, n)
            dinv = (1.0 / dg)[:, None]
            t0 = time.perf_counter()
            # stop rule |r_rec| <= 2 tol on the normalised system; tol = 5e-9 targets a 1e-8 residual
            xk, k, _ = run_batched_cg(mm, b[:, None], torch.zeros_like(b[:, None]), 100000, 5e-9,
                                      precond=lambda r: dinv * r)
            t_used += time.perf_counter() - t0
            x = xk[:, 0]
            iters.append(k)
        rr = float((b - Acsr @ x).norm() / b.norm())
        worst = rr if (rr != rr or worst != worst) else max(worst, rr)  # a NaN stays visible
        done += 1
        s += 1
    kind = "reference" if cola_ref is not None else "port"
    what = (f"cola.linalg.inv(PSD({op_kind}), CG(tol=5e-9, P=Diagonal(1/diag))) @ b of the reference package"
            if cola_ref is not None else "the reference CG loop restated on torch CPU ops")
    return {"value": done / t_used, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": f"{done} of the {fam.num_systems} instances, {what}, float64, "
                      f"{statistics.mean(iters):.0f} iterations each, max true relres {worst:.2e}",
            "seconds": t_used}


def _reference_csr(cola_ref, indptr, indices, vals, n):
    """The reference's Sparse operator for a CSR matrix; where its construction reorders the values
    (an unstable argsort, operators.py:64-76), the same CSR product (Sparse._matmat, operators.py:77-78)
    in the reference's LinearOperator base class.  Returns (operator, description)."""
    indptr, indices = indptr.long(), indices.long()
    rows = torch.repeat_interleave(torch.arange(n), indptr[1:] - indptr[:-1])
    Acsr = torch.sparse_csr_tensor(indptr, indices, vals, (n, n))
    A0 = cola_ref.ops.Sparse(vals, rows, indices, (n, n))
    probe = torch.randn(n, dtype=vals.dtype, generator=torch.Generator().manual_seed(0))
    if torch.allclose(A0 @ probe, Acsr @ probe, rtol=1e-5, atol=1e-6):
        return A0, "Sparse"

    class _CSR(cola_ref.ops.LinearOperator):
        def __init__(self, M):
            super().__init__(dtype=M.dtype, shape=M.shape)
            self.M = M

        def _matmat(self, X):
            return self.M @ X
    return _CSR(Acsr), "LinearOperator(CSR @ X)"


def _reference_lanczos_step_seconds(cola_ref, op, rhs, m, k_steps=3):
    """Seconds per step of the reference's own Lanczos (lanczos_fact's body, lanczos.py:238-253) on the
    operator and start block, with the (bs, n, m + 2) basis of an m-step run: its loop driver is
    replaced for the duration by one that runs k_steps of the body (after one untimed step) and stops.
    The reference reorthogonalises against all m + 2 columns at every step (lanczos.py:287-296), so every
    step costs the same and a run costs m of them."""
    from cola.linalg.decompositions import lanczos as ref_lanczos
    xnp = op.xnp
    timing = {}
    original = xnp.while_loop_winfo

    def bounded(error, tol, max_iters, pbar=False, **kw):
        def while_fn(cond_fun, body_fun, state):
            state = body_fun(state)
            t0 = time.perf_counter()
            for _ in range(k_steps):
                state = body_fun(state)
            timing["t"] = (time.perf_counter() - t0) / k_steps
            return state
        return while_fn, {}
    xnp.while_loop_winfo = bounded
    try:
        init = ref_lanczos.init_lanczos(xnp, rhs, m, op.dtype)
        ref_lanczos.lanczos_fact(op, init, max_iters=m, tol=0.0)
    finally:
        xnp.while_loop_winfo = original
    return timing["t"]


def config_reference_cpu(config):
    """The reference package on the host cores (all threads) for a benchmark configuration, on a bounded
    sample of the workload (stated in `sample`), same inputs as the GPU line.  None without the package."""
    cola_ref = reference_package()
    if cola_ref is None:
        return {"unavailable": "the reference package is not installed in baseline/_ref"}
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    from cola_gb300 import workloads as W
    out = {"kind": "reference", "cores": threads}
    if config == "c1":
        A, b, _ = W.dense_spd(2048, seed=0, lo=1e-2, hi=1e2, dtype=torch.float32)
        t0 = time.perf_counter()
        Ainv = cola_ref.linalg.inv(cola_ref.PSD(cola_ref.ops.Dense(A)), cola_ref.linalg.CG(tol=1e-6, max_iters=2000))
        x = Ainv @ b
        t = time.perf_counter() - t0
        out.update(value=1.0 / t, unit="solves/s", seconds=t,
                   sample=f"one full FP32 solve, {int(Ainv.info['iterations'])} CG iterations")
    elif config == "c2":
        ip, ix, v = W.diffusion_3d(m=128, device="cpu")
        n = ip.numel() - 1
        A, kind = _reference_csr(cola_ref, ip, ix, v, n)
        rows = torch.repeat_interleave(torch.arange(n), (ip[1:] - ip[:-1]).long())
        dg = torch.zeros(n).index_add_(0, rows, torch.where(rows == ix.long(), v, torch.zeros_like(v)))
        Bm = torch.randn(n, 32, generator=torch.Generator().manual_seed(2))
        its = 50
        alg = cola_ref.linalg.CG(tol=1e-30, max_iters=its, P=cola_ref.ops.Diagonal(1.0 / dg))
        t0 = time.perf_counter()
        X = cola_ref.linalg.inv(cola_ref.PSD(A), alg) @ Bm
        t = time.perf_counter() - t0
        steps = 427  # Jacobi-PCG steps to a 1e-8 FP64 residual on this operator (the GPU line's count)
        out.update(value=32.0 / (t / its * steps), unit="rhs/s", seconds=t,
                   sample=f"{its} Jacobi-PCG iterations of all 32 right-hand sides on the reference's {kind} "
                          f"(FP32), extrapolated to the {steps} iterations a 1e-8 residual takes")
    elif config == "c3a":
        mats, rhs, meta = W.rbf_systems(num=256, seed=3, device="cpu")
        done, t = 0, 0.0
        for A, b in zip(mats, rhs):
            t0 = time.perf_counter()
            cola_ref.linalg.inv(cola_ref.PSD(cola_ref.ops.Dense(A)), cola_ref.linalg.CG(tol=1e-6, max_iters=2000)) @ b
            t += time.perf_counter() - t0
            done += 1
            if t > 20.0:
                break
        out.update(value=done / t, unit="systems/s", seconds=t,
                   sample=f"the first {done} of the 256 systems, one reference CG call each (FP32)")
    elif config == "c3b":
        Ks, _ = W.kron_rbf(seed=4, device="cpu")
        K = cola_ref.ops.Kronecker(*[cola_ref.ops.Dense(k) for k in Ks])
        op = cola_ref.PSD(K + 0.01 * cola_ref.ops.I_like(K))
        bs, steps = 8, 100
        from cola_gb300.linalg.prng import randn as keyed_randn
        Z = torch.sign(keyed_randn(op.shape[0], 64, dtype=torch.float32, key=5))[:, :bs].contiguous()
        t = _reference_lanczos_step_seconds(cola_ref, op, Z, steps)
        total = t * steps * (64 / bs)
        out.update(value=1.0 / total, unit="logdets/s", seconds=t,
                   sample=f"3 steps of the reference's own Lanczos on {bs} of the 64 probes with the 102-column "
                          f"basis (per step {t:.2f} s), times {steps} steps and 64/{bs}")
    elif config == "c5":
        A1, _, _ = W.dense_spd(1024, seed=6, lo=1e-2, hi=1e1, dtype=torch.float32)
        A2, _, _ = W.dense_spd(1024, seed=61, lo=1e-2, hi=1e1, dtype=torch.float32)
        n = 1 << 20
        ip, ix, v = W.rgg_laplacian(n, 0.002, seed=7, device="cpu")
        L, kind = _reference_csr(cola_ref, ip, ix, v, n)
        op = cola_ref.SelfAdjoint(cola_ref.ops.Kronecker(cola_ref.ops.Dense(A1), cola_ref.ops.Dense(A2)) + L)
        steps = 256
        from cola_gb300.linalg.prng import PRNGKey, randn as keyed_randn
        start = keyed_randn(n, dtype=torch.float32, key=PRNGKey(42))[:, None]
        t = _reference_lanczos_step_seconds(cola_ref, op, start, steps)
        out.update(value=1.0 / (t * steps), unit="eigensolves/s", seconds=t,
                   sample=f"3 steps of the reference's own Lanczos (Kronecker + {kind}, 258-column basis; per step "
                          f"{t:.2f} s), times {steps} steps")
    return out


def run_reference(args, world, rank):
    if rank != 0:
        return None
    from cola_gb300.workloads import diffusion_family_2d
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    fam, B, _, _ = diffusion_family_2d(range(TEST_SEEDS0, TEST_SEEDS0 + max(1, args.ref_systems)), m=args.m,
                                       device=dev)
    vals = []
    cb = None
    if args.warmup > 0:  # untimed: one bounded sample warms the host's thread pool and caches
        cpu_baseline(args, fam, B, sample_s=0.5)
    for _ in range(args.steps):
        cb = cpu_baseline(args, fam, B, sample_s=args.ref_seconds)
        vals.append(cb["value"])
    v = statistics.mean(vals)
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "grid": f"{args.m}x{args.m}", "method": "jacobi-cg (reference)",
                       "tol": 1e-8},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cb["cores"], "kind": cb["kind"],
                             "sample": cb["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c4", choices=["c1", "c2", "c3a", "c3b", "c4", "c5"],
                    help="c4 (default): the headline family; the others print one measurement line each")
    ap.add_argument("--method", default="learned", choices=["learned", "fsai", "jacobi", "plain"])
    ap.add_argument("--compare", default="plain,jacobi,fsai",
                    help="methods timed once each beside the headline (same schedule): plain CG, Jacobi PCG, "
                         "closed-form FSAI PCG ('none': no comparison)")
    ap.add_argument("--systems", type=int, default=SYSTEMS)
    ap.add_argument("--m", type=int, default=M)
    ap.add_argument("--inner-tol", type=float, default=None)
    ap.add_argument("--mode", default="reliable", choices=["reliable", "restart"])
    ap.add_argument("--schedule", default="auto", choices=["auto", "grid", "cluster8", "cluster16", "onchip"])
    ap.add_argument("--spare", default="auto", choices=["off", "auto"],
                    help="on-chip schedule: also solve systems on the SMs its clusters leave free")
    ap.add_argument("--cpu-baseline", type=int, default=1)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-seconds", type=float, default=20.0)
    ap.add_argument("--ref-systems", type=int, default=4)
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.config != "c4":
        from cola_gb300 import _capi, configs
        _capi.load()
        if rank == 0:
            line = configs.RUNNERS[args.config]()
            roof = line.get("roofline")
            if isinstance(roof, dict) and roof.get("bound") == "hbm" and "achieved_gbs" in roof:
                roof["peak"], roof["peak_kind"] = peaks()
                roof["unit"] = "GB/s"
                roof["frac"] = roof["achieved_gbs"] / roof["peak"]
            if args.cpu_baseline:
                line["cpu_reference"] = config_reference_cpu(args.config)
            print(json.dumps(line))
        return
    if args.impl == "reference":
        out = run_reference(args, world, rank)
    else:
        out = run_ours(args, world, rank, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
