"""Schedule autotuner for the batched shared-pattern solver, with a persistent JSON cache.

``solve_batched(..., schedule="tuned")`` picks, per (GPU, pattern signature, n, nnz, systems,
preconditioner, matvec storage), the schedule whose measured time per CG step and system is lowest
among the ones the pattern supports (on-chip, 8- or 16-CTA clusters, cooperative grid).  The first
solve of a new key runs each candidate once on a few of the systems with the step count capped
(a short timed probe, CUDA events on the current stream) and records the winner; later solves read
it from the cache.  The cache lives in ``$COLA_GB300_TUNE_CACHE`` (default
``~/.cache/cola_gb300/tune.json``); deleting the file re-tunes.

The chosen schedule changes only the order of floating-point reductions, never the algorithm: a tuned
solve returns exactly what an explicit ``schedule=<winner>`` solve returns.
"""
from __future__ import annotations

import hashlib
import json
import os
import threading
import time
from pathlib import Path

import torch

CANDIDATES = ("onchip", "cluster8", "cluster16", "grid", "block")
_lock = threading.Lock()
_mem: dict | None = None


def cache_path() -> Path:
    p = os.environ.get("COLA_GB300_TUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "cola_gb300" / "tune.json"


def _load() -> dict:
    global _mem
    path = cache_path()
    if _mem is not None and _mem.get("__path__") == str(path):
        return _mem
    data = {}
    try:
        data = json.loads(path.read_text())
    except (OSError, ValueError):
        data = {}
    data["__path__"] = str(path)
    _mem = data
    return data


def _save(data: dict) -> None:
    path = cache_path()
    path.parent.mkdir(parents=True, exist_ok=True)
    out = {k: v for k, v in data.items() if k != "__path__"}
    tmp = path.with_suffix(".tmp")
    tmp.write_text(json.dumps(out, indent=1, sort_keys=True))
    os.replace(tmp, path)


def gpu_key(dev: torch.device) -> str:
    p = torch.cuda.get_device_properties(dev)
    return f"{p.name}|sm{p.major}{p.minor}|{p.multi_processor_count}"


def pattern_signature(indptr: torch.Tensor, indices: torch.Tensor) -> str:
    """A short hash of the CSR pattern's row lengths and column offsets (first 4096 rows) -- what
    decides which schedules apply and how they perform."""
    ip = indptr[: 4097].to("cpu", torch.int64)
    ix = indices[: int(ip[-1])].to("cpu", torch.int64)
    rows = torch.repeat_interleave(torch.arange(ip.numel() - 1), ip[1:] - ip[:-1])
    h = hashlib.sha256()
    h.update((ip[1:] - ip[:-1]).numpy().tobytes())
    h.update((ix - rows).numpy().tobytes())
    return h.hexdigest()[:16]


def key_of(A, systems: int, precond: str, matvec: str, dev: torch.device) -> str:
    return "|".join([gpu_key(dev), pattern_signature(A.indptr, A.indices), f"n{A.n}", f"nnz{A.indices.numel()}",
                     f"S{systems}", f"P{precond}", f"mv{matvec}"])


def choose(key: str, measure) -> str:
    """The cached schedule for `key`, or the fastest of `measure(schedule) -> seconds per step`
    (None for a schedule that does not apply), recorded in the cache."""
    with _lock:
        data = _load()
        hit = data.get(key)
        if hit is not None:
            return hit["schedule"]
    times = {}
    for sched in CANDIDATES:
        t = measure(sched)
        if t is not None:
            times[sched] = t
    if not times:
        raise RuntimeError("schedule autotuner: no schedule applies to this family")
    best = min(times, key=times.get)
    with _lock:
        data = _load()
        data[key] = {"schedule": best, "us_per_step_system": {k: 1e6 * v for k, v in times.items()},
                     "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
        _save(data)
    return best


def probe_measure(solve, A, B, precond: str, fsai, matvec: str, probe_systems: int = 16, probe_steps: int = 300):
    """measure(schedule): one capped solve of the first `probe_systems` systems (after an untimed one
    that pays for set-up), returning seconds per CG step and system; None if the schedule refuses."""
    from .linalg.batched import BatchedCSR
    S = B.shape[0]
    m = min(S, probe_systems)
    sub = A if A.shared else BatchedCSR(A.indptr, A.indices, A.values[:m])
    Bs = B[:m]
    fs = None
    if fsai is not None:
        fs = (fsai[0], fsai[1][:m])

    def measure(sched):
        kw = dict(precond=precond, fsai=fs, schedule=sched, matvec=matvec, max_inner_iters=probe_steps,
                  max_sweeps=1000, tol=1e-30)
        try:
            solve(sub, Bs, **kw)
        except NotImplementedError:
            return None
        st = torch.cuda.current_stream(Bs.device)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        _, info = solve(sub, Bs, **kw)
        b.record(st)
        torch.cuda.synchronize()
        steps = max(1, int(info["iterations"].sum()))
        return a.elapsed_time(b) / 1e3 / steps
    return measure
