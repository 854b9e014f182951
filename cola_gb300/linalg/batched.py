"""Many independent SPD systems that share one CSR sparsity pattern (a family of operators on one
mesh), solved together to a true FP64 relative residual.

The reference solves each system with its own ``cola.linalg.solve(PSD(Sparse(...)), b, CG(P=...))``
call (inv.py:24-69, cg.py:94-154).  ``solve_batched`` advances all of them in one persistent
launch per call (colagb_cg_batched_csr_solve): FP32 preconditioned CG inner solves, FP64
iterative refinement, per-system convergence masks.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from .. import _capi


def lower_pattern(indptr: torch.Tensor, indices: torch.Tensor):
    """Lower-triangular part (j <= i) of a CSR pattern.

    Returns (g_indptr, g_indices, src) with src[e] = position in the full pattern of G entry e."""
    n = indptr.numel() - 1
    dev = indptr.device
    counts = (indptr[1:] - indptr[:-1]).to(torch.int64)
    rows = torch.repeat_interleave(torch.arange(n, device=dev), counts)
    keep = indices.to(torch.int64) <= rows
    src = torch.nonzero(keep).flatten()
    g_rows = rows[src]
    g_counts = torch.bincount(g_rows, minlength=n)
    g_indptr = torch.zeros(n + 1, dtype=torch.int64, device=dev)
    g_indptr[1:] = torch.cumsum(g_counts, 0)
    return g_indptr.to(torch.int32), indices[src].to(torch.int32).contiguous(), src


def transpose_pattern(indptr: torch.Tensor, indices: torch.Tensor):
    """CSR pattern of the transpose plus perm (entry e of the transpose = entry perm[e] of the original)."""
    n = indptr.numel() - 1
    dev = indptr.device
    counts = (indptr[1:] - indptr[:-1]).to(torch.int64)
    rows = torch.repeat_interleave(torch.arange(n, device=dev), counts)
    cols = indices.to(torch.int64)
    order = torch.argsort(cols * n + rows, stable=True)
    t_counts = torch.bincount(cols, minlength=n)
    t_indptr = torch.zeros(n + 1, dtype=torch.int64, device=dev)
    t_indptr[1:] = torch.cumsum(t_counts, 0)
    return t_indptr.to(torch.int32), rows[order].to(torch.int32).contiguous(), order.to(torch.int32).contiguous()


@dataclass
class BatchedCSR:
    """S systems on one CSR pattern: indptr (n+1), indices (nnz), values (S, nnz) float32.

    values of shape (1, nnz) with ``shared=True`` is one matrix used by every system (many
    right-hand sides solved with independent convergence)."""
    indptr: torch.Tensor
    indices: torch.Tensor
    values: torch.Tensor
    shared: bool = False

    @property
    def n(self) -> int:
        return self.indptr.numel() - 1

    @property
    def num_systems(self) -> int:
        return self.values.shape[0]

    def matvec(self, X: torch.Tensor) -> torch.Tensor:
        """Y[s] = A_s X[s] in FP64 (host-side helper for checks; uses torch sparse ops)."""
        out = []
        for s in range(X.shape[0]):
            A = torch.sparse_csr_tensor(self.indptr.to(torch.int64), self.indices.to(torch.int64),
                                        self.values[0 if self.shared else s].double(), (self.n, self.n))
            out.append(A @ X[s].double())
        return torch.stack(out)


def solve_dense_batched(matrices, rhs, tol: float = 1e-6, max_iters: int = 1000, refine: bool = False,
                        inner_tol: float = 1e-3, max_sweeps: int = 30):
    """Independent dense SPD systems of uneven sizes, all solved by FP32 CG in one persistent launch.

    Each system reproduces ``cola.linalg.solve(PSD(Dense(A_s)), b_s, CG(tol, max_iters))`` with its
    own stop test (cg.py:94-154).  ``matrices``: list of (n_s, n_s) CUDA tensors; ``rhs``: list of
    (n_s,) tensors.  Returns (list of solutions, per-system iterations, per-system status).

    ``refine=True`` adds FP64 iterative refinement, which the reference does not have: the solution
    accumulates in FP64, the residual b - A x is recomputed in FP64 after every FP32 CG pass (each pass
    to a relative ``inner_tol`` of the current residual, at most ``max_iters`` steps) and a system stops
    once its FP64 true relative residual is <= tol.  Ill-conditioned systems (the RBF K + s^2 I with
    s^2 ~ 1e-3) then reach the requested residual that FP32 CG alone stagnates above.  Solutions are
    then FP64 and the iteration counts are summed over the passes."""
    if len(matrices) != len(rhs):
        raise ValueError("one right-hand side per matrix")
    S = len(matrices)
    if S == 0:
        return [], torch.zeros(0, dtype=torch.int32), torch.zeros(0, dtype=torch.int32)
    _capi.require_cuda(*matrices, *rhs)
    dev = matrices[0].device
    sizes = [int(A.shape[0]) for A in matrices]
    for A, b in zip(matrices, rhs):
        if A.shape != (b.shape[0], b.shape[0]):
            raise ValueError(f"matrix {tuple(A.shape)} and right-hand side {tuple(b.shape)} do not match")
    a_off = [0]
    v_off = [0]
    for n in sizes[:-1]:
        a_off.append(a_off[-1] + n * n)
        v_off.append(v_off[-1] + n)
    vals = torch.cat([A.to(torch.float32).reshape(-1) for A in matrices])
    total = sum(sizes)
    t_sizes = torch.tensor(sizes, dtype=torch.int32, device=dev)
    t_aoff = torch.tensor(a_off, dtype=torch.int64, device=dev)
    t_voff = torch.tensor(v_off, dtype=torch.int64, device=dev)
    lib = _capi.load()
    nbytes = C.c_size_t()
    _capi.check(lib.colagb_cg_dense_batched_workspace_bytes(S, total, C.byref(nbytes)), "dense batched cg")
    ws = _capi.workspace(nbytes.value, dev)

    def fp32_pass(B32, tol_pass):
        X = torch.empty_like(B32)
        iters = torch.zeros(S, dtype=torch.int32, device=dev)
        status = torch.zeros(S, dtype=torch.int32, device=dev)
        _capi.check(lib.colagb_cg_dense_batched_solve(S, t_sizes.data_ptr(), t_aoff.data_ptr(), t_voff.data_ptr(),
                                                      total, vals.data_ptr(), B32.data_ptr(), X.data_ptr(),
                                                      float(tol_pass), int(max_iters), iters.data_ptr(),
                                                      status.data_ptr(), ws.data_ptr(), nbytes.value,
                                                      _capi.stream_ptr(dev)), "dense batched cg")
        return X, iters, status

    if not refine:
        B = torch.cat([b.to(torch.float32).reshape(-1) for b in rhs])
        X, iters, status = fp32_pass(B, tol)
        return list(torch.split(X, sizes)), iters, status
    B64 = torch.cat([b.to(torch.float64).reshape(-1) for b in rhs])
    X64 = torch.zeros_like(B64)
    R64 = torch.empty_like(B64)
    rr = torch.zeros(S, dtype=torch.float64, device=dev)
    seg = torch.repeat_interleave(torch.arange(S, device=dev), torch.tensor(sizes, device=dev))
    bn = torch.zeros(S, dtype=torch.float64, device=dev).index_add_(0, seg, B64 * B64).sqrt()
    iters = torch.zeros(S, dtype=torch.int32, device=dev)
    status = torch.full((S,), 2, dtype=torch.int32, device=dev)  # COLAGB_SYS_MAX_ITERS until converged

    def residual():
        _capi.check(lib.colagb_dense_batched_residual64(S, t_sizes.data_ptr(), t_aoff.data_ptr(), t_voff.data_ptr(),
                                                        total, vals.data_ptr(), B64.data_ptr(), X64.data_ptr(),
                                                        R64.data_ptr(), rr.data_ptr(), _capi.stream_ptr(dev)),
                    "dense residual")
        return rr.sqrt() / bn.clamp_min(1e-300)

    relres = residual()
    for _ in range(max_sweeps):
        done = (relres <= tol) | (bn == 0)
        status = torch.where(done, torch.ones_like(status), status)
        if bool(done.all()):
            break
        # converged systems get a zero right-hand side: the FP32 pass leaves them at once
        R32 = torch.where(done[seg], torch.zeros_like(R64), R64).to(torch.float32)
        D, it, _ = fp32_pass(R32, inner_tol)
        iters += torch.where(done, torch.zeros_like(it), it)
        X64 += D.to(torch.float64)
        relres = residual()
    done = (relres <= tol) | (bn == 0)
    status = torch.where(done, torch.ones_like(status), status)
    return list(torch.split(X64, sizes)), iters, status


class FsaiPattern:
    """Pattern data of G (lower part of A's pattern) and of G^T, shared by all systems."""

    def __init__(self, indptr: torch.Tensor, indices: torch.Tensor):
        self.g_indptr, self.g_indices, self.src = lower_pattern(indptr, indices)
        self.gt_indptr, self.gt_indices, self.gt_perm = transpose_pattern(self.g_indptr, self.g_indices)
        self.g_nnz = self.g_indices.numel()


_PREC = {"none": _capi.PREC_NONE, None: _capi.PREC_NONE, "jacobi": _capi.PREC_JACOBI, "fsai": _capi.PREC_FSAI}
_SCHED = {"auto": 0, "grid": 1, "cluster8": 2, "cluster16": 3, "onchip": 4, "block": 5}
_SCHED_NAME = {v: k for k, v in _SCHED.items()}


def onchip_schedule_info(n: int, halo: int) -> dict:
    """Geometry of the on-chip schedule for n-row systems whose diagonals reach `halo` rows off the
    main diagonal: cluster size (0: does not fit), rows per CTA, clusters resident at once, shared
    memory per CTA in bytes."""
    info = (C.c_int32 * 4)()
    _capi.check(_capi.load().colagb_onchip_schedule_info(int(n), int(halo), info), "onchip info")
    return {"cluster_size": info[0], "rows_per_cta": info[1], "clusters_in_flight": info[2],
            "smem_per_cta": info[3]}


def solve_batched(A: BatchedCSR, B: torch.Tensor, precond: str = "jacobi", tol: float = 1e-8,
                  inner_tol: float | None = None, max_sweeps: int = 200, max_inner_iters: int = 50000,
                  fsai: tuple | None = None, fallback: bool = True, mode: str = "reliable",
                  schedule: str = "auto", wait: bool = True, spin_limit: int = 0, matvec: str = "fp32",
                  spare: str = "auto"):
    """Solve A_s x_s = b_s for every system s to |b_s - A_s x_s| / |b_s| <= tol (FP64 residual).

    Args:
        A: the family (float32 values); n must be a multiple of 4.
        B: (S, n) right-hand sides (any float dtype, promoted to float64).
        precond: "none", "jacobi" or "fsai" (then ``fsai=(FsaiPattern, g_values (S, g_nnz))``).
        mode: "reliable" -- FP32 CG whose residual is replaced by the FP64 b - A x each time it has
            dropped by inner_tol (default 0.01: about five replacements on the way to 1e-8), the
            recurrence continues; "restart" -- classic
            iterative refinement, every FP64 residual starts a new FP32 CG run (default inner_tol 1e-4).
        max_sweeps: FP64 residual replacements per system; max_inner_iters: CG steps per system.
        schedule: "onchip" -- one thread-block cluster per system with p, r and the FP32 correction in
            the cluster's shared memory and the matrix stored by diagonals (patterns of at most 9
            constant-offset diagonals, n <= 262144); "cluster8" / "cluster16" -- one cluster per system
            on the CSR pattern, vectors in global memory; "grid" -- one cooperative grid that advances
            every system together; "block" -- shared-values families: every right-hand side a column
            of one (n, k) block advancing in lockstep, the matrix read once per step for all of them;
            "auto" (default) -- "block" for shared-values families of >= 4 right-hand sides (no FSAI,
            FP32 matvec), else "onchip" when it applies, else a cluster;
            "tuned" -- the fastest applicable schedule for this GPU, pattern, size and preconditioner,
            measured once and kept in the autotuner's JSON cache (cola_gb300.tuning).
        wait: False returns once the solve is enqueued on the current stream (the on-chip and cluster
            schedules); X and the per-system tensors of info are then ready in stream order and
            info["sweeps"] is None.  The scratch buffer is per stream, so solves on other streams may
            run meanwhile.
        spin_limit: naps a CTA of the "grid" schedule may take in one grid barrier before the solve
            gives up with COLAGB_ERR_TIMEOUT (a ColagbError); 0 keeps the library default (seconds).
        matvec: "fp32" -- the inner CG multiplies by the FP32 values; "bf16" -- by BF16 off-diagonal
            values with an FP32 diagonal made consistent with them (within 2^-9 of A in the energy norm
            for weighted-Laplacian-type operators), on the cluster schedules; the FP64 residual
            replacements always use the FP32 values.
        spare: the on-chip schedule's use of the SMs its clusters leave free (40 of 152 for 512 x 512):
            "auto" -- one CTA per free SM also solves whole systems (same algorithm and stop rule,
            vectors in global memory) while more than ~28 systems per cluster remain, so the clusters
            finish the tail (default; on the 256-system 512 x 512 batch: 482 -> 454 ms per solve call);
            "off" -- clusters only, bit-reproducible run to run; "only" -- every system on those CTAs.
    Returns (X (S, n) float64, info) with per-system iterations, status and FP64 relative residuals.
    """
    _capi.require_cuda(A.values, B)
    if schedule == "tuned":
        from .. import tuning
        S_t = B.shape[0]
        key = tuning.key_of(A, S_t, precond, matvec, A.values.device)
        schedule = tuning.choose(key, tuning.probe_measure(solve_batched, A, B, precond, fsai, matvec))
    lib = _capi.load()
    dev = A.values.device
    n = A.n
    S = B.shape[0] if A.shared else A.num_systems
    if A.shared and A.values.shape[0] != 1:
        raise ValueError("a shared-values family holds exactly one value array")
    if B.shape != (S, n):
        raise ValueError(f"B must be ({S}, {n}), got {tuple(B.shape)}")
    vals = A.values.to(torch.float32).contiguous()
    Bd = B.to(torch.float64).contiguous()
    X = torch.empty((S, n), dtype=torch.float64, device=dev)
    pk = _PREC[precond]
    desc = _capi.BatchedCsr(n=n, nnz=A.indices.numel(), num_systems=S, indptr=A.indptr.data_ptr(),
                            indices=A.indices.data_ptr(), values=vals.data_ptr(),
                            shared_values=1 if A.shared else 0)
    keep = [vals, Bd]
    if pk == _capi.PREC_FSAI:
        if fsai is None:
            raise ValueError("precond='fsai' needs fsai=(FsaiPattern, g_values)")
        pat, gv = fsai
        gv = gv.to(torch.float32).contiguous()
        keep.append(gv)
        desc.g_nnz = pat.g_nnz
        desc.g_indptr, desc.g_indices = pat.g_indptr.data_ptr(), pat.g_indices.data_ptr()
        desc.gt_indptr, desc.gt_indices = pat.gt_indptr.data_ptr(), pat.gt_indices.data_ptr()
        desc.gt_perm, desc.g_values = pat.gt_perm.data_ptr(), gv.data_ptr()
    if mode not in ("reliable", "restart"):
        raise ValueError("mode must be 'reliable' or 'restart'")
    if inner_tol is None:
        inner_tol = 0.01 if mode == "reliable" else 1e-4
    prm = _capi.IrParams(tol=float(tol), inner_tol=float(inner_tol), max_sweeps=int(max_sweeps),
                         max_inner_iters=int(max_inner_iters), preconditioner=pk, fallback=1 if fallback else 0,
                         spin_limit=int(spin_limit), mode=_capi.IR_RELIABLE if mode == "reliable" else _capi.IR_RESTART,
                         schedule=_SCHED[schedule], no_wait=0 if wait else 1,
                         matvec={"fp32": _capi.MATVEC_FP32, "bf16": _capi.MATVEC_BF16}[matvec],
                         spare={"auto": _capi.SPARE_AUTO, "off": _capi.SPARE_OFF, "only": _capi.SPARE_ONLY}[spare])
    iters = torch.zeros(S, dtype=torch.int32, device=dev)
    status = torch.zeros(S, dtype=torch.int32, device=dev)
    relres = torch.zeros(S, dtype=torch.float64, device=dev)
    nbytes = C.c_size_t()
    _capi.check(lib.colagb_cg_batched_csr_workspace_bytes(C.byref(desc), C.byref(prm), C.byref(nbytes)), "batched cg")
    ws = _capi.workspace(nbytes.value, dev)
    res = _capi.IrResult()
    _capi.check(lib.colagb_cg_batched_csr_solve(C.byref(desc), Bd.data_ptr(), X.data_ptr(), C.byref(prm),
                                                iters.data_ptr(), status.data_ptr(), relres.data_ptr(), ws.data_ptr(),
                                                nbytes.value, C.byref(res), _capi.stream_ptr(dev)), "batched cg")
    swp = int(res.sweeps) if res.sweeps >= 0 else None
    info = {"iterations": iters, "status": status, "relres": relres, "replacements": swp,
            "sweeps": swp, "max_iterations": int(res.total_inner_iters),
            "schedule": _SCHED_NAME.get(int(res.schedule), "auto"),
            "companion_systems": int(res.companion_systems) if res.companion_systems >= 0 else None}
    return X, info
