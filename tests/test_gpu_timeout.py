"""The cooperative kernels' grid barrier gives up after `spin_limit` naps and the call returns
COLAGB_ERR_TIMEOUT; the CUDA context stays usable and the next call solves normally.

The wait is made to run out by a spin limit of one nap: a CTA that arrives at a barrier before the
last CTA of the grid (always the case on a grid of hundreds of CTAs) gives up at once, so no GPU
fault, trap or endless loop is involved."""
import ctypes as C

import pytest
import torch

import cola_gb300 as cola
from cola_gb300 import _capi
from cola_gb300.lowering import Lowered

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")


def _dense_cg(op, B, spin_limit):
    lib = _capi.load()
    low = Lowered(op)
    n, k = B.shape
    X = torch.zeros_like(B)
    prm = _capi.CgParams(tol=0.0, max_iters=200, check_every=16, allow_fused=1, graph=0, spin_limit=spin_limit)
    res = _capi.CgResult()
    nb = C.c_size_t()
    _capi.check(lib.colagb_cg_workspace_bytes(low.handle, None, k, C.byref(nb)), "ws")
    ws = torch.empty(nb.value, dtype=torch.uint8, device=DEV)
    st = lib.colagb_cg_solve(low.handle, None, B.data_ptr(), k, X.data_ptr(), k, k, C.byref(prm), None,
                             ws.data_ptr(), nb.value, C.byref(res), _capi.stream_ptr(DEV))
    torch.cuda.synchronize()
    return st, res, X


def test_fused_cg_grid_barrier_times_out_and_context_survives():
    # a 3072 x 3072 FP32 matrix (37.7 MB) is above the single-cluster limit, so the fused solve runs
    # on the cooperative grid with its software barrier
    n = 3072
    g = torch.Generator().manual_seed(0)
    M = (torch.randn(n, n, generator=g) / n ** 0.5).to(DEV)
    A = M @ M.T + 2.0 * torch.eye(n, device=DEV)
    op = cola.PSD(cola.ops.Dense(A))
    B = torch.randn(n, 1, generator=g).to(DEV)
    st, res, _ = _dense_cg(op, B, spin_limit=1)
    assert res.fused == 1
    assert st == _capi.ERR_TIMEOUT and res.status == _capi.ERR_TIMEOUT
    assert b"timed out" in _capi.load().colagb_last_error()
    # same call with the default limit: completes, and the solution is right
    st, res, X = _dense_cg(op, B, spin_limit=0)
    assert st == _capi.OK and res.status == 0 and res.iterations == 200
    rel = float((A @ X - B).norm() / B.norm())
    assert rel < 1e-4, rel


def test_batched_grid_schedule_times_out_and_context_survives():
    from cola_gb300.linalg.batched import solve_batched
    from cola_gb300.workloads import diffusion_family_2d
    fam, B, _, _ = diffusion_family_2d(range(5000, 5004), m=32, device=DEV)
    with pytest.raises(_capi.ColagbError, match="timed out"):
        solve_batched(fam, B, precond="jacobi", tol=1e-8, schedule="grid", spin_limit=1)
    X, info = solve_batched(fam, B, precond="jacobi", tol=1e-8, schedule="grid")
    assert bool((info["status"] == 1).all()) and float(info["relres"].max()) <= 1e-8
