"""colagb_cg_solve_noalloc: CG for callers that cannot allocate device memory (a host runtime with its
own fixed pool, or code where cudaMalloc is not allowed).  Its scratch is a fixed array inside the
library, so it must give the same answers as colagb_cg_solve with a caller workspace -- also on the
second call, when the array still holds the first call's data.  Named to run after every other test
file."""
import ctypes as C

import numpy as np
import pytest
import torch

from cola_gb300 import _capi
from cola_gb300.lowering import Lowered
import cola_gb300 as cola

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")


def _solve(op, B, x0, allocating: bool, tol=1e-7, max_iters=600, P=None, allow_fused=1):
    lib = _capi.load()
    low = Lowered(op)
    lowp = Lowered(P) if P is not None else None
    ph = lowp.handle if lowp is not None else None
    k = B.shape[1]
    X = x0.clone()
    prm = _capi.CgParams(tol=tol, max_iters=max_iters, check_every=16, allow_fused=allow_fused, graph=0,
                         spin_limit=0)
    res = _capi.CgResult()
    st = _capi.stream_ptr(DEV)
    if allocating:
        nb = C.c_size_t()
        _capi.check(lib.colagb_cg_workspace_bytes(low.handle, ph, k, C.byref(nb)), "ws")
        ws = torch.empty(nb.value, dtype=torch.uint8, device=DEV)
        _capi.check(lib.colagb_cg_solve(low.handle, ph, B.data_ptr(), k, X.data_ptr(), k, k, C.byref(prm), None,
                                        ws.data_ptr(), nb.value, C.byref(res), st), "cg")
    else:
        _capi.check(lib.colagb_cg_solve_noalloc(low.handle, ph, B.data_ptr(), k, X.data_ptr(), k, k, C.byref(prm),
                                                None, C.byref(res), st), "cg noalloc")
    torch.cuda.synchronize()
    return X, res.iterations, res.fused


def _dense_spd(n, seed):
    g = torch.Generator().manual_seed(seed)
    Q, _ = torch.linalg.qr(torch.randn(n, n, generator=g, dtype=torch.float64))
    lam = torch.exp(torch.empty(n, dtype=torch.float64).uniform_(np.log(0.1), np.log(10.0), generator=g))
    return ((Q * lam) @ Q.T).float()


@pytest.mark.parametrize("kind", ["dense", "sparse"])
def test_noalloc_matches_workspace_entry_two_calls_in_a_row(kind):
    if kind == "dense":
        op = cola.PSD(cola.ops.Dense(_dense_spd(300, 1).to(DEV)))
        n, k = 300, 2
    else:
        from cola_gb300.workloads import grid_pattern_2d, diffusion_values_2d
        m = 24
        ip, ix, ok = grid_pattern_2d(m, DEV)
        a = torch.exp(torch.randn(1, m, m, device=DEV, dtype=torch.float64))
        op = cola.PSD(cola.ops.Sparse.from_csr(ip, ix, diffusion_values_2d(a, ok)[0], (m * m, m * m)))
        n, k = m * m, 3
    for call in range(2):  # the second call runs on a scratch array still holding the first call's data
        g = torch.Generator(device="cpu").manual_seed(10 + call)
        B = torch.randn(n, k, generator=g).to(DEV)
        x0 = torch.zeros_like(B)
        X_ref, it_ref, _ = _solve(op, B, x0, allocating=True)
        X_na, it_na, _ = _solve(op, B, x0, allocating=False)
        assert it_na == it_ref
        rel = float((X_na - X_ref).norm() / X_ref.norm())
        assert rel < 1e-6, (call, rel)


@pytest.mark.parametrize("pkind", ["jacobi", "explicit"])
def test_noalloc_generic_loop_fp64_with_preconditioner_two_calls_in_a_row(pkind):
    """The multi-launch loop (fused kernel disabled) in FP64 with a preconditioner keeps the operator's
    own workspace, and for an explicit P the preconditioned residual, inside the shared array too."""
    n, k = 200, 2
    A = _dense_spd(n, 3).double().to(DEV)
    op = cola.PSD(cola.ops.Dense(A))
    if pkind == "jacobi":
        P = cola.ops.Diagonal(1.0 / torch.diagonal(A))
    else:  # a general operator program: Jacobi written as a Sum of two scaled diagonals
        d = 1.0 / torch.diagonal(A)
        P = cola.ops.Diagonal(0.5 * d) + cola.ops.Diagonal(0.5 * d)
    for call in range(2):
        g = torch.Generator(device="cpu").manual_seed(20 + call)
        B = torch.randn(n, k, generator=g, dtype=torch.float64).to(DEV)
        x0 = torch.zeros_like(B)
        X_ref, it_ref, f_ref = _solve(op, B, x0, allocating=True, tol=1e-10, P=P, allow_fused=0)
        X_na, it_na, f_na = _solve(op, B, x0, allocating=False, tol=1e-10, P=P, allow_fused=0)
        assert f_ref == 0 and f_na == 0
        assert it_na == it_ref
        rel = float((X_na - X_ref).norm() / X_ref.norm())
        assert rel < 1e-12, (call, rel)


def test_noalloc_rejects_problems_beyond_its_scratch():
    lib = _capi.load()
    n, k = 1 << 20, 4  # ~50 MB of CG vectors: far beyond the 8 MiB array
    op = cola.PSD(cola.ops.Diagonal(torch.ones(n, device=DEV)))
    low = Lowered(op)
    B = torch.ones(n, k, device=DEV)
    X = torch.zeros_like(B)
    prm = _capi.CgParams(tol=1e-6, max_iters=10, check_every=16, allow_fused=1, graph=0, spin_limit=0)
    res = _capi.CgResult()
    st = lib.colagb_cg_solve_noalloc(low.handle, None, B.data_ptr(), k, X.data_ptr(), k, k, C.byref(prm), None,
                                     C.byref(res), _capi.stream_ptr(DEV))
    assert st == _capi.ERR_INVALID
    assert b"8388608" in lib.colagb_last_error()
