"""The Kronecker matvec's tensor-core contractions (tcgen05 + TMA, csrc/tc_gemm.cu) against an FP64
dense product (Kronecker._matmat, cola/ops/operators.py:216-223).

Shapes cover every operand form of the kernel: the per-block transposed operand with a 3-D tensor map
(several blocks), one block (2-D map), the row form (q = 1), output widths that are not a multiple of
the tile, reduction lengths that are not a multiple of 64 or of 8, BF16-stored factors, and beta != 0.
Tolerances: the three-product split ("bf16x3") is within 3e-5 of FP64 in relative Frobenius norm (each
product is exact to ~2^-16), single BF16 products ("bf16") within 1e-2."""
import ctypes as C

import numpy as np
import pytest
import torch

import cola_gb300 as cola
from cola_gb300 import _capi
from cola_gb300.lowering import Lowered

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")
TOL = {"bf16x3": 3e-5, "bf16": 1e-2}


def kron_apply64(factors, X):
    """(F_0 x F_1 x ...) @ X in FP64 on the device, one factor contraction at a time (never dense)."""
    k = X.shape[1]
    T = X.double().to(DEV).reshape(*[f.shape[1] for f in factors], k)
    for i, f in enumerate(factors):
        T = torch.tensordot(f.double().to(DEV), T, dims=([1], [i])).movedim(0, i)
    return T.reshape(-1, k)


def matmat(op, X, Y=None, alpha=1.0, beta=0.0):
    lib = _capi.load()
    low = Lowered(op)
    k = X.shape[1]
    if Y is None:
        Y = torch.zeros(op.shape[0], k, device=DEV, dtype=X.dtype)
    nb = C.c_size_t()
    _capi.check(lib.colagb_matmat_workspace_bytes(low.handle, k, C.byref(nb)), "ws")
    ws = torch.empty(max(nb.value, 1), dtype=torch.uint8, device=DEV)
    _capi.check(lib.colagb_matmat(low.handle, X.data_ptr(), k, Y.data_ptr(), k, k, alpha, beta, ws.data_ptr(),
                                  nb.value, _capi.stream_ptr(DEV)), "matmat")
    torch.cuda.synchronize()
    return Y


def rel(a, b):
    return float((a.double().cpu() - b.double().cpu()).norm() / b.double().cpu().norm())


CASES = [
    # (factor shapes, k): exercises
    ([(64, 64), (64, 64), (64, 64)], 4),     # q = 16384 / 256 / 4 -> transposed 2-D and 3-D forms, SIMT for q=4
    ([(96, 72), (48, 40)], 1),               # K not a multiple of 64; q = 40 (3-D), then q = 1 (row form)
    ([(100, 30), (200, 136)], 1),            # N not a multiple of the tile, K = 30 (padded to 32)
    ([(256, 256), (128, 128)], 2),           # wider tiles, q = 256 then q = 2 (SIMT)
    ([(1024, 1024), (64, 64)], 1),           # C5-like first factor, 2-D map with many tiles
]


@pytest.mark.parametrize("prec", ["bf16x3", "bf16"])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_kron_tensor_core_contraction_matches_fp64(prec, case):
    shapes, k = CASES[case]
    g = torch.Generator().manual_seed(case)
    Fs = [torch.randn(r, c, generator=g) / c ** 0.5 for r, c in shapes]
    op = cola.ops.Kronecker(*[cola.ops.Dense(f.to(DEV)) for f in Fs], precision=prec)
    ncols = int(np.prod([c for _, c in shapes]))
    X = torch.randn(ncols, k, generator=g)
    Y = matmat(op, X.to(DEV))
    ref = kron_apply64(Fs, X)
    assert rel(Y, ref) < TOL[prec], rel(Y, ref)
    # the FP32 SIMT path agrees with FP64 to FP32 rounding
    op32 = cola.ops.Kronecker(*[cola.ops.Dense(f.to(DEV)) for f in Fs], precision="fp32")
    assert rel(matmat(op32, X.to(DEV)), ref) < 1e-5


def test_kron_tensor_core_bf16_factor_and_beta():
    g = torch.Generator().manual_seed(7)
    F1 = (torch.randn(128, 128, generator=g) / 12).bfloat16()
    F2 = torch.randn(256, 256, generator=g) / 16
    op = cola.ops.Kronecker(cola.ops.Dense(F1.to(DEV)), cola.ops.Dense(F2.to(DEV)), precision="bf16x3")
    X = torch.randn(128 * 256, 1, generator=g)  # k = 1: the last factor runs in row form with beta
    Y0 = torch.randn(128 * 256, 1, generator=g)
    Y = matmat(op, X.to(DEV), Y0.clone().to(DEV), alpha=0.5, beta=-2.0)
    ref = 0.5 * kron_apply64([F1.float(), F2], X) - 2.0 * Y0.double().to(DEV)
    assert rel(Y, ref) < TOL["bf16x3"], rel(Y, ref)


def test_kron_auto_uses_tensor_cores_only_for_large_contractions():
    """auto: a 1024 x 1024 factor (2^30 multiply-adds at k = 1) runs on the tensor cores, a small
    Kronecker stays on the FP32 path (its result equals the forced-FP32 result bit for bit)."""
    g = torch.Generator().manual_seed(3)
    small = [torch.randn(8, 8, generator=g) for _ in range(2)]
    X = torch.randn(64, 2, generator=g).to(DEV)
    ya = matmat(cola.ops.Kronecker(*[cola.ops.Dense(f.to(DEV)) for f in small]), X)
    yf = matmat(cola.ops.Kronecker(*[cola.ops.Dense(f.to(DEV)) for f in small], precision="fp32"), X)
    assert torch.equal(ya, yf)
    big = [torch.randn(1024, 1024, generator=g) / 32 for _ in range(2)]
    Xb = torch.randn(1024 * 1024, 1, generator=g).to(DEV)
    ya = matmat(cola.ops.Kronecker(*[cola.ops.Dense(f.to(DEV)) for f in big]), Xb)
    yt = matmat(cola.ops.Kronecker(*[cola.ops.Dense(f.to(DEV)) for f in big], precision="bf16x3"), Xb)
    assert torch.equal(ya, yt)
    Xm = Xb.reshape(1024, 1024).double()
    ref = (big[0].double().to(DEV) @ Xm @ big[1].double().to(DEV).T).reshape(-1, 1)
    assert rel(ya, ref) < TOL["bf16x3"]
