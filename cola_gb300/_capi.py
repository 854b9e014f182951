"""ctypes binding of libcolagb (declared in include/colagb.h).

The library is built in-tree by ``cola_gb300._build.build()``.  There is no
fallback: every compute entry point of this package goes through this module,
and importing a compute function without the library raises at call time with
the reason.
"""
from __future__ import annotations

import collections
import ctypes as C
import threading
from pathlib import Path

import torch

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libcolagb.so"

OK = 0
ERR_INVALID = 1
ERR_CUDA = 2
ERR_TIMEOUT = 3
ERR_UNSUPPORTED = 4
ERR_WORKSPACE = 5

F32, F64, BF16 = 0, 1, 2

OP_DENSE, OP_CSR, OP_DIAG, OP_SCALAR, OP_IDENTITY, OP_SUM, OP_PRODUCT, OP_KRON, OP_BLOCKDIAG = range(1, 10)
KRON_PRECISION = {"auto": 0, "fp32": 1, "bf16": 2, "bf16x3": 3}

PREC_NONE, PREC_JACOBI, PREC_FSAI = 0, 1, 2
IR_RELIABLE, IR_RESTART = 0, 1
MATVEC_FP32, MATVEC_BF16 = 0, 1
SPARE_OFF, SPARE_AUTO, SPARE_ONLY = 0, 1, 2

SYS_RUNNING, SYS_CONVERGED, SYS_MAX_ITERS, SYS_BREAKDOWN, SYS_NAN, SYS_FALLBACK = range(6)
SYS_STATUS_NAMES = {0: "running", 1: "converged", 2: "max_iters", 3: "breakdown", 4: "nan", 5: "fallback"}

TORCH_TO_CODE = {torch.float32: F32, torch.float64: F64, torch.bfloat16: BF16}
CODE_TO_TORCH = {v: k for k, v in TORCH_TO_CODE.items()}


class OpNode(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("dtype", C.c_int32), ("rows", C.c_int64), ("cols", C.c_int64),
        ("data", C.c_void_p), ("ld", C.c_int64), ("indptr", C.c_void_p), ("indices", C.c_void_p),
        ("nnz", C.c_int64), ("scalar", C.c_double), ("children", C.POINTER(C.c_int32)),
        ("num_children", C.c_int32), ("multiplicities", C.POINTER(C.c_int64)),
        ("precision", C.c_int32), ("reserved", C.c_int32), ("perm", C.c_void_p),
    ]


class CgParams(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iters", C.c_int32), ("check_every", C.c_int32),
                ("allow_fused", C.c_int32), ("graph", C.c_int32), ("spin_limit", C.c_int64)]


class CgResult(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("fused", C.c_int32), ("status", C.c_int32), ("graph", C.c_int32)]


class BatchedCsr(C.Structure):
    _fields_ = [
        ("n", C.c_int64), ("nnz", C.c_int64), ("num_systems", C.c_int64),
        ("indptr", C.c_void_p), ("indices", C.c_void_p), ("values", C.c_void_p),
        ("g_nnz", C.c_int64), ("g_indptr", C.c_void_p), ("g_indices", C.c_void_p),
        ("gt_indptr", C.c_void_p), ("gt_indices", C.c_void_p), ("gt_perm", C.c_void_p),
        ("g_values", C.c_void_p), ("shared_values", C.c_int32), ("reserved", C.c_int32),
    ]


class IrParams(C.Structure):
    _fields_ = [("tol", C.c_double), ("inner_tol", C.c_double), ("max_sweeps", C.c_int32),
                ("max_inner_iters", C.c_int32), ("preconditioner", C.c_int32), ("fallback", C.c_int32),
                ("spin_limit", C.c_int64), ("mode", C.c_int32), ("schedule", C.c_int32), ("no_wait", C.c_int32),
                ("matvec", C.c_int32), ("spare", C.c_int32)]


class IrResult(C.Structure):
    _fields_ = [("sweeps", C.c_int32), ("total_inner_iters", C.c_int32), ("status", C.c_int32),
                ("schedule", C.c_int32), ("companion_systems", C.c_int32)]


class LanczosParams(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iters", C.c_int32), ("check_every", C.c_int32)]


# name -> (restype, argtypes); every symbol declared in include/colagb.h
_vp, _i64, _i32, _d, _sz = C.c_void_p, C.c_int64, C.c_int32, C.c_double, C.c_size_t
_P = C.POINTER
SIGNATURES = {
    "colagb_last_error": (C.c_char_p, []),
    "colagb_version": (C.c_int, [_P(_i32), _P(_i32)]),
    "colagb_op_create": (C.c_int, [_P(OpNode), _i32, _i32, _P(_vp)]),
    "colagb_op_free": (C.c_int, [_vp]),
    "colagb_op_info": (C.c_int, [_vp, _P(_i64), _P(_i64), _P(_i32)]),
    "colagb_matmat_workspace_bytes": (C.c_int, [_vp, _i64, _P(_sz)]),
    "colagb_matmat": (C.c_int, [_vp, _vp, _i64, _vp, _i64, _i64, _d, _d, _vp, _sz, _vp]),
    "colagb_cg_workspace_bytes": (C.c_int, [_vp, _vp, _i64, _P(_sz)]),
    "colagb_cg_solve": (C.c_int, [_vp, _vp, _vp, _i64, _vp, _i64, _i64, _P(CgParams), _vp, _vp, _sz,
                                  _P(CgResult), _vp]),
    "colagb_cg_solve_noalloc": (C.c_int, [_vp, _vp, _vp, _i64, _vp, _i64, _i64, _P(CgParams), _vp, _P(CgResult),
                                          _vp]),
    "colagb_cg_batched_csr_workspace_bytes": (C.c_int, [_P(BatchedCsr), _P(IrParams), _P(_sz)]),
    "colagb_cg_batched_csr_solve": (C.c_int, [_P(BatchedCsr), _vp, _vp, _P(IrParams), _vp, _vp, _vp, _vp, _sz,
                                              _P(IrResult), _vp]),
    "colagb_onchip_schedule_info": (C.c_int, [_i64, _i32, _vp]),
    "colagb_cg_dense_batched_workspace_bytes": (C.c_int, [_i64, _i64, _P(_sz)]),
    "colagb_dense_batched_residual64": (C.c_int, [_i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp]),
    "colagb_cg_dense_batched_solve": (C.c_int, [_i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _d, _i32, _vp, _vp, _vp,
                                                _sz, _vp]),
    "colagb_lanczos_workspace_bytes": (C.c_int, [_vp, _i64, _i32, _P(_sz)]),
    "colagb_arnoldi_workspace_bytes": (C.c_int, [_vp, _i64, _i32, _P(_sz)]),
    "colagb_arnoldi": (C.c_int, [_vp, _vp, _i64, _i64, _P(LanczosParams), _vp, _vp, _P(_i32), _vp, _sz, _vp]),
    "colagb_lanczos": (C.c_int, [_vp, _vp, _i64, _i64, _P(LanczosParams), _vp, _vp, _vp, _P(_i32), _vp, _sz,
                                 _vp]),
    "colagb_basis_combine": (C.c_int, [_vp, _i64, _i64, _i32, _vp, _i64, _vp, _i32, _vp]),
    "colagb_tridiag_eig_f64": (C.c_int, [_vp, _vp, _i64, _i64, _vp, _vp, _vp, _vp, _vp]),
    "colagb_tridiag_eig_f32": (C.c_int, [_vp, _vp, _i64, _i64, _vp, _vp, _vp, _vp, _vp]),
    "colagb_grid5_stencil": (C.c_int, [_vp, _vp, _vp, _i64, _i64, _i64, _vp, _vp, _vp]),
    "colagb_fsai_features": (C.c_int, [_vp, _i64, _i64, _vp, _vp]),
    "colagb_fsai_assemble": (C.c_int, [_vp, _vp, _i64, _i64, _vp, _vp]),
    "colagb_fsai_compact": (C.c_int, [_vp, _vp, _i64, _i64, _i64, _vp, _vp]),
    "colagb_fsai_net_build": (C.c_int, [_vp, _vp, _i64, _i64, _i64, _vp, _i64, _vp, _vp, _vp]),
    "colagb_fsai_closed_build": (C.c_int, [_vp, _i64, _i64, _vp, _i64, _vp, _vp]),
    "colagb_conv3x3_forward": (C.c_int, [_vp, _i64, _i32, _i32, _i64, _i64, _vp, _vp, _i32, _vp, _vp]),
    "colagb_conv3x3_backward_scratch_bytes": (C.c_int, [_i32, _i32, _P(_sz)]),
    "colagb_conv3x3_backward": (C.c_int, [_vp, _vp, _vp, _i64, _i32, _i32, _i64, _i64, _vp, _vp, _vp, _vp, _sz,
                                          _vp]),
    "colagb_fsai_loss_grad": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _i64, _i64, _vp, _vp, _vp, _sz, _vp]),
    "colagb_fsai_rq_loss_grad": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _i64, _i64, _vp, _vp, _vp, _sz, _vp]),
    "colagb_adam_step": (C.c_int, [_vp, _vp, _vp, _vp, _i64, C.c_float, C.c_float, C.c_float, C.c_float, _i32,
                                   _vp]),
    "colagb_read_bandwidth_probe": (C.c_int, [_vp, _sz, _i32, _vp, _vp]),
    "colagb_matmat_vjp": (C.c_int, [_vp, _vp, _i64, _vp, _i64, _i64, _d, _vp, _vp]),
}

_lib = None
_lock = threading.Lock()


class ColagbError(RuntimeError):
    pass


def load(path: Path | None = None):
    """Load libcolagb.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise ColagbError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        lib = C.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status: int, what: str = "") -> None:
    """Map a colagb status code to the exception type the reference raises for that condition."""
    if status == OK:
        return
    msg = load().colagb_last_error().decode(errors="replace")
    text = f"{what}: {msg}" if what else msg
    if status in (ERR_INVALID, ERR_WORKSPACE):
        raise ValueError(text)
    if status == ERR_UNSUPPORTED:
        raise NotImplementedError(text)
    raise ColagbError(text)


def stream_ptr(device: torch.device | None = None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def require_cuda(*tensors: torch.Tensor) -> None:
    for t in tensors:
        if t is None:
            continue
        if not t.is_cuda:
            raise ValueError("cola_gb300 computes on the GPU: pass CUDA tensors (got a tensor on "
                             f"{t.device}); there is no CPU execution path")


_ws_cache: "collections.OrderedDict" = collections.OrderedDict()
_WS_CACHE_STREAMS = 8


def workspace(nbytes: int, device: torch.device) -> torch.Tensor:
    """A device scratch buffer of at least nbytes for work on the device's current stream, cached per
    (device, stream) and grown on demand: calls on one stream reuse it in stream order (also calls
    that return before their kernels finish, e.g. a batched solve with wait=False), calls on
    different streams never share it.  The cache keeps the buffers of the 8 most recently used
    streams; an older stream's buffer is dropped, and torch's allocator hands its memory out again
    only in that stream's order, so work still queued there is not disturbed."""
    idx = device.index if device.index is not None else torch.cuda.current_device()
    key = (device.type, idx, stream_ptr(torch.device(device.type, idx)))
    buf = _ws_cache.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
        _ws_cache[key] = buf
    _ws_cache.move_to_end(key)
    while len(_ws_cache) > _WS_CACHE_STREAMS:
        _ws_cache.popitem(last=False)
    return buf
