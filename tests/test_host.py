"""Host-side logic that needs no GPU: the C ABI library loads and exports every declared symbol,
operator lowering, argument validation and error mapping, dispatch rules, pattern helpers."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest
import torch

import cola_gb300 as cola
from cola_gb300 import _capi
from cola_gb300.linalg import CG, Lanczos
from cola_gb300.linalg.batched import lower_pattern, transpose_pattern
from cola_gb300.lowering import Lowered

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "colagb.h").read_text()
    return sorted(set(re.findall(r"\b(colagb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _capi.load()
    names = declared_symbols()
    assert len(names) >= 14
    for name in names:
        assert hasattr(lib, name), name
        assert name in _capi.SIGNATURES, f"{name} has no ctypes signature"


def test_version():
    lib = _capi.load()
    v, a = C.c_int32(), C.c_int32()
    assert lib.colagb_version(C.byref(v), C.byref(a)) == 0
    assert a.value == 1003


STRUCTS = {
    "colagb_op_node": _capi.OpNode, "colagb_cg_params": _capi.CgParams, "colagb_cg_result": _capi.CgResult,
    "colagb_batched_csr": _capi.BatchedCsr, "colagb_ir_params": _capi.IrParams,
    "colagb_ir_result": _capi.IrResult, "colagb_lanczos_params": _capi.LanczosParams,
}


def test_struct_layouts_match_header(tmp_path):
    """Every ctypes struct has the size and field offsets the C compiler gives the header's struct."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{ROOT / "include" / "colagb.h"}"',
             "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in STRUCTS.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_lowering_structure():
    A = torch.randn(6, 6)
    D = cola.ops.Dense(A)
    op = cola.kron(D, cola.ops.Diagonal(torch.ones(2))) + 0.5 * cola.ops.I_like(cola.kron(D, torch.eye(2)))
    low = Lowered(op)
    kinds = [n.kind for n in low.nodes]
    assert kinds[-1] == _capi.OP_SUM
    assert _capi.OP_KRON in kinds and _capi.OP_SCALAR in kinds
    rows, cols, cdt = C.c_int64(), C.c_int64(), C.c_int32()
    assert _capi.load().colagb_op_info(low.handle, C.byref(rows), C.byref(cols), C.byref(cdt)) == 0
    assert (rows.value, cols.value, cdt.value) == (12, 12, _capi.F32)
    assert Lowered(cola.ops.Dense(A.double())).compute_dtype == torch.float64


def test_blockdiag_and_product_lowering_and_workspace():
    D1, D2 = cola.ops.Dense(torch.randn(3, 3)), cola.ops.Dense(torch.randn(2, 2))
    BD = cola.ops.BlockDiag(D1, D2, multiplicities=[2, 3])
    P = cola.ops.Product(cola.ops.Dense(torch.randn(12, 12)), BD)
    low = Lowered(P)
    nb = C.c_size_t()
    assert _capi.load().colagb_matmat_workspace_bytes(low.handle, 4, C.byref(nb)) == 0
    assert nb.value >= 12 * 4 * 4  # the product's intermediate


def test_invalid_operator_is_value_error():
    nd = _capi.OpNode(kind=_capi.OP_DENSE, dtype=_capi.F32, rows=4, cols=4, data=None, ld=4)
    h = C.c_void_p()
    st = _capi.load().colagb_op_create(C.byref(nd), 1, 0, C.byref(h))
    assert st == _capi.ERR_INVALID
    with pytest.raises(ValueError):
        _capi.check(st, "op")
    # shape mismatch in a Sum
    with pytest.raises(ValueError):
        cola.ops.Sum(cola.ops.Dense(torch.randn(3, 3)), cola.ops.Dense(torch.randn(4, 4)))
    with pytest.raises(ValueError):
        cola.ops.Product(cola.ops.Dense(torch.randn(3, 4)), cola.ops.Dense(torch.randn(3, 3)))


def test_unknown_kind_and_cycle_rejected():
    lib = _capi.load()
    kids = (C.c_int32 * 1)(0)
    nd = _capi.OpNode(kind=_capi.OP_SUM, rows=2, cols=2, children=C.cast(kids, C.POINTER(C.c_int32)), num_children=1)
    h = C.c_void_p()
    assert lib.colagb_op_create(C.byref(nd), 1, 0, C.byref(h)) == _capi.ERR_INVALID
    assert b"cycle" in lib.colagb_last_error()
    nd2 = _capi.OpNode(kind=77, rows=2, cols=2)
    assert lib.colagb_op_create(C.byref(nd2), 1, 0, C.byref(h)) == _capi.ERR_INVALID


def test_compute_requires_cuda_tensors():
    op = cola.PSD(cola.ops.Dense(torch.eye(3)))
    with pytest.raises(ValueError, match="GPU"):
        op @ torch.ones(3)
    with pytest.raises(ValueError, match="GPU"):
        cola.linalg.inverse.cg(op, torch.ones(3))


def test_dispatch_rules():
    D = cola.ops.Dense(torch.eye(3))
    with pytest.raises(AssertionError):
        cola.inv(D, CG())
    Ainv = cola.inv(cola.PSD(D), CG(tol=1e-3))
    assert isinstance(Ainv, cola.linalg.IterativeOperatorWInfo)
    d = cola.ops.Diagonal(torch.tensor([2.0, 4.0]))
    assert torch.allclose(cola.inv(d, CG()).diag, torch.tensor([0.5, 0.25]))
    K = cola.ops.Kronecker(cola.PSD(D), cola.PSD(D))
    Kinv = cola.inv(K, CG())
    assert isinstance(Kinv, cola.ops.Kronecker) and all(isinstance(M, cola.linalg.IterativeOperatorWInfo) for M in Kinv.Ms)
    assert isinstance(cola.inv(cola.ops.I_like(D), CG()), cola.ops.Identity)
    with pytest.raises(AssertionError):
        cola.eig(D, 2, "LM", Lanczos())
    assert cola.linalg.get_slice(3, "LM") == slice(-3, None) and cola.linalg.get_slice(2, "SM") == slice(0, 2)


def test_annotations_inference():
    D = cola.PSD(cola.ops.Dense(torch.eye(4)))
    assert (D + 0.1 * cola.ops.I_like(D)).isa(cola.PSD)
    assert cola.kron(D, D).isa(cola.PSD)
    assert not cola.ops.Dense(torch.eye(4)).isa(cola.PSD)
    assert (2.0 * D).isa(cola.PSD)


def test_reference_randn_recipe():
    from cola_gb300.linalg.prng import PRNGKey, next_key, randn, sha_hash
    assert PRNGKey(42) == sha_hash(42) and next_key(7) == sha_hash(7)
    torch.manual_seed(PRNGKey(42))
    a = torch.randn(13, 4, dtype=torch.float64)
    assert torch.equal(a, randn(13, 4, dtype=torch.float64, key=PRNGKey(42)))


def test_pattern_helpers():
    from cola_gb300.workloads import grid_pattern_2d
    ip, ix, _ = grid_pattern_2d(5)
    gip, gix, src = lower_pattern(ip, ix)
    n = 25
    rows = torch.repeat_interleave(torch.arange(n), (gip[1:] - gip[:-1]).long())
    assert torch.all(gix.long() <= rows)
    assert gix.numel() == (ix.numel() + n) // 2
    tip, tix, perm = transpose_pattern(gip, gix)
    # entry e of G^T at (i, tix[e]) is entry perm[e] of G at (tix[e], i)
    trow = torch.repeat_interleave(torch.arange(n), (tip[1:] - tip[:-1]).long())
    assert torch.all(rows[perm.long()] == tix.long()) and torch.all(gix[perm.long()].long() == trow)


def test_sparse_csr_build_host():
    S = cola.ops.Sparse(torch.tensor([1.0, 2.0, 3.0]), torch.tensor([1, 0, 1]), torch.tensor([0, 1, 0]), (2, 2))
    assert S.indptr.tolist() == [0, 1, 2] and S.indices.tolist() == [1, 0]
    assert S.values.tolist() == [2.0, 4.0]
    assert torch.equal(S.to_dense(), torch.tensor([[0.0, 2.0], [4.0, 0.0]]))


def test_workload_generators_small():
    from cola_gb300.workloads import diffusion_family_2d
    fam, B, coeff, params = diffusion_family_2d([5000, 5001], m=12, device="cpu")
    assert fam.values.shape == (2, fam.indices.numel()) and B.shape == (2, 144)
    for (ell, var) in params:
        assert 0.05 <= ell <= 0.2 and 0.5 <= var <= 2.0
    n = 144
    for s in range(2):
        A = torch.sparse_csr_tensor(fam.indptr.long(), fam.indices.long(), fam.values[s].double(), (n, n)).to_dense()
        assert torch.allclose(A, A.T)
        assert torch.linalg.eigvalsh(A)[0] > 0


def _bf16_round(x: np.ndarray) -> np.ndarray:
    """float32 -> bfloat16 (round to nearest, ties to even) -> float32, as __float2bfloat16_rn."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def test_bfloat16_preconditioner_boost_keeps_it_spd():
    """The on-chip schedule stores M = G^T G in bfloat16 with each main-diagonal entry raised by
    2^-7 times its row's absolute sum (kMBoost, cg_onchip.cu).  For any symmetric M that makes the
    stored M' - M diagonally dominant with a non-negative diagonal, so M' >= M: checked here on
    FSAI-shaped banded matrices and on dense symmetric ones with large off-diagonals, including M
    that is barely positive definite."""
    rng = np.random.default_rng(7)
    m, n = 8, 64
    cases = []
    for _ in range(20):  # G lower with offsets {0, -1, -m}, M = G^T G (7 diagonals)
        G = np.diag(rng.uniform(0.5, 2.0, n))
        G += np.diag(-rng.uniform(0.0, 1.0, n - 1), -1) + np.diag(-rng.uniform(0.0, 1.0, n - m), -m)
        cases.append((G.T @ G).astype(np.float32))
    for _ in range(20):  # dense symmetric, shifted to be barely positive definite
        B = rng.standard_normal((32, 32)).astype(np.float32)
        S = B + B.T
        cases.append((S - (np.linalg.eigvalsh(S.astype(np.float64))[0] - 1e-3) * np.eye(32)).astype(np.float32))
    for M in cases:
        Mp = _bf16_round(M)
        np.fill_diagonal(Mp, _bf16_round(np.diag(M) + np.float32(1 / 128) * np.abs(M).sum(1, dtype=np.float32)))
        assert np.array_equal(Mp, Mp.T)
        assert np.linalg.eigvalsh((Mp - M).astype(np.float64))[0] >= -1e-12 * np.abs(M).max()
        assert np.linalg.eigvalsh(Mp.astype(np.float64))[0] > 0


def test_bench_byte_model_and_launch_count():
    """The roofline's algorithmic bytes and the launch count the bench reports: on-chip steps move
    only the matrix diagonals (A in FP32, M = G^T G in bfloat16); the CSR schedules move the values
    and six vector streams; each timed step launches the build (two kernels per 64 systems), the
    pattern analysis and the solve."""
    import sys
    sys.path.insert(0, str(ROOT))
    import bench
    n, nnz = 512 * 512, 1308672
    assert bench.bytes_per_system_iter(n, nnz, "learned", "onchip", 5, 7) == (5 * 4 + 7 * 2) * n
    assert bench.bytes_per_system_iter(n, nnz, "jacobi", "onchip", 5, 7) == 5 * 4 * n + 4 * n
    assert bench.bytes_per_system_iter(n, nnz, "plain", "cluster8") == nnz * 4 + 6 * n * 4
    assert bench.launches_per_solve("onchip", "learned", 256) == 4 * 2 + (1 + 2 * 2)
    assert bench.launches_per_solve("onchip", "plain", 256) == 1 + 2
    assert bench.launches_per_solve("cluster8", "jacobi", 2048) == 2
    assert bench.launches_per_solve("onchip", "learned", 256, "auto") == 4 * 2 + (1 + 2 * 2) + 1
    comp = bench.companion_roofline(40, 1000.0, n, 5, 7, 0.5, 6754.8)
    assert comp["bytes_per_row_step"] == 5 * 4 + 7 * 2 + 48
    assert comp["dram_bytes_est"] == 40 * 1000.0 * 82 * n
    assert bench.companion_roofline(None, 1000.0, n, 5, 7, 0.5, 6754.8) is None


def test_reference_lanczos_step_timer_runs_the_reference_body():
    """The per-configuration CPU timing drives the reference's own Lanczos body for a few steps with
    the basis of a full run, and puts its loop driver back afterwards."""
    import sys
    sys.path.insert(0, str(ROOT))
    import bench
    cola_ref = bench.reference_package()
    if cola_ref is None:
        pytest.skip("the reference package is not installed in baseline/_ref")
    A = torch.randn(64, 64, dtype=torch.float64, generator=torch.Generator().manual_seed(0))
    op = cola_ref.PSD(cola_ref.ops.Dense(A @ A.T + 64 * torch.eye(64, dtype=torch.float64)))
    before = op.xnp.while_loop_winfo
    t = bench._reference_lanczos_step_seconds(cola_ref, op, torch.randn(64, 2, dtype=torch.float64), 20, k_steps=2)
    assert t > 0 and op.xnp.while_loop_winfo is before


def test_c_program_links_and_calls_the_abi(tmp_path):
    """The drop-in boundary from C, without Python: a program compiled against include/colagb.h and
    linked to libcolagb.so calls entry points that need no GPU (version, argument validation and the
    per-thread error text) and gets the documented status codes."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = _capi.LIB_PATH
    src = tmp_path / "abi.c"
    src.write_text(r'''
#include <stdio.h>
#include <string.h>
#include "colagb.h"
int main(void) {
  int32_t v = 0, a = 0;
  if (colagb_version(&v, &a) != COLAGB_OK || a != 1003) return 1;
  /* a null output pointer is an argument error with a message */
  if (colagb_onchip_schedule_info(1024, 32, NULL) != COLAGB_ERR_INVALID) return 2;
  if (strlen(colagb_last_error()) == 0) return 3;
  /* an empty operator description is rejected before any device work */
  colagb_op* h = NULL;
  if (colagb_op_create(NULL, 0, 0, &h) == COLAGB_OK) return 4;
  printf("ok %d\n", (int)v);
  return 0;
}
''')
    exe = tmp_path / "abi"
    subprocess.run([cc, str(src), "-I", str(ROOT / "include"), "-L", str(lib.parent), "-lcolagb",
                    f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stderr)
    assert out.stdout.startswith("ok ")
