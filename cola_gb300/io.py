"""Matrix Market input for the sparse operators.

``load_mtx(path, device)`` reads a Matrix Market coordinate file -- field ``real``, ``integer`` or
``pattern``, symmetry ``general``, ``symmetric`` or ``skew-symmetric`` -- and returns a
``cola_gb300.ops.Sparse``.

- The text is parsed on the host; that is the only host step.
- The (row, col, value) triplets go to the device in one copy each.
- The CSR (row sort, duplicate summing, column order) is built there by ``Sparse``.
- Symmetric files list one triangle; the mirrored entries are added on the device.

This replaces the host scipy COO -> CSR conversion of the reference's ``Sparse`` (operators.py:64-75)
for files in the format its tests read (``tests/data/*.mtx``).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import torch

from . import ops as O


def _header(f):
    line = f.readline()
    if isinstance(line, bytes):
        line = line.decode()
    parts = line.strip().lower().split()
    if len(parts) < 5 or parts[0] != "%%matrixmarket" or parts[1] != "matrix":
        raise ValueError("not a Matrix Market matrix file")
    fmt, field, symmetry = parts[2], parts[3], parts[4]
    if fmt != "coordinate":
        raise NotImplementedError("only coordinate (sparse) Matrix Market files are read")
    if field not in ("real", "integer", "pattern", "double"):
        raise NotImplementedError(f"Matrix Market field {field!r} is not supported")
    if symmetry not in ("general", "symmetric", "skew-symmetric"):
        raise NotImplementedError(f"Matrix Market symmetry {symmetry!r} is not supported")
    return field, symmetry


def load_mtx(path, device="cuda", dtype=torch.float32) -> O.Sparse:
    """Read a Matrix Market coordinate file into a device CSR operator."""
    path = Path(path)
    with open(path, "rb") as f:
        field, symmetry = _header(f)
        line = f.readline()
        while line.lstrip().startswith(b"%") or not line.strip():
            line = f.readline()
        rows, cols, nnz = (int(x) for x in line.split()[:3])
        ncol = 2 if field == "pattern" else 3
        data = np.loadtxt(f, dtype=np.float64, ndmin=2, max_rows=nnz) if nnz else np.zeros((0, ncol))
    if data.shape[0] != nnz or (nnz and data.shape[1] < ncol):
        raise ValueError(f"{path}: expected {nnz} entries of {ncol} columns, found {data.shape}")
    r = torch.from_numpy(data[:, 0].astype(np.int64) - 1)
    c = torch.from_numpy(data[:, 1].astype(np.int64) - 1)
    v = torch.ones(nnz, dtype=torch.float64) if field == "pattern" else torch.from_numpy(data[:, 2].copy())
    if nnz and (int(r.min()) < 0 or int(c.min()) < 0 or int(r.max()) >= rows or int(c.max()) >= cols):
        raise ValueError(f"{path}: entry index outside the {rows} x {cols} matrix")
    r, c, v = r.to(device), c.to(device), v.to(device=device, dtype=dtype)
    if symmetry != "general":
        off = r != c
        sign = -1.0 if symmetry == "skew-symmetric" else 1.0
        r, c, v = torch.cat([r, c[off]]), torch.cat([c, r[off]]), torch.cat([v, sign * v[off]])
    return O.Sparse(v, r, c, (rows, cols))
