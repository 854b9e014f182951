"""A Matrix Market file straight into the device CG (the reference's tests read tests/data/*.mtx)."""
import numpy as np
import pytest
import scipy.io
import scipy.sparse
import scipy.sparse.linalg
import torch

from cola_gb300.annotations import PSD
from cola_gb300.io import load_mtx
from cola_gb300.linalg.inverse import cg

pytestmark = pytest.mark.gpu


def test_symmetric_mtx_solves_with_device_cg(tmp_path):
    m = 20
    T = scipy.sparse.diags([-1, 2.2, -1], [-1, 0, 1], shape=(m, m))
    A = (scipy.sparse.kron(T, scipy.sparse.eye(m)) + scipy.sparse.kron(scipy.sparse.eye(m), T)).tocoo()
    p = tmp_path / "lap.mtx"
    scipy.io.mmwrite(str(p), A, symmetry="symmetric")
    op = load_mtx(p, device="cuda", dtype=torch.float64)
    b = np.random.default_rng(0).standard_normal(m * m)
    x, info = cg(PSD(op), torch.tensor(b, device="cuda"), tol=1e-10, max_iters=2000)
    xs = scipy.sparse.linalg.spsolve(A.tocsc(), b)
    np.testing.assert_allclose(x.cpu().numpy(), xs, rtol=1e-7, atol=1e-9)
    assert op.nnz == A.nnz
