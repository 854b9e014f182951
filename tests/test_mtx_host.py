"""Matrix Market reading (host parsing; the CSR build runs where the tensors live -- the CPU here,
so only the assembled pattern and values are checked, no compute call)."""
import numpy as np
import pytest
import scipy.io
import scipy.sparse
import torch

from cola_gb300.io import load_mtx


def _write(tmp_path, M, symmetry="general", field="real"):
    p = tmp_path / f"m_{symmetry}_{field}.mtx"
    scipy.io.mmwrite(str(p), M, symmetry=symmetry, field=field)
    return p


def _dense(op):
    D = torch.zeros(op.shape, dtype=torch.float64)
    rows = torch.repeat_interleave(torch.arange(op.shape[0]), (op.indptr[1:] - op.indptr[:-1]).long())
    D.index_put_((rows, op.indices.long()), op.values.double(), accumulate=True)
    return D.numpy()


@pytest.mark.parametrize("symmetry", ["general", "symmetric", "skew-symmetric"])
def test_coordinate_files_round_trip(tmp_path, symmetry):
    rng = np.random.default_rng(0)
    A = scipy.sparse.random(30, 30, density=0.1, random_state=1, format="coo").toarray()
    if symmetry == "symmetric":
        A = A + A.T
    elif symmetry == "skew-symmetric":
        A = A - A.T
    p = _write(tmp_path, scipy.sparse.coo_matrix(A), symmetry=symmetry)
    op = load_mtx(p, device="cpu", dtype=torch.float64)
    np.testing.assert_allclose(_dense(op), scipy.io.mmread(str(p)).toarray(), rtol=1e-14, atol=1e-14)
    # CSR invariants: sorted columns within each row, no duplicates
    ip, ix = op.indptr.long(), op.indices.long()
    for i in range(op.shape[0]):
        row = ix[ip[i]: ip[i + 1]]
        assert torch.all(row[1:] > row[:-1])
    assert rng is not None


def test_pattern_and_integer_fields(tmp_path):
    A = scipy.sparse.coo_matrix(np.array([[2, 0, 1], [0, 3, 0], [4, 0, 5]]))
    p = _write(tmp_path, A, field="integer")
    np.testing.assert_allclose(_dense(load_mtx(p, device="cpu", dtype=torch.float64)), A.toarray())
    p2 = _write(tmp_path, A, field="pattern")
    np.testing.assert_allclose(_dense(load_mtx(p2, device="cpu", dtype=torch.float64)), (A.toarray() != 0) * 1.0)


def test_rejects_dense_and_bad_files(tmp_path):
    p = tmp_path / "dense.mtx"
    scipy.io.mmwrite(str(p), np.eye(3))
    with pytest.raises(NotImplementedError):
        load_mtx(p, device="cpu")
    q = tmp_path / "bad.mtx"
    q.write_text("%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 1.0\n4 1 2.0\n")
    with pytest.raises(ValueError):
        load_mtx(q, device="cpu")
    r = tmp_path / "junk.mtx"
    r.write_text("hello\n")
    with pytest.raises(ValueError):
        load_mtx(r, device="cpu")
