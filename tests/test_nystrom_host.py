"""The Nystrom construction (get_nys_approx) against the reference's own outputs, on the host with a
plain FP64 tensor for A (the device operator path is in test_gpu_parity.py)."""
import numpy as np
import pytest
import torch

from cola_gb300.linalg.preconditioning import get_nys_approx
from cola_gb300.linalg.prng import PRNGKey, randn


def _golden(name):
    import pathlib
    return np.load(pathlib.Path(__file__).parent / "golden" / f"{name}.npz")


def test_nystrom_construction_matches_reference_f64():
    g = _golden("nystrom_f64")
    A = torch.from_numpy(g["A"])
    Omega = randn(A.shape[0], int(g["rank"]), dtype=torch.float64, key=PRNGKey(42))
    lam, U = get_nys_approx(A, Omega, eps=float(g["eps"]))
    np.testing.assert_allclose(lam.numpy(), g["Lambda"], rtol=1e-10, atol=1e-12)
    # P = I + U diag(min(lam) / lam - 1) U^T with mu = 0, which does not depend on U's signs
    s = lam.min() / lam - 1
    P = torch.eye(A.shape[0], dtype=torch.float64) + U @ torch.diag(s) @ U.T
    np.testing.assert_allclose(P.numpy(), g["P"], rtol=0, atol=1e-10)


def test_nystrom_construction_matches_reference_f32():
    g = _golden("nystrom_f32")
    A = torch.from_numpy(g["A"])
    Omega = randn(A.shape[0], int(g["rank"]), dtype=torch.float32, key=PRNGKey(42))
    lam, U = get_nys_approx(A, Omega, eps=float(g["eps"]))
    np.testing.assert_allclose(lam.numpy(), g["Lambda"], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("tag", ["f32", "f64"])
def test_nystrom_golden_is_a_preconditioner(tag):
    """The recorded P maps the top approximated eigenvalues of A down to min(Lambda): P A has a
    smaller spread than A."""
    g = _golden(f"nystrom_{tag}")
    A, P = g["A"].astype(np.float64), g["P"].astype(np.float64)
    ev_a = np.linalg.eigvalsh(A)
    ev_pa = np.sort(np.linalg.eigvals(P @ A).real)
    assert ev_pa[-1] / ev_pa[0] < ev_a[-1] / ev_a[0]
