"""Seeded synthetic inputs with the shapes and value distributions of the benchmark configurations
(no public dataset is involved).  Generation uses tensor ops on the target device; it is set-up
work, not part of any timed Krylov loop.
"""
from __future__ import annotations

import math

import torch

from .linalg.batched import BatchedCSR


# ---------------------------------------------------------------------------------------------
# dense SPD with a log-uniform spectrum (Q from the QR of an N(0,1) matrix)

def dense_spd(n: int = 2048, seed: int = 0, lo: float = 1e-2, hi: float = 1e2, dtype=torch.float32, device="cpu"):
    """A = Q diag(lam) Q^T, lam log-uniform in [lo, hi]; b ~ N(0, 1).  Returns (A, b, lam)."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    M = torch.randn(n, n, dtype=torch.float64, generator=g)
    Q, _ = torch.linalg.qr(M)
    lam = torch.exp(torch.empty(n, dtype=torch.float64).uniform_(math.log(lo), math.log(hi), generator=g))
    A = ((Q * lam) @ Q.T)
    A = 0.5 * (A + A.T)
    b = torch.randn(n, dtype=torch.float64, generator=g)
    return A.to(dtype).to(device), b.to(dtype).to(device), lam


# ---------------------------------------------------------------------------------------------
# 2-D / 3-D variable-coefficient diffusion (finite volumes, harmonic-mean faces, Dirichlet walls)

def grid_pattern_2d(m: int, device="cpu"):
    """CSR pattern of the 5-point stencil on an m x m grid, rows i*m + j, columns sorted."""
    n = m * m
    p = torch.arange(n, device=device)
    i, j = p // m, p % m
    cand = torch.stack([p - m, p - 1, p, p + 1, p + m], 1)
    ok = torch.stack([i > 0, j > 0, torch.ones_like(i, dtype=torch.bool), j < m - 1, i < m - 1], 1)
    counts = ok.sum(1)
    indptr = torch.zeros(n + 1, dtype=torch.int64, device=device)
    indptr[1:] = torch.cumsum(counts, 0)
    indices = cand[ok]
    return indptr.to(torch.int32), indices.to(torch.int32), ok


def diffusion_values_2d(a: torch.Tensor, ok: torch.Tensor) -> torch.Tensor:
    """CSR values (float32, pattern order of grid_pattern_2d) for cell coefficients a (S, m, m)."""
    S, m, _ = a.shape
    a = a.double()

    def harm(x, y):
        return 2 * x * y / (x + y)
    tN = torch.full_like(a, 0.0)
    tS = torch.full_like(a, 0.0)
    tW = torch.full_like(a, 0.0)
    tE = torch.full_like(a, 0.0)
    tN[:, 1:, :] = harm(a[:, 1:, :], a[:, :-1, :])   # face to row i-1
    tN[:, 0, :] = 2 * a[:, 0, :]
    tS[:, :-1, :] = harm(a[:, :-1, :], a[:, 1:, :])  # face to row i+1
    tS[:, -1, :] = 2 * a[:, -1, :]
    tW[:, :, 1:] = harm(a[:, :, 1:], a[:, :, :-1])
    tW[:, :, 0] = 2 * a[:, :, 0]
    tE[:, :, :-1] = harm(a[:, :, :-1], a[:, :, 1:])
    tE[:, :, -1] = 2 * a[:, :, -1]
    diag = tN + tS + tW + tE
    full = torch.stack([-tN, -tW, diag, -tE, -tS], -1).reshape(S, m * m, 5)
    return full[:, ok].to(torch.float32)


def matern32_field(m: int, ell: float, var: float, gen: torch.Generator, device) -> torch.Tensor:
    """Gaussian random field with Matern-3/2 covariance on the unit square (m x m cells), by
    circulant embedding on a periodic 2m x 2m grid (spectral density (3/ell^2 + 4 pi^2 |k|^2)^-5/2)."""
    N = 2 * m
    h = 1.0 / m
    k = torch.fft.fftfreq(N, d=h, device=device, dtype=torch.float64)
    k2 = k[:, None] ** 2 + k[None, :] ** 2
    S = (3.0 / ell**2 + 4 * math.pi**2 * k2) ** (-2.5)
    w = torch.randn(N, N, generator=gen, device=device, dtype=torch.float64)
    f = torch.fft.ifft2(torch.fft.fft2(w) * torch.sqrt(S)).real
    f = f * math.sqrt(var / S.mean().item())
    return f[:m, :m]


def diffusion_family_2d(seeds, m: int = 512, device="cuda", ell_range=(0.05, 0.2), var_range=(0.5, 2.0)):
    """The learned-preconditioner family: one operator per seed on a shared m x m 5-point pattern.

    Coefficient field exp(f), f a Matern-3/2 GRF with lengthscale ~ U[0.05, 0.2] and variance
    ~ U[0.5, 2]; b ~ N(0, 1).  Returns (BatchedCSR, B (S, n) float64, coeff (S, m, m) float32,
    params list)."""
    indptr, indices, ok = grid_pattern_2d(m, device)
    vals, Bs, coeffs, params = [], [], [], []
    for s in seeds:
        gen = torch.Generator(device=device).manual_seed(int(s))
        u = torch.rand(2, generator=gen, device=device, dtype=torch.float64).cpu()
        ell = ell_range[0] + (ell_range[1] - ell_range[0]) * float(u[0])
        var = var_range[0] + (var_range[1] - var_range[0]) * float(u[1])
        f = matern32_field(m, ell, var, gen, device)
        a = torch.exp(f)
        coeffs.append(a.float())
        vals.append(diffusion_values_2d(a[None], ok)[0])
        Bs.append(torch.randn(m * m, generator=gen, device=device, dtype=torch.float64))
        params.append((ell, var))
    return BatchedCSR(indptr, indices, torch.stack(vals)), torch.stack(Bs), torch.stack(coeffs), params


def rbf_systems(num: int = 256, seed: int = 3, n_range=(500, 8000), device="cuda"):
    """Dense RBF-kernel systems K + s^2 I: n_i uniform in n_range, points uniform in [0,1]^3, lengthscale
    uniform in [0.05, 0.5], s^2 log-uniform in [1e-3, 1e-1], FP32, one N(0,1) right-hand side each."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    mats, rhs, meta = [], [], []
    for _ in range(num):
        n = int(torch.randint(n_range[0], n_range[1] + 1, (1,), generator=g))
        ell = 0.05 + 0.45 * float(torch.rand(1, generator=g))
        s2 = math.exp(math.log(1e-3) + (math.log(1e-1) - math.log(1e-3)) * float(torch.rand(1, generator=g)))
        pts = torch.rand(n, 3, generator=g, dtype=torch.float64).to(device)
        d2 = torch.cdist(pts, pts).pow(2)
        K = torch.exp(-d2 / (2 * ell * ell))
        K.diagonal().add_(s2)
        mats.append(K.float())
        rhs.append(torch.randn(n, generator=g).to(device))
        meta.append((n, ell, s2))
    return mats, rhs, meta


def rbf_grid_kernel(m: int, ell: float, dtype=torch.float64, device="cuda"):
    """m x m RBF kernel on a uniform 1-D grid of [0, 1]."""
    x = torch.linspace(0, 1, m, dtype=dtype, device=device)
    return torch.exp(-((x[:, None] - x[None, :]) ** 2) / (2 * ell * ell))


def kron_rbf(seed: int = 4, m: int = 64, factors: int = 3, device="cuda", dtype=torch.float32):
    """Factors of Kronecker(K1, K2, K3): RBF kernels on 1-D grids, lengthscales uniform in [0.05, 0.3]."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    ells = [0.05 + 0.25 * float(torch.rand(1, generator=g)) for _ in range(factors)]
    return [rbf_grid_kernel(m, ell, device=device).to(dtype) for ell in ells], ells


def rgg_laplacian(num_points: int = 1 << 20, radius: float = 0.002, seed: int = 7, device="cuda"):
    """Unweighted graph Laplacian D - W of a random geometric graph: points uniform in [0,1]^2, an edge
    between points closer than `radius`.  Neighbours are found by binning points into cells of side
    >= radius and testing the 3x3 surrounding cells.  Returns CSR (indptr, indices, values float32)."""
    g = torch.Generator(device=device).manual_seed(seed)
    pts = torch.rand(num_points, 2, generator=g, device=device, dtype=torch.float64)
    nc = max(1, int(1.0 / radius))
    cell = (pts * nc).long().clamp_(0, nc - 1)
    cid = cell[:, 0] * nc + cell[:, 1]
    order = torch.argsort(cid)
    cid_sorted = cid[order]
    counts = torch.bincount(cid_sorted, minlength=nc * nc)
    start = torch.zeros(nc * nc + 1, dtype=torch.int64, device=device)
    start[1:] = torch.cumsum(counts, 0)
    maxc = int(counts.max())
    rows, cols = [], []
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            cx, cy = cell[:, 0] + dx, cell[:, 1] + dy
            ok = (cx >= 0) & (cx < nc) & (cy >= 0) & (cy < nc)
            nb = (cx.clamp(0, nc - 1) * nc + cy.clamp(0, nc - 1))
            s0, cnt = start[nb], counts[nb] * ok
            for k in range(maxc):
                has = cnt > k
                idx = torch.nonzero(has).flatten()
                if idx.numel() == 0:
                    break
                j = order[s0[idx] + k]
                d2 = ((pts[idx] - pts[j]) ** 2).sum(1)
                keep = (d2 < radius * radius) & (j != idx)
                rows.append(idx[keep])
                cols.append(j[keep])
    r = torch.cat(rows)
    c = torch.cat(cols)
    deg = torch.bincount(r, minlength=num_points).to(torch.float32)
    # CSR of D - W with columns sorted per row
    r_all = torch.cat([r, torch.arange(num_points, device=device)])
    c_all = torch.cat([c, torch.arange(num_points, device=device)])
    v_all = torch.cat([-torch.ones(r.numel(), device=device), deg])
    key = r_all * num_points + c_all
    o = torch.argsort(key)
    r_all, c_all, v_all = r_all[o], c_all[o], v_all[o]
    indptr = torch.zeros(num_points + 1, dtype=torch.int64, device=device)
    indptr[1:] = torch.cumsum(torch.bincount(r_all, minlength=num_points), 0)
    return indptr.to(torch.int32), c_all.to(torch.int32), v_all.to(torch.float32)


def diffusion_3d(m: int = 128, seed: int = 1, shift: float = 1e-3, device="cuda"):
    """7-point variable-coefficient diffusion on an m^3 grid, cell coefficients exp(g), g ~ N(0,1)
    i.i.d. per cell, harmonic-mean faces, Dirichlet walls, plus shift * I.  Returns CSR arrays."""
    n = m**3
    gen = torch.Generator(device=device).manual_seed(seed)
    a = torch.exp(torch.randn(m, m, m, generator=gen, device=device, dtype=torch.float64))
    p = torch.arange(n, device=device)
    z, y, x = p // (m * m), (p // m) % m, p % m
    offs = [(-m * m, z > 0, (-1, 0, 0)), (-m, y > 0, (0, -1, 0)), (-1, x > 0, (0, 0, -1)), (0, None, None),
            (1, x < m - 1, (0, 0, 1)), (m, y < m - 1, (0, 1, 0)), (m * m, z < m - 1, (1, 0, 0))]
    af = a.reshape(-1)
    diag = torch.full((n,), shift, dtype=torch.float64, device=device)
    cols, vals, oks = [], [], []
    for off, valid, _ in offs:
        if off == 0:
            continue
        nb = (p + off).clamp(0, n - 1)
        t_int = 2 * af * af[nb] / (af + af[nb])
        t = torch.where(valid, t_int, 2 * af)
        diag += t
    for off, valid, _ in offs:
        if off == 0:
            cols.append(p)
            vals.append(diag)
            oks.append(torch.ones(n, dtype=torch.bool, device=device))
        else:
            nb = (p + off).clamp(0, n - 1)
            t_int = 2 * af * af[nb] / (af + af[nb])
            cols.append(p + off)
            vals.append(-t_int)
            oks.append(valid)
    C = torch.stack(cols, 1)
    V = torch.stack(vals, 1)
    OK = torch.stack(oks, 1)
    counts = OK.sum(1)
    indptr = torch.zeros(n + 1, dtype=torch.int64, device=device)
    indptr[1:] = torch.cumsum(counts, 0)
    return indptr.to(torch.int32), C[OK].to(torch.int32), V[OK].to(torch.float32)
