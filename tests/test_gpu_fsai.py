"""Learned FSAI preconditioner: kernels against the float64 CPU oracle (oracle/fsai.py), gradients of
the hand-written backward pass, and what the preconditioner buys inside the batched solver."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle.fsai as OF
from cola_gb300 import _capi
from cola_gb300.linalg.batched import FsaiPattern, solve_batched
from cola_gb300.precond import learned_fsai as L
from cola_gb300.workloads import diffusion_family_2d

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")


def rel(a, b):
    a, b = a.detach().double().cpu(), b.detach().double().cpu()
    return float((a - b).norm() / b.norm().clamp_min(1e-300))


@pytest.fixture(scope="module")
def small_family():
    fam, B, coeff, _ = diffusion_family_2d([101, 102, 103], m=16, device=DEV)
    return fam, B


def test_stencil_and_features(small_family):
    fam, _ = small_family
    st = L.stencil(fam)
    m = 16
    n = m * m
    for s in range(fam.num_systems):
        A = torch.sparse_csr_tensor(fam.indptr.long(), fam.indices.long(), fam.values[s].double(), (n, n)).to_dense()
        x = torch.randn(n, dtype=torch.float64, device=DEV)
        y = OF.apply_A(st[s: s + 1].double(), x.view(1, m, m)).view(-1)
        assert rel(y, A @ x) < 1e-6
    f = L.features(st)
    assert rel(f, OF.features(st.double().cpu())) < 1e-6


def test_conv_forward_matches_float64(small_family):
    fam, _ = small_family
    net = L.FsaiNet(DEV, seed=3)
    net.params.add_(0.05 * torch.randn_like(net.params))  # non-zero last layer
    st = L.stencil(fam)
    acts = net.forward(L.features(st))
    ref = OF.net_forward(net.params.double().cpu(), OF.features(st.double().cpu()))
    assert rel(acts[-1], ref) < 1e-5


def test_assemble_compact_and_closed_form(small_family):
    fam, _ = small_family
    st = L.stencil(fam)
    o = 0.1 * torch.randn((fam.num_systems, 3, 16, 16), device=DEV)
    g = L.assemble(st, o)
    gN, gW, gC = OF.assemble(st.double().cpu(), o.double().cpu())
    assert rel(g[:, 0], gN) < 1e-6 and rel(g[:, 1], gW) < 1e-6 and rel(g[:, 2], gC) < 1e-6
    pat = FsaiPattern(fam.indptr, fam.indices)
    gv = L.compact(g, pat)
    # compact CSR G applied to x equals the stencil form
    n = 256
    for s in range(fam.num_systems):
        G = torch.sparse_csr_tensor(pat.g_indptr.long(), pat.g_indices.long(), gv[s].double(), (n, n)).to_dense()
        x = torch.randn(n, dtype=torch.float64, device=DEV)
        y = OF.apply_G(g[s: s + 1, 0].double(), g[s: s + 1, 1].double(), g[s: s + 1, 2].double(), x.view(1, 16, 16))
        assert rel(G @ x, y.view(-1)) < 1e-6
    # closed-form FSAI row: (G A G^T)_pp = 1 on the pattern's Schur complement
    g0 = L.assemble(st, None)
    A = torch.sparse_csr_tensor(fam.indptr.long(), fam.indices.long(), fam.values[0].double(), (n, n)).to_dense()
    G0 = torch.sparse_csr_tensor(pat.g_indptr.long(), pat.g_indices.long(), L.compact(g0, pat)[0].double(),
                                 (n, n)).to_dense()
    assert torch.allclose(torch.diagonal(G0 @ A @ G0.T), torch.ones(n, dtype=torch.float64, device=DEV), atol=1e-5)


def test_gradients_match_cpu_oracle(small_family):
    fam, _ = small_family
    m, n, S = 16, 256, fam.num_systems
    net = L.FsaiNet(DEV, seed=5)
    net.params.add_(0.05 * torch.randn(net.params.shape, generator=torch.Generator().manual_seed(1)).to(DEV))
    st = L.stencil(fam)
    r = torch.randn((S, m, m), device=DEV)
    e = torch.empty_like(r)
    for s in range(S):
        A = torch.sparse_csr_tensor(fam.indptr.long(), fam.indices.long(), fam.values[s].double(), (n, n)).to_dense()
        e[s] = torch.linalg.solve(A, r[s].reshape(-1).double()).float().view(m, m)
    acts = net.forward(L.features(st))
    o = acts[-1]
    gst = L.assemble(st, o)
    loss, dout = L.loss_and_grad(st, o, gst, r, e)
    grad = net.backward(acts, dout)
    loss_o, grad_o, dout_o, _ = OF.loss_and_grads(net.params.cpu(), st.cpu(), r.cpu(), e.cpu())
    assert abs(float(loss) - loss_o) < 1e-4 * abs(loss_o) + 1e-6
    assert rel(dout, dout_o) < 2e-3
    assert rel(grad, grad_o) < 2e-3
    # per layer as well (the first layer's gradient flows through two ReLU masks)
    for li in range(3):
        off, ln = net.layer_slice(li)
        assert rel(grad[off: off + ln], grad_o[off: off + ln]) < 5e-3, li


def test_spectral_loss_gradients_match_cpu_oracle(small_family):
    """The Rayleigh-quotient (log-condition proxy) loss: value, d/d(o) and d/d(params) against float64
    autograd, with one pair of each kind (white-noise error weighted +1, smooth error -1)."""
    fam, _ = small_family
    m, n, S = 16, 256, fam.num_systems
    net = L.FsaiNet(DEV, seed=7)
    net.params.add_(0.05 * torch.randn(net.params.shape, generator=torch.Generator().manual_seed(2)).to(DEV))
    st = L.stencil(fam)
    e = torch.randn((S, m, m), device=DEV)
    e[1] = torch.linspace(0, 1, m, device=DEV)[:, None] * torch.linspace(0, 1, m, device=DEV)[None, :]  # smooth
    r = torch.stack([OF.apply_A(st[s: s + 1].double(), e[s: s + 1].double())[0] for s in range(S)]).float()
    w = torch.tensor([0.5, -1.0, 0.5], device=DEV)
    acts = net.forward(L.features(st))
    o = acts[-1]
    gst = L.assemble(st, o)
    loss, dout = L.rq_loss_and_grad(st, o, gst, r, e, w)
    grad = net.backward(acts, dout)
    loss_o, grad_o, dout_o, _ = OF.rq_loss_and_grads(net.params.cpu(), st.cpu(), r.cpu(), e.cpu(), w.cpu())
    assert abs(float(loss) - loss_o) < 1e-4 * abs(loss_o) + 1e-5
    assert rel(dout, dout_o) < 2e-3
    assert rel(grad, grad_o) < 2e-3


def test_adam_step():
    p = torch.randn(1000, device=DEV)
    g = torch.randn(1000, device=DEV)
    m1 = torch.zeros_like(p)
    m2 = torch.zeros_like(p)
    p0 = p.clone()
    L.adam_step(p, g, m1, m2, 1, 1e-2)
    # first bias-corrected Adam step moves every parameter by lr * sign(g) (up to eps)
    assert torch.allclose(p0 - p, 1e-2 * torch.sign(g), atol=1e-6)


def test_training_reduces_loss_and_preconditioner_converges():
    fam, B, _, _ = diffusion_family_2d(list(range(200, 208)), m=32, device=DEV)
    m = 32
    X, info = solve_batched(fam, B, precond="jacobi", tol=1e-7)
    nrm = B.norm(dim=1, keepdim=True)
    st = L.stencil(fam, m)
    r = (B / nrm).float().view(-1, m, m)
    e = (X / nrm).float().view(-1, m, m)
    net = L.FsaiNet(DEV, seed=0)
    hist = L.train(net, st, r, e, epochs=12, batch=4, lr=3e-3, log=lambda *_: None)
    assert hist[-1] < hist[0]
    fam2, B2, _, _ = diffusion_family_2d(list(range(300, 306)), m=32, device=DEV)
    res = {}
    for name, kw in [("jacobi", dict(precond="jacobi")),
                     ("fsai", dict(precond="fsai", fsai=L.g_values(fam2, None))),
                     ("learned", dict(precond="fsai", fsai=L.g_values(fam2, net)))]:
        Xs, inf = solve_batched(fam2, B2, tol=1e-8, **kw)
        assert float(inf["relres"].max()) <= 1e-8
        res[name] = float(inf["iterations"].double().mean())
    # closed-form FSAI needs fewer iterations than Jacobi
    assert res["fsai"] < res["jacobi"], res


@pytest.mark.skipif(not L.WEIGHTS.exists(), reason="trained weights not present")
def test_trained_network_beats_jacobi_on_held_out_512():
    """What the shipped factor gains over Jacobi-PCG and over closed-form FSAI, measured in CG
    iterations on held-out 512 x 512 instances (seeds never used in fitting)."""
    fam, B, _, _ = diffusion_family_2d(list(range(4100, 4108)), m=512, device=DEV)
    net = L.FsaiNet.load(device=DEV)
    _, ij = solve_batched(fam, B, precond="jacobi", tol=1e-8)
    _, il = solve_batched(fam, B, precond="fsai", fsai=L.g_values(fam, net), tol=1e-8)
    assert float(il["relres"].max()) <= 1e-8 and float(ij["relres"].max()) <= 1e-8
    it_j = float(ij["iterations"].double().mean())
    it_l = float(il["iterations"].double().mean())
    assert it_l < 0.8 * it_j, (it_l, it_j)
    # and over closed-form FSAI on the same pattern (the fitted over-relaxation of its off-diagonals)
    _, ic = solve_batched(fam, B, precond="fsai", fsai=L.g_values(fam, None), tol=1e-8)
    it_c = float(ic["iterations"].double().mean())
    assert it_l < it_c, (it_l, it_c)


@pytest.mark.parametrize("m", [20, 45, 64])
def test_fused_build_matches_layered_path(m):
    """colagb_fsai_net_build (features, three convolutions and the assembly of a 32 x 32 tile in
    shared memory) gives the values of the layer-by-layer kernels; every layer random, biases too,
    grids whose side is not a multiple of the tile.  Both evaluate the same FMAs in the same order,
    so the comparison is to 1 ulp-level (2e-6 relative)."""
    fam, _, _, _ = diffusion_family_2d(list(range(700, 705)), m=m, device=DEV)
    net = L.FsaiNet(DEV, seed=3)
    g = torch.Generator().manual_seed(11)
    net.params.copy_((0.3 * torch.randn(net.params.shape, generator=g)).to(DEV))
    pat = FsaiPattern(fam.indptr, fam.indices)
    _, fused = L.g_values(fam, net, pat, batch=3)
    _, layered = L.g_values_layered(fam, net, pat, batch=3)
    assert torch.isfinite(fused).all()
    assert (fused - layered).abs().max().item() <= 2e-6 * layered.abs().max().item()
    _, cf = L.g_values(fam, None, pat)
    _, cl = L.g_values_layered(fam, None, pat)
    assert torch.equal(cf, cl)


def test_fused_build_rejects_other_network_shapes():
    fam, _, _, _ = diffusion_family_2d([1], m=16, device=DEV)
    pat = FsaiPattern(fam.indptr, fam.indices)
    st = L.stencil(fam, 16)
    out = torch.empty((1, pat.g_nnz), dtype=torch.float32, device=DEV)
    bad = torch.zeros(100, dtype=torch.float32, device=DEV)
    rc = _capi.load().colagb_fsai_net_build(st.data_ptr(), bad.data_ptr(), bad.numel(), 16, 1, pat.g_indptr.data_ptr(),
                                            pat.g_nnz, out.data_ptr(), None, _capi.stream_ptr(DEV))
    assert rc != 0


def test_overlapped_build_and_no_wait_pipeline_matches_sequential():
    """The bench's pipeline: family i + 1's learned factor is built on a side stream while family i
    solves (wait=False returns at once); every solution equals the sequential calls' bit for bit."""
    from cola_gb300.linalg.batched import BatchedCSR
    fam, B, _, _ = diffusion_family_2d(list(range(80, 88)), m=64, device=DEV)
    fam2 = BatchedCSR(fam.indptr, fam.indices, fam.values.flip(0).contiguous())
    net = L.FsaiNet.load(device=DEV) if L.WEIGHTS.exists() else L.FsaiNet(DEV, seed=1)
    pat = FsaiPattern(fam.indptr, fam.indices)
    seq = [solve_batched(f, B, precond="fsai", fsai=L.g_values(f, net, pat), tol=1e-8)[0] for f in (fam, fam2)]
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    side = torch.cuda.Stream()
    X0, i0 = solve_batched(fam, B, precond="fsai", fsai=L.g_values(fam, net, pat), tol=1e-8, wait=False)
    with torch.cuda.stream(side):
        fs1 = L.g_values(fam2, net, pat)
        ready = torch.cuda.Event()
        ready.record(side)
    st.wait_event(ready)
    fs1[1].record_stream(st)
    X1, i1 = solve_batched(fam2, B, precond="fsai", fsai=fs1, tol=1e-8, wait=False)
    torch.cuda.synchronize()
    assert i0["schedule"] == "onchip" and i0["sweeps"] is None
    assert torch.equal(X0, seq[0]) and torch.equal(X1, seq[1])
    assert bool((i1["status"] == 1).all())


def test_no_wait_solves_on_two_streams_do_not_share_scratch():
    """Two batched solves enqueued with wait=False on different streams at once: each stream has its
    own library scratch (the on-chip schedule's diagonal slots and system counter live there), so
    both give the sequential solutions bit for bit."""
    from cola_gb300.linalg.batched import BatchedCSR
    fam, B, _, _ = diffusion_family_2d(list(range(90, 96)), m=64, device=DEV)
    fam2 = BatchedCSR(fam.indptr, fam.indices, (1.5 * fam.values).contiguous())
    seq = [solve_batched(f, B, precond="jacobi", tol=1e-8)[0] for f in (fam, fam2)]
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    X0, _ = solve_batched(fam, B, precond="jacobi", tol=1e-8, wait=False)
    with torch.cuda.stream(side):
        X1, _ = solve_batched(fam2, B, precond="jacobi", tol=1e-8, wait=False)
    torch.cuda.synchronize()
    assert torch.equal(X0, seq[0]) and torch.equal(X1, seq[1])
