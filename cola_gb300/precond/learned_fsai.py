"""Learned FSAI preconditioner for families of 5-point operators on an m x m grid.

A three-layer 3x3 convolutional network (6 -> 16 -> 16 -> 3 channels, ReLU) reads scale-free
features of each operator's coefficients and outputs per-cell scalings of the closed-form FSAI
factor G on the operator's lower pattern; the CG preconditioner is P = G^T G (it plugs into the
CG(P=...) hook, cola/linalg/inverse/cg.py:124, 150 -- see ``learned_preconditioner``).  The last
layer starts at zero, so an untrained network reproduces closed-form FSAI; Jacobi-PCG stays the
fallback and the FP64 true residual the judge (colagb_cg_batched_csr_solve).

What the shipped weights are, in plain words: the network's last layer is zero and its bias is the
constant (0, atanh 0.9, atanh 0.775), a global over-relaxation of the two off-diagonals of G found
by direct search on PCG iteration counts.  Gradient training with this project's kernels lowered
its losses but not the iteration count, and no per-cell or per-operator output has beaten the
constant: choosing the best over-relaxation separately for each operator saves at most 1.0 % of
the iterations on 128 training instances (train_fsai --headroom), about the run-to-run spread of
FP32 CG step counts.  With this 3-entry factor pattern there is nothing left for a prediction to
gain, so the "learned" factor is a fitted constant on top of closed-form FSAI (4-5 % fewer steps).

Every forward, backward, loss and optimiser step runs in libcolagb kernels
(colagb_conv3x3_forward/backward, colagb_fsai_*, colagb_adam_step); torch only holds memory.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import torch

from .. import _capi
from ..linalg.batched import BatchedCSR, FsaiPattern

WEIGHTS = Path(__file__).resolve().parent / "fsai_net.pt"
LAYERS = [(6, 16, True), (16, 16, True), (16, 3, False)]


def _lib():
    return _capi.load()


def _sp(t):
    return _capi.stream_ptr(t.device)


class FsaiNet:
    """Parameters in one flat float32 buffer: per layer W (cout, cin, 3, 3) then b (cout)."""

    def __init__(self, device="cuda", seed: int = 0):
        self.device = torch.device(device)
        sizes = []
        for cin, cout, _ in LAYERS:
            sizes += [cout * cin * 9, cout]
        self.sizes = sizes
        self.params = torch.zeros(sum(sizes), dtype=torch.float32, device=self.device)
        g = torch.Generator(device="cpu").manual_seed(seed)
        for li, (cin, cout, _) in enumerate(LAYERS[:-1]):
            W, _ = self.layer(li)
            W.copy_(torch.randn(W.shape, generator=g) * math.sqrt(2.0 / (cin * 9)))

    def layer(self, li):
        off = sum(self.sizes[: 2 * li])
        cin, cout, _ = LAYERS[li]
        W = self.params[off: off + cout * cin * 9].view(cout, cin, 3, 3)
        b = self.params[off + cout * cin * 9: off + cout * cin * 9 + cout]
        return W, b

    def layer_slice(self, li):
        off = sum(self.sizes[: 2 * li])
        cin, cout, _ = LAYERS[li]
        return off, cout * cin * 9 + cout

    # ---- forward / backward on (B, 6, H, W) features ----------------------------------------
    def forward(self, feats: torch.Tensor):
        lib = _lib()
        B, _, H, W = feats.shape
        acts = [feats]
        x = feats
        for li, (cin, cout, relu) in enumerate(LAYERS):
            Wt, b = self.layer(li)
            y = torch.empty((B, cout, H, W), dtype=torch.float32, device=feats.device)
            _capi.check(lib.colagb_conv3x3_forward(x.data_ptr(), B, cin, cout, H, W, Wt.data_ptr(), b.data_ptr(),
                                                   1 if relu else 0, y.data_ptr(), _sp(x)), "conv3x3 forward")
            acts.append(y)
            x = y
        return acts  # [features, h1, h2, o]

    def backward(self, acts, dout: torch.Tensor) -> torch.Tensor:
        lib = _lib()
        B, _, H, W = dout.shape
        grad = torch.zeros_like(self.params)
        g = dout
        for li in reversed(range(len(LAYERS))):
            cin, cout, relu = LAYERS[li]
            Wt, _ = self.layer(li)
            x_in, y = acts[li], acts[li + 1]
            gin = torch.empty_like(x_in) if li > 0 else None
            nb = C.c_size_t()
            _capi.check(lib.colagb_conv3x3_backward_scratch_bytes(cin, cout, C.byref(nb)), "conv scratch")
            scratch = _capi.workspace(nb.value, dout.device)
            off, ln = self.layer_slice(li)
            gw = grad[off: off + ln]
            _capi.check(lib.colagb_conv3x3_backward(g.data_ptr(), y.data_ptr() if relu else None, x_in.data_ptr(), B,
                                                    cin, cout, H, W, Wt.data_ptr(),
                                                    gin.data_ptr() if gin is not None else None, gw.data_ptr(),
                                                    scratch.data_ptr(), nb.value, _sp(g)), "conv3x3 backward")
            g = gin
        return grad

    def state_dict(self):
        return {"params": self.params.detach().cpu(), "layers": LAYERS}

    def load_state_dict(self, d):
        self.params.copy_(d["params"].to(self.device))

    @classmethod
    def load(cls, path=WEIGHTS, device="cuda"):
        d = torch.load(path, map_location="cpu", weights_only=False)
        net = cls(device)
        net.load_state_dict(d)
        return net


# ---------------------------------------------------------------------------------------------
# operator-side kernels

def grid_side(fam: BatchedCSR) -> int:
    m = int(round(math.sqrt(fam.n)))
    if m * m != fam.n:
        raise ValueError("learned FSAI needs an m x m grid operator")
    return m


def stencil(fam: BatchedCSR, m: int | None = None, err: torch.Tensor | None = None) -> torch.Tensor:
    """(S, 5, m, m) [N, W, C, E, S] stencil of every operator of the family.

    With ``err`` (a device int32 flag) the pattern check is left to the caller, who reads the flag
    once after several calls; without it the flag is read here."""
    m = m or grid_side(fam)
    S = fam.num_systems
    st = torch.empty((S, 5, m, m), dtype=torch.float32, device=fam.values.device)
    own = err is None
    if own:
        err = torch.zeros(1, dtype=torch.int32, device=fam.values.device)
    vals = fam.values.to(torch.float32).contiguous()
    _capi.check(_lib().colagb_grid5_stencil(fam.indptr.data_ptr(), fam.indices.data_ptr(), vals.data_ptr(),
                                            fam.indices.numel(), m, S, st.data_ptr(), err.data_ptr(), _sp(st)), "stencil")
    if own:
        check_stencil(err)
    return st


def check_stencil(err: torch.Tensor):
    if int(err.item()) != 0:
        raise ValueError("operator pattern is not the 5-point stencil of an m x m grid")


def features(st: torch.Tensor) -> torch.Tensor:
    S, _, m, _ = st.shape
    f = torch.empty((S, 6, m, m), dtype=torch.float32, device=st.device)
    _capi.check(_lib().colagb_fsai_features(st.data_ptr(), m, S, f.data_ptr(), _sp(st)), "features")
    return f


def assemble(st: torch.Tensor, o: torch.Tensor | None) -> torch.Tensor:
    S, _, m, _ = st.shape
    g = torch.empty((S, 3, m, m), dtype=torch.float32, device=st.device)
    _capi.check(_lib().colagb_fsai_assemble(st.data_ptr(), o.data_ptr() if o is not None else None, m, S, g.data_ptr(),
                                            _sp(st)), "assemble")
    return g


def compact(gst: torch.Tensor, pat: FsaiPattern, out: torch.Tensor | None = None) -> torch.Tensor:
    """G values on the CSR pattern of G, (S, g_nnz); ``out``: a contiguous tensor of that shape."""
    S, _, m, _ = gst.shape
    if out is None:
        out = torch.empty((S, pat.g_nnz), dtype=torch.float32, device=gst.device)
    _capi.check(_lib().colagb_fsai_compact(gst.data_ptr(), pat.g_indptr.data_ptr(), m, S, pat.g_nnz, out.data_ptr(),
                                           _sp(gst)), "compact")
    return out


def loss_and_grad(st, o, gst, r, e, want_grad=True):
    """Mean pair loss over systems and d(loss)/d(o)."""
    S, _, m, _ = st.shape
    n = m * m
    terms = torch.empty((3, S), dtype=torch.float64, device=st.device)
    scratch = _capi.workspace(3 * S * n * 4, st.device)
    dout = torch.empty((S, 3, m, m), dtype=torch.float32, device=st.device) if want_grad else None
    _capi.check(_lib().colagb_fsai_loss_grad(st.data_ptr(), o.data_ptr() if o is not None else None, gst.data_ptr(),
                                             r.data_ptr(), e.data_ptr(), m, S,
                                             dout.data_ptr() if dout is not None else None, terms.data_ptr(),
                                             scratch.data_ptr(), scratch.numel(), _sp(st)), "fsai loss")
    er, vAv, vr = terms[0], terms[1], terms[2]
    loss = ((vAv - 2 * vr + er) / er).mean()
    return loss, dout


def rq_loss_and_grad(st, o, gst, r, e, w, want_grad=True):
    """Spectral loss sum_s w_s log(|G r_s|^2 / e_s^T r_s) and d(loss)/d(o)."""
    S, _, m, _ = st.shape
    n = m * m
    terms = torch.empty((2, S), dtype=torch.float64, device=st.device)
    scratch = _capi.workspace(S * n * 4, st.device)
    dout = torch.empty((S, 3, m, m), dtype=torch.float32, device=st.device) if want_grad else None
    _capi.check(_lib().colagb_fsai_rq_loss_grad(st.data_ptr(), o.data_ptr() if o is not None else None, gst.data_ptr(),
                                                r.data_ptr(), e.data_ptr(), w.data_ptr(), m, S,
                                                dout.data_ptr() if dout is not None else None, terms.data_ptr(),
                                                scratch.data_ptr(), scratch.numel(), _sp(st)), "fsai rq loss")
    loss = (w.double() * torch.log(terms[1] / terms[0])).sum()
    return loss, dout


# ---------------------------------------------------------------------------------------------
# inference and training

def g_values(fam: BatchedCSR, net: FsaiNet | None, pat: FsaiPattern | None = None, batch: int = 64):
    """Compact G values (S, g_nnz) for the batched solver; net=None gives closed-form FSAI.

    Two kernels per batch of systems: the stencil extraction and the fused build
    (colagb_fsai_net_build: features, the network and the assembly in shared memory, or
    colagb_fsai_closed_build)."""
    m = grid_side(fam)
    pat = pat or FsaiPattern(fam.indptr, fam.indices)
    out = torch.empty((fam.num_systems, pat.g_nnz), dtype=torch.float32, device=fam.values.device)
    err = torch.zeros(1, dtype=torch.int32, device=fam.values.device)
    counter = torch.empty(1, dtype=torch.int32, device=fam.values.device)  # tiles in arrival order
    lib = _lib()
    for s0 in range(0, fam.num_systems, batch):
        sub = BatchedCSR(fam.indptr, fam.indices, fam.values[s0: s0 + batch])
        st = stencil(sub, m, err)
        dst = out[s0: s0 + batch]
        if net is not None:
            _capi.check(lib.colagb_fsai_net_build(st.data_ptr(), net.params.data_ptr(), net.params.numel(), m,
                                                  sub.num_systems, pat.g_indptr.data_ptr(), pat.g_nnz,
                                                  dst.data_ptr(), counter.data_ptr(), _sp(st)), "net build")
        else:
            _capi.check(lib.colagb_fsai_closed_build(st.data_ptr(), m, sub.num_systems, pat.g_indptr.data_ptr(),
                                                     pat.g_nnz, dst.data_ptr(), _sp(st)), "closed build")
    check_stencil(err)  # one host read for all batches
    return pat, out


def g_values_layered(fam: BatchedCSR, net: FsaiNet | None, pat: FsaiPattern | None = None, batch: int = 32):
    """The same values as ``g_values``, layer by layer (features, each convolution, assembly and
    compaction as separate kernels with their fields in device memory) -- the path training runs."""
    m = grid_side(fam)
    pat = pat or FsaiPattern(fam.indptr, fam.indices)
    out = torch.empty((fam.num_systems, pat.g_nnz), dtype=torch.float32, device=fam.values.device)
    for s0 in range(0, fam.num_systems, batch):
        sub = BatchedCSR(fam.indptr, fam.indices, fam.values[s0: s0 + batch])
        st = stencil(sub, m)
        o = net.forward(features(st))[-1] if net is not None else None
        compact(assemble(st, o), pat, out[s0: s0 + batch])
    return pat, out


def preconditioner_for(fam: BatchedCSR, coeff=None, net: FsaiNet | None = None, weights=WEIGHTS):
    """(FsaiPattern, G values) for solve_batched(..., precond='fsai', fsai=...) from the trained network."""
    if net is None:
        if not Path(weights).exists():
            raise FileNotFoundError(f"trained weights {weights} not found")
        net = FsaiNet.load(weights, device=fam.values.device)
    return g_values(fam, net)


def adam_step(params, grad, m1, m2, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    _capi.check(_lib().colagb_adam_step(params.data_ptr(), grad.data_ptr(), m1.data_ptr(), m2.data_ptr(),
                                        params.numel(), lr, b1, b2, eps, step, _sp(params)), "adam")


def train(net: FsaiNet, st_train: torch.Tensor, r_train: torch.Tensor, e_train: torch.Tensor, epochs: int = 10,
          batch: int = 16, lr: float = 3e-3, seed: int = 0, log=print, on_epoch=None, kind=None, state=None):
    """Minimise a loss over training systems (stencils st_train (N, 5, m, m), pairs (N, m*m)).
    kind None: the A-norm pair loss; kind (N,) int tensor: the spectral loss with kind 1 = white-noise
    error (top of the spectrum), 0 = smooth error (bottom); every batch holds both kinds.
    `on_epoch(ep, mean_loss)` runs after every epoch (validation, checkpointing).  `state`: a dict
    carrying the Adam moments and step count across calls (created when empty)."""
    N = st_train.shape[0]
    state = {} if state is None else state
    if "m1" not in state:
        state.update(m1=torch.zeros_like(net.params), m2=torch.zeros_like(net.params), step=0)
    m1, m2 = state["m1"], state["m2"]
    g = torch.Generator(device="cpu").manual_seed(seed)
    step = state["step"]
    hist = []
    for ep in range(epochs):
        perm = torch.randperm(N, generator=g)
        if kind is not None:  # alternate the two kinds so every batch holds both
            k_cpu = kind.cpu()
            hi, lo = perm[k_cpu[perm] == 1], perm[k_cpu[perm] == 0]
            q = min(hi.numel(), lo.numel())
            perm = torch.stack([hi[:q], lo[:q]], 1).flatten()
            N_eff = perm.numel()
        else:
            N_eff = N
        tot, cnt = 0.0, 0
        for s0 in range(0, N_eff - batch + 1, batch):
            idx = perm[s0: s0 + batch].to(st_train.device)
            st = st_train.index_select(0, idx).contiguous()
            r = r_train.index_select(0, idx).contiguous()
            e = e_train.index_select(0, idx).contiguous()
            acts = net.forward(features(st))
            o = acts[-1]
            gst = assemble(st, o)
            if kind is None:
                loss, dout = loss_and_grad(st, o, gst, r, e)
            else:
                kb = kind.index_select(0, idx).float()
                nh = kb.sum().clamp_min(1.0)
                nl = (1 - kb).sum().clamp_min(1.0)
                w = (kb / nh - (1 - kb) / nl).contiguous()
                loss, dout = rq_loss_and_grad(st, o, gst, r, e, w)
            grad = net.backward(acts, dout)
            step += 1
            state["step"] = step
            adam_step(net.params, grad, m1, m2, step, lr)
            tot += float(loss)
            cnt += 1
        hist.append(tot / max(cnt, 1))
        log(f"pass {ep}: mean loss {hist[-1]:.5f}")
        if on_epoch is not None:
            on_epoch(ep, hist[-1])
    return hist


# ---------------------------------------------------------------------------------------------
# the CG(P=...) hook: P = G^T G as a LinearOperator

def factor_operator(pat: FsaiPattern, g: torch.Tensor):
    """P = G^T G of one system as a LinearOperator (a Product of the two CSR factors), for the
    reference's preconditioner hook ``CG(P=...)`` (cola/linalg/inverse/cg.py:124, 150): CG applies it
    as P @ r on the device with the structured-matvec runtime.  ``g``: the (g_nnz,) G values of one
    system in the lower pattern's CSR order."""
    from .. import ops as O
    n = pat.g_indptr.numel() - 1
    g = g.to(torch.float32).contiguous()
    G = O.Sparse.from_csr(pat.g_indptr, pat.g_indices, g, (n, n))
    Gt = O.Sparse.from_csr(pat.gt_indptr, pat.gt_indices, g[pat.gt_perm.long()].contiguous(), (n, n))
    return O.Product(Gt, G)


def learned_preconditioner(A, net: FsaiNet | None = None, weights=WEIGHTS, closed_form: bool = False):
    """The trained network's FSAI preconditioner of a 5-point operator A (a Sparse LinearOperator on an
    m x m grid, rows i * m + j, FP32 values) as a LinearOperator P = G^T G, ready for
    ``cola.linalg.solve(PSD(A), b, CG(P=learned_preconditioner(A)))``.  ``closed_form`` builds the
    closed-form FSAI factor instead of the network's."""
    from .. import ops as O
    A0 = A  # PSD(...) / SelfAdjoint(...) keep the operator's class
    if not isinstance(A0, O.Sparse):
        raise NotImplementedError("the learned FSAI preconditioner is built for Sparse 5-point operators")
    fam = BatchedCSR(A0.indptr, A0.indices, A0.values.to(torch.float32)[None, :])
    if not closed_form and net is None:
        if not Path(weights).exists():
            raise FileNotFoundError(f"trained weights {weights} not found")
        net = FsaiNet.load(weights, device=A0.values.device)
    pat, g = g_values(fam, None if closed_form else net)
    return factor_operator(pat, g[0])
