"""Learned-FSAI network, G assembly and pair loss restated on the CPU in float64 -- TEST
INFRASTRUCTURE ONLY (the gradient oracle for the hand-written training kernels).

Uses torch CPU autograd for the derivatives; the forward follows the same equations as
cola_gb300/csrc/fsai.cu (stencil [N, W, C, E, S] on an m x m grid, features, three 3x3 conv
layers with ReLU, closed-form FSAI reshaped by the network output and renormalised to
diag(G A G^T) = 1, loss
||G^T G r - e||_A^2 / ||e||_A^2 averaged over systems).
"""
from __future__ import annotations

import torch
import torch.nn.functional as F

LAYERS = [(6, 16, True), (16, 16, True), (16, 3, False)]


def unpack(params):
    out, off = [], 0
    for cin, cout, relu in LAYERS:
        W = params[off: off + cout * cin * 9].view(cout, cin, 3, 3)
        off += cout * cin * 9
        b = params[off: off + cout]
        off += cout
        out.append((W, b, relu))
    return out


def features(st):
    N, W_, C, E, S = st[:, 0], st[:, 1], st[:, 2], st[:, 3], st[:, 4]
    d = C
    f4 = torch.zeros_like(d)
    f5 = torch.zeros_like(d)
    f4[:, 1:, :] = torch.log(d[:, 1:, :] / d[:, :-1, :])
    f5[:, :, 1:] = torch.log(d[:, :, 1:] / d[:, :, :-1])
    return torch.stack([-N / d, -W_ / d, -E / d, -S / d, f4, f5], 1)


def net_forward(params, feats):
    x = feats
    for W, b, relu in unpack(params):
        x = F.conv2d(x, W, b, padding=1)
        if relu:
            x = torch.relu(x)
    return x


def closed_form(st):
    N, W_, C = st[:, 0], st[:, 1], st[:, 2]
    dN = torch.zeros_like(C)
    dW = torch.zeros_like(C)
    dN[:, 1:, :] = C[:, :-1, :]
    dW[:, :, 1:] = C[:, :, :-1]
    hasN = torch.zeros_like(C, dtype=torch.bool)
    hasW = torch.zeros_like(C, dtype=torch.bool)
    hasN[:, 1:, :] = True
    hasW[:, :, 1:] = True
    sch = C - torch.where(hasN, N * N / torch.where(hasN, dN, 1.0), 0.0) - \
        torch.where(hasW, W_ * W_ / torch.where(hasW, dW, 1.0), 0.0)
    inv = 1.0 / torch.sqrt(sch)
    fN = torch.where(hasN, -N / torch.where(hasN, dN, 1.0), 0.0) * inv
    fW = torch.where(hasW, -W_ / torch.where(hasW, dW, 1.0), 0.0) * inv
    return fN, fW, inv


def assemble(st, o):
    """H = (fN (1 + tanh o1), fW (1 + tanh o2), fC), each row renormalised so that (G A G^T)_pp = 1."""
    fN, fW, fC = closed_form(st)
    hN, hW, hC = (1 + torch.tanh(o[:, 1])) * fN, (1 + torch.tanh(o[:, 2])) * fW, fC
    C = st[:, 2]
    dN = torch.zeros_like(C)
    dW = torch.zeros_like(C)
    aN = torch.zeros_like(C)
    aW = torch.zeros_like(C)
    dN[:, 1:, :] = C[:, :-1, :]
    dW[:, :, 1:] = C[:, :, :-1]
    aN[:, 1:, :] = st[:, 0, 1:, :]
    aW[:, :, 1:] = st[:, 1, :, 1:]
    s = hC * hC * C + hN * hN * dN + hW * hW * dW + 2 * hC * (hN * aN + hW * aW)
    inv = 1.0 / torch.sqrt(s)
    return hN * inv, hW * inv, hC * inv


def apply_G(gN, gW, gC, x):
    y = gC * x
    y[:, 1:, :] += gN[:, 1:, :] * x[:, :-1, :]
    y[:, :, 1:] += gW[:, :, 1:] * x[:, :, :-1]
    return y


def apply_GT(gN, gW, gC, x):
    y = gC * x
    y[:, :-1, :] += gN[:, 1:, :] * x[:, 1:, :]
    y[:, :, :-1] += gW[:, :, 1:] * x[:, :, 1:]
    return y


def apply_A(st, x):
    y = st[:, 2] * x
    y[:, 1:, :] += st[:, 0, 1:, :] * x[:, :-1, :]
    y[:, :, 1:] += st[:, 1, :, 1:] * x[:, :, :-1]
    y[:, :, :-1] += st[:, 3, :, :-1] * x[:, :, 1:]
    y[:, :-1, :] += st[:, 4, :-1, :] * x[:, 1:, :]
    return y


def pair_loss(st, o, r, e):
    gN, gW, gC = assemble(st, o)
    v = apply_GT(gN, gW, gC, apply_G(gN, gW, gC, r))
    w = apply_A(st, v)
    er = (e * r).sum((1, 2))
    return (((v * w).sum((1, 2)) - 2 * (v * r).sum((1, 2)) + er) / er).mean()


def loss_and_grads(params, st, r, e):
    """Loss, d/d(params) and d/d(o) in float64 on the CPU."""
    params = params.detach().double().clone().requires_grad_(True)
    st, r, e = st.double(), r.double(), e.double()
    o = net_forward(params, features(st))
    o.retain_grad()
    loss = pair_loss(st, o, r, e)
    loss.backward()
    return float(loss), params.grad.clone(), o.grad.clone(), o.detach()


def rq_loss(st, o, r, e, w):
    """Spectral loss sum_s w_s log(|G r_s|^2 / e_s^T r_s)."""
    gN, gW, gC = assemble(st, o)
    t = apply_G(gN, gW, gC, r)
    R = (t * t).sum((1, 2)) / (e * r).sum((1, 2))
    return (w * torch.log(R)).sum()


def rq_loss_and_grads(params, st, r, e, w):
    """Spectral loss, d/d(params) and d/d(o) in float64 on the CPU."""
    params = params.detach().double().clone().requires_grad_(True)
    st, r, e, w = st.double(), r.double(), e.double(), w.double()
    o = net_forward(params, features(st))
    o.retain_grad()
    loss = rq_loss(st, o, r, e, w)
    loss.backward()
    return float(loss), params.grad.clone(), o.grad.clone(), o.detach()
