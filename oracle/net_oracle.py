"""CPU oracle of the learned preconditioner network (test infrastructure only).

A plain torch restatement, FP64 by default, of the network the device kernels implement
(ifgf2d_gb300/csrc/precond_net.cuh): features per point, six circular 1D convolutions of
kernel 7 (6 -> 64 -> 64 x4 with residual connections -> 2), ReLU, the mean squared error
against (e - 2 r) e^{-i phi} / sigma, and M(r) = 2 r + sigma e^{i phi} (o_0 + i o_1), with
sigma = RMS(r) and the canonical phase phi = arg(sum r^2) / 2.  With bf16=True every tensor the
device stores in BF16 (features, weights, layer outputs) is rounded to BF16 on the way
forward; the backward pass treats the rounding as the identity.  Gradients of the device
kernels are checked against this module's autograd gradients, and this module's gradients
against finite differences.
"""
from __future__ import annotations

import numpy as np

LAYERS, TAPS, HIDDEN, IN_PAD, OUT_PAD, FEATURES, OUTPUTS = 6, 7, 64, 16, 16, 6, 2
BASE = 2.0
HALO = 3


def cin(l):
    return IN_PAD if l == 0 else HIDDEN


def cout(l):
    return OUT_PAD if l == LAYERS - 1 else HIDDEN


def num_params():
    return sum(cout(l) * TAPS * cin(l) + cout(l) for l in range(LAYERS))


def unpack(params):
    """flat parameters -> per layer (W[cout][7][cin], b[cout]) as numpy arrays"""
    out, off = [], 0
    for l in range(LAYERS):
        n = cout(l) * TAPS * cin(l)
        W = np.asarray(params[off:off + n]).reshape(cout(l), TAPS, cin(l))
        off += n
        b = np.asarray(params[off:off + cout(l)])
        off += cout(l)
        out.append((W, b))
    return out


def random_params(seed, scale_last=0.05):
    """seeded parameters with every layer nonzero (the device's fresh net has a zero output layer)"""
    rng = np.random.default_rng(seed)
    p = []
    for l in range(LAYERS):
        ci_real = FEATURES if l == 0 else HIDDEN
        co_real = OUTPUTS if l == LAYERS - 1 else HIDDEN
        sd = np.sqrt(2.0 / (TAPS * ci_real)) * (scale_last if l == LAYERS - 1 else (1.0 if l == 0 else 0.5))
        W = np.zeros((cout(l), TAPS, cin(l)))
        W[:co_real, :, :ci_real] = rng.normal(0.0, sd, (co_real, TAPS, ci_real))
        b = np.zeros(cout(l))
        b[:co_real] = rng.normal(0.0, 0.02, co_real)
        p += [W.ravel(), b]
    return np.concatenate(p).astype(np.float32)


def _torch():
    import torch
    return torch


def _round(x, bf16):
    if not bf16:
        return x
    torch = _torch()
    return x + (x.to(torch.bfloat16).to(x.dtype) - x).detach()


def features(r, geom, k, bf16=False):
    """(16, n) feature tensor of one sample, its sigma and its canonical phase factor e^{i phi}"""
    torch = _torch()
    r = torch.as_tensor(r)
    g = torch.as_tensor(geom).reshape(-1, 4)
    sigma = torch.sqrt(torch.mean(r.real ** 2 + r.imag ** 2))
    s2 = torch.sum(r * r)
    phi = 0.5 * torch.atan2(s2.imag, s2.real)
    c, s = torch.cos(phi), torch.sin(phi)
    if bf16:   # the device keeps sigma and the phase factor in FP32
        sigma = sigma.to(torch.float32).to(torch.float64)
        c = c.to(torch.float32).to(torch.float64)
        s = s.to(torch.float32).to(torch.float64)
    f = torch.zeros((IN_PAD, r.shape[0]), dtype=torch.float64)
    f[0] = (r.real * c + r.imag * s) / sigma
    f[1] = (r.imag * c - r.real * s) / sigma
    f[2] = g[:, 0] / k
    f[3] = g[:, 1]
    f[4] = g[:, 2]
    f[5] = k * g[:, 3]
    return _round(f, bf16), sigma, (c, s)


def _conv(x, W, b, bf16):
    torch = _torch()
    import torch.nn.functional as F
    xw = F.pad(x[None], (HALO, HALO), mode="circular")
    Wc = _round(W, bf16).permute(0, 2, 1)   # (cout, cin, taps)
    return F.conv1d(xw, Wc)[0] + b[:, None]


def forward(params_t, r, geom, k, bf16=False):
    """the two output channels o (2, n) for one sample; params_t: list of (W, b) torch tensors"""
    torch = _torch()
    x, sigma, rot = features(r, geom, k, bf16)
    W0, b0 = params_t[0]
    x = _round(torch.relu(_conv(x, W0, b0, bf16)), bf16)
    for l in range(1, LAYERS - 1):
        W, b = params_t[l]
        y = _round(torch.relu(_conv(x, W, b, bf16)), bf16)
        x = _round(y + x, bf16)
    W, b = params_t[LAYERS - 1]
    o = _conv(x, W, b, bf16)
    return o[:OUTPUTS], sigma, rot


def loss_and_grad(params, samples, bf16=False):
    """MSE over all points and both channels of every sample (r, e, geom, k) and its gradient
    w.r.t. the flat parameters (FP64 autograd)"""
    torch = _torch()
    flat = torch.tensor(np.asarray(params, dtype=np.float64), requires_grad=True)
    pt, off = [], 0
    for l in range(LAYERS):
        n = cout(l) * TAPS * cin(l)
        W = flat[off:off + n].reshape(cout(l), TAPS, cin(l))
        off += n
        b = flat[off:off + cout(l)]
        off += cout(l)
        pt.append((W, b))
    tot, cnt = 0.0, 0
    for (r, e, geom, k) in samples:
        o, sigma, (c, s) = forward(pt, r, geom, k, bf16)
        rt, et = torch.as_tensor(r), torch.as_tensor(e)
        dr, di = et.real - BASE * rt.real, et.imag - BASE * rt.imag
        t = torch.stack([(dr * c + di * s) / sigma, (di * c - dr * s) / sigma])
        tot = tot + torch.sum((o - t) ** 2)
        cnt += 2 * len(r)
    L = tot / cnt
    L.backward()
    return float(L.detach()), flat.grad.numpy().copy()


def apply(params, r, geom, k, bf16=False):
    """M(r) = 2 r + sigma e^{i phi} (o_0 + i o_1) for one sample"""
    torch = _torch()
    pt = [(torch.tensor(W), torch.tensor(b)) for (W, b) in unpack(np.asarray(params, dtype=np.float64))]
    with torch.no_grad():
        o, sigma, (c, s) = forward(pt, r, geom, k, bf16)
    o = o.numpy()
    return BASE * np.asarray(r) + float(sigma) * complex(float(c), float(s)) * (o[0] + 1j * o[1]), o
