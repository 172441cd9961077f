"""CPU oracle of the learned coarse-velocity corrector (torch, float64).

TEST INFRASTRUCTURE ONLY: imported by tests/ and bench.py's CPU leg, never by
the product path.  The corrector has no counterpart in the reference; this
module restates the network of libvlagpu's vg_corr_* kernels in PyTorch on
the CPU so that their forward pass, loss and parameter gradients can be
checked:

- ``forward`` / ``loss_and_grads(..., emulate=False)`` is the plain FP64
  network, gradients by torch autograd.
- ``emulate=True`` rounds to bfloat16 at exactly the points where the CUDA
  kernels hold BF16 values (input features, weights, activations, the loss
  gradient and the back-propagated data gradients) and accumulates in FP64
  otherwise.  Its backward pass is written out by hand, in the kernels'
  order: weight gradients from the BF16 operands, data gradients masked by
  the ReLU of the stored BF16 activation, then rounded.

Parameter vector (float32 on the device, PyTorch conv1d order): W1 [64][16][5]
(input channels 0..3 used: d/s, v/vmax, row feature, d_prev/s), b1 [64], W2 [64][64][5],
b2, W3, b3, W4 [1][64][5], b4 [1].
"""

from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as F

NV = 128
C_IN, HID = 16, 64
SHAPES = [("W1", (HID, C_IN, 5)), ("b1", (HID,)), ("W2", (HID, HID, 5)), ("b2", (HID,)),
          ("W3", (HID, HID, 5)), ("b3", (HID,)), ("W4", (1, HID, 5)), ("b4", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(params):
    """Flat parameter vector -> dict of float64 CPU tensors (views of a copy)."""
    p = torch.as_tensor(np.asarray(params, dtype=np.float64))
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([d[name].detach().reshape(-1).numpy() for name, _ in SHAPES]).astype(np.float32)


def bf(t):
    """Round to bfloat16 (round to nearest even) and back to float64."""
    return t.to(torch.bfloat16).to(torch.float64)


def row_scale(g32):
    """RMS of each row in float32, as the features kernel computes it (a
    pairwise tree over the 128 squares) plus 1e-30."""
    sq = (g32 * g32).to(torch.float32)
    n = sq.shape[1]
    while n > 1:
        n //= 2
        sq = sq[:, :n] + sq[:, n:2 * n]
    return torch.sqrt(sq[:, 0] / NV) + torch.tensor(1e-30, dtype=torch.float32)


def group_mean(g32, group_rows):
    """float64 mean of each group of group_rows consecutive rows (summed in
    row order, as the group-mean kernel does), broadcast back to the rows."""
    rows = g32.shape[0]
    gg = g32.to(torch.float64).reshape(rows // group_rows, group_rows, NV)
    acc = torch.zeros((rows // group_rows, NV), dtype=torch.float64)
    for r in range(group_rows):
        acc = acc + gg[:, r]
    return (acc / group_rows).repeat_interleave(group_rows, dim=0)


def mean_pair(g32, group_rows):
    """The group mean as the kernels carry it: an FP32 pair (hi, lo) with
    hi + lo = the float64 mean (to ~1e-14)."""
    m = group_mean(g32, group_rows)
    hi = m.to(torch.float32)
    lo = (m - hi.to(torch.float64)).to(torch.float32)
    return hi, lo


def deviation(g, group_rows):
    """Rows minus their group mean in FP32 as (g - hi) - lo (the rows
    themselves without groups)."""
    g32 = torch.as_tensor(np.asarray(g, dtype=np.float32))
    if not group_rows:
        return g32
    hi, lo = mean_pair(g32, group_rows)
    return (g32 - hi) - lo


def features(g, row_feat, vmax, emulate, group_rows=0, prev=None):
    """[rows][16][128] input of the first layer."""
    g32 = deviation(g, group_rows)
    rows = g32.shape[0]
    s = row_scale(g32)
    dv = np.float32(2.0 * vmax / NV)
    v = (np.float32(-vmax) + dv * (np.arange(NV, dtype=np.float32) + np.float32(0.5))).astype(np.float32)
    x = torch.zeros((rows, C_IN, NV), dtype=torch.float64)
    x[:, 0] = (g32 / s[:, None]).to(torch.float64)
    x[:, 1] = torch.as_tensor(v / np.float32(vmax)).to(torch.float64)[None, :]
    if row_feat is not None:
        x[:, 2] = torch.as_tensor(np.asarray(row_feat, dtype=np.float32)).to(torch.float64)[:, None]
    if prev is not None:
        x[:, 3] = (deviation(prev, group_rows) / s[:, None]).to(torch.float64)
    if emulate:
        x = bf(x)
    return x, s.to(torch.float64)


def high_pass(t, protect_modes):
    """Remove the v-Fourier modes |m| < protect_modes of each row ([rows][128])."""
    if not protect_modes:
        return t
    z = torch.fft.rfft(t, dim=-1)
    z[..., :protect_modes] = 0
    return torch.fft.irfft(z, n=t.shape[-1], dim=-1)


def _weights(p, emulate):
    return {k: (bf(v) if (emulate and k.startswith("W")) else v) for k, v in p.items()}


def forward(params, g, row_feat, vmax, emulate=False, group_rows=0, prev=None):
    """Network output [rows][128] and the intermediates."""
    p = _weights(unpack(params), emulate)
    x0, s = features(g, row_feat, vmax, emulate, group_rows, prev)
    acts = [x0]
    a = x0
    for i in (1, 2, 3):
        z = F.conv1d(a, p[f"W{i}"], p[f"b{i}"], padding=2)
        a = torch.relu(z)
        if emulate:
            a = bf(a)
        acts.append(a)
    pred = F.conv1d(a, p["W4"], p["b4"], padding=2)[:, 0]
    return pred, s, acts, p


def loss_and_grads(params, g, row_feat, target, vmax, tau, emulate=False, group_rows=0, protect_modes=0,
                   prev=None):
    """(loss, flat gradient float64) of mean((P(net - (dt - dg) / (s tau)))^2),
    dg and dt the rows minus their group means (or the rows themselves), P
    the removal of the modes |m| < protect_modes."""
    g64 = deviation(g, group_rows).to(torch.float64)
    t64 = deviation(target, group_rows).to(torch.float64)
    if not emulate:
        p = {k: v.clone().requires_grad_(True) for k, v in unpack(params).items()}
        x0, s = features(g, row_feat, vmax, False, group_rows, prev)
        a = x0
        for i in (1, 2, 3):
            a = torch.relu(F.conv1d(a, p[f"W{i}"], p[f"b{i}"], padding=2))
        pred = F.conv1d(a, p["W4"], p["b4"], padding=2)[:, 0]
        want = (t64 - g64) / (s[:, None] * tau)
        loss = torch.mean(high_pass(pred - want, protect_modes) ** 2)
        loss.backward()
        return float(loss.detach()), np.concatenate([p[name].grad.reshape(-1).numpy() for name, _ in SHAPES])
    pred, s, acts, p = forward(params, g, row_feat, vmax, emulate=True, group_rows=group_rows, prev=prev)
    want = (t64 - g64) / (s[:, None] * tau)
    d = high_pass(pred - want, protect_modes)
    n = d.numel()
    loss = float(torch.mean(d * d))
    dy = torch.zeros((d.shape[0], 1, NV), dtype=torch.float64)
    dy[:, 0] = bf(2.0 * d / n)
    grads = {}
    for i in (4, 3, 2, 1):
        a_in = acts[i - 1]
        # dW[o][c][t] = sum_rows sum_p dy[o][p] a_in[c][p + t - 2]
        a_pad = F.pad(a_in, (2, 2))
        cols = torch.stack([a_pad[:, :, t:t + NV] for t in range(5)], dim=-1)  # [rows][c][p][t]
        grads[f"W{i}"] = torch.einsum("rop,rcpt->oct", dy, cols)
        grads[f"b{i}"] = dy.sum(dim=(0, 2))
        if i > 1:
            dx = F.conv_transpose1d(dy, p[f"W{i}"], padding=2)
            dx = dx * (acts[i - 1] > 0)
            dy = bf(dx)
    return loss, np.concatenate([grads[name].reshape(-1).numpy() for name, _ in SHAPES])


def apply(params, g, row_feat, vmax, tau, emulate=True, group_rows=0, protect_modes=0, prev=None):
    """Corrected rows (float64): m + P'd + (Pd + c) min(1, |Pd| / |Pd + c|)
    per row, m the group mean, d = g - m, P the removal of the modes |m| <
    protect_modes, P' = 1 - P, c = P(s tau net)."""
    pred, s, _, _ = forward(params, g, row_feat, vmax, emulate, group_rows, prev)
    g32 = torch.as_tensor(np.asarray(g, dtype=np.float32))
    d = deviation(g, group_rows).to(torch.float64)
    dh = high_pass(d, protect_modes)
    hn = dh + high_pass(s[:, None] * tau * pred, protect_modes)
    old, new = (dh * dh).sum(1), (hn * hn).sum(1)
    factor = torch.where(new > old, torch.sqrt(old / new), torch.ones_like(old))
    dn = (d - dh) + hn * factor[:, None]
    if not group_rows:
        return dn.numpy()
    hi, lo = mean_pair(g32, group_rows)
    return (hi.to(torch.float64) + (lo.to(torch.float64) + dn)).numpy()
