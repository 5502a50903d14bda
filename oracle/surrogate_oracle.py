"""ORACLE — test infrastructure, never the product.

FP64 numpy restatement of the waveform surrogate's network (fwant_gb300/surrogate.py):
3x3x3 convolutions with zero padding 1 and stride 1 or 2, dense layers, leaky ReLU and
the mean-squared-error loss, forward and hand-derived backward.  The tests feed it the
BF16-rounded weights the GPU kernels read and compare every gradient; the backward here
is itself checked against central finite differences.
"""
from __future__ import annotations

import numpy as np


def bf16_round(a):
    """Round float32 values to the nearest BF16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(a, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _pad(x):
    return np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1), (1, 1)))


def conv3d(x, w, b, stride):
    """x (B, Ci, D, H, W), w (Co, Ci, 3, 3, 3), b (Co,) or None -> (B, Co, Do, Ho, Wo)."""
    B, Ci, D, H, W = x.shape
    Co = w.shape[0]
    Do, Ho, Wo = (D - 1) // stride + 1, (H - 1) // stride + 1, (W - 1) // stride + 1
    xp = _pad(x)
    y = np.zeros((B, Co, Do, Ho, Wo))
    for kd in range(3):
        for kh in range(3):
            for kw in range(3):
                patch = xp[:, :, kd:kd + stride * (Do - 1) + 1:stride, kh:kh + stride * (Ho - 1) + 1:stride,
                           kw:kw + stride * (Wo - 1) + 1:stride]
                y += np.einsum("bcdhw,oc->bodhw", patch, w[:, :, kd, kh, kw])
    if b is not None:
        y += b[None, :, None, None, None]
    return y


def conv3d_bwd(x, w, dy, stride):
    """(dx, dw, db) of conv3d."""
    B, Ci, D, H, W = x.shape
    _, Co, Do, Ho, Wo = dy.shape
    xp = _pad(x)
    dxp = np.zeros_like(xp)
    dw = np.zeros_like(w)
    for kd in range(3):
        for kh in range(3):
            for kw in range(3):
                sl = (slice(None), slice(None), slice(kd, kd + stride * (Do - 1) + 1, stride),
                      slice(kh, kh + stride * (Ho - 1) + 1, stride), slice(kw, kw + stride * (Wo - 1) + 1, stride))
                dw[:, :, kd, kh, kw] = np.einsum("bodhw,bcdhw->oc", dy, xp[sl])
                dxp[sl] += np.einsum("bodhw,oc->bcdhw", dy, w[:, :, kd, kh, kw])
    return dxp[:, :, 1:-1, 1:-1, 1:-1], dw, dy.sum(axis=(0, 2, 3, 4))


def lrelu(x, slope):
    return np.where(x > 0, x, slope * x)


def lrelu_bwd(y, dy, slope):
    return np.where(y > 0, dy, slope * dy)


class Net:
    """Same layer stack as fwant_gb300.surrogate.Net; params is a dict of float64 arrays."""

    def __init__(self, convs, dense, slope):
        self.convs = convs      # [(cin, cout, stride)]
        self.dense = dense      # [(in, out)]
        self.slope = slope

    def forward(self, p, x):
        acts = [x]
        h = x
        for n, (_, _, s) in enumerate(self.convs):
            h = lrelu(conv3d(h, p[f"conv{n}.w"], p[f"conv{n}.b"], s), self.slope)
            acts.append(h)
        h = h.reshape(h.shape[0], -1)
        acts.append(h)
        for n in range(len(self.dense)):
            h = h @ p[f"fc{n}.w"].T + p[f"fc{n}.b"]
            if n + 1 < len(self.dense):
                h = lrelu(h, self.slope)
            acts.append(h)
        return h, acts

    def loss_and_grads(self, p, x, t):
        y, acts = self.forward(p, x)
        n = y.size
        loss = float(np.sum((y - t) ** 2) / n)
        g = {}
        dy = 2.0 * (y - t) / n
        nd = len(self.dense)
        for q in reversed(range(nd)):
            hin = acts[len(self.convs) + 1 + q]
            g[f"fc{q}.w"] = dy.T @ hin
            g[f"fc{q}.b"] = dy.sum(axis=0)
            dy = dy @ p[f"fc{q}.w"]
            if q > 0:
                dy = lrelu_bwd(hin, dy, self.slope)
        dy = lrelu_bwd(acts[len(self.convs) + 1], dy, self.slope).reshape(acts[len(self.convs)].shape)
        for q in reversed(range(len(self.convs))):
            _, _, s = self.convs[q]
            dx, dw, db = conv3d_bwd(acts[q], p[f"conv{q}.w"], dy, s)
            g[f"conv{q}.w"] = dw
            g[f"conv{q}.b"] = db
            if q > 0:
                dy = lrelu_bwd(acts[q], dx, self.slope)
        return loss, g
