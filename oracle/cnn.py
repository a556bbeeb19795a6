"""Oracle (test infrastructure only): the 3D convolutional coarse-correction
network in numpy FP64 — forward, backward (data and weight gradients) and
the relative-MSE loss — used to check the GPU training kernels.

Network: L layers of 3x3x3 convolutions with zero padding, ReLU between
layers, no activation after the last; input channels = residual (re, im)
plus static features, output channels = error (re, im).
"""
from __future__ import annotations

import numpy as np


def conv3d(x, W, b):
    """x: (B, Ci, D, H, W); W: (Co, Ci, 3, 3, 3); b: (Co,). Zero padding 1."""
    B, Ci, D, H, Wd = x.shape
    Co = W.shape[0]
    xp = np.zeros((B, Ci, D + 2, H + 2, Wd + 2))
    xp[:, :, 1:-1, 1:-1, 1:-1] = x
    out = np.zeros((B, Co, D, H, Wd))
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                patch = xp[:, :, dz:dz + D, dy:dy + H, dx:dx + Wd]
                out += np.einsum("oi,bidhw->bodhw", W[:, :, dz, dy, dx], patch)
    return out + b[None, :, None, None, None]


def conv3d_grad(x, W, gout):
    """Gradients of conv3d w.r.t. x, W and b."""
    B, Ci, D, H, Wd = x.shape
    xp = np.zeros((B, Ci, D + 2, H + 2, Wd + 2))
    xp[:, :, 1:-1, 1:-1, 1:-1] = x
    gxp = np.zeros_like(xp)
    gW = np.zeros_like(W)
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                patch = xp[:, :, dz:dz + D, dy:dy + H, dx:dx + Wd]
                gW[:, :, dz, dy, dx] = np.einsum("bodhw,bidhw->oi", gout, patch)
                gxp[:, :, dz:dz + D, dy:dy + H, dx:dx + Wd] += np.einsum("oi,bodhw->bidhw", W[:, :, dz, dy, dx], gout)
    gb = gout.sum(axis=(0, 2, 3, 4))
    return gxp[:, :, 1:-1, 1:-1, 1:-1], gW, gb


def forward(x, Ws, bs):
    acts = [x]
    pres = []
    h = x
    for l, (W, b) in enumerate(zip(Ws, bs)):
        z = conv3d(h, W, b)
        pres.append(z)
        h = np.maximum(z, 0.0) if l + 1 < len(Ws) else z
        acts.append(h)
    return h, acts, pres


def loss_and_grads(x, target, Ws, bs):
    """Relative MSE over the batch: sum_b ||y_b - t_b||^2 / ||t_b||^2 / B."""
    y, acts, pres = forward(x, Ws, bs)
    B = x.shape[0]
    tn = np.sum(target ** 2, axis=(1, 2, 3, 4))
    diff = y - target
    L = float(np.mean(np.sum(diff ** 2, axis=(1, 2, 3, 4)) / tn))
    g = 2.0 * diff / (B * tn[:, None, None, None, None])
    gWs, gbs = [None] * len(Ws), [None] * len(Ws)
    for l in reversed(range(len(Ws))):
        if l + 1 < len(Ws):
            g = g * (pres[l] > 0)
        gx, gWs[l], gbs[l] = conv3d_grad(acts[l], Ws[l], g)
        g = gx
    return L, gWs, gbs
