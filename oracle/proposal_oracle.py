"""CPU oracle of the learned rotation proposal -- TEST INFRASTRUCTURE ONLY.

float64 numpy restatement of the proposal network's forward and backward
passes (3x3x3 zero-padded convolutions with ReLU, rotational correlation of
two feature fields at zero translation, softmax cross-entropy), used to check
the GPU kernels' values and gradients.  Nothing in the product imports it.  The rotation's voxel map is the
reference's nearest-voxel gather (rot_mrc, VESPER_1_prob_new.py:296-348) with
every in-bounds voxel accepted.
"""
from __future__ import annotations

import numpy as np

from . import vesper_oracle as orc


def src_map(d, F):
    """Destination -> source voxel index (-1: none) of one rotation."""
    old, dst = orc.rot_positions(d, F)
    ok = np.all((old >= 0) & (old < d), axis=1)
    oi = old.astype(np.float64).astype(np.int64)
    src = (oi[:, 0] * d + oi[:, 1]) * d + oi[:, 2]
    out = np.full(d ** 3, -1, np.int64)
    rows = np.nonzero(ok)[0]
    out[dst[rows]] = src[rows]       # numpy assigns in order: the last row wins
    return out


def conv_fwd(x, W, b, relu):
    """x [Cin][d][d][d], W [Cout][Cin][27], b [Cout]."""
    cin, d = x.shape[0], x.shape[1]
    cout = W.shape[0]
    xp = np.zeros((cin, d + 2, d + 2, d + 2))
    xp[:, 1:-1, 1:-1, 1:-1] = x
    out = np.zeros((cout, d, d, d))
    for o in range(27):
        dx, dy, dz = o // 9, (o // 3) % 3, o % 3
        sl = xp[:, dx:dx + d, dy:dy + d, dz:dz + d]
        out += np.einsum("oc,cxyz->oxyz", W[:, :, o], sl)
    out += b[:, None, None, None]
    return np.maximum(out, 0) if relu else out


def conv_bwd(g, out, relu, x, W):
    """(dx, dW, db) for one layer; g = dL/d(out)."""
    if relu:
        g = np.where(out > 0, g, 0.0)
    cin, d = x.shape[0], x.shape[1]
    xp = np.zeros((cin, d + 2, d + 2, d + 2))
    xp[:, 1:-1, 1:-1, 1:-1] = x
    dW = np.zeros_like(W)
    dxp = np.zeros_like(xp)
    for o in range(27):
        dx, dy, dz = o // 9, (o // 3) % 3, o % 3
        sl = xp[:, dx:dx + d, dy:dy + d, dz:dz + d]
        dW[:, :, o] = np.einsum("oxyz,cxyz->oc", g, sl)
        dxp[:, dx:dx + d, dy:dy + d, dz:dz + d] += np.einsum("oc,oxyz->cxyz", W[:, :, o], g)
    db = g.sum(axis=(1, 2, 3))
    return dxp[:, 1:-1, 1:-1, 1:-1], dW, db


def encoder_fwd(x, layers):
    """layers: list of (W, b, relu).  Returns the list of activations."""
    acts = [x]
    for W, b, relu in layers:
        acts.append(conv_fwd(acts[-1], W, b, relu))
    return acts


def encoder_bwd(acts, layers, g):
    grads = [None] * len(layers)
    for i in range(len(layers) - 1, -1, -1):
        W, b, relu = layers[i]
        gx, dW, db = conv_bwd(g, acts[i + 1], relu, acts[i], W)
        grads[i] = (dW, db)
        g = gx
    return grads


def score_fwd(ET, EQ, maps):
    """ET, EQ [K][N]; maps: list of src maps.  s[r] = sum ET[:, v] EQ[:, src(v)]."""
    s = np.zeros(len(maps))
    for r, m in enumerate(maps):
        ok = m >= 0
        s[r] = np.sum(ET[:, ok] * EQ[:, m[ok]])
    return s


def score_bwd(ET, EQ, maps, g):
    gT = np.zeros_like(ET)
    gQ = np.zeros_like(EQ)
    for r, m in enumerate(maps):
        ok = np.nonzero(m >= 0)[0]
        gT[:, ok] += g[r] * EQ[:, m[ok]]
        np.add.at(gQ, (slice(None), m[ok]), g[r] * ET[:, ok])
    return gT, gQ


def softmax_ce(s, q, tau):
    """Cross-entropy of softmax(u / tau) against q, u = the scores standardised
    over the rotations (population std + 1e-6); returns (loss, dL/ds)."""
    mu = s.mean()
    sd = np.sqrt(np.mean((s - mu) ** 2)) + 1e-6
    u = (s - mu) / sd
    z = u / tau
    z = z - z.max()
    lp = z - np.log(np.exp(z).sum())
    p = np.exp(lp)
    gu = (p - q) / tau
    gs = (gu - gu.mean() - u * np.mean(gu * u)) / sd
    return -np.sum(q * lp), gs
