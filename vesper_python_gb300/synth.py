"""Seeded synthetic density maps with the shapes and value distributions of the
benchmark workloads (there is no public dataset for this path).

Map1: an S^3 float32 grid at 1.0 A voxels, the sum of isotropic Gaussian blobs
(sigma = 1.5 A, peak amplitude U[0.5, 1.5]) at uniform positions inside a
sphere centred on the grid, plus N(0, 0.01) noise (sigma = 0.01).
Map2: an (S/2)^3 crop of map1 taken after a seeded random ZYZ rotation
(nearest-grid resample) and a U[-5, 5] A translation, with fresh noise.

Arrays are returned in the ``[x][y][z]`` index order that the reference uses
after its x<->z swap of the MRC data (VESPER_1_prob_new.py:43).
"""
from __future__ import annotations

import dataclasses

import numpy as np

__all__ = ["MapPair", "make_blob_map", "rotated_crop", "make_pair", "prob_channels",
           "WORKLOADS", "workload_pair"]


@dataclasses.dataclass
class MapPair:
    map1: np.ndarray          # [x][y][z] float32
    map2: np.ndarray          # [x][y][z] float32
    orig1: np.ndarray         # origin (A) of map1
    orig2: np.ndarray         # origin (A) of map2
    width: float              # voxel width (A)
    rot_zyz: np.ndarray       # generating ZYZ Euler angles (deg)
    shift: np.ndarray         # generating translation (A)
    prob1: np.ndarray | None = None   # (X, Y, Z, 4) in the file order of the .npy input
    prob2: np.ndarray | None = None


def _blob_positions(rng, nblob, radius):
    u = rng.random(nblob)
    r = radius * np.cbrt(u)
    v = rng.normal(size=(nblob, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v * r[:, None]


def make_blob_map(rng, side, nblob, radius, sigma=1.5, noise=0.01):
    """Sum of Gaussian blobs inside a centred sphere, plus Gaussian noise."""
    cen = side * 0.5
    pos = _blob_positions(rng, nblob, radius) + cen
    amp = rng.uniform(0.5, 1.5, size=nblob)
    out = np.zeros((side, side, side), np.float64)
    half = int(np.ceil(4.0 * sigma))
    off = np.arange(-half, half + 1)
    inv2s2 = 1.0 / (2.0 * sigma * sigma)
    for p, a in zip(pos, amp):
        base = np.floor(p).astype(int)
        ix = base[0] + off
        iy = base[1] + off
        iz = base[2] + off
        gx = np.exp(-(ix - p[0]) ** 2 * inv2s2)
        gy = np.exp(-(iy - p[1]) ** 2 * inv2s2)
        gz = np.exp(-(iz - p[2]) ** 2 * inv2s2)
        mx = (ix >= 0) & (ix < side)
        my = (iy >= 0) & (iy < side)
        mz = (iz >= 0) & (iz < side)
        blk = a * gx[mx][:, None, None] * gy[my][None, :, None] * gz[mz][None, None, :]
        out[np.ix_(ix[mx], iy[my], iz[mz])] += blk
    out += rng.normal(0.0, noise, size=out.shape)
    return out.astype(np.float32)


def _zyz_matrix(angles_deg):
    a, b, c = np.deg2rad(angles_deg)

    def rz(t):
        return np.array([[np.cos(t), -np.sin(t), 0.0], [np.sin(t), np.cos(t), 0.0], [0.0, 0.0, 1.0]])

    def ry(t):
        return np.array([[np.cos(t), 0.0, np.sin(t)], [0.0, 1.0, 0.0], [-np.sin(t), 0.0, np.cos(t)]])

    return rz(a) @ ry(b) @ rz(c)


def rotated_crop(rng, map1, side2, rot_zyz, shift, noise=0.01, extra=None):
    """Nearest-grid resample of ``map1`` onto a ``side2`` cube centred on map1's
    centre, rotated by ``rot_zyz`` and shifted by ``shift`` (voxel units).
    ``extra`` arrays (same grid as map1, any trailing channel dims) are
    resampled with the same voxel map and no noise."""
    s1 = map1.shape[0]
    m = _zyz_matrix(rot_zyz)
    q = np.indices((side2, side2, side2)).reshape(3, -1).T.astype(np.float64) - side2 * 0.5
    src = q @ m.T + s1 * 0.5 + shift
    idx = np.rint(src).astype(np.int64)
    ok = np.all((idx >= 0) & (idx < s1), axis=1)
    flat = np.zeros(q.shape[0], np.float64)
    ii = idx[ok]
    flat[ok] = map1[ii[:, 0], ii[:, 1], ii[:, 2]]
    out = flat.reshape(side2, side2, side2) + rng.normal(0.0, noise, size=(side2,) * 3)
    extras = []
    for e in extra or []:
        tail = e.shape[3:]
        ef = np.zeros((q.shape[0],) + tail, e.dtype)
        ef[ok] = e[ii[:, 0], ii[:, 1], ii[:, 2]]
        extras.append(ef.reshape((side2,) * 3 + tail))
    return out.astype(np.float32), extras


def prob_channels(rng, density, threshold):
    """Four per-voxel probability channels drawn Dirichlet(0.5) inside the
    thresholded mask of ``density`` and zero outside; shape (X, Y, Z, 4)."""
    mask = density >= threshold
    p = rng.dirichlet([0.5] * 4, size=int(mask.sum())).astype(np.float32)
    out = np.zeros(density.shape + (4,), np.float32)
    out[mask] = p
    return out


def make_pair(seed, side1, nblob, radius, with_prob=False, threshold=0.1):
    rng = np.random.default_rng(seed)
    map1 = make_blob_map(rng, side1, nblob, radius)
    side2 = side1 // 2
    a = rng.uniform(0.0, 360.0)
    b = np.rad2deg(np.arccos(rng.uniform(-1.0, 1.0)))
    c = rng.uniform(0.0, 360.0)
    rot = np.array([a, b, c])
    shift = rng.uniform(-5.0, 5.0, size=3)
    prob1 = prob_channels(rng, map1, threshold) if with_prob else None
    extra = [prob1] if with_prob else None
    map2, extras = rotated_crop(rng, map1, side2, rot, shift, extra=extra)
    prob2 = extras[0] if with_prob else None
    if with_prob:
        # zero the channels wherever the noisy crop falls below the threshold
        prob2 = np.where((map2 >= threshold)[..., None], prob2, 0.0).astype(np.float32)
    orig1 = np.zeros(3)
    orig2 = np.full(3, (side1 - side2) * 0.5)
    return MapPair(map1, map2, orig1, orig2, 1.0, rot, shift, prob1, prob2)


# Workload table: generator sizes and search parameters of the benchmark
# configurations.  t, T: thresholds; g: Gaussian bandwidth; s: coarse voxel
# spacing; A: angle step; N: top-N.
WORKLOADS = {
    "pair128_s7_a30": dict(side1=128, nblob=400, radius=40.0, t=0.1, T=0.1, g=16.0, s=7.0, A=30.0, N=10,
                           modes=("V",)),
    "pair200_s2_a10": dict(side1=200, nblob=1500, radius=70.0, t=0.1, T=0.1, g=16.0, s=2.0, A=10.0, N=10,
                           modes=("V", "O", "C", "P", "L")),
    "prop128_s3_a10": dict(side1=128, nblob=400, radius=40.0, t=0.1, T=0.1, g=16.0, s=3.0, A=10.0, N=10,
                           modes=("V",)),
    "prob128_s3_a15": dict(side1=128, nblob=400, radius=40.0, t=0.1, T=0.1, g=16.0, s=3.0, A=15.0, N=10,
                           modes=("V",), alpha=0.5, prob=True, pad=64),
}

UNEVEN_SIDES = (64, 96, 128, 160, 192, 256)
UNEVEN_WORKLOAD = dict(pairs=64, t=0.1, T=0.1, g=16.0, s=4.0, A=15.0, N=10)


def uneven_spec(index, seed_base=1000):
    """(generator seed, map1 side, blob count, sphere radius) of pair ``index``
    of the uneven batch: side drawn from UNEVEN_SIDES, blob count
    proportional to volume, radius proportional to side."""
    rng = np.random.default_rng(seed_base + index)
    side = int(rng.choice(UNEVEN_SIDES))
    scale = side / 128.0
    return seed_base * 7 + index, side, max(8, int(round(400 * scale ** 3))), 40.0 * scale


def workload_pair(name, seed=0):
    w = WORKLOADS[name]
    return make_pair(seed, w["side1"], w["nblob"], w["radius"], with_prob=w.get("prob", False),
                     threshold=w["t"])


def uneven_pair(index, seed_base=1000):
    """One pair of the uneven batch (uneven_spec), generated with numpy."""
    seed, side, nblob, radius = uneven_spec(index, seed_base)
    return make_pair(seed, side, nblob, radius)
