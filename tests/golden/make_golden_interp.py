"""Golden vectors of the probability-map hole filling (interpolate,
interpolation_functions.py:6-135): the UNMODIFIED reference function run
under the stand-in modules of refshim.py on small seeded arrays.

    VESPER_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden_interp.py

Under the identity jit the reference's mean accumulates in float32 (numpy
scalars), where numba accumulates in float64; the inputs are multiples of
1/16 below 8, so every sum is exact in float32 and the two agree bit for bit
(means of 2 and 4 are exact scalings; a mean of 6 rounds the same exact
quotient either way).  Output: interp_small.npz (inputs and outputs).
"""
from __future__ import annotations

import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refshim  # noqa: E402


def sparse_prob_map(rng, shape, parity, holes=0.15):
    """Values on the voxels of one parity class (every other voxel per axis),
    zero elsewhere, with some of those voxels zero too."""
    nx, ny, nz = shape
    a = np.zeros((nx, ny, nz, 4), np.float32)
    px, py, pz = parity
    v = rng.integers(1, 128, size=a[px::2, py::2, pz::2].shape).astype(np.float32) / 16.0
    v[rng.random(v.shape) < holes] = 0.0
    a[px::2, py::2, pz::2] = v
    return a


def main():
    refshim.import_reference()          # installs the stand-ins and the reference path
    interp = importlib.import_module("interpolation_functions")
    rng = np.random.default_rng(2024)
    cases = [((9, 10, 11), (0, 0, 0)), ((8, 8, 8), (1, 0, 1)), ((12, 7, 9), (1, 1, 1)), ((5, 6, 7), (0, 1, 0))]
    out = {}
    for n, (shape, parity) in enumerate(cases):
        a = sparse_prob_map(rng, shape, parity)
        out[f"in{n}"] = a.copy()
        interp.interpolate(a)
        out[f"out{n}"] = a
    np.savez_compressed(os.path.join(HERE, "interp_small.npz"), **out)


if __name__ == "__main__":
    main()
