"""Import the unmodified reference module ``VESPER_1_prob_new`` under stand-in
modules for its three absent third-party dependencies, for golden-vector
generation only (see make_golden.py).  Nothing at test time imports this.

Stand-ins:
* ``numba.jit``      -> identity decorator (the jitted functions run as Python);
* ``pyfftw``         -> ``scipy.fft`` rfftn/irfftn with FFTW's conventions:
                        unnormalised forward, ``normalise_idft=False`` gives the
                        unnormalised backward (x N), single precision for
                        float32 plans, ``next_fast_len`` restated from pyFFTW's
                        documented rule (2^a 3^b 5^c 7^d 11^e 13^f, e+f <= 1);
* ``mrcfile``        -> stub (callers build ``mrc_obj`` instances directly).

Pinned numpy 1.21 semantics: ``np.fft.rfftn`` computed in float64 for every
input dtype (numpy >= 2.0 computes float32 input in float32), so the target
spectra are complex128 as in the reference's declared environment.
"""
from __future__ import annotations

import importlib
import os
import sys
import types

import numpy as np
import scipy.fft


def next_fast_len_fftw(n: int) -> int:
    n = int(n)
    if n <= 1:
        return max(n, 1)
    m = n
    while True:
        k = m
        for p in (2, 3, 5, 7):
            while k % p == 0:
                k //= p
        if k in (1, 11, 13):
            return m
        m += 1


class _FFTW:
    def __init__(self, a, b, axes=(0, 1, 2), direction="FFTW_FORWARD", normalise_idft=True, **kw):
        self.input_array = a
        self.output_array = b
        self.axes = tuple(axes)
        self.direction = direction
        self.normalise_idft = normalise_idft

    def __call__(self, input_array=None, output_array=None, **kw):
        if input_array is not None and input_array is not self.input_array:
            np.copyto(self.input_array, input_array)
        a = self.input_array
        if self.direction == "FFTW_FORWARD":
            r = scipy.fft.rfftn(a, axes=self.axes)
        else:
            shape = [self.output_array.shape[ax] for ax in self.axes]
            r = scipy.fft.irfftn(a, s=shape, axes=self.axes)
            if not self.normalise_idft:
                r = r * np.prod(shape)
        np.copyto(self.output_array, r)
        return self.output_array


def _install_standins():
    numba = types.ModuleType("numba")

    def jit(*args, **kw):
        if args and callable(args[0]) and not kw:
            return args[0]
        return lambda f: f

    numba.jit = jit
    numba.njit = jit
    sys.modules["numba"] = numba

    pyfftw = types.ModuleType("pyfftw")
    pyfftw.config = types.SimpleNamespace(PLANNER_EFFORT="FFTW_MEASURE", NUM_THREADS=1)
    pyfftw.empty_aligned = lambda shape, dtype="float64", **kw: np.empty(shape, dtype=dtype)
    pyfftw.next_fast_len = next_fast_len_fftw
    pyfftw.FFTW = _FFTW
    sys.modules["pyfftw"] = pyfftw

    mrcfile = types.ModuleType("mrcfile")

    def _open(*a, **k):
        raise RuntimeError("mrcfile stand-in: build mrc_obj instances directly")

    mrcfile.open = _open
    sys.modules["mrcfile"] = mrcfile

    _rfftn = np.fft.rfftn

    def rfftn_f64(a, *args, **kw):
        a = np.asarray(a)
        if a.dtype != np.float64:
            a = a.astype(np.float64)
        return _rfftn(a, *args, **kw)

    np.fft.rfftn = rfftn_f64


def import_reference(ref_dir: str | None = None):
    ref_dir = ref_dir or os.environ.get("VESPER_REFERENCE_DIR")
    if not ref_dir:
        raise RuntimeError("set VESPER_REFERENCE_DIR to a checkout of the reference (VESPER_Python)")
    _install_standins()
    if ref_dir not in sys.path:
        sys.path.insert(0, ref_dir)
    sys.dont_write_bytecode = True
    return importlib.import_module("VESPER_1_prob_new")


def make_mrc_obj(ref, data_xyz, width, orig):
    """An ``mrc_obj`` as the reference's constructor would build it from a map
    with ``data_xyz`` (already swapped to [x][y][z]), float32 voxel width and
    float32 origin."""
    o = ref.mrc_obj.__new__(ref.mrc_obj)
    o.xdim, o.ydim, o.zdim = data_xyz.shape
    # The voxel width is held as float64: under numpy >= 2 (NEP 50) a float32
    # width would turn ``dreso / src_xwidth`` in doFastVEC into float32
    # arithmetic, unlike numba and numpy 1.21, where it is float64.  Widths
    # used here are exact in float32, so the value is the same.
    o.xwidth = o.ywidth = o.zwidth = np.float64(np.float32(width))
    o.cent = np.array([o.xdim * 0.5, o.ydim * 0.5, o.zdim * 0.5])
    o.orig = np.array([np.float32(v) for v in orig])
    o.data = np.array(data_xyz, copy=True)
    o.dens = np.swapaxes(o.data, 0, 2).flatten()
    o.vec = np.zeros(data_xyz.shape + (3,), dtype="float32")
    o.dsum = o.Nact = o.ave = o.std_norm_ave = o.std = None
    return o
