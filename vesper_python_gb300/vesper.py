"""Host layer of the GB300 VESPER path, mirroring the reference module
``VESPER_1_prob_new.py`` function by function (same names, argument meaning,
printed output and exceptions), with every hot step executed by the sm_103a
kernels of ``libvesper_gb300.so``:

  fastVEC              -> vesper_fastvec         (VESPER_1_prob_new.py:145-257)
  rot_mrc/rot_mrc_prob -> vesper_rot_gather      (:279-354, :1211-1299)
  target spectra       -> vesper_target_spectra  (:601-628, :846-864)
  rotation loops       -> vesper_search          (:644-655, :724-736, :880-962, :1025-1080)
  sorted(...)[:TopN]   -> vesper_topn            (:664, :739, :992, :1082)
  get_score            -> vesper_rescore         (:1302-1393)

Map set-up (mrc_set_vox_size), the angle grid, rotation matrices (scipy, as
the reference), output geometry and the PDB writer stay on the host: they are
O(R) or O(d^3) bookkeeping, not the hot path.

Printed values follow the reference's pinned numpy 1.21 semantics where
numpy 2 differs: scaled scores are float64 (numpy 1.21 promotes float32
scalar x Python float to float64) and scalars print like Python floats/ints.
"""
from __future__ import annotations

import copy
import ctypes
import dataclasses
from datetime import datetime
from pathlib import Path

import numpy as np
import torch
from scipy.spatial.transform import Rotation as R

from . import _native
from .mrc import read_mrc

__all__ = [
    "mrc_obj", "mrc_set_vox_size", "fastVEC", "search_map_fft", "search_map_fft_prob", "rot_mrc", "rot_mrc_prob",
    "get_score", "calc_angle_comb", "euler2rot", "convert_trans", "show_vec", "next_fast_len", "rot_matrices",
    "Device", "MODE_CODES",
]

MODE_CODES = {"VecProduct": 0, "Overlap": 1, "CC": 2, "PCC": 3, "Laplacian": 4, "prob": 5}


# ----------------------------------------------------------------------------
# device plumbing
# ----------------------------------------------------------------------------

def _raw_stream(index):
    return torch.cuda.current_stream(index).cuda_stream


if hasattr(torch._C, "_cuda_getCurrentRawStream"):
    _raw_stream = torch._C._cuda_getCurrentRawStream   # noqa: F811  (same value, without the Stream object)


class Device:
    """CUDA device, stream and cached scratch buffers for the C-ABI calls."""

    def __init__(self, device="cuda:0"):
        if not torch.cuda.is_available():
            raise RuntimeError("the GB300 VESPER path needs a CUDA device; none is available")
        self.device = torch.device(device)
        self.index = self.device.index if self.device.index is not None else torch.cuda.current_device()
        self.lib = _native.load()
        self._ws = {}

    @property
    def stream(self):
        """The current CUDA stream of this device (a capture stream inside
        torch.cuda.graph), as the raw handle the C-ABI takes."""
        return ctypes.c_void_p(_raw_stream(self.index))

    def workspace(self, key, nbytes):
        """Scratch buffer for ``key`` on the current stream (work on different
        streams never shares scratch)."""
        key = key + (_raw_stream(self.index),)
        buf = self._ws.get(key)
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=self.device)
            self._ws[key] = buf
        return buf

    def to_dev_async(self, a):
        """Small host array -> device without waiting on the stream: staged in
        pinned memory (torch's caching host allocator keeps the staging block
        until the copy has run)."""
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        return t.to(self.device, non_blocking=True)

    def to_dev(self, a, dtype=None):
        t = torch.as_tensor(np.ascontiguousarray(a))
        if dtype is not None:
            t = t.to(dtype)
        return t.to(self.device, non_blocking=False)


_DEV = None


def default_device() -> Device:
    global _DEV
    if _DEV is None:
        _DEV = Device()
    return _DEV


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _host_d3(v):
    return (ctypes.c_double * 3)(*[float(x) for x in v])


# ----------------------------------------------------------------------------
# printing helpers (numpy 1.21 scalar formatting)
# ----------------------------------------------------------------------------

def _py(v):
    if isinstance(v, np.generic):
        return v.item()
    if isinstance(v, tuple):
        return tuple(_py(x) for x in v)
    return v


# ----------------------------------------------------------------------------
# map objects and set-up (host)
# ----------------------------------------------------------------------------

class mrc_obj:
    """A density map with the fields of the reference's ``mrc_obj``
    (VESPER_1_prob_new.py:18-56): data in [x][y][z] order after the x<->z swap."""

    def __init__(self, path):
        m = read_mrc(path)
        self.xdim = int(m.nx)
        self.ydim = int(m.ny)
        self.zdim = int(m.nz)
        self.xwidth = m.voxel_size[0]
        self.ywidth = m.voxel_size[1]
        self.zwidth = m.voxel_size[2]
        self.cent = np.array([self.xdim * 0.5, self.ydim * 0.5, self.zdim * 0.5])
        self.orig = np.array([m.origin[0], m.origin[1], m.origin[2]])
        self.data = np.swapaxes(copy.deepcopy(m.data), 0, 2)
        self.dens = m.data.flatten()
        self.vec = np.zeros((self.xdim, self.ydim, self.zdim, 3), dtype="float32")
        self.dsum = None
        self.Nact = None
        self.ave = None
        self.std_norm_ave = None
        self.std = None

    @classmethod
    def from_array(cls, data_xyz, width=1.0, orig=(0.0, 0.0, 0.0)):
        """A map object for an in-memory [x][y][z] float32 array (width and
        origin held as float32, as an MRC header stores them)."""
        o = cls.__new__(cls)
        o.xdim, o.ydim, o.zdim = data_xyz.shape
        o.xwidth = o.ywidth = o.zwidth = np.float32(width)
        o.cent = np.array([o.xdim * 0.5, o.ydim * 0.5, o.zdim * 0.5])
        o.orig = np.array([np.float32(v) for v in orig])
        o.data = np.array(data_xyz, dtype=np.float32, copy=True)
        o.dens = np.swapaxes(o.data, 0, 2).flatten()
        o.vec = np.zeros(o.data.shape + (3,), dtype="float32")
        o.dsum = o.Nact = o.ave = o.std_norm_ave = o.std = None
        return o


def next_fast_len(n: int) -> int:
    """pyFFTW's next_fast_len (VESPER_1_prob_new.py:97): the smallest m >= n of
    the form 2^a 3^b 5^c 7^d 11^e 13^f with e + f <= 1."""
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


def mrc_set_vox_size(mrc, th=0.00, voxel_size=7.0):
    """VESPER_1_prob_new.py:59-118: threshold in place, size the coarse grid and
    return (mrc, mrc_new)."""
    if th < 0:
        mrc.dens = mrc.dens - th
        th = 0.0
    mrc.dens[mrc.dens < th] = 0.0
    mrc.data[mrc.data < th] = 0.0
    non_zero_index_list = np.array(np.nonzero(mrc.data)).T
    cent_arr = np.array(mrc.cent)
    d2_list = np.linalg.norm(non_zero_index_list - cent_arr, axis=1)
    dmax = max(d2_list)  # ValueError on an empty map, as in the reference
    print()
    print("#dmax=" + str(_py(dmax / np.float64(mrc.xwidth))))
    dmax = dmax * np.float64(mrc.xwidth)
    new_cent = mrc.cent * np.float64(mrc.xwidth) + mrc.orig
    tmp_size = 2 * dmax / voxel_size
    new_xdim = next_fast_len(int(tmp_size))
    new_orig = new_cent - 0.5 * new_xdim * voxel_size
    mrc_new = copy.deepcopy(mrc)
    mrc_new.orig = new_orig
    mrc_new.xdim = new_xdim
    mrc_new.ydim = new_xdim
    mrc_new.zdim = new_xdim
    mrc_new.cent = new_cent
    mrc_new.xwidth = mrc_new.ywidth = mrc_new.zwidth = voxel_size
    print("Nvox= " + str(mrc_new.xdim) + ", " + str(mrc_new.ydim) + ", " + str(mrc_new.zdim))
    print("cent= " + str(_py(new_cent[0])) + ", " + str(_py(new_cent[1])) + ", " + str(_py(new_cent[2])))
    print("ori= " + str(_py(new_orig[0])) + ", " + str(_py(new_orig[1])) + ", " + str(_py(new_orig[2])))
    return mrc, mrc_new


# ----------------------------------------------------------------------------
# fastVEC
# ----------------------------------------------------------------------------

def fastvec_device(src_data, src_width, src_orig, dim, dest_width, dest_orig, dreso, dev=None, want_f32=True):
    """vesper_fastvec on device arrays.  ``src_data`` is a host [x][y][z] array or
    a float32 CUDA tensor.  Returns (data f64, data f32 or None when not
    ``want_f32``, vec f32) CUDA tensors."""
    dev = dev or default_device()
    src = src_data if isinstance(src_data, torch.Tensor) else dev.to_dev(np.asarray(src_data, np.float32))
    if src.dtype != torch.float32 or not src.is_contiguous():
        src = src.to(torch.float32).contiguous()
    sx, sy, sz = src.shape
    ws_bytes = _native.size_query("vesper_fastvec_workspace_size", sx, sy, sz, dim)
    ws = dev.workspace(("fastvec", sx, sy, sz, dim), ws_bytes)
    data = torch.empty((dim, dim, dim), dtype=torch.float64, device=dev.device)
    data32 = torch.empty((dim, dim, dim), dtype=torch.float32, device=dev.device) if want_f32 else None
    vec = torch.empty((dim, dim, dim, 3), dtype=torch.float32, device=dev.device)
    _native.check(dev.lib.vesper_fastvec(_ptr(src), sx, sy, sz, float(src_width), _host_d3(src_orig), int(dim),
                                         float(dest_width), _host_d3(dest_orig), float(dreso), _ptr(data),
                                         _ptr(data32), _ptr(vec), _ptr(ws), ws.numel(), dev.stream))
    return data, data32, vec


def _fastvec_stats(dest_data):
    dsum = np.sum(dest_data)
    Nact = np.count_nonzero(dest_data)
    pos = dest_data[dest_data > 0]
    ave = np.mean(pos)
    std = np.linalg.norm(pos)
    std_norm_ave = np.linalg.norm(pos - ave)
    return dsum, Nact, ave, std, std_norm_ave


def fastVEC(src, dest, dreso=16.0, dev=None):
    """VESPER_1_prob_new.py:145-177 on the GPU.  ``dest.data``'s dtype (float64
    in orig mode, float32 in prob mode, main.py:43/345) is kept."""
    dev = dev or default_device()
    f32 = np.asarray(dest.data).dtype == np.float32
    data, data32, vec = fastvec_device(src.data, np.float64(src.xwidth), np.asarray(src.orig, np.float64),
                                       int(dest.xdim), float(dest.xwidth), np.asarray(dest.orig, np.float64),
                                       dreso, dev)
    dest_data = (data32 if f32 else data).cpu().numpy()
    dest_vec = vec.cpu().numpy()
    dsum, Nact, ave, std, std_norm_ave = _fastvec_stats(dest_data)
    print("#MAP SUM={sum} COUNT={cnt} AVE={ave} STD={std} STD_norm={std_norm}".format(
        sum=_py(dsum), cnt=Nact, ave=_py(ave), std=_py(std), std_norm=_py(std_norm_ave)))
    dest.data = dest_data
    dest.vec = dest_vec
    dest.dsum = dsum
    dest.Nact = Nact
    dest.ave = ave
    dest.std = std
    dest.std_norm_ave = std_norm_ave
    # keep the device copies for the search
    dest._dev = {"data": data if not f32 else data32.to(torch.float64), "vec": vec, "data32": data32}
    return dest


# ----------------------------------------------------------------------------
# angles and rotations
# ----------------------------------------------------------------------------

def calc_angle_comb(ang_interval):
    """VESPER_1_prob_new.py:1396-1415."""
    x_angle = []
    y_angle = []
    z_angle = []
    i = 0
    while i < 360:
        x_angle.append(i)
        y_angle.append(i)
        i += ang_interval
    i = 0
    while i <= 180:
        z_angle.append(i)
        i += ang_interval
    return np.array(np.meshgrid(x_angle, y_angle, z_angle)).T.reshape(-1, 3)


def rot_matrices(angles) -> np.ndarray:
    """float32 [n][3][3]: np.flip of the ZYX Euler matrix with |m| < 1e-15
    zeroed, per rotation (VESPER_1_prob_new.py:305-310)."""
    angles = np.asarray(angles, dtype=np.float64).reshape(-1, 3)
    if len(angles) == 0:
        return np.zeros((0, 3, 3), np.float32)
    # one vectorised scipy call gives the same matrices as one call per angle
    mtx = R.from_euler("ZYX", angles, degrees=True).as_matrix()
    mtx[np.isclose(mtx, 0, atol=1e-15)] = 0
    return np.ascontiguousarray(np.flip(mtx, axis=(1, 2)).astype(np.float32))


_ROT_CACHE = {}


def rot_matrices_device(angles, dev, key=None):
    """Device copy of rot_matrices(angles), cached by ``key`` (the angle step)."""
    if key is not None and (key, dev.device) in _ROT_CACHE:
        return _ROT_CACHE[(key, dev.device)]
    t = dev.to_dev(rot_matrices(angles))
    if key is not None:
        _ROT_CACHE[(key, dev.device)] = t
    return t


_REFINE_OFFSETS = np.array(np.meshgrid([-5, 0, 5], [-5, 0, 5], [-5, 0, 5])).T.reshape(-1, 3)


def refine_angle_list(sorted_topN_angles):
    """VESPER_1_prob_new.py:693-713, vectorised: per top angle the 27
    offsets of +-5 degrees in the reference's meshgrid order, filtered and
    wrapped as there, concatenated in the same order."""
    tops = np.asarray(sorted_topN_angles, dtype=np.float64).reshape(-1, 3)
    cand = (tops[:, None, :] + _REFINE_OFFSETS[None, :, :]).reshape(-1, 3)
    cand = cand[(cand[:, 0] < 360) & (cand[:, 1] < 360) & (cand[:, 2] < 180)]
    cand[cand < 0] += 360
    return cand


_LATTICE = {}
LATTICE_STEP = 5.0
LATTICE_N = 72


def lattice_rot_matrices_device(dev):
    """rot_matrices of every angle of the 5-degree lattice [0, 360)^3
    (373,248 rotations, 13 MB), computed once per device.  The angle grids
    with steps that are multiples of 5 degrees and their +-5 degree
    refinement sets all lie on it, so their matrices are rows of this table
    (scipy's vectorised result is row-for-row the per-angle result)."""
    m = _LATTICE.get(dev.device)
    if m is None:
        k = np.arange(LATTICE_N) * LATTICE_STEP
        lat = np.stack(np.meshgrid(k, k, k, indexing="ij"), -1).reshape(-1, 3)
        m = _LATTICE[dev.device] = dev.to_dev(rot_matrices(lat))
    return m


def lattice_index(angles):
    """Row of each angle in the 5-degree lattice, or None when an angle is
    off the lattice."""
    a = np.asarray(angles, dtype=np.float64).reshape(-1, 3)
    q = a / LATTICE_STEP
    k = np.rint(q)
    if not (np.all(q == k) and np.all((k >= 0) & (k < LATTICE_N))):
        return None
    k = k.astype(np.int64)
    return (k[:, 0] * LATTICE_N + k[:, 1]) * LATTICE_N + k[:, 2]


def rot_matrices_lattice(angles, dev):
    """Device rot_matrices(angles): rows of the lattice table when the angles
    are on it (a small index copy), else computed and copied."""
    idx = lattice_index(angles)
    if idx is None:
        return dev.to_dev_async(rot_matrices(angles))
    return lattice_rot_matrices_device(dev).index_select(0, dev.to_dev_async(idx))


def _dev_fields(m, dev):
    """(data f64, vec f32) CUDA tensors of a map object."""
    d = getattr(m, "_dev", None)
    if d is None:
        d = {"data": dev.to_dev(np.asarray(m.data, np.float64)), "vec": dev.to_dev(np.asarray(m.vec, np.float32))}
        m._dev = d
    return d["data"], d["vec"]


def rot_gather_device(data, vec, rotmats, probs=None, dev=None):
    dev = dev or default_device()
    d = data.shape[0]
    n = rotmats.shape[0]
    data_out = torch.empty((n, d, d, d), dtype=torch.float64, device=dev.device)
    vec_out = torch.empty((n, d, d, d, 3), dtype=torch.float32, device=dev.device)
    probs_out = torch.empty((n, 4, d, d, d), dtype=torch.float32, device=dev.device) if probs is not None else None
    _native.check(dev.lib.vesper_rot_gather(_ptr(data), _ptr(vec), _ptr(probs), d, _ptr(rotmats), n,
                                            _ptr(data_out), _ptr(vec_out), _ptr(probs_out), dev.stream))
    return data_out, vec_out, probs_out


def rot_mrc(orig_mrc_data, orig_mrc_vec, angle, dev=None):
    """VESPER_1_prob_new.py:279-354 on the GPU: (new_vec, new_data)."""
    dev = dev or default_device()
    data = dev.to_dev(np.asarray(orig_mrc_data, np.float64))
    vec = dev.to_dev(np.asarray(orig_mrc_vec, np.float32))
    mats = dev.to_dev(rot_matrices([angle]))
    dout, vout, _ = rot_gather_device(data, vec, mats, dev=dev)
    return vout[0].cpu().numpy(), dout[0].cpu().numpy().astype(np.asarray(orig_mrc_data).dtype)


def rot_mrc_prob(orig_mrc_data, orig_mrc_vec, p1, p2, p3, p4, angle, dev=None):
    """VESPER_1_prob_new.py:1211-1299 on the GPU."""
    dev = dev or default_device()
    data = dev.to_dev(np.asarray(orig_mrc_data, np.float64))
    vec = dev.to_dev(np.asarray(orig_mrc_vec, np.float32))
    probs = dev.to_dev(np.stack([np.asarray(p, np.float32) for p in (p1, p2, p3, p4)]))
    mats = dev.to_dev(rot_matrices([angle]))
    dout, vout, pout = rot_gather_device(data, vec, mats, probs=probs, dev=dev)
    pout = pout[0].cpu().numpy()
    return (vout[0].cpu().numpy(), dout[0].cpu().numpy().astype(np.asarray(orig_mrc_data).dtype),
            pout[0], pout[1], pout[2], pout[3])


# ----------------------------------------------------------------------------
# search primitives on device
# ----------------------------------------------------------------------------

def target_spectra_device(data, vec, mode, ave, probs=None, dev=None):
    dev = dev or default_device()
    d = int(data.shape[0]) if data is not None else int(vec.shape[0])
    code = mode if isinstance(mode, int) else MODE_CODES[mode]
    nbytes = _native.size_query("vesper_spectra_bytes", d, code)
    spec = torch.empty(nbytes // 8, dtype=torch.complex64, device=dev.device)
    ws = dev.workspace(("target", d, code), _native.size_query("vesper_target_workspace_size", d, code))
    _native.check(dev.lib.vesper_target_spectra(_ptr(data), _ptr(vec), _ptr(probs), d, code, float(ave or 0.0),
                                                _ptr(spec), _ptr(ws), ws.numel(), dev.stream))
    return spec


_TUNED = {}          # (device, side, mode) -> the autotuner's launch shape
_SEARCH_SIZES = {}   # (device, side, mode, mixed, batch, rotations, options) -> (scores per rotation,
#                      workspace tensor, options array)


def search_device(spec, data, vec, mode, ave, rotmats, probs=None, mix=None, batch=0, dev=None, profile=None,
                  opts=None, tuned=False, out=None):
    """vesper_search: (scores f32 [n][nscore], lin int32 [n][nscore]) CUDA tensors,
    written into ``out`` = (scores, lin) when given (contiguous, those shapes).
    With ``profile`` (a dict), vesper_search_profile runs instead and the dict
    receives the per-pass device milliseconds and launch counts.  With
    ``tuned``, the autotuned launch shape is used."""
    dev = dev or default_device()
    d = int(data.shape[0])
    code = mode if isinstance(mode, int) else MODE_CODES[mode]
    n = int(rotmats.shape[0])
    if tuned and opts is None and batch == 0 and not isinstance(mode, int):
        tk = (dev.device, d, mode)
        t = _TUNED.get(tk)
        if t is None:
            from . import autotune
            t = autotune.tune(dev, spec, data, vec, mode, ave, rotmats, probs=probs, mix=mix)
            _TUNED[tk] = t
        batch = int(t["batch"])
        opts = (-1, int(t["cchunk"]), int(t["W"]))
    # per call shape: scores per rotation, the workspace size and the options
    # array (the workspace itself is looked up per call: it belongs to the
    # current stream, and searches on different streams run concurrently)
    sk = (dev.device, d, code, mix is not None, int(batch), max(n, 1), tuple(opts) if opts is not None else None)
    ent = _SEARCH_SIZES.get(sk)
    if ent is None:
        ws_bytes = _native.size_query("vesper_search_workspace_size", d, code, int(batch), max(n, 1))
        ent = _SEARCH_SIZES[sk] = (dev.lib.vesper_search_nscore(code, 1 if mix is not None else 0), ws_bytes,
                                   (ctypes.c_int * 3)(*[int(v) for v in opts]) if opts is not None else None)
    nscore, ws_bytes, copts = ent
    ws = dev.workspace(("search", d, code, int(batch)), ws_bytes)
    if out is not None:
        scores, lin = out
        if (tuple(scores.shape) != (n, nscore) or tuple(lin.shape) != (n, nscore) or not scores.is_contiguous()
                or not lin.is_contiguous()):
            raise ValueError("search_device: out tensors must be contiguous [n][nscore]")
    else:
        scores = torch.empty((n, nscore), dtype=torch.float32, device=dev.device)
        lin = torch.empty((n, nscore), dtype=torch.int32, device=dev.device)
    mixarr = (ctypes.c_double * 5)(*[float(v) for v in mix]) if mix is not None else None
    args = (_ptr(spec), _ptr(data), _ptr(vec), _ptr(probs), d, code, float(ave or 0.0), _ptr(rotmats), n, mixarr,
            _ptr(scores), _ptr(lin), int(batch), _ptr(ws), ws.numel(), dev.stream)
    if profile is not None:
        ms = (ctypes.c_float * 4)()
        nl = (ctypes.c_int * 4)()
        _native.check(dev.lib.vesper_search_profile(*args, ms, nl, copts))
        for k in range(4):
            profile.setdefault("pass_ms", [0.0] * 4)[k] += ms[k]
            profile.setdefault("pass_launches", [0] * 4)[k] += nl[k]
        # (side, mode code, rotations, mixed pass, kernel family) of every
        # profiled call
        path = search_plan(d, code, int(batch), 1, tuple(opts) if opts is not None else None, dev)[0]
        profile.setdefault("calls", []).append((d, code, n, mix is not None, path))
    elif copts is not None:
        _native.check(dev.lib.vesper_search_tuned(*args, copts))
    else:
        _native.check(dev.lib.vesper_search(*args))
    return scores, lin


def search_device_sharded(spec, data, vec, mode, ave, rotmats, group=None, probs=None, mix=None, dev=None, **kw):
    """search_device over every rotation of ``rotmats``; with a
    torch.distributed process group, this rank searches only its contiguous
    block of the rotations on its own GPU and the blocks' per-rotation results
    are gathered in rotation order (shard.search_sharded), so every rank holds
    what one process would have computed.  Returns device tensors as
    search_device does."""
    dev = dev or default_device()
    if group is None:
        return search_device(spec, data, vec, mode, ave, rotmats, probs=probs, mix=mix, dev=dev, **kw)
    from . import shard
    code = mode if isinstance(mode, int) else MODE_CODES[mode]
    nscore = dev.lib.vesper_search_nscore(code, 1 if mix is not None else 0)

    def block(lo, hi):
        if hi <= lo:
            return np.zeros((0, nscore), np.float32), np.zeros((0, nscore), np.int32)
        sc, ln = search_device(spec, data, vec, mode, ave, rotmats[lo:hi], probs=probs, mix=mix, dev=dev, **kw)
        return sc.cpu().numpy(), ln.cpu().numpy()

    sc, ln = shard.search_sharded(block, int(rotmats.shape[0]), group)
    return dev.to_dev(sc), dev.to_dev(ln)


_PLANS = {}


def search_plan(dim, mode, batch=0, nrot=1, opts=None, dev=None):
    """vesper_search_plan: (kernel family 0 radix / 1 register / 2 fused,
    kernel launches of one search call)."""
    dev = dev or default_device()
    code = mode if isinstance(mode, int) else MODE_CODES[mode]
    key = (dev.device, int(dim), code, int(batch), int(nrot), tuple(opts) if opts is not None else None)
    got = _PLANS.get(key)
    if got is not None:
        return got
    path = ctypes.c_int(0)
    nl = ctypes.c_int(0)
    copts = (ctypes.c_int * 3)(*[int(v) for v in opts]) if opts is not None else None
    _native.check(dev.lib.vesper_search_plan(int(dim), code, int(batch), int(nrot), copts, ctypes.byref(path),
                                             ctypes.byref(nl)))
    _PLANS[key] = (path.value, nl.value)
    return path.value, nl.value


def topn_device(scores, topn, column=0, dev=None):
    """Stable top-N indices of scores[:, column] (int32 CUDA tensor, -1 padded)."""
    dev = dev or default_device()
    n = int(scores.shape[0])
    stride = int(scores.shape[1]) if scores.dim() == 2 else 1
    out = torch.empty(max(int(topn), 1), dtype=torch.int32, device=dev.device)
    base = scores[:, column] if scores.dim() == 2 else scores
    _native.check(dev.lib.vesper_topn(ctypes.c_void_p(base.data_ptr()), n, stride, int(topn), _ptr(out),
                                      dev.stream))
    return out[:int(topn)]


def unravel(lin, d):
    lin = int(lin)
    return (lin // (d * d), (lin // d) % d, lin % d)


def score_scale(mode, target):
    if mode == "CC":
        return 1.0 / target.std ** 2
    if mode == "PCC":
        return 1.0 / target.std_norm_ave ** 2
    return None


# ----------------------------------------------------------------------------
# output geometry and final scoring
# ----------------------------------------------------------------------------

def euler2rot(euler):
    """VESPER_1_prob_new.py:1549-1551."""
    return R.from_euler("xyz", euler, degrees=True)


def convert_trans(cen1, cen2, r, trans, xwidth2, dim):
    """VESPER_1_prob_new.py:1554-1566."""
    trans = np.array(trans)
    if trans[0] > 0.5 * dim:
        trans[0] -= dim
    if trans[1] > 0.5 * dim:
        trans[1] -= dim
    if trans[2] > 0.5 * dim:
        trans[2] -= dim
    cen2 = r.apply(cen2)
    return cen1 - (cen2 + trans * xwidth2)


@dataclasses.dataclass
class ScoreResult:
    overlap: float
    nm: int
    total: int
    cc: float
    pcc: float
    score: float
    sco_arr: np.ndarray | None


def get_score_device(target_map, sdata, svec, trans, want_arr=True, dev=None):
    dev = dev or default_device()
    tdata, tvec = _dev_fields(target_map, dev)
    d = int(tdata.shape[0])
    res = torch.empty(8, dtype=torch.float64, device=dev.device)
    sco = torch.empty((d, d, d), dtype=torch.float64, device=dev.device) if want_arr else None
    tr = (ctypes.c_int32 * 3)(*[int(t) for t in trans])
    ws = dev.workspace(("rescore", d), _native.size_query("vesper_rescore_workspace_size", d))
    _native.check(dev.lib.vesper_rescore(_ptr(tdata), _ptr(tvec), float(target_map.ave), float(target_map.std),
                                         float(target_map.std_norm_ave), _ptr(sdata), _ptr(svec), d, tr, _ptr(res),
                                         _ptr(sco), _ptr(ws), ws.numel(), dev.stream))
    r = res.cpu().numpy()
    nm, total = int(r[0]), int(r[1])
    return ScoreResult(float(nm) / float(total), nm, total, float(r[2]), float(r[3]), float(r[4]),
                       sco.cpu().numpy() if want_arr else None)


def _print_score(sr: ScoreResult):
    print("Overlap=" + str(sr.overlap) + " " + str(sr.nm) + "/" + str(sr.total) + " CC=" + str(sr.cc) + " PCC=" +
          str(sr.pcc))
    print("Score=", sr.score)


def get_score(target_map, search_map_data, search_map_vec, trans, dev=None):
    """VESPER_1_prob_new.py:1302-1393 in float64 on the GPU; prints the same two
    lines and returns the per-voxel dot-product array."""
    dev = dev or default_device()
    sdata = dev.to_dev(np.asarray(search_map_data, np.float64))
    svec = dev.to_dev(np.asarray(search_map_vec, np.float32))
    sr = get_score_device(target_map, sdata, svec, trans, dev=dev)
    _print_score(sr)
    return sr.sco_arr


def show_vec(origin, sampled_mrc_vec, sampled_mrc_data, score_arr, score, sample_width, trans, angle, folder_path,
             rank):
    """VESPER_1_prob_new.py:1144-1208: write the rotated, translated query map as
    CA (voxel) / CB (voxel + vector) atom pairs."""
    dim = sampled_mrc_data.shape[0]
    filename = "R_{:02d}-S_{:>7.3f}.pdb".format(rank, score).replace(" ", "_")
    filepath = Path(folder_path) / filename
    origin = np.array([origin[0], origin[1], origin[2]])
    trans = np.array(trans)
    if trans[0] > 0.5 * dim:
        trans[0] -= dim
    if trans[1] > 0.5 * dim:
        trans[1] -= dim
    if trans[2] > 0.5 * dim:
        trans[2] -= dim
    add = origin - trans * sample_width
    nz = np.argwhere(sampled_mrc_data != 0.0)   # C order == the reference's x, y, z loops
    lines = []
    natm = 1
    nres = 1
    for x, y, z in nz:
        tmp = np.array([x, y, z]) * sample_width + add
        lines.append("ATOM{:>7d}  CA  ALA{:>6d}    ".format(natm, nres) +
                     "{:8.3f}{:8.3f}{:8.3f}{:6.2f}{:6.2f}".format(tmp[0], tmp[1], tmp[2], 1.0, score_arr[x][y][z]))
        natm += 1
        tmp = (np.array([x, y, z]) + sampled_mrc_vec[x][y][z]) * sample_width + add
        lines.append("ATOM{:>7d}  CB  ALA{:>6d}    ".format(natm, nres) +
                     "{:8.3f}{:8.3f}{:8.3f}{:6.2f}{:6.2f}".format(tmp[0], tmp[1], tmp[2], 1.0, score_arr[x][y][z]))
        natm += 1
        nres += 1
    with open(filepath, "w") as f:
        f.write("".join(line + "\n" for line in lines))


def _print_model(prefix, i, angle, new_trans):
    print(prefix + str(i), "Rotation=", "(" + str(_py(angle[0])), str(_py(angle[1])), str(_py(angle[2])) + ")",
          "Translation=", "(" + "{:.3f}".format(new_trans[0]), "{:.3f}".format(new_trans[1]),
          "{:.3f}".format(new_trans[2]) + ")")


def _out_folder(folder):
    if folder is not None:
        folder_path = Path.cwd() / folder
    else:
        folder_path = Path.cwd() / ("VESPER_RUN_" + datetime.now().strftime('%m%d_%H%M'))
    Path.mkdir(folder_path)
    return folder_path


# ----------------------------------------------------------------------------
# search entry points
# ----------------------------------------------------------------------------

def search_map_fft(mrc_target, mrc_search, TopN=10, ang=30, mode="VecProduct", is_eval_mode=False, save_path=".",
                   showPDB=False, folder=None, dev=None, batch=0, timings=None, group=None):
    """VESPER_1_prob_new.py:568-795 with the rotation loops on the GPU.  With a
    torch.distributed process ``group`` the rotations are split across its
    ranks (one GPU each) and every rank returns the single-process result."""
    dev = dev or default_device()
    if is_eval_mode:
        print("#For Evaluation Mode")
        print("#Please use the same coordinate system and map size for map1 and map2.")
        print("#Example:")
        print("#In Chimera command line: open map1 and map2 as #0 and #1, then type")
        print("#> open map1.mrc")
        print("#> open map2.mrc")
        print("#> vop #1 resample onGrid #0")
        print("#> volume #2 save new.mrc")
        print("#Chimera will generate the resampled map2.mrc as new.mrc")
        _ = get_score(mrc_target, mrc_search.data, mrc_search.vec, [0, 0, 0], dev=dev)
        return None
    if mode not in MODE_CODES or mode == "prob":
        raise NameError(f"name 'X1' is not defined (unknown mode {mode!r})")
    tdata, tvec = _dev_fields(mrc_target, dev)
    qdata, qvec = _dev_fields(mrc_search, dev)
    d = int(mrc_target.xdim)
    rd3 = 1.0 / d ** 3
    spec = target_spectra_device(tdata, tvec, mode, mrc_target.ave, dev=dev)
    angle_comb = calc_angle_comb(ang)
    mats = rot_matrices_device(angle_comb, dev, key=("grid", float(ang)))
    print("###Start Searching###")
    scores, lin = search_device_sharded(spec, qdata, qvec, mode, mrc_target.ave, mats, group, batch=batch, dev=dev,
                                        tuned=True)
    top = topn_device(scores, TopN, dev=dev)
    scale = score_scale(mode, mrc_target)
    raw = scores[:, 0].cpu().numpy()
    lin_h = lin[:, 0].cpu().numpy()
    top_h = [int(i) for i in top.cpu().numpy() if i >= 0]

    def scaled(r):
        v = np.float64(raw[r])
        if scale is not None:
            v = v * scale
        return v * rd3

    score_arr = raw.astype(np.float64)
    if scale is not None:
        score_arr = score_arr * scale
    score_arr = score_arr * rd3
    ave_s = np.mean(score_arr)
    std_s = np.std(score_arr)
    print("\nStd= " + str(_py(std_s)) + " Ave= " + str(_py(ave_s)) + "\n")
    sorted_topN = [{"angle": angle_comb[r], "vec_score": scaled(r), "vec_trans": unravel(lin_h[r], d)}
                   for r in top_h]
    for i, result_mrc in enumerate(sorted_topN):
        r = euler2rot(result_mrc["angle"])
        new_trans = convert_trans(mrc_target.cent, mrc_search.cent, r, result_mrc["vec_trans"], mrc_search.xwidth,
                                  mrc_search.xdim)
        _print_model("M", i, result_mrc["angle"], new_trans)
    print()
    if ang > 5.0:
        refine_ang_arr = refine_angle_list([s["angle"] for s in sorted_topN])
        # the overlapping +-5 degree sets repeat angles (kept, as in the
        # reference); each distinct angle is searched once and its result
        # copied to every position it holds
        uang, uinv = np.unique(refine_ang_arr, axis=0, return_inverse=True)
        rmats = dev.to_dev(rot_matrices(uang))
        rscores, rlin = search_device_sharded(spec, qdata, qvec, mode, mrc_target.ave, rmats, group, batch=batch,
                                              dev=dev, tuned=True)
        sel_u = dev.to_dev(uinv.reshape(-1).astype(np.int64))
        rscores, rlin = rscores.index_select(0, sel_u), rlin.index_select(0, sel_u)
        rtop = [int(i) for i in topn_device(rscores, TopN, dev=dev).cpu().numpy() if i >= 0]
        rraw = rscores[:, 0].cpu().numpy()
        rlin_h = rlin[:, 0].cpu().numpy()
        sel = dev.to_dev(np.ascontiguousarray(rot_matrices(refine_ang_arr[rtop])))
        gd, gv, _ = rot_gather_device(qdata, qvec, sel, dev=dev)
        refined_list = []
        for k, r in enumerate(rtop):
            v = np.float64(rraw[r])
            if scale is not None:
                v = v * scale
            refined_list.append({"angle": tuple(refine_ang_arr[r]), "vec_score": v * rd3,
                                 "vec_trans": unravel(rlin_h[r], d), "_dev": (gd[k], gv[k])})
    else:
        refined_list = sorted_topN
    if showPDB:
        folder_path = _out_folder(folder)
        print("\n###Writing results to PDB files###")
    else:
        print()
    for i, result_mrc in enumerate(refined_list):
        r = euler2rot(result_mrc["angle"])
        new_trans = convert_trans(mrc_target.cent, mrc_search.cent, r, result_mrc["vec_trans"], mrc_search.xwidth,
                                  mrc_search.xdim)
        _print_model("\n#", i, result_mrc["angle"], new_trans)
        if "_dev" not in result_mrc:
            raise KeyError("data")  # the reference indexes result_mrc["data"] here (:778)
        sd, sv = result_mrc.pop("_dev")
        sr = get_score_device(mrc_target, sd, sv, result_mrc["vec_trans"], want_arr=True, dev=dev)
        _print_score(sr)
        result_mrc["data"] = sd.cpu().numpy()
        result_mrc["vec"] = sv.cpu().numpy()
        if showPDB:
            show_vec(mrc_target.orig, result_mrc["vec"], result_mrc["data"], sr.sco_arr, result_mrc["vec_score"],
                     mrc_search.xwidth, result_mrc["vec_trans"], result_mrc["angle"], folder_path, i)
    return refined_list


def search_map_fft_prob(mrc_P1, mrc_P2, mrc_P3, mrc_P4, mrc_target, mrc_search, mrc_search_p1, mrc_search_p2,
                        mrc_search_p3, mrc_search_p4, ang, alpha=0.0, TopN=10, num_proc=4, vave=-10, vstd=-10,
                        pave=-10, pstd=-10, showPDB=False, folder=None, dev=None, batch=0, group=None):
    """VESPER_1_prob_new.py:798-1141 with both rotation passes and the
    refinement on the GPU.  With a torch.distributed process ``group`` each
    pass splits the rotations across its ranks; the statistics between the
    passes are taken over the gathered scores of every rotation, so they equal
    the single-process values."""
    dev = dev or default_device()
    tdata, tvec = _dev_fields(mrc_target, dev)
    qdata, qvec = _dev_fields(mrc_search, dev)
    tprobs = dev.to_dev(np.stack([np.asarray(m.data, np.float32) for m in (mrc_P1, mrc_P2, mrc_P3, mrc_P4)]))
    qprobs = dev.to_dev(np.stack([np.asarray(m.data, np.float32)
                                  for m in (mrc_search_p1, mrc_search_p2, mrc_search_p3, mrc_search_p4)]))
    d = int(mrc_target.xdim)
    rd3 = 1.0 / (d ** 3)
    spec = target_spectra_device(tdata, tvec, "prob", 0.0, probs=tprobs, dev=dev)
    angle_comb = calc_angle_comb(ang)
    mats = rot_matrices_device(angle_comb, dev, key=("grid", float(ang)))
    print()
    print("###Start Searching###")
    if vave >= 0 and vstd >= 0 and pstd >= 0 and pave >= 0:
        pass
    else:
        s1, _ = search_device_sharded(spec, qdata, qvec, "prob", 0.0, mats, group, probs=qprobs, batch=batch, dev=dev)
        s1 = s1.cpu().numpy().astype(np.float64) * rd3
        vstd = np.std(s1[:, 0])
        vave = np.mean(s1[:, 0])
        pstd = np.std(s1[:, 1])
        pave = np.mean(s1[:, 1])
    print()
    print("DotScore Std=", _py(vstd), "DotScore Ave=", _py(vave))
    print("ProbScore Std=", _py(pstd), "ProbScore Ave=", _py(pave))
    print()
    mix = (alpha, vstd, vave, pstd, pave)
    s2, l2 = search_device_sharded(spec, qdata, qvec, "prob", 0.0, mats, group, probs=qprobs, mix=mix, batch=batch,
                                   dev=dev)
    top = [int(i) for i in topn_device(s2, TopN, column=2, dev=dev).cpu().numpy() if i >= 0]
    s2h = s2.cpu().numpy()
    l2h = l2.cpu().numpy()

    def entry(angle, sc, ln):
        return {"angle": angle, "vec_score": np.float64(sc[0]) * rd3, "vec_trans": unravel(ln[0], d),
                "prob_score": np.float64(sc[1]) * rd3, "prob_trans": unravel(ln[1], d),
                "mixed_score": np.float64(sc[2]) * rd3, "mixed_trans": unravel(ln[2], d)}

    sorted_topN = [entry(angle_comb[r], s2h[r], l2h[r]) for r in top]
    for idx, x in enumerate(sorted_topN):
        print("M", str(idx + 1), {k: _py(v) for k, v in x.items()})
    if ang > 5.0:
        print("\n###Start Refining###")
        refine_ang_list = refine_angle_list([s["angle"] for s in sorted_topN])
        # each distinct angle searched once (the mixed score of a rotation
        # depends on it alone once the statistics are fixed), then expanded
        uang, uinv = np.unique(refine_ang_list, axis=0, return_inverse=True)
        rmats = dev.to_dev(rot_matrices(uang))
        rs, rl = search_device_sharded(spec, qdata, qvec, "prob", 0.0, rmats, group, probs=qprobs, mix=mix,
                                       batch=batch, dev=dev)
        sel_u = dev.to_dev(uinv.reshape(-1).astype(np.int64))
        rs, rl = rs.index_select(0, sel_u), rl.index_select(0, sel_u)
        rtop = [int(i) for i in topn_device(rs, TopN, column=2, dev=dev).cpu().numpy() if i >= 0]
        rsh = rs.cpu().numpy()
        rlh = rl.cpu().numpy()
        sel = dev.to_dev(np.ascontiguousarray(rot_matrices(refine_ang_list[rtop])))
        gd, gv, _ = rot_gather_device(qdata, qvec, sel, dev=dev)
        refined_list = []
        for k, r in enumerate(rtop):
            e = entry(tuple(refine_ang_list[r]), rsh[r], rlh[r])
            e["_dev"] = (gd[k], gv[k])
            refined_list.append(e)
    else:
        refined_list = sorted_topN
    if showPDB:
        folder_path = _out_folder(folder)
        print("###Writing results to PDB files###")
    else:
        print()
    for i, result_mrc in enumerate(refined_list):
        r = euler2rot(result_mrc["angle"])
        new_trans = convert_trans(mrc_target.cent, mrc_search.cent, r, result_mrc["mixed_trans"], mrc_search.xwidth,
                                  mrc_search.xdim)
        _print_model("\n#", i, result_mrc["angle"], new_trans)
        print("Translation=", str(_py(result_mrc["vec_trans"])), "Probability Score=",
              str(_py(result_mrc["prob_score"])), "Probability Translation=", str(_py(result_mrc["prob_trans"])))
        if "_dev" not in result_mrc:
            raise KeyError("data")  # the reference indexes result_mrc["data"] here (:1124)
        sd, sv = result_mrc.pop("_dev")
        sr = get_score_device(mrc_target, sd, sv, result_mrc["vec_trans"], want_arr=True, dev=dev)
        _print_score(sr)
        result_mrc["data"] = sd.cpu().numpy()
        result_mrc["vec"] = sv.cpu().numpy()
        if showPDB:
            show_vec(mrc_target.orig, result_mrc["vec"], result_mrc["data"], sr.sco_arr, result_mrc["mixed_score"],
                     mrc_search.xwidth, result_mrc["mixed_trans"], result_mrc["angle"], folder_path, i)
    return refined_list


# ----------------------------------------------------------------------------
# probability-map hole filling (interpolation_functions.py:6-135)
# ----------------------------------------------------------------------------

def interpolate_device(data, dev=None):
    """vesper_prob_interpolate in place on a CUDA float32 [X][Y][Z][C] tensor."""
    dev = dev or default_device()
    if data.dtype != torch.float32 or not data.is_contiguous() or data.dim() != 4:
        raise ValueError("interpolate_device: a contiguous float32 [X][Y][Z][C] CUDA tensor is needed")
    ws = dev.workspace(("interp",), 8)
    nx, ny, nz, nc = (int(v) for v in data.shape)
    _native.check(dev.lib.vesper_prob_interpolate(_ptr(data), nx, ny, nz, nc, _ptr(ws), ws.numel(), dev.stream))
    found = ctypes.c_int(0)
    _native.check(dev.lib.vesper_prob_interpolate_found(_ptr(ws), ctypes.byref(found), dev.stream))
    if not found.value:
        raise UnboundLocalError("local variable 'ref_x' referenced before assignment")
    return data


def interpolate(data):
    """interpolation_functions.interpolate on the GPU: fills the zero voxels
    of the [X][Y][Z][C] probability array in place and returns None, as the
    reference does."""
    arr = np.asarray(data)
    t = torch.as_tensor(np.ascontiguousarray(arr, np.float32)).to(default_device().device)
    interpolate_device(t)
    out = t.cpu().numpy()
    if isinstance(data, np.ndarray):
        data[...] = out.astype(data.dtype, copy=False)
    return None
