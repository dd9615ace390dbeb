"""CPU oracle for the VESPER alignment hot path -- TEST INFRASTRUCTURE ONLY.

A numpy/scipy restatement of the reference algorithm (KawaiR/VESPER_Python,
``VESPER_1_prob_new.py`` and ``main.py``), with the order-sensitive scalar
loops in ``vesper_oracle.c``.  Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` import this module; the product
path never does.

Numeric conventions follow the reference's pinned environment
(requirements.txt: numpy 1.21, scipy 1.7, pyFFTW 0.12):

* target spectra are ``conj(np.fft.rfftn(x))`` computed in float64 ->
  complex128 (numpy 1.21 has no single-precision FFT);
* the query FFTs are single precision (pyFFTW float32 plans), here
  ``scipy.fft`` in float32; the product ``target * query`` is complex128 and
  is cast to complex64 before the unnormalised float32 inverse;
* ``vec_score * rd3`` is float64 (numpy 1.21 promotes a float32 scalar times a
  Python float to float64), so ranking by scaled score equals ranking by the
  raw float32 score;
* ``sorted(..., reverse=True)`` is stable: equal scores keep rotation order.

Parity status: pinned against golden vectors produced by importing the
unmodified reference module under stand-in modules (tests/golden/).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np
import scipy.fft
from scipy.spatial.transform import Rotation

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libvesper_oracle.so")
_lib = None
_lib_lock = threading.Lock()

MODES = {"V": "VecProduct", "O": "Overlap", "C": "CC", "P": "PCC", "L": "Laplacian"}


def build(force: bool = False) -> str:
    """Compile vesper_oracle.c (gcc, OpenMP, no FP contraction)."""
    os.makedirs(os.path.dirname(_LIB_PATH), exist_ok=True)
    src = os.path.join(_HERE, "vesper_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        tmp = _LIB_PATH + f".{os.getpid()}.tmp"
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
                               src, "-o", tmp, "-lm"])
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    with _lib_lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            vp = ctypes.c_void_p
            L.orc_fastvec.argtypes = [vp, vp, ctypes.c_double, vp, vp, ctypes.c_double, vp, ctypes.c_double,
                                      vp, vp, vp, ctypes.c_int64, ctypes.c_int]
            L.orc_fastvec.restype = None
            L.orc_rot_gather.argtypes = [vp, vp, vp, ctypes.c_int, vp, vp, vp, vp]
            L.orc_rot_gather.restype = None
            L.orc_rot_positions.argtypes = [ctypes.c_int, vp, vp, vp]
            L.orc_rot_positions.restype = None
            _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


# --------------------------------------------------------------------------
# grid sizing, angles, rotation matrices
# --------------------------------------------------------------------------

def next_fast_len(n: int) -> int:
    """pyFFTW 0.12 ``next_fast_len`` (VESPER_1_prob_new.py:97): the smallest
    m >= n of the form 2^a 3^b 5^c 7^d 11^e 13^f with e + f <= 1."""
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


def calc_angle_comb(ang_interval):
    """VESPER_1_prob_new.py:1396-1415: rows (x, y, z) with z slowest, x middle,
    y fastest; x, y in [0, 360), z in [0, 180] by repeated addition."""
    xs, zs = [], []
    i = 0
    while i < 360:
        xs.append(i)
        i += ang_interval
    i = 0
    while i <= 180:
        zs.append(i)
        i += ang_interval
    return np.array(np.meshgrid(xs, xs, zs)).T.reshape(-1, 3)


def rot_matrix_f32(angle) -> np.ndarray:
    """np.flip of the ZYX Euler matrix with |m| < 1e-15 zeroed, as float32
    (VESPER_1_prob_new.py:305-310, :341)."""
    mtx = Rotation.from_euler("ZYX", angle, degrees=True).as_matrix()
    mtx[np.isclose(mtx, 0, atol=1e-15)] = 0
    return np.ascontiguousarray(np.flip(mtx).astype(np.float32))


def refine_angles(top_angles):
    """Refinement angle set (VESPER_1_prob_new.py:693-713): +-5 deg meshgrid per
    top angle, keep x<360, y<360, z<180, then add 360 to negatives."""
    out = []
    for ang in top_angles:
        a = np.array(np.meshgrid([ang[0] - 5, ang[0], ang[0] + 5],
                                 [ang[1] - 5, ang[1], ang[1] + 5],
                                 [ang[2] - 5, ang[2], ang[2] + 5])).T.reshape(-1, 3)
        a = a[(a[:, 0] < 360) & (a[:, 1] < 360) & (a[:, 2] < 180)]
        a[a < 0] += 360
        out.append(a)
    return np.concatenate(out, axis=0)


# --------------------------------------------------------------------------
# map set-up (mrc_set_vox_size, main.py grid unification)
# --------------------------------------------------------------------------

class OMap:
    """The fields of the reference's ``mrc_obj`` the hot path reads."""

    def __init__(self, data_xyz, width, orig):
        self.data = np.array(data_xyz, copy=True)
        self.xdim, self.ydim, self.zdim = self.data.shape
        self.xwidth = np.float32(width)
        self.orig = np.array([np.float32(v) for v in orig])
        self.cent = np.array([self.xdim * 0.5, self.ydim * 0.5, self.zdim * 0.5])
        self.vec = None
        self.dsum = self.Nact = self.ave = self.std = self.std_norm_ave = None


def set_vox_size(m: OMap, th, voxel_size):
    """mrc_set_vox_size (VESPER_1_prob_new.py:59-118) without the prints:
    thresholds m.data in place and returns (new_dim, new_orig, new_cent, dmax_vox)."""
    if th < 0:
        th = 0.0
    m.data[m.data < th] = 0.0
    nz = np.array(np.nonzero(m.data)).T
    d2 = np.linalg.norm(nz - np.array(m.cent), axis=1)
    dmax = max(d2)
    dmax_vox = dmax / m.xwidth
    dmax = dmax * m.xwidth
    new_cent = m.cent * m.xwidth + m.orig
    tmp = 2 * dmax / voxel_size
    new_dim = next_fast_len(int(tmp))
    new_orig = new_cent - 0.5 * new_dim * voxel_size
    return new_dim, new_orig, new_cent, dmax_vox


def unify(dim1, orig1, cent1, dim2, orig2, cent2, voxel_spacing):
    """main.py:166-178: the smaller grid grows to the larger side and its
    origin is recomputed from its centre."""
    orig1 = np.array(orig1, dtype=np.float64)
    orig2 = np.array(orig2, dtype=np.float64)
    if dim1 > dim2:
        dim = dim1
        for a in range(3):
            orig2[a] = cent2[a] - 0.5 * voxel_spacing * dim
    else:
        dim = dim2
        for a in range(3):
            orig1[a] = cent1[a] - 0.5 * voxel_spacing * dim
    return dim, orig1, orig2


# --------------------------------------------------------------------------
# fastVEC
# --------------------------------------------------------------------------

def fastvec(src_data, src_width, src_orig, dest_dim, dest_width, dest_orig, dreso,
            idx=None, nthreads=0, data_dtype=np.float64):
    """doFastVEC (VESPER_1_prob_new.py:180-257) via the C restatement.
    Returns (data, vec).  ``data_dtype`` float32 reproduces prob mode, where the
    destination array is float32 (main.py:345)."""
    src = np.ascontiguousarray(src_data, dtype=np.float32)
    sd = np.array(src.shape, np.int32)
    dd = np.array([dest_dim] * 3, np.int32)
    so = np.array(src_orig, np.float64)
    do = np.array(dest_orig, np.float64)
    data = np.zeros((dest_dim,) * 3, np.float64)
    vec = np.zeros((dest_dim,) * 3 + (3,), np.float32)
    ix = None if idx is None else np.ascontiguousarray(idx, np.int64)
    lib().orc_fastvec(_p(src), _p(sd), float(src_width), _p(so), _p(dd), float(dest_width), _p(do),
                      float(dreso), _p(data), _p(vec), _p(ix), 0 if ix is None else ix.size, int(nthreads))
    return data.astype(data_dtype), vec


def fastvec_stats(data):
    """fastVEC statistics (VESPER_1_prob_new.py:157-161)."""
    dsum = np.sum(data)
    nact = np.count_nonzero(data)
    pos = data[data > 0]
    ave = np.mean(pos)
    std = np.linalg.norm(pos)
    std_norm_ave = np.linalg.norm(pos - ave)
    return dsum, nact, ave, std, std_norm_ave


# --------------------------------------------------------------------------
# rotation of the query map
# --------------------------------------------------------------------------

def rot_mrc(data, vec, angle, F=None):
    """rot_mrc (VESPER_1_prob_new.py:279-354).  Returns (new_vec, new_data)."""
    d = vec.shape[0]
    F = rot_matrix_f32(angle) if F is None else F
    dd = np.ascontiguousarray(data, np.float64)
    vv = np.ascontiguousarray(vec, np.float32)
    od = np.zeros_like(dd)
    ov = np.zeros_like(vv)
    lib().orc_rot_gather(_p(dd), _p(vv), None, d, _p(F), _p(od), _p(ov), None)
    return ov, od.astype(data.dtype)


def rot_mrc_prob(data, vec, p1, p2, p3, p4, angle, F=None):
    """rot_mrc_prob (VESPER_1_prob_new.py:1211-1299): returns
    (new_vec, new_data, new_p1, new_p2, new_p3, new_p4)."""
    d = vec.shape[0]
    F = rot_matrix_f32(angle) if F is None else F
    dd = np.ascontiguousarray(data, np.float64)
    vv = np.ascontiguousarray(vec, np.float32)
    ps = [np.ascontiguousarray(p, np.float32) for p in (p1, p2, p3, p4)]
    od = np.zeros_like(dd)
    ov = np.zeros_like(vv)
    ops = [np.zeros_like(p) for p in ps]
    pin = (ctypes.c_void_p * 4)(*[p.ctypes.data for p in ps])
    pout = (ctypes.c_void_p * 4)(*[p.ctypes.data for p in ops])
    lib().orc_rot_gather(_p(dd), _p(vv), pin, d, _p(F), _p(od), _p(ov), pout)
    return (ov, od.astype(data.dtype), *ops)


def rot_mrc_numpy(data, vec, F, probs=None):
    """rot_mrc / rot_mrc_prob (VESPER_1_prob_new.py:279-354, :1211-1299) in
    whole-array numpy operations, the form the reference runs: float32 matmul
    of the centred new positions by the transposed matrix, in-bounds mask,
    truncation, density (or per-channel) non-zero mask, fancy-index gather,
    float32 matmul of the vectors, fancy-index scatter (rows in the
    reference's order, z slowest, x middle, y fastest, so the last row wins a
    collision).  For the CPU-baseline timing; the C gather above is the
    checked form.  Returns (new_vec, new_data[, new_probs list])."""
    d = vec.shape[0]
    cent = 0.5 * float(d)
    ar = np.arange(d)
    z, x, y = np.meshgrid(ar, ar, ar, indexing="ij")
    new_pos = np.stack([x.reshape(-1), y.reshape(-1), z.reshape(-1)], axis=1) - cent
    Ff = np.asarray(F, np.float32)
    old = new_pos.astype(np.float32) @ Ff.T + np.float32(cent)
    inb = np.all((old >= 0) & (old < d), axis=1)
    src = old[inb].astype(np.int32)
    dst = (new_pos[inb].astype(np.int32) + cent).astype(np.int64)
    si, sj, sk = src[:, 0], src[:, 1], src[:, 2]
    di, dj, dk = dst[:, 0], dst[:, 1], dst[:, 2]
    keep = data[si, sj, sk] != 0.0
    new_vec = np.zeros_like(vec)
    new_data = np.zeros_like(data)
    new_vec[di[keep], dj[keep], dk[keep]] = vec[si[keep], sj[keep], sk[keep]].astype(np.float32) @ Ff
    new_data[di[keep], dj[keep], dk[keep]] = data[si[keep], sj[keep], sk[keep]]
    if probs is None:
        return new_vec, new_data
    outs = []
    for p in probs:
        m = p[si, sj, sk] != 0.0
        o = np.zeros_like(p)
        o[di[m], dj[m], dk[m]] = p[si[m], sj[m], sk[m]]
        outs.append(o)
    return new_vec, new_data, outs


def rot_positions(d, F):
    """float32 old positions and destination indices of every new_pos row."""
    n = d ** 3
    old = np.zeros((n, 3), np.float32)
    dst = np.zeros(n, np.int64)
    lib().orc_rot_positions(d, _p(np.ascontiguousarray(F, np.float32)), _p(old), _p(dst))
    return old, dst


# --------------------------------------------------------------------------
# scalar-mode transforms and target spectra
# --------------------------------------------------------------------------

def laplacian_filter(arr):
    """laplacian_filter (VESPER_1_prob_new.py:494-526): -6 a + x+1 + x-1 + y+1
    + y-1 + z+1 + z-1 where a > 0, missing neighbours skipped, float64."""
    a = np.asarray(arr)
    out = np.zeros_like(a)
    m = a > 0
    acc = -6.0 * a
    z = np.zeros_like(a)

    def sh(axis, step):
        s = np.zeros_like(a)
        src = [slice(None)] * 3
        dst = [slice(None)] * 3
        if step > 0:
            src[axis] = slice(1, None)
            dst[axis] = slice(0, -1)
        else:
            src[axis] = slice(0, -1)
            dst[axis] = slice(1, None)
        s[tuple(dst)] = a[tuple(src)]
        return s

    for axis in range(3):
        for step in (1, -1):
            acc = acc + sh(axis, step)  # a missing neighbour adds +0.0
    out[m] = acc[m]
    del z
    return out


def mode_field(mode, data, vec=None, ave=None):
    """The real field correlated for each mode (VESPER_1_prob_new.py:601-615,
    :546-555).  Returns a list of arrays (3 for V, 1 otherwise)."""
    if mode in ("V", "VecProduct"):
        return [vec[..., 0], vec[..., 1], vec[..., 2]]
    if mode in ("O", "Overlap"):
        return [np.where(data > 0, 1.0, 0.0)]
    if mode in ("C", "CC"):
        return [np.where(data > 0, data, 0.0)]
    if mode in ("P", "PCC"):
        return [np.where(data > 0, data - ave, 0.0)]
    if mode in ("L", "Laplacian"):
        return [laplacian_filter(data)]
    raise ValueError(f"unknown mode {mode!r}")


def target_spectra(fields):
    """conj(np.fft.rfftn(x)) in float64 -> complex128 (VESPER_1_prob_new.py:621-628)."""
    return [np.conj(np.fft.rfftn(np.asarray(f, np.float64))) for f in fields]


def correlate(target_list, query_list, fp64=False, workers=None):
    """fft_search_best_dot (VESPER_1_prob_new.py:464-491): per channel the
    unnormalised inverse of (target * rfftn_f32(query)) -> float32 volumes.
    ``workers`` is scipy.fft's thread count (the reference's FFTW plans use
    every CPU, VESPER_1_prob_new.py:15)."""
    out = []
    for T, q in zip(target_list, query_list):
        shape = q.shape
        if fp64:
            Q = scipy.fft.rfftn(np.asarray(q, np.float64), workers=workers)
            r = scipy.fft.irfftn(T * Q, s=shape, workers=workers) * np.prod(shape)
            out.append(r)
        else:
            Q = scipy.fft.rfftn(np.asarray(q, np.float32), workers=workers).astype(np.complex128)
            P = (T * Q).astype(np.complex64)
            r = (scipy.fft.irfftn(P, s=shape, workers=workers) * np.float32(np.prod(shape))).astype(np.float32)
            out.append(r)
    return out


def best_trans(vols):
    """find_best_trans_list (VESPER_1_prob_new.py:357-374): sum, amax, first
    argmax in C order."""
    s = np.zeros_like(vols[0])
    for v in vols:
        s = s + v
    best = np.amax(s)
    return best, np.unravel_index(s.argmax(), s.shape)


def best_trans_mixed(vvols, pvols, alpha, vstd, vave, pstd, pave, promotion="numpy1"):
    """find_best_trans_mixed (VESPER_1_prob_new.py:1530-1545).

    promotion="numpy1" (the reference's pinned numpy 1.21): float32 volumes
    combined with float64 scalars stay float32.  promotion="numpy2" (NEP 50):
    the np.float64 statistics promote the arithmetic to float64; this variant
    exists only to compare with golden vectors recorded under numpy 2."""
    sv = sum(vvols)
    sp = sum(pvols)
    if promotion == "numpy2":
        sv = (sv - np.float64(vave)) / np.float64(vstd)
        sp = (sp - np.float64(pave)) / np.float64(pstd)
        mixed = (1 - alpha) * sv + alpha * sp
    else:
        sv = (sv - np.float32(vave)) / np.float32(vstd)
        sp = (sp - np.float32(pave)) / np.float32(pstd)
        mixed = np.float32(1 - alpha) * sv + np.float32(alpha) * sp
    return mixed.max(), np.unravel_index(mixed.argmax(), mixed.shape)


def score_scale(mode, target_std, target_std_norm_ave):
    """CC and PCC scale factors (VESPER_1_prob_new.py:1452-1457)."""
    if mode in ("C", "CC"):
        return 1.0 / target_std ** 2
    if mode in ("P", "PCC"):
        return 1.0 / target_std_norm_ave ** 2
    return 1.0


def rot_and_search(tgt_spec, mode, qdata, qvec, angle, target_ave, fp64=False, workers=None):
    """rot_and_search_fft (VESPER_1_prob_new.py:1418-1459) without the CC/PCC
    scale: returns (raw float32 score, (i, j, k), new_vec, new_data)."""
    new_vec, new_data = rot_mrc(qdata, qvec, angle)
    q = mode_field(mode, new_data, new_vec, target_ave)
    best, trans = best_trans(correlate(tgt_spec, q, fp64=fp64, workers=workers))
    return best, tuple(int(t) for t in trans), new_vec, new_data


def search(tgt_spec, mode, qdata, qvec, angles, target_ave, fp64=False, workers=None):
    """Per-rotation (raw score, trans) over ``angles``."""
    sc = np.zeros(len(angles), np.float64 if fp64 else np.float32)
    tr = np.zeros((len(angles), 3), np.int64)
    for r, ang in enumerate(angles):
        s, t, _, _ = rot_and_search(tgt_spec, mode, qdata, qvec, ang, target_ave, fp64=fp64, workers=workers)
        sc[r] = s
        tr[r] = t
    return sc, tr


def topn(scores, n):
    """Stable descending order, ties by lower index (VESPER_1_prob_new.py:664)."""
    order = sorted(range(len(scores)), key=lambda i: float(scores[i]), reverse=True)
    return np.array(order[:n], np.int64)


# --------------------------------------------------------------------------
# final scoring and output geometry
# --------------------------------------------------------------------------

def wrap_trans(trans, dim):
    t = np.array(trans)
    for a in range(3):
        if t[a] > 0.5 * dim:
            t[a] -= dim
    return t


def get_score(tdata, tvec, tave, tstd, tstd_norm_ave, sdata, svec, trans):
    """get_score (VESPER_1_prob_new.py:1302-1393) without the prints: returns
    (overlap, Nm, total, cc, pcc, score, sco_arr).  Keeps the reference's
    ``d2 = where(d2 <= 0, 0, d1)`` (:1357)."""
    ave2 = np.mean(sdata[sdata > 0])
    std2 = np.linalg.norm(sdata[sdata > 0])
    pstd2 = np.linalg.norm(sdata[sdata > 0] - ave2)
    dim = tdata.shape[0]
    t = wrap_trans(trans, dim)
    tpos = np.array(np.meshgrid(np.arange(dim), np.arange(dim), np.arange(dim))).T.reshape(-1, 3)
    spos = tpos + t
    total = np.count_nonzero(tdata[tpos[:, 0], tpos[:, 1], tpos[:, 2]])
    comb = np.hstack((tpos, spos))
    comb = comb[(comb[:, 3] >= 0) & (comb[:, 4] >= 0) & (comb[:, 5] >= 0)
                & (comb[:, 3] < dim) & (comb[:, 4] < dim) & (comb[:, 5] < dim)]
    tpos = comb[:, 0:3]
    spos = comb[:, 3:6]
    d1 = tdata[tpos[:, 0], tpos[:, 1], tpos[:, 2]]
    d2 = sdata[spos[:, 0], spos[:, 1], spos[:, 2]]
    d1 = np.where(d1 <= 0, 0.0, d1)
    d2 = np.where(d2 <= 0, 0.0, d1)
    pd1 = np.where(d1 <= 0, 0.0, d1 - tave)
    pd2 = np.where(d2 <= 0, 0.0, d2 - ave2)
    cc = np.sum(np.multiply(d1, d2))
    pcc = np.sum(np.multiply(pd1, pd2))
    tz = tdata[tpos[:, 0], tpos[:, 1], tpos[:, 2]] == 0
    tnz = tdata[tpos[:, 0], tpos[:, 1], tpos[:, 2]] > 0
    snz = sdata[spos[:, 0], spos[:, 1], spos[:, 2]] > 0
    total += np.count_nonzero(np.multiply(tz, snz))
    tv = tvec[tpos[:, 0], tpos[:, 1], tpos[:, 2]]
    sv = svec[spos[:, 0], spos[:, 1], spos[:, 2]]
    sco_arr = np.zeros_like(sdata)
    sco = np.einsum("ij,ij->i", tv, sv)
    sco_arr[spos[:, 0], spos[:, 1], spos[:, 2]] = sco
    score = np.sum(sco_arr)
    nm = np.count_nonzero(np.multiply(tnz, snz))
    return float(nm) / float(total), nm, total, cc / (tstd * std2), pcc / (tstd_norm_ave * pstd2), score, sco_arr


def euler2rot(euler):
    """VESPER_1_prob_new.py:1549-1551 ('xyz' convention, unlike rot_mrc's 'ZYX')."""
    return Rotation.from_euler("xyz", euler, degrees=True)


def convert_trans(cen1, cen2, r, trans, xwidth2, dim):
    """VESPER_1_prob_new.py:1554-1566."""
    t = wrap_trans(trans, dim)
    return cen1 - (r.apply(cen2) + t * xwidth2)


# --------------------------------------------------------------------------
# prob mode
# --------------------------------------------------------------------------

def rot_and_search_prob(tgt_spec7, qdata, qvec, qprobs, angle, alpha, stats=None, fp64=False,
                        promotion="numpy1"):
    """rot_and_search_fft_prob (VESPER_1_prob_new.py:1462-1527).  ``stats`` is
    (vstd, vave, pstd, pave) or None.  Returns (vec_score, vec_trans,
    prob_score, prob_trans, mixed_score, mixed_trans) with raw scores."""
    r = rot_mrc_prob(qdata, qvec, *qprobs, angle)
    nv = r[0]
    qv = [nv[..., 0], nv[..., 1], nv[..., 2]]
    qp = list(r[2:6])
    cv = correlate(tgt_spec7[:3], qv, fp64=fp64)
    cp = correlate(tgt_spec7[3:], qp, fp64=fp64)
    vs, vt = best_trans(cv)
    ps, pt = best_trans(cp)
    ms, mt = None, None
    if stats is not None:
        vstd, vave, pstd, pave = stats
        ms, mt = best_trans_mixed(cv, cp, alpha, vstd, vave, pstd, pave, promotion=promotion)
        mt = tuple(int(t) for t in mt)
    return vs, tuple(int(t) for t in vt), ps, tuple(int(t) for t in pt), ms, mt


def prob_stats(vscores, pscores, rd3):
    """Pass-1 statistics (VESPER_1_prob_new.py:920-926): np.std (ddof=0) and
    np.mean of the rd3-scaled per-rotation scores (float64)."""
    v = np.asarray(vscores, np.float64) * rd3
    p = np.asarray(pscores, np.float64) * rd3
    return np.std(v), np.mean(v), np.std(p), np.mean(p)


# --------------------------------------------------------------------------
# probability-map hole filling (interpolation_functions.py:6-135)
# --------------------------------------------------------------------------

def interpolate(data):
    """interpolate, in place on a [X][Y][Z][C] float32 array: the parity of
    the first voxel (C order) with channel 0 > 0 fixes the reference lattice;
    zero voxels whose parity differs on one axis (x, y, z), then on two (xy,
    xz, yz), then on all three take the float64 mean of their neighbours along
    the differing axes (x pair, y pair, z pair in that order), rounded to
    float32.  Index -1 wraps to the last element and each axis stops before
    its last index, as the reference's loops do."""
    pos = np.argwhere(data[..., 0] > 0)
    if len(pos) == 0:
        raise ValueError("interpolate: no voxel with a positive first channel (the reference's ref_x is unbound)")
    ref = [int(v) % 2 for v in pos[0]]
    shape = data.shape[:3]
    for m in (1, 2, 4, 3, 5, 6, 7):
        start = [(r + 1) % 2 if m & (1 << a) else r for a, r in enumerate(ref)]
        idx = [np.arange(start[a], shape[a] - 1, 2) for a in range(3)]
        if any(len(i) == 0 for i in idx):
            continue
        cell = data[np.ix_(*idx)]
        acc = np.zeros(cell.shape, np.float64)
        n = 0
        for a in range(3):
            if m & (1 << a):
                up = list(idx)
                dn = list(idx)
                up[a] = idx[a] + 1
                dn[a] = idx[a] - 1          # -1 indexes the last element, as in Python
                acc += data[np.ix_(*up)]
                acc += data[np.ix_(*dn)]
                n += 2
        data[np.ix_(*idx)] = np.where(cell == 0, (acc / n).astype(np.float32), cell)
