"""The float-float arithmetic of the fastVEC kernels (k_fvf_z/y/x), restated in
numpy with float32 operations, against the float64 C restatement of the
reference loop (doFastVEC, VESPER_1_prob_new.py:180-257): the precision the
GPU path relies on, checked on the CPU.

Each partial sum is a pair (hi, lo) of float32 values.  Products: TwoProd of
the high parts (the exact error of a float32 product is computed here in
float64, which holds a 24 x 24-bit product exactly) plus the cross terms with
fmaf; sums: TwoSum, the low parts, then FastTwoSum.  The same operation order
as the kernels.
"""
import contextlib
import io

import numpy as np

from oracle import vesper_oracle as orc

f32, f64 = np.float32, np.float64


def _fma(a, b, c):
    return (a.astype(f64) * b.astype(f64) + c.astype(f64)).astype(f32)


def _mul_f(h, l, v):
    ph = (h * v).astype(f32)
    e = (h.astype(f64) * v.astype(f64) - ph.astype(f64)).astype(f32)
    return ph, _fma(l, v, e)


def _mul(ah, al, bh, bl):
    ph = (ah * bh).astype(f32)
    e = (ah.astype(f64) * bh.astype(f64) - ph.astype(f64)).astype(f32)
    e = _fma(ah, bl, e)
    return ph, _fma(al, bh, e)


def _add(sh, sl, th, tl):
    s = (sh + th).astype(f32)
    bb = (s - sh).astype(f32)
    e = ((sh - (s - bb).astype(f32)).astype(f32) + (th - bb).astype(f32)).astype(f32)
    e = (e + (sl + tl).astype(f32)).astype(f32)
    h = (s + e).astype(f32)
    return h, (e - (h - s).astype(f32)).astype(f32)


def _split(x):
    h = x.astype(f32)
    return h, (x - h.astype(f64)).astype(f32)


def _tables(S, d, sw, sorig, dw, dorig, dreso):
    q = dreso / sw
    fsiv = 1.0 / (q * 0.5) ** 2
    fmaxd = q * 2.0
    WB = int(2.0 * fmaxd) + 3
    T = []
    for a in range(3):
        p = ((np.arange(d) * dw + dorig[a]) - sorig[a]) / sw
        stp = np.maximum((p - fmaxd).astype(np.int64), 0)
        endp = np.minimum(((p + fmaxd) + 1.0).astype(np.int64), S[a])
        ln = np.clip(endp - stp, 0, WB)
        k = np.arange(WB)[:, None]
        r = (stp[None, :] + k) - p[None, :]
        w = np.where(k < ln[None, :], np.exp(-1.5 * (r * r) * fsiv), 0.0)
        T.append(dict(pos=p, stp=stp, len=ln, idx=np.where((p >= 0) & (p < S[a]), p.astype(np.int64), -1),
                      w=_split(w), wp=_split(w * (stp[None, :] + k))))
    return T, WB


def fastvec_float_float(src, sw, sorig, d, dw, dorig, dreso):
    S = src.shape
    T, WB = _tables(S, d, sw, sorig, dw, dorig, dreso)
    src = src.astype(f32)
    zero = lambda shape: [np.zeros(shape, f32), np.zeros(shape, f32)]
    A0, A1 = zero((S[0], S[1], d)), zero((S[0], S[1], d))
    tz = T[2]
    for k in range(WB):
        m = (k < tz["len"])[None, None, :]
        v = np.where(m, src[:, :, np.minimum(tz["stp"] + k, S[2] - 1)], f32(0))
        for acc, (wh, wl) in ((A0, tz["w"]), (A1, tz["wp"])):
            th, tl = _mul_f(np.broadcast_to(wh[k], v.shape), np.broadcast_to(wl[k], v.shape), v)
            acc[0], acc[1] = _add(acc[0], acc[1], th, tl)
    ty = T[1]
    B = [zero((S[0], d, d)) for _ in range(3)]
    for k in range(WB):
        iy = np.minimum(ty["stp"] + k, S[1] - 1)
        m = (k < ty["len"])[None, :, None]
        a0 = [np.where(m, A0[0][:, iy, :], f32(0)), np.where(m, A0[1][:, iy, :], f32(0))]
        a1 = [np.where(m, A1[0][:, iy, :], f32(0)), np.where(m, A1[1][:, iy, :], f32(0))]
        W = lambda t: [np.broadcast_to(t[0][k][None, :, None], a0[0].shape),
                       np.broadcast_to(t[1][k][None, :, None], a0[0].shape)]
        for acc, x, wt in ((B[0], a0, ty["w"]), (B[1], a0, ty["wp"]), (B[2], a1, ty["w"])):
            ww = W(wt)
            th, tl = _mul(x[0], x[1], ww[0], ww[1])
            acc[0], acc[1] = _add(acc[0], acc[1], th, tl)
    tx = T[0]
    D = [zero((d, d, d)) for _ in range(4)]
    for k in range(WB):
        ix = np.minimum(tx["stp"] + k, S[0] - 1)
        m = (k < tx["len"])[:, None, None]
        b = [[np.where(m, B[j][0][ix], f32(0)), np.where(m, B[j][1][ix], f32(0))] for j in range(3)]
        W = lambda t: [np.broadcast_to(t[0][k][:, None, None], b[0][0].shape),
                       np.broadcast_to(t[1][k][:, None, None], b[0][0].shape)]
        for acc, x, wt in ((D[0], b[0], tx["w"]), (D[1], b[0], tx["wp"]), (D[2], b[1], tx["w"]), (D[3], b[2], tx["w"])):
            ww = W(wt)
            th, tl = _mul(x[0], x[1], ww[0], ww[1])
            acc[0], acc[1] = _add(acc[0], acc[1], th, tl)
    dt, px, py, pz = [D[j][0].astype(f64) + D[j][1].astype(f64) for j in range(4)]
    ix_, iy_, iz_ = T[0]["idx"], T[1]["idx"], T[2]["idx"]
    valid = (ix_[:, None, None] >= 0) & (iy_[None, :, None] >= 0) & (iz_[None, None, :] >= 0)
    valid &= src[np.maximum(ix_, 0)][:, np.maximum(iy_, 0)][:, :, np.maximum(iz_, 0)] != 0
    dt = np.where(valid, dt, 0.0)
    ok = valid & (dt != 0)
    with np.errstate(all="ignore"):
        t0 = px * (1.0 / dt) - T[0]["pos"][:, None, None]
        t1 = py * (1.0 / dt) - T[1]["pos"][None, :, None]
        t2 = pz * (1.0 / dt) - T[2]["pos"][None, None, :]
        dv = np.sqrt(t0 * t0 + t1 * t1 + t2 * t2)
        dv = np.where(dv == 0, 1.0, dv)
        vec = np.stack([t0 * (1.0 / dv), t1 * (1.0 / dv), t2 * (1.0 / dv)], -1).astype(f32)
    return dt, np.where(ok[..., None], vec, f32(0))


def _check(src, sw, so, d, dw, do, g, rel_tol=1e-12):
    ref_d, ref_v = orc.fastvec(src, sw, so, d, dw, do, g)
    data, vec = fastvec_float_float(src, sw, np.asarray(so, f64), d, dw, np.asarray(do, f64), g)
    nz = ref_d != 0
    assert np.array_equal(data != 0, nz)
    assert np.max(np.abs(data - ref_d)[nz] / np.abs(ref_d[nz])) < rel_tol
    assert np.max(np.abs(vec - ref_v)) < 2e-6


def test_float_float_golden_cases(golden_dir):
    g = np.load(f"{golden_dir}/fastvec_small.npz")
    for i in range(3):
        S, sw, so0, so1, so2, dd, dw, do0, do1, do2, gg = g[f"c{i}_params"]
        _check(g[f"c{i}_src"], sw, [so0, so1, so2], int(dd), dw, [do0, do1, do2], gg, rel_tol=1e-13)


def test_float_float_blob_map():
    """A 48^3 generator map at s = 3, g = 16 (33-voxel bands, the learned-proposal
    workload's band width)."""
    from vesper_python_gb300 import synth
    from vesper_python_gb300 import vesper as vg
    rng = np.random.default_rng(5)
    src = synth.make_blob_map(rng, 48, 60, 15.0)
    m = vg.mrc_obj.from_array(src, 1.0, (0.0, 0.0, 0.0))
    with contextlib.redirect_stdout(io.StringIO()):
        _, mn = vg.mrc_set_vox_size(m, 0.1, 3.0)
    _check(m.data, np.float64(m.xwidth), m.orig.astype(f64), mn.xdim, 3.0, mn.orig, 16.0, rel_tol=1e-13)


def test_float_float_noncubic_sources(golden_dir):
    g = np.load(f"{golden_dir}/fastvec_noncubic.npz")
    for i in range(2):
        sw, so0, so1, so2, dd, dw, do0, do1, do2, gg = g[f"c{i}_params"]
        data, vec = fastvec_float_float(g[f"c{i}_src"], sw, np.array([so0, so1, so2], f64), int(dd), dw,
                                        np.array([do0, do1, do2], f64), gg)
        rd = g[f"c{i}_data"]
        assert np.array_equal(data != 0, rd != 0)
        assert np.max(np.abs(data - rd)[rd != 0] / np.abs(rd[rd != 0])) < 1e-13
        assert np.max(np.abs(vec - g[f"c{i}_vec"])) < 2e-6
