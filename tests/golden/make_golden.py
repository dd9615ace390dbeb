"""Generate the golden vectors under tests/golden/ by running the UNMODIFIED
reference module (imported under stand-in modules, see refshim.py).

Run in a container that has the reference checkout:

    VESPER_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py

Outputs (committed):
  angles.npz          calc_angle_comb for several steps
  rot_small.npz       rot_mrc / rot_mrc_prob digests over every rotation of
                      the 30-degree grid at small sides, plus full outputs of
                      a few rotations
  fastvec_small.npz   doFastVEC (pure-Python reference loop) on tiny maps
  search_pair128.npz  mrc_set_vox_size, per-rotation raw (score, trans) for
                      modes V/O/C/P/L, refined top-N, on the seed-0
                      128^3/64^3 pair at s=7, A=30
  search_pair128_*.txt  the reference's stdout for each mode
  prob_pair128.npz    prob-mode per-rotation results, statistics and top-N
  prob_pair128.txt    the reference's stdout
  voxsize_cases.npz   mrc_set_vox_size on small maps (thresholds incl. the
                      negative-shift path, two voxel sizes): digests of data
                      and dens, the new grid and the printed lines
  show_vec_cases.npz  show_vec's PDB files (names and text) for two models
  fastvec_noncubic.npz doFastVEC on non-cubic sources (windows clipped)

The coarse fields feeding the search goldens come from the C restatement of
doFastVEC (the pure-Python reference loop is far too slow at 65^3 windows);
that restatement is itself pinned by fastvec_small.npz.
"""
from __future__ import annotations

import contextlib
import hashlib
import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import refshim  # noqa: E402
from oracle import vesper_oracle as orc  # noqa: E402
from vesper_python_gb300 import synth  # noqa: E402

ref = refshim.import_reference()


def digest(*arrays):
    h = hashlib.sha1()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def gen_angles():
    out = {}
    # steps that divide 360 and steps that do not (the grid's range ends)
    for a in (30.0, 15.0, 10.0, 45.0, 60.0, 20.0, 90.0, 7.0, 25.0, 7.5, 50.0, 100.0):
        out[f"A{a:g}"] = ref.calc_angle_comb(a)
    np.savez_compressed(os.path.join(HERE, "angles.npz"), **out)


def small_field(rng, d, zero_frac=0.4, dtype=np.float64):
    data = rng.uniform(0.1, 2.0, size=(d, d, d))
    data[rng.random((d, d, d)) < zero_frac] = 0.0
    vec = rng.normal(size=(d, d, d, 3))
    vec /= np.linalg.norm(vec, axis=-1, keepdims=True)
    vec[data == 0] = 0
    return data.astype(dtype), vec.astype(np.float32)


def gen_rot_small():
    rng = np.random.default_rng(7)
    out = {}
    angles = ref.calc_angle_comb(30.0)
    for d in (8, 9, 12, 15):
        data, vec = small_field(rng, d)
        out[f"d{d}_data"] = data
        out[f"d{d}_vec"] = vec
        dig = []
        for ang in angles:
            nv, nd = ref.rot_mrc(data, vec, ang)
            dig.append(digest(nv, nd))
        out[f"d{d}_digest"] = np.array(dig)
        for r in (0, 1, 13, 144, 500, 1007):
            nv, nd = ref.rot_mrc(data, vec, angles[r])
            out[f"d{d}_r{r}_vec"] = nv
            out[f"d{d}_r{r}_data"] = nd
    # 10-degree grid (every 37th rotation) and odd refinement angles
    angles10 = ref.calc_angle_comb(10.0)[::37]
    extra = np.array([[355.0, 5.0, 175.0], [5.0, 355.0, 35.0], [25.0, 65.0, 5.0], [0.0, 0.0, 5.0]])
    for d in (12, 15):
        data, vec = out[f"d{d}_data"], out[f"d{d}_vec"]
        out[f"d{d}_a10_digest"] = np.array([digest(*ref.rot_mrc(data, vec, a)) for a in angles10])
        out[f"d{d}_extra_digest"] = np.array([digest(*ref.rot_mrc(data, vec, a)) for a in extra])
    out["angles10_sub"] = angles10
    out["extra_angles"] = extra
    # prob variant (float32 data, per-channel masks)
    for d in (9, 12):
        data, vec = small_field(rng, d, dtype=np.float32)
        probs = []
        for c in range(4):
            p = rng.dirichlet([0.5] * 4, size=(d, d, d))[..., c].astype(np.float32)
            p[rng.random((d, d, d)) < 0.5] = 0.0
            probs.append(p)
        out[f"p{d}_data"] = data
        out[f"p{d}_vec"] = vec
        out[f"p{d}_probs"] = np.stack(probs)
        sel = angles[::11]
        out[f"p{d}_digest"] = np.array([digest(*ref.rot_mrc_prob(data, vec, *probs, a)) for a in sel])
    np.savez_compressed(os.path.join(HERE, "rot_small.npz"), **out)


def gen_fastvec_small():
    rng = np.random.default_rng(11)
    out = {}
    cases = [
        # (src side, src width, src orig, dest dim, dest width, dest orig, dreso)
        (18, 1.0, (0.0, 0.0, 0.0), 6, 3.0, (0.3, -0.7, 1.1), 4.0),
        (16, 1.0, (2.5, -1.0, 0.0), 7, 2.5, (1.0, -2.0, 0.25), 3.0),
        (14, 1.5, (0.0, 0.0, 0.0), 5, 4.0, (-3.0, 2.0, 1.0), 5.0),
    ]
    for i, (S, sw, so, dd, dw, do, g) in enumerate(cases):
        src = synth.make_blob_map(rng, S, 12, S * 0.3, sigma=1.2).astype(np.float32)
        src[src < 0.1] = 0.0
        sobj = refshim.make_mrc_obj(ref, src, sw, so)
        dobj = refshim.make_mrc_obj(ref, np.zeros((dd,) * 3), dw, (0, 0, 0))
        dobj.orig = np.array(do, np.float64)
        dobj.xwidth = dw
        with contextlib.redirect_stdout(io.StringIO()):
            res = ref.fastVEC(sobj, dobj, dreso=g)
        out[f"c{i}_src"] = src
        out[f"c{i}_params"] = np.array([S, sw, *so, dd, dw, *do, g], np.float64)
        out[f"c{i}_data"] = res.data
        out[f"c{i}_vec"] = res.vec
        out[f"c{i}_stats"] = np.array([res.dsum, res.Nact, res.ave, res.std, res.std_norm_ave], np.float64)
    np.savez_compressed(os.path.join(HERE, "fastvec_small.npz"), **out)


def gen_fastvec_noncubic():
    """doFastVEC (pure-Python reference loop) on non-cubic sources, with the
    destination grid reaching past the source on some axes (windows clipped at
    both ends)."""
    rng = np.random.default_rng(12)
    out = {}
    cases = [
        # (src shape, src width, src orig, dest dim, dest width, dest orig, dreso)
        ((20, 14, 17), 1.0, (0.0, 1.5, -2.0), 7, 3.0, (-1.0, 0.5, 0.0), 4.0),
        ((12, 19, 15), 1.25, (3.0, 0.0, 0.0), 6, 3.5, (2.0, -4.0, 1.5), 3.0),
    ]
    for i, (shape, sw, so, dd, dw, do, g) in enumerate(cases):
        src = np.zeros(shape, np.float32)
        m = synth.make_blob_map(rng, max(shape), 10, min(shape) * 0.35, sigma=1.2).astype(np.float32)
        src[...] = m[:shape[0], :shape[1], :shape[2]]
        src[src < 0.1] = 0.0
        sobj = refshim.make_mrc_obj(ref, src, sw, so)
        dobj = refshim.make_mrc_obj(ref, np.zeros((dd,) * 3), dw, (0, 0, 0))
        dobj.orig = np.array(do, np.float64)
        dobj.xwidth = dw
        with contextlib.redirect_stdout(io.StringIO()):
            res = ref.fastVEC(sobj, dobj, dreso=g)
        out[f"c{i}_src"] = src
        out[f"c{i}_params"] = np.array([sw, *so, dd, dw, *do, g], np.float64)
        out[f"c{i}_data"] = res.data
        out[f"c{i}_vec"] = res.vec
    np.savez_compressed(os.path.join(HERE, "fastvec_noncubic.npz"), **out)


def _patch_fastvec_with_oracle():
    """doFastVEC -> the C restatement, same arguments and outputs."""

    def do_fast_vec(src_xwidth, src_orig, src_dims, src_data, dest_xwidth, dest_orig, dest_dims, dest_data,
                    dest_vec, dreso=16.0):
        data, vec = orc.fastvec(src_data, src_xwidth, src_orig, int(dest_dims[0]), dest_xwidth, dest_orig, dreso)
        dest_data[...] = data.astype(dest_data.dtype)
        dest_vec[...] = vec
        return dest_data, dest_vec

    ref.doFastVEC = do_fast_vec


def prepare_orig_pair(pair, t, T, g, s):
    """main.py:158-191 with the reference's own functions."""
    mrc1 = refshim.make_mrc_obj(ref, pair.map1, pair.width, pair.orig1)
    mrc2 = refshim.make_mrc_obj(ref, pair.map2, pair.width, pair.orig2)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        mrc1, n1 = ref.mrc_set_vox_size(mrc1, t, s)
        mrc2, n2 = ref.mrc_set_vox_size(mrc2, T, s)
        if n1.xdim > n2.xdim:
            dim = n2.xdim = n2.ydim = n2.zdim = n1.xdim
            n2.orig[0] = n2.cent[0] - 0.5 * s * n2.xdim
            n2.orig[1] = n2.cent[1] - 0.5 * s * n2.xdim
            n2.orig[2] = n2.cent[2] - 0.5 * s * n2.xdim
        else:
            dim = n1.xdim = n1.ydim = n1.zdim = n2.xdim
            n1.orig[0] = n1.cent[0] - 0.5 * s * n1.xdim
            n1.orig[1] = n1.cent[1] - 0.5 * s * n1.xdim
            n1.orig[2] = n1.cent[2] - 0.5 * s * n1.xdim
        for n in (n1, n2):
            n.dens = np.zeros((dim ** 3, 1))
            n.vec = np.zeros((dim, dim, dim, 3), dtype="float32")
            n.data = np.zeros((dim, dim, dim))
        print()
        n1 = ref.fastVEC(mrc1, n1, g)
        n2 = ref.fastVEC(mrc2, n2, g)
        print()
    return n1, n2, buf.getvalue()


def gen_search_pair128():
    _patch_fastvec_with_oracle()
    w = synth.WORKLOADS["pair128_s7_a30"]
    pair = synth.workload_pair("pair128_s7_a30", seed=0)
    n1, n2, setup_out = prepare_orig_pair(pair, w["t"], w["T"], w["g"], w["s"])
    out = {
        "dim": n1.xdim, "orig1": n1.orig, "orig2": n2.orig, "cent1": n1.cent, "cent2": n2.cent,
        "data1": n1.data, "vec1": n1.vec, "data2": n2.data, "vec2": n2.vec,
        "stats1": np.array([n1.dsum, n1.Nact, n1.ave, n1.std, n1.std_norm_ave], np.float64),
        "stats2": np.array([n2.dsum, n2.Nact, n2.ave, n2.std, n2.std_norm_ave], np.float64),
    }
    with open(os.path.join(HERE, "search_pair128_setup.txt"), "w") as f:
        f.write(setup_out)
    real_ras = ref.rot_and_search_fft
    for mode_letter, mode in orc.MODES.items():
        rec = []

        def recording(data, vec, angle, target_list, mrc_target, mode="VecProduct"):
            r = real_ras(data, vec, angle, target_list, mrc_target, mode=mode)
            rec.append((np.array(angle, np.float64), r[0], tuple(int(t) for t in r[1])))
            return r

        ref.rot_and_search_fft = recording
        buf = io.StringIO()
        with contextlib.redirect_stdout(buf), contextlib.redirect_stderr(io.StringIO()):
            refined = ref.search_map_fft(n1, n2, TopN=w["N"], ang=w["A"], mode=mode)
        ref.rot_and_search_fft = real_ras
        out[f"{mode_letter}_angles"] = np.array([r[0] for r in rec])
        out[f"{mode_letter}_score"] = np.array([r[1] for r in rec], np.float64)
        out[f"{mode_letter}_trans"] = np.array([r[2] for r in rec], np.int64)
        out[f"{mode_letter}_refined_angle"] = np.array([r["angle"] for r in refined], np.float64)
        out[f"{mode_letter}_refined_score"] = np.array([r["vec_score"] for r in refined], np.float64)
        out[f"{mode_letter}_refined_trans"] = np.array([r["vec_trans"] for r in refined], np.int64)
        with open(os.path.join(HERE, f"search_pair128_{mode_letter}.txt"), "w") as f:
            f.write(buf.getvalue())
    np.savez_compressed(os.path.join(HERE, "search_pair128.npz"), **out)


def gen_prob_pair():
    """Prob mode on the seed-0 128^3 pair with four channels, s=7, A=30."""
    _patch_fastvec_with_oracle()
    t = T = 0.1
    g, s, A, N, alpha = 16.0, 7.0, 30.0, 10, 0.5
    pair = synth.make_pair(0, 128, 400, 40.0, with_prob=True, threshold=t)
    mk = lambda d, o: refshim.make_mrc_obj(ref, d, pair.width, o)  # noqa: E731
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        mrc1, mrc2 = mk(pair.map1, pair.orig1), mk(pair.map2, pair.orig2)
        p1 = [mk(pair.prob1[..., c], pair.orig1) for c in range(4)]
        p2 = [mk(pair.prob2[..., c], pair.orig2) for c in range(4)]
        mrc1, n1 = ref.mrc_set_vox_size(mrc1, t, s)
        mrc2, n2 = ref.mrc_set_vox_size(mrc2, T, s)
        np1 = [ref.mrc_set_vox_size(p, th=0.0, voxel_size=s)[1] for p in p1]
        np2 = [ref.mrc_set_vox_size(p, th=0.0, voxel_size=s)[1] for p in p2]
        lst = [n1, n2] + np1 + np2
        md = np.max([m.xdim for m in lst])
        for m in lst:
            if m.xdim != md:
                m.xdim = m.ydim = m.zdim = md
                m.orig = m.cent - 0.5 * s * m.xdim
        for m in lst:
            m.dens = np.zeros((md ** 3, 1), dtype="float32")
            m.data = np.zeros((md, md, md), dtype="float32")
            m.vec = np.zeros((md, md, md, 3), dtype="float32")
        n1 = ref.fastVEC(mrc1, n1, dreso=g)
        np1 = [ref.fastVEC(p, q, dreso=g) for p, q in zip(p1, np1)]
        n2 = ref.fastVEC(mrc2, n2, dreso=g)
        np2 = [ref.fastVEC(p, q, dreso=g) for p, q in zip(p2, np2)]
    setup = buf.getvalue()
    out = {"dim": md, "data1": n1.data, "vec1": n1.vec, "data2": n2.data, "vec2": n2.vec,
           "probs1": np.stack([p.data for p in np1]), "probs2": np.stack([p.data for p in np2]),
           "cent1": n1.cent, "cent2": n2.cent}
    rec = []
    real = ref.rot_and_search_fft_prob

    def recording(*a, **k):
        r = real(*a, **k)
        rec.append((np.array(a[6], np.float64), r[0], r[1], r[2], r[3], r[4], r[5]))
        return r

    ref.rot_and_search_fft_prob = recording
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf), contextlib.redirect_stderr(io.StringIO()):
        refined = ref.search_map_fft_prob(np1[0], np1[1], np1[2], np1[3], n1, n2, np2[0], np2[1], np2[2], np2[3],
                                          ang=A, alpha=alpha, TopN=N)
    ref.rot_and_search_fft_prob = real
    R = len(ref.calc_angle_comb(A))
    p1rec, p2rec = rec[:R], rec[R:]
    out["pass1_vscore"] = np.array([r[1] for r in p1rec], np.float64)
    out["pass1_vtrans"] = np.array([r[2] for r in p1rec], np.int64)
    out["pass1_pscore"] = np.array([r[3] for r in p1rec], np.float64)
    out["pass1_ptrans"] = np.array([r[4] for r in p1rec], np.int64)
    out["pass2_mscore"] = np.array([r[5] for r in p2rec], np.float64)
    out["pass2_mtrans"] = np.array([r[6] for r in p2rec], np.int64)
    out["refined_angle"] = np.array([r["angle"] for r in refined], np.float64)
    out["refined_mixed"] = np.array([r["mixed_score"] for r in refined], np.float64)
    out["refined_mtrans"] = np.array([r["mixed_trans"] for r in refined], np.int64)
    out["refined_vtrans"] = np.array([r["vec_trans"] for r in refined], np.int64)
    np.savez_compressed(os.path.join(HERE, "prob_pair128.npz"), **out)
    with open(os.path.join(HERE, "prob_pair128.txt"), "w") as f:
        f.write(setup + buf.getvalue())


def gen_voxsize():
    """mrc_set_vox_size (VESPER_1_prob_new.py:59-118) on small random maps with
    negative values: thresholds 0, 0.25 and -0.3 (the shift path), voxel
    sizes 2 and 5, non-cubic maps and non-zero origins; the thresholded data,
    dens, the new grid (xdim, orig, cent) and the printed lines."""
    rng = np.random.default_rng(77)
    out = {}
    k = 0
    for si, (shape, orig, width) in enumerate((((24, 28, 20), (1.5, -2.0, 0.25), 1.0),
                                               ((31, 31, 31), (0.0, 0.0, 0.0), 1.5))):
        base = (rng.normal(size=shape) * 0.4).astype(np.float32)
        out[f"src{si}"] = base
        for th in (0.0, 0.25, -0.3):
            for vs in (2.0, 5.0):
                m = refshim.make_mrc_obj(ref, base, width, orig)
                buf = io.StringIO()
                with contextlib.redirect_stdout(buf):
                    m, n = ref.mrc_set_vox_size(m, th, vs)
                out[f"c{k}_params"] = np.array([si, width, *orig, th, vs], np.float64)
                # thresholded data and dens as digests of their bytes (float32 / float64)
                out[f"c{k}_digest"] = np.array([digest(np.asarray(m.data, np.float32)),
                                                digest(np.asarray(m.dens, np.float64).reshape(-1))])
                out[f"c{k}_grid"] = np.array([n.xdim, *n.orig, *n.cent], np.float64)
                out[f"c{k}_print"] = np.array(buf.getvalue())
                k += 1
    out["ncase"] = np.array(k)
    np.savez_compressed(os.path.join(HERE, "voxsize_cases.npz"), **out)


def gen_show_vec():
    """show_vec (VESPER_1_prob_new.py:1144-1208): the PDB files the reference
    writes for two small models (translations wrapping past d/2 and negative
    scores included), stored as text."""
    import tempfile
    from pathlib import Path
    rng = np.random.default_rng(91)
    out = {}
    for k, (d, trans, score, rank) in enumerate(((5, (4, 1, 0), 12.3456, 3), (7, (0, 6, 3), -3.25, 11))):
        data = np.where(rng.random((d, d, d)) < 0.35, rng.uniform(0.5, 2, (d, d, d)), 0.0)
        vec = rng.normal(size=(d, d, d, 3)).astype(np.float32)
        sco = rng.normal(size=(d, d, d))
        origin = rng.uniform(-20, 20, size=3)
        with tempfile.TemporaryDirectory() as tmp:
            with contextlib.redirect_stdout(io.StringIO()):
                ref.show_vec(origin, vec, data, sco, score, 7.0, trans, (0, 0, 0), Path(tmp), rank)
            names = sorted(os.listdir(tmp))
            assert len(names) == 1
            out[f"c{k}_name"] = np.array(names[0])
            with open(os.path.join(tmp, names[0])) as f:
                out[f"c{k}_text"] = np.array(f.read())
        out[f"c{k}_data"], out[f"c{k}_vec"], out[f"c{k}_sco"] = data, vec, sco
        out[f"c{k}_params"] = np.array([*origin, *trans, score, rank], np.float64)
    np.savez_compressed(os.path.join(HERE, "show_vec_cases.npz"), **out)


if __name__ == "__main__":
    which = sys.argv[1:] or ["angles", "rot", "fastvec", "search", "prob", "voxsize", "showvec", "noncubic"]
    if "angles" in which:
        gen_angles()
    if "rot" in which:
        gen_rot_small()
    if "fastvec" in which:
        gen_fastvec_small()
    if "search" in which:
        gen_search_pair128()
    if "prob" in which:
        gen_prob_pair()
    if "voxsize" in which:
        gen_voxsize()
    if "showvec" in which:
        gen_show_vec()
    if "noncubic" in which:
        gen_fastvec_noncubic()
