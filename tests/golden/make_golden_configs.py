"""Golden vectors at the benchmarked configurations, made by running the
UNMODIFIED reference module (imported under stand-in modules, refshim.py) over
the FULL angle grid of each configuration.

    VESPER_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden_configs.py [jobs...]

Jobs (each runs in its own spawned process; the slowest, pair200 mode L,
takes about 1.6 h on one core):

  pair200:<mode>   the seed-0 200^3 / 100^3 pair at s = 2, A = 10, grid side
                   75, mode V/O/C/P/L: search_map_fft over all 24,624
                   rotations, its refinement and its printed output
  prob64           the seed-0 128^3 / 64^3 pair with four probability
                   channels, s = 3, every grid padded to 64^3, A = 15,
                   alpha = 0.5: search_map_fft_prob over all 7,488 rotations
                   (statistics pass and mixed pass), refinement, output
  uneven           one pair of the uneven 64-pair batch for every grid side
                   the batch produces (11 ... 44), s = 4, A = 15, mode V:
                   search_map_fft over all 7,488 rotations, refinement, output

Outputs (committed): search_pair200.npz + search_pair200_<mode>.txt,
prob_pair128_pad64.npz + .txt, uneven_sides.npz.  Coarse fields are stored
sparse (flat indices of the non-zero voxels and their values), since most
voxels of a thresholded blob map are zero.

Stand-in environment (beyond refshim): the coarse fields come from the C
restatement of doFastVEC (pinned by fastvec_small.npz; the pure-Python loop is
far too slow at these sizes).  Two numpy 2 (NEP 50) promotions are set back to
those of numpy 1.21, the reference's pinned version, at the call boundaries
only (every reference function runs unmodified): the per-rotation scores the
searches return reach their caller as np.float64, so ``score * rd3`` and the
prob statistics are float64; and find_best_trans_mixed receives its
statistics as Python floats, so the z-scores of the float32 volumes are
float32 arithmetic.
"""
from __future__ import annotations

import contextlib
import io
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PARTS = os.environ.get("VESPER_GOLDEN_PARTS", "/tmp/vesper_golden_parts")

PAIR200_MODES = ("V", "O", "C", "P", "L")
MODE_NAMES = {"V": "VecProduct", "O": "Overlap", "C": "CC", "P": "PCC", "L": "Laplacian"}


def _setup():
    for p in (ROOT, HERE):
        if p not in sys.path:
            sys.path.insert(0, p)
    import make_golden as mg   # imports the reference under the stand-ins
    mg._patch_fastvec_with_oracle()
    return mg


def sparse(prefix, arr):
    """{prefix_idx, prefix_val}: flat indices of the non-zero voxels (over the
    first three axes) and their values."""
    a = np.asarray(arr)
    mask = np.any(a.reshape(a.shape[:3] + (-1,)) != 0, axis=3)
    idx = np.flatnonzero(mask).astype(np.int32)
    return {f"{prefix}_idx": idx, f"{prefix}_val": a.reshape((-1,) + a.shape[3:])[idx],
            f"{prefix}_shape": np.array(a.shape, np.int64)}


def dense(g, prefix):
    """Inverse of sparse()."""
    shape = tuple(int(v) for v in g[f"{prefix}_shape"])
    val = g[f"{prefix}_val"]
    out = np.zeros((int(np.prod(shape[:3])),) + shape[3:], val.dtype)
    out[g[f"{prefix}_idx"]] = val
    return out.reshape(shape)


def _record_search(mg, n1, n2, mode_letter, A, N):
    """search_map_fft with every rot_and_search_fft call recorded."""
    ref = mg.ref
    real = ref.rot_and_search_fft
    rec = []

    def recording(data, vec, angle, target_list, mrc_target, mode="VecProduct"):
        r = real(data, vec, angle, target_list, mrc_target, mode=mode)
        rec.append((np.array(angle, np.float64), float(r[0]), tuple(int(t) for t in r[1])))
        # numpy 1.21 promotes np.float32 * Python float (the caller's
        # ``vec_score * rd3``) to float64; numpy 2 keeps float32
        return (np.float64(r[0]),) + tuple(r[1:])

    ref.rot_and_search_fft = recording
    buf = io.StringIO()
    try:
        with contextlib.redirect_stdout(buf), contextlib.redirect_stderr(io.StringIO()):
            refined = ref.search_map_fft(n1, n2, TopN=N, ang=A, mode=MODE_NAMES[mode_letter])
    finally:
        ref.rot_and_search_fft = real
    R = len(ref.calc_angle_comb(A))
    glob, refine = rec[:R], rec[R:]
    out = {
        "score": np.array([r[1] for r in glob], np.float64),
        "trans": np.array([r[2] for r in glob], np.int16),
        "refine_angles": np.array([r[0] for r in refine], np.float64).reshape(-1, 3),
        "refine_score": np.array([r[1] for r in refine], np.float64),
        "refine_trans": np.array([r[2] for r in refine], np.int16).reshape(-1, 3),
        "refined_angle": np.array([r["angle"] for r in refined], np.float64),
        "refined_score": np.array([r["vec_score"] for r in refined], np.float64),
        "refined_trans": np.array([r["vec_trans"] for r in refined], np.int64),
        "stdout": np.array(buf.getvalue()),
    }
    assert np.array_equal(np.array([r[0] for r in glob]), ref.calc_angle_comb(A))
    return out


def _fields(n1, n2):
    out = {"dim": np.array(n1.xdim), "orig1": n1.orig, "orig2": n2.orig, "cent1": n1.cent, "cent2": n2.cent,
           "stats1": np.array([n1.dsum, n1.Nact, n1.ave, n1.std, n1.std_norm_ave], np.float64),
           "stats2": np.array([n2.dsum, n2.Nact, n2.ave, n2.std, n2.std_norm_ave], np.float64),
           "xwidth2": np.array(n2.xwidth, np.float64)}
    out.update(sparse("data1", n1.data))
    out.update(sparse("vec1", n1.vec))
    out.update(sparse("data2", n2.data))
    out.update(sparse("vec2", n2.vec))
    return out


def job_pair200(mode_letter):
    mg = _setup()
    from vesper_python_gb300 import synth
    w = synth.WORKLOADS["pair200_s2_a10"]
    pair = synth.workload_pair("pair200_s2_a10", seed=0)
    n1, n2, setup_out = mg.prepare_orig_pair(pair, w["t"], w["T"], w["g"], w["s"])
    out = {f"{mode_letter}_{k}": v for k, v in _record_search(mg, n1, n2, mode_letter, w["A"], w["N"]).items()}
    if mode_letter == "V":
        out.update(_fields(n1, n2))
        out["setup"] = np.array(setup_out)
    return out


def job_prob64():
    mg = _setup()
    ref = mg.ref
    from vesper_python_gb300 import synth
    w = synth.WORKLOADS["prob128_s3_a15"]
    t, T, g, s, A, N, alpha, pad = w["t"], w["T"], w["g"], w["s"], w["A"], w["N"], w["alpha"], int(w["pad"])
    pair = synth.workload_pair("prob128_s3_a15", seed=0)
    mk = lambda d, o: mg.refshim.make_mrc_obj(ref, d, pair.width, o)  # noqa: E731
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
        assert max(m.xdim for m in lst) <= pad
        # every grid padded to pad^3 about its centre (main.py:317-327's rule
        # for the smaller grids, applied to all)
        for m in lst:
            m.xdim = m.ydim = m.zdim = pad
            m.orig = m.cent - 0.5 * s * m.xdim
            m.dens = np.zeros((pad ** 3, 1), dtype="float32")
            m.data = np.zeros((pad, pad, pad), dtype="float32")
            m.vec = np.zeros((pad, pad, pad, 3), dtype="float32")
        n1 = ref.fastVEC(mrc1, n1, dreso=g)
        np1 = [ref.fastVEC(p, q, dreso=g) for p, q in zip(p1, np1)]
        n2 = ref.fastVEC(mrc2, n2, dreso=g)
        np2 = [ref.fastVEC(p, q, dreso=g) for p, q in zip(p2, np2)]
    setup = buf.getvalue()
    out = {"dim": np.array(pad), "cent1": n1.cent, "cent2": n2.cent, "xwidth2": np.array(n2.xwidth, np.float64),
           "setup": np.array(setup)}
    out.update(sparse("data1", n1.data))
    out.update(sparse("vec1", n1.vec))
    out.update(sparse("data2", n2.data))
    out.update(sparse("vec2", n2.vec))
    out.update(sparse("probs1", np.stack([p.data for p in np1], axis=-1)))
    out.update(sparse("probs2", np.stack([p.data for p in np2], axis=-1)))
    rec, mixed_rec, rot_rec = [], [], []
    real = ref.rot_and_search_fft_prob
    real_mixed = ref.find_best_trans_mixed
    real_rot = ref.rot_mrc_prob

    def recording(*a, **k):
        r = real(*a, **k)
        rec.append((float(r[0]), r[1], float(r[2]), r[3], None if r[4] is None else float(r[4]), r[5]))
        # numpy 1.21 promotion of the caller's ``score * rd3`` (float64)
        return (np.float64(r[0]), r[1], np.float64(r[2]), r[3], None if r[4] is None else np.float64(r[4]), r[5])

    def mixed_numpy1(v, p, alpha_, vstd, vave, pstd, pave):
        # the statistics as Python floats (float32 z-scores, numpy 1.21's
        # value-based casting), the best score handed back as float64
        best, trans = real_mixed(v, p, float(alpha_), float(vstd), float(vave), float(pstd), float(pave))
        mixed_rec.append((float(best), tuple(int(t) for t in trans)))
        return np.float64(best), trans

    def rot_recording(*a, **k):
        rot_rec.append(np.array(a[6], np.float64))
        return real_rot(*a, **k)

    ref.rot_and_search_fft_prob = recording
    ref.find_best_trans_mixed = mixed_numpy1
    ref.rot_mrc_prob = rot_recording
    buf = io.StringIO()
    try:
        with contextlib.redirect_stdout(buf), contextlib.redirect_stderr(io.StringIO()):
            refined = ref.search_map_fft_prob(np1[0], np1[1], np1[2], np1[3], n1, n2, np2[0], np2[1], np2[2],
                                              np2[3], ang=A, alpha=alpha, TopN=N)
    finally:
        ref.rot_and_search_fft_prob = real
        ref.find_best_trans_mixed = real_mixed
        ref.rot_mrc_prob = real_rot
    R = len(ref.calc_angle_comb(A))
    # the refinement loop runs its searches inline (not through
    # rot_and_search_fft_prob): its calls are the last ones of the gather and
    # of the mixed-score function
    p1rec, p2rec = rec[:R], rec[R:2 * R]
    refrec = [(None, None, None, None, m, t) for (m, t) in mixed_rec[R:]]
    out["refine_angles"] = np.array(rot_rec[2 * R:], np.float64).reshape(-1, 3)
    assert len(refrec) == len(out["refine_angles"])
    out["pass1_vscore"] = np.array([r[0] for r in p1rec], np.float64)
    out["pass1_vtrans"] = np.array([r[1] for r in p1rec], np.int16)
    out["pass1_pscore"] = np.array([r[2] for r in p1rec], np.float64)
    out["pass1_ptrans"] = np.array([r[3] for r in p1rec], np.int16)
    out["pass2_mscore"] = np.array([r[4] for r in p2rec], np.float64)
    out["pass2_mtrans"] = np.array([r[5] for r in p2rec], np.int16)
    out["refine_mscore"] = np.array([r[4] for r in refrec], np.float64)
    out["refine_mtrans"] = np.array([r[5] for r in refrec], np.int16).reshape(-1, 3)
    out["refined_angle"] = np.array([r["angle"] for r in refined], np.float64)
    out["refined_mixed"] = np.array([r["mixed_score"] for r in refined], np.float64)
    out["refined_mtrans"] = np.array([r["mixed_trans"] for r in refined], np.int64)
    out["refined_vtrans"] = np.array([r["vec_trans"] for r in refined], np.int64)
    out["stdout"] = np.array(buf.getvalue())
    return out


def uneven_side_pairs():
    """{grid side: first pair index of the uneven batch with that side}."""
    from oracle import vesper_oracle as orc
    from vesper_python_gb300 import synth
    w = synth.UNEVEN_WORKLOAD
    first = {}
    for i in range(w["pairs"]):
        p = synth.uneven_pair(i)
        m1, m2 = orc.OMap(p.map1, 1.0, p.orig1), orc.OMap(p.map2, 1.0, p.orig2)
        d1, o1, c1, _ = orc.set_vox_size(m1, w["t"], w["s"])
        d2, o2, c2, _ = orc.set_vox_size(m2, w["T"], w["s"])
        dim = orc.unify(d1, o1, c1, d2, o2, c2, w["s"])[0]
        first.setdefault(int(dim), i)
    return dict(sorted(first.items()))


def job_uneven(sides):
    mg = _setup()
    from vesper_python_gb300 import synth
    w = synth.UNEVEN_WORKLOAD
    first = uneven_side_pairs()
    out = {}
    for d in sides:
        i = first[d]
        pair = synth.uneven_pair(i)
        n1, n2, setup_out = mg.prepare_orig_pair(pair, w["t"], w["T"], w["g"], w["s"])
        assert n1.xdim == d
        rec = _record_search(mg, n1, n2, "V", w["A"], w["N"])
        f = _fields(n1, n2)
        f["pair_index"] = np.array(i)
        f["setup"] = np.array(setup_out)
        f.update(rec)
        out.update({f"d{d}_{k}": v for k, v in f.items()})
    return out


def _run(job):
    t0 = time.time()
    kind, _, arg = job.partition(":")
    if kind == "pair200":
        out = job_pair200(arg)
    elif kind == "prob64":
        out = job_prob64()
    elif kind == "uneven":
        out = job_uneven([int(v) for v in arg.split(",")])
    else:
        raise ValueError(job)
    os.makedirs(PARTS, exist_ok=True)
    np.savez(os.path.join(PARTS, job.replace(":", "_").replace(",", "-") + ".npz"), **out)
    return job, time.time() - t0


def _compact(z):
    """float64 arrays whose values are all float32 numbers (raw float32
    scores) stored as float32."""
    out = {}
    for k, v in z.items():
        if isinstance(v, np.ndarray) and v.dtype == np.float64 and v.size > 64 and \
                np.array_equal(v.astype(np.float32).astype(np.float64), v):
            v = v.astype(np.float32)
        out[k] = v
    return out


def combine():
    import glob
    parts = sorted(glob.glob(os.path.join(PARTS, "*.npz")))
    p200 = {}
    unev = {}
    for p in parts:
        name = os.path.basename(p)
        z = _compact(dict(np.load(p)))
        if name.startswith("pair200_"):
            p200.update(z)
        elif name.startswith("uneven_"):
            unev.update(z)
        elif name.startswith("prob64"):
            txt = str(z.pop("setup")) + str(z["stdout"])
            np.savez_compressed(os.path.join(HERE, "prob_pair128_pad64.npz"), **z)
            with open(os.path.join(HERE, "prob_pair128_pad64.txt"), "w") as f:
                f.write(txt)
    if p200:
        # jobs run separately add their modes to those already in the fixture
        old = os.path.join(HERE, "search_pair200.npz")
        if os.path.exists(old):
            p200 = dict(np.load(old), **p200)
        for m in PAIR200_MODES:
            if f"{m}_stdout" in p200:
                with open(os.path.join(HERE, f"search_pair200_{m}.txt"), "w") as f:
                    f.write(str(p200[f"{m}_stdout"]))
        np.savez_compressed(os.path.join(HERE, "search_pair200.npz"), **p200)
    if unev:
        sides = sorted({int(k[1:].split("_")[0]) for k in unev})
        unev["sides"] = np.array(sides)
        np.savez_compressed(os.path.join(HERE, "uneven_sides.npz"), **unev)


DEFAULT_JOBS = [f"pair200:{m}" for m in PAIR200_MODES] + ["prob64", "uneven:11,12,13,16,18,21,22,24,27",
                                                          "uneven:28,30,32,33,35,44"]

if __name__ == "__main__":
    args = sys.argv[1:]
    if args == ["combine"]:
        combine()
        sys.exit(0)
    jobs = args or DEFAULT_JOBS
    ctx = mp.get_context("spawn")
    with ctx.Pool(len(jobs)) as pool:
        for job, secs in pool.imap_unordered(_run, jobs):
            print(f"{job}: {secs:.0f} s", flush=True)
    combine()
