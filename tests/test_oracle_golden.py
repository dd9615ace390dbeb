"""The CPU oracle against the golden vectors recorded from the unmodified
reference (tests/golden/make_golden.py, make_golden_configs.py and
make_golden_interp.py).  No GPU needed."""
import hashlib
import os

import numpy as np
import pytest

from oracle import vesper_oracle as orc


def _g(golden_dir, name):
    return np.load(os.path.join(golden_dir, name))


def digest(*arrays):
    h = hashlib.sha1()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_angle_grids(golden_dir):
    g = _g(golden_dir, "angles.npz")
    for key in g.files:
        a = float(key[1:])
        assert np.array_equal(orc.calc_angle_comb(a), g[key]), key
    # row order: z slowest, x middle, y fastest
    ac = g["A30"]
    assert tuple(ac[1]) == (0, 30, 0) and tuple(ac[12]) == (30, 0, 0) and tuple(ac[144]) == (0, 0, 30)
    assert len(g["A10"]) == 24624 and len(g["A15"]) == 7488 and len(ac) == 1008


@pytest.mark.parametrize("d", [8, 9, 12, 15])
def test_rot_mrc_all_rotations(golden_dir, d):
    g = _g(golden_dir, "rot_small.npz")
    data, vec = g[f"d{d}_data"], g[f"d{d}_vec"]
    ang = orc.calc_angle_comb(30.0)
    dig = g[f"d{d}_digest"]
    bad = [r for r, a in enumerate(ang) if digest(*orc.rot_mrc(data, vec, a)) != dig[r]]
    assert not bad
    for r in (0, 1, 13, 144, 500, 1007):
        nv, nd = orc.rot_mrc(data, vec, ang[r])
        assert np.array_equal(nv, g[f"d{d}_r{r}_vec"]) and np.array_equal(nd, g[f"d{d}_r{r}_data"])


def test_rot_mrc_fine_and_refinement_angles(golden_dir):
    g = _g(golden_dir, "rot_small.npz")
    for d in (12, 15):
        data, vec = g[f"d{d}_data"], g[f"d{d}_vec"]
        for a, dg in zip(g["angles10_sub"], g[f"d{d}_a10_digest"]):
            assert digest(*orc.rot_mrc(data, vec, a)) == dg
        for a, dg in zip(g["extra_angles"], g[f"d{d}_extra_digest"]):
            assert digest(*orc.rot_mrc(data, vec, a)) == dg


@pytest.mark.parametrize("d", [9, 12])
def test_rot_mrc_prob(golden_dir, d):
    g = _g(golden_dir, "rot_small.npz")
    data, vec, probs = g[f"p{d}_data"], g[f"p{d}_vec"], g[f"p{d}_probs"]
    ang = orc.calc_angle_comb(30.0)[::11]
    for a, dg in zip(ang, g[f"p{d}_digest"]):
        assert digest(*orc.rot_mrc_prob(data, vec, *probs, a)) == dg


@pytest.mark.parametrize("d", [9, 12])
def test_rot_mrc_numpy_form_matches_reference(golden_dir, d):
    """The whole-array numpy gather timed by the CPU baseline gives the
    reference's outputs (digests over every rotation of the 30-degree grid,
    odd side included; prob channels with their own masks)."""
    g = _g(golden_dir, "rot_small.npz")
    data, vec = g[f"d{d}_data"], g[f"d{d}_vec"]
    ang = orc.calc_angle_comb(30.0)
    dig = g[f"d{d}_digest"]
    bad = [r for r, a in enumerate(ang) if digest(*orc.rot_mrc_numpy(data, vec, orc.rot_matrix_f32(a))) != dig[r]]
    assert not bad
    data, vec, probs = g[f"p{d}_data"], g[f"p{d}_vec"], g[f"p{d}_probs"]
    for a, dg in zip(ang[::11], g[f"p{d}_digest"]):
        nv, nd, ps = orc.rot_mrc_numpy(data, vec, orc.rot_matrix_f32(a), list(probs))
        assert digest(nv, nd, *ps) == dg


def test_odd_side_collision_rule():
    """Odd d: destination index (d-1)/2 takes the later of two source rows and
    the last plane stays empty (identity rotation)."""
    d = 15
    data = np.arange(1, d ** 3 + 1, dtype=np.float64).reshape(d, d, d)
    vec = np.ones((d, d, d, 3), np.float32)
    _, nd = orc.rot_mrc(data, vec, (0.0, 0.0, 0.0))
    assert np.all(nd[14] == 0) and np.all(nd[:, 14] == 0) and np.all(nd[:, :, 14] == 0)
    assert nd[7, 7, 7] == data[8, 8, 8]
    assert nd[3, 3, 3] == data[3, 3, 3] and nd[10, 10, 10] == data[11, 11, 11]


def test_fastvec_c_restatement(golden_dir):
    """C restatement of doFastVEC vs the pure-Python reference loop: data within
    2 ulp-scale (numpy vs libm exp), vectors identical."""
    g = _g(golden_dir, "fastvec_small.npz")
    for i in range(3):
        S, sw, so0, so1, so2, dd, dw, do0, do1, do2, gg = g[f"c{i}_params"]
        data, vec = orc.fastvec(g[f"c{i}_src"], sw, np.float32([so0, so1, so2]), int(dd), dw, [do0, do1, do2], gg)
        rd = g[f"c{i}_data"]
        assert np.array_equal(data != 0, rd != 0)
        assert np.max(np.abs(data - rd) / np.maximum(np.abs(rd), 1e-300)) < 1e-15
        assert np.array_equal(vec, g[f"c{i}_vec"])
        st = np.array(orc.fastvec_stats(data), np.float64)
        assert np.allclose(st, g[f"c{i}_stats"], rtol=1e-14)


@pytest.mark.parametrize("mode", ["V", "O", "C", "P", "L"])
def test_search_per_rotation_bit_exact(golden_dir, mode):
    g = _g(golden_dir, "search_pair128.npz")
    s1 = g["stats1"]
    ts = orc.target_spectra(orc.mode_field(mode, g["data1"], g["vec1"], s1[2]))
    ang = g[f"{mode}_angles"]
    sc, tr = orc.search(ts, mode, g["data2"], g["vec2"], ang, s1[2])
    scale = orc.score_scale(mode, s1[3], s1[4])
    assert np.array_equal(sc.astype(np.float64) * scale, g[f"{mode}_score"])
    assert np.array_equal(tr, g[f"{mode}_trans"])
    R = len(orc.calc_angle_comb(30.0))
    top = orc.topn(sc[:R], 10)
    assert np.array_equal(orc.refine_angles(ang[top]), ang[R:])
    rtop = orc.topn(sc[R:], 10)
    assert np.array_equal(ang[R:][rtop], g[f"{mode}_refined_angle"])
    assert np.array_equal(tr[R:][rtop], g[f"{mode}_refined_trans"])


def test_set_vox_size_matches_reference_prints(golden_dir):
    from vesper_python_gb300 import synth
    g = _g(golden_dir, "search_pair128.npz")
    pair = synth.workload_pair("pair128_s7_a30", seed=0)
    m1 = orc.OMap(pair.map1, 1.0, pair.orig1)
    m2 = orc.OMap(pair.map2, 1.0, pair.orig2)
    d1, o1, c1, _ = orc.set_vox_size(m1, 0.1, 7.0)
    d2, o2, c2, _ = orc.set_vox_size(m2, 0.1, 7.0)
    dim, o1, o2 = orc.unify(d1, o1, c1, d2, o2, c2, 7.0)
    assert dim == int(g["dim"])
    assert np.array_equal(o1, g["orig1"]) and np.array_equal(o2, g["orig2"])
    data1, vec1 = orc.fastvec(m1.data, np.float64(m1.xwidth), m1.orig.astype(np.float64), dim, 7.0, o1, 16.0)
    assert np.array_equal(data1, g["data1"]) and np.array_equal(vec1, g["vec1"])
    txt = open(os.path.join(golden_dir, "search_pair128_setup.txt")).read()
    assert "Nvox= 12, 12, 12" in txt and "Nvox= 13, 13, 13" in txt


def test_prob_passes(golden_dir):
    g = _g(golden_dir, "prob_pair128.npz")
    d = int(g["dim"])
    tspec = orc.target_spectra([g["vec1"][..., 0], g["vec1"][..., 1], g["vec1"][..., 2]] + list(g["probs1"]))
    ang = orc.calc_angle_comb(30.0)[::9]
    idx = np.arange(0, 1008, 9)
    for a, r in zip(ang, idx):
        vs, vt, ps, pt, _, _ = orc.rot_and_search_prob(tspec, g["data2"], g["vec2"], g["probs2"], a, 0.5)
        assert np.float64(vs) == g["pass1_vscore"][r] and tuple(vt) == tuple(g["pass1_vtrans"][r])
        assert np.float64(ps) == g["pass1_pscore"][r] and tuple(pt) == tuple(g["pass1_ptrans"][r])
    st = orc.prob_stats(g["pass1_vscore"], g["pass1_pscore"], 1.0 / d ** 3)
    for a, r in zip(ang, idx):
        res = orc.rot_and_search_prob(tspec, g["data2"], g["vec2"], g["probs2"], a, 0.5, st, promotion="numpy2")
        assert np.float64(res[4]) == g["pass2_mscore"][r] and tuple(res[5]) == tuple(g["pass2_mtrans"][r])
    txt = open(os.path.join(golden_dir, "prob_pair128.txt")).read()
    assert f"DotScore Std= {float(st[0])!r} DotScore Ave= {float(st[1])!r}" in txt


def test_next_fast_len():
    assert [orc.next_fast_len(n) for n in (1, 2, 11, 13, 17, 19, 23, 29, 37, 74, 97, 143, 169)] == \
        [1, 2, 11, 13, 18, 20, 24, 30, 39, 75, 98, 144, 175]
    # 11*13 and 13*13 need e+f = 2 -> skipped
    assert orc.next_fast_len(143) == 144


def test_interpolate_oracle_matches_golden(golden_dir):
    """The oracle's probability-map hole filling against the reference
    function's outputs (interpolation_functions.py:6-135), bit for bit."""
    g = np.load(os.path.join(golden_dir, "interp_small.npz"))
    for n in range(4):
        a = g[f"in{n}"].copy()
        orc.interpolate(a)
        np.testing.assert_array_equal(a, g[f"out{n}"])


@pytest.mark.parametrize("mode", ["V", "O", "C", "P", "L"])
def test_get_score_matches_reference_prints(golden_dir, mode):
    """The oracle's get_score (the checker of the GPU rescoring) against the
    reference's own printed get_score lines of every refined model of the
    128^3/64^3 seed-0 pair (search_pair128_<mode>.txt, recorded by
    make_golden.py from the reference's search_map_fft): Overlap, Nm/total,
    CC, PCC and Score."""
    import re
    g = _g(golden_dir, "search_pair128.npz")
    txt = open(f"{golden_dir}/search_pair128_{mode}.txt").read()
    printed = re.findall(r"Overlap=(\S+) (\d+)/(\d+) CC=(\S+) PCC=(\S+)\nScore= (\S+)", txt)
    angles, trans = g[f"{mode}_refined_angle"], g[f"{mode}_refined_trans"]
    assert len(printed) == len(angles) > 0
    st1 = g["stats1"]
    for k in range(len(angles)):
        vec, data = orc.rot_mrc(g["data2"], g["vec2"], angles[k])
        ov, nm, total, cc, pcc, score, _ = orc.get_score(g["data1"], g["vec1"], st1[2], st1[3], st1[4], data, vec,
                                                         trans[k])
        p_ov, p_nm, p_total, p_cc, p_pcc, p_score = printed[k]
        assert (nm, total) == (int(p_nm), int(p_total))
        assert ov == float(p_ov)
        for got, want in ((cc, p_cc), (pcc, p_pcc), (score, p_score)):
            assert abs(got - float(want)) <= 1e-12 * max(1.0, abs(float(want))), (k, got, want)


@pytest.mark.parametrize("mode", ["V", "O", "C", "P", "L"])
def test_refined_model_translations_match_reference_prints(golden_dir, mode):
    """convert_trans with euler2rot (the oracle's restatement of :1549-1566)
    reproduces the reference's printed translation of every refined model,
    to the printed three decimals."""
    import re
    g = _g(golden_dir, "search_pair128.npz")
    txt = open(f"{golden_dir}/search_pair128_{mode}.txt").read()
    printed = re.findall(r"\n#(\d+) Rotation= \((\S+) (\S+) (\S+)\) Translation= \((\S+) (\S+) (\S+)\)", txt)
    angles, trans = g[f"{mode}_refined_angle"], g[f"{mode}_refined_trans"]
    assert len(printed) == len(angles) > 0
    d = int(g["dim"])
    for k, row in enumerate(printed):
        assert int(row[0]) == k
        assert np.allclose([float(v) for v in row[1:4]], angles[k])
        t = orc.convert_trans(g["cent1"], g["cent2"], orc.euler2rot(angles[k]), trans[k], 7.0, d)
        assert ["{:.3f}".format(v) for v in t] == list(row[4:7]), (k, t, row)


@pytest.mark.parametrize("mode", ["V", "O", "C", "P", "L"])
def test_global_top_n_matches_reference_prints(golden_dir, mode):
    """The oracle's stable top-N (score descending, ties to the lower index,
    :664) over the reference's recorded per-rotation scores of the 30-degree
    grid gives the rotations the reference printed as M0..M9, in order."""
    import re
    g = _g(golden_dir, "search_pair128.npz")
    txt = open(f"{golden_dir}/search_pair128_{mode}.txt").read()
    printed = re.findall(r"\nM(\d+) Rotation= \((\S+) (\S+) (\S+)\)", txt)
    grid = orc.calc_angle_comb(30.0)
    angles, scores = g[f"{mode}_angles"], g[f"{mode}_score"]
    assert np.array_equal(angles[:len(grid)], np.asarray(grid, np.float64))   # the grid comes first, in order
    top = orc.topn(scores[:len(grid)], len(printed))
    assert len(printed) == 10
    for k, (i, a, b, c) in enumerate(printed):
        assert int(i) == k
        assert np.allclose(grid[top[k]], [float(a), float(b), float(c)]), (k, grid[top[k]], (a, b, c))


def test_prob_refined_models_match_reference(golden_dir):
    """The oracle's mixed pass (with the statistics of its own first pass)
    over the reference's refined prob-mode models: mixed score times 1/d^3,
    and the mixed and vector translations of every model."""
    g = _g(golden_dir, "prob_pair128.npz")
    d = int(g["dim"])
    rd3 = 1.0 / d ** 3
    tspec = orc.target_spectra([g["vec1"][..., 0], g["vec1"][..., 1], g["vec1"][..., 2]] + list(g["probs1"]))
    st = orc.prob_stats(g["pass1_vscore"], g["pass1_pscore"], rd3)
    for k, a in enumerate(g["refined_angle"]):
        res = orc.rot_and_search_prob(tspec, g["data2"], g["vec2"], g["probs2"], a, 0.5, st, promotion="numpy2")
        assert abs(np.float64(res[4]) * rd3 - g["refined_mixed"][k]) <= 1e-15 * abs(g["refined_mixed"][k])
        assert tuple(res[5]) == tuple(g["refined_mtrans"][k]) and tuple(res[1]) == tuple(g["refined_vtrans"][k])


@pytest.mark.parametrize("mode", ["V", "O", "C", "P", "L"])
def test_refinement_angle_list_matches_reference(golden_dir, mode):
    """The refinement angles the reference searched (its recorded calls after
    the 30-degree grid, duplicates included, in order) are refine_angle_list
    of its top-N, for the oracle's loop and the package's vectorised form."""
    from vesper_python_gb300 import vesper as vg
    g = _g(golden_dir, "search_pair128.npz")
    grid = orc.calc_angle_comb(30.0)
    angles, scores = g[f"{mode}_angles"], g[f"{mode}_score"]
    top = orc.topn(scores[:len(grid)], 10)
    want = angles[len(grid):]
    tops = [grid[t] for t in top]
    assert np.array_equal(vg.refine_angle_list(tops), want)
    assert np.array_equal(np.asarray(orc.refine_angles(tops), np.float64), want)


@pytest.mark.parametrize("mode", ["V", "O", "C", "P", "L"])
def test_refined_top_n_matches_reference(golden_dir, mode):
    """The stable top-N over the reference's recorded refinement scores
    (duplicated angles included: ties go to the first occurrence) is its
    refined model list, angles and translations in order."""
    g = _g(golden_dir, "search_pair128.npz")
    n = len(orc.calc_angle_comb(30.0))
    angles, scores, trans = g[f"{mode}_angles"][n:], g[f"{mode}_score"][n:], g[f"{mode}_trans"][n:]
    top = orc.topn(scores, len(g[f"{mode}_refined_angle"]))
    assert np.array_equal(angles[top], g[f"{mode}_refined_angle"])
    assert np.array_equal(trans[top], g[f"{mode}_refined_trans"])


def test_fastvec_noncubic_sources(golden_dir):
    """C restatement of doFastVEC on non-cubic sources whose windows are
    clipped at both ends, against the reference loop."""
    g = _g(golden_dir, "fastvec_noncubic.npz")
    for i in range(2):
        sw, so0, so1, so2, dd, dw, do0, do1, do2, gg = g[f"c{i}_params"]
        data, vec = orc.fastvec(g[f"c{i}_src"], sw, np.float32([so0, so1, so2]), int(dd), dw, [do0, do1, do2], gg)
        rd = g[f"c{i}_data"]
        assert np.count_nonzero(rd) > 10
        assert np.array_equal(data != 0, rd != 0)
        assert np.max(np.abs(data - rd) / np.maximum(np.abs(rd), 1e-300)) < 1e-15
        assert np.array_equal(vec, g[f"c{i}_vec"])


# ---------------------------------------------------------------------------
# The benchmarked configurations (make_golden_configs.py: the unmodified
# reference over the full angle grids).  The oracle is checked bit for bit on
# rotations spread over each grid and over each refinement set; the GPU tests
# compare every rotation.
# ---------------------------------------------------------------------------
def _dense(g, prefix):
    """A fixture field stored sparse (flat indices of its non-zero voxels
    and their values) as a dense array."""
    shape = tuple(int(v) for v in g[f"{prefix}_shape"])
    val = g[f"{prefix}_val"]
    out = np.zeros((int(np.prod(shape[:3])),) + shape[3:], val.dtype)
    out[g[f"{prefix}_idx"]] = val
    return out.reshape(shape)


def _spread(n, k):
    return np.unique(np.linspace(0, n - 1, k).astype(int))


@pytest.mark.parametrize("mode", ["V", "O", "C", "P", "L"])
def test_pair200_sampled_rotations_bit_exact(golden_dir, mode):
    """The 200^3 / 100^3 pair at s = 2 (grid side 75), A = 10."""
    g = _g(golden_dir, "search_pair200.npz")
    s1 = g["stats1"]
    assert int(g["dim"]) == 75
    ts = orc.target_spectra(orc.mode_field(mode, _dense(g, "data1"), _dense(g, "vec1"), s1[2]))
    qd, qv = _dense(g, "data2"), _dense(g, "vec2")
    scale = orc.score_scale(mode, s1[3], s1[4])
    grid = orc.calc_angle_comb(10.0)
    assert len(grid) == len(g[f"{mode}_score"]) == 24624
    for angles, key in ((grid, ""), (g[f"{mode}_refine_angles"], "refine_")):
        sel = _spread(len(angles), 16)
        sc, tr = orc.search(ts, mode, qd, qv, angles[sel], s1[2])
        assert np.array_equal(sc.astype(np.float64) * scale, g[f"{mode}_{key}score"][sel]), key or "global"
        assert np.array_equal(tr, g[f"{mode}_{key}trans"][sel]), key or "global"
    # the refinement set is that of the reference's own global top-10, and
    # the refined models its top-10
    top = orc.topn(np.asarray(g[f"{mode}_score"], np.float64), 10)
    assert np.array_equal(orc.refine_angles(grid[top]), g[f"{mode}_refine_angles"])
    rtop = orc.topn(np.asarray(g[f"{mode}_refine_score"], np.float64), 10)
    assert np.array_equal(g[f"{mode}_refine_angles"][rtop], g[f"{mode}_refined_angle"])


def test_prob_pad64_sampled_rotations_bit_exact(golden_dir):
    """The prob pair with every grid padded to 64^3, A = 15: both passes and
    the refinement set."""
    g = _g(golden_dir, "prob_pair128_pad64.npz")
    d = int(g["dim"])
    assert d == 64
    tvec, tprobs = _dense(g, "vec1"), np.moveaxis(_dense(g, "probs1"), 3, 0).copy()
    qd, qv, qp = _dense(g, "data2"), _dense(g, "vec2"), list(np.moveaxis(_dense(g, "probs2"), 3, 0).copy())
    tspec = orc.target_spectra([tvec[..., 0], tvec[..., 1], tvec[..., 2]] + list(tprobs))
    grid = orc.calc_angle_comb(15.0)
    assert len(grid) == len(g["pass1_vscore"])
    for r in _spread(len(grid), 12):
        vs, vt, ps, pt, _, _ = orc.rot_and_search_prob(tspec, qd, qv, qp, grid[r], 0.5)
        assert np.float64(vs) == g["pass1_vscore"][r] and tuple(vt) == tuple(g["pass1_vtrans"][r])
        assert np.float64(ps) == g["pass1_pscore"][r] and tuple(pt) == tuple(g["pass1_ptrans"][r])
    st = orc.prob_stats(g["pass1_vscore"], g["pass1_pscore"], 1.0 / d ** 3)
    for r in _spread(len(grid), 12):
        res = orc.rot_and_search_prob(tspec, qd, qv, qp, grid[r], 0.5, st)
        assert np.float64(res[4]) == g["pass2_mscore"][r] and tuple(res[5]) == tuple(g["pass2_mtrans"][r])
    ra = g["refine_angles"]
    assert np.array_equal(ra, orc.refine_angles(grid[orc.topn(g["pass2_mscore"], 10)]))
    for r in _spread(len(ra), 8):
        res = orc.rot_and_search_prob(tspec, qd, qv, qp, ra[r], 0.5, st)
        assert np.float64(res[4]) == g["refine_mscore"][r] and tuple(res[5]) == tuple(g["refine_mtrans"][r])


def test_uneven_sides_sampled_rotations_bit_exact(golden_dir):
    """One pair of the uneven 64-pair batch for every grid side it produces
    (11 ... 44, fused sides included), s = 4, A = 15, mode V."""
    g = _g(golden_dir, "uneven_sides.npz")
    grid = orc.calc_angle_comb(15.0)
    sides = [int(s) for s in g["sides"]]
    assert {11, 18, 22, 44} <= set(sides)
    for side in sides:
        pre = f"d{side}_"
        assert int(g[pre + "dim"]) == side
        s1 = g[pre + "stats1"]
        ts = orc.target_spectra(orc.mode_field("V", _dense(g, pre + "data1"), _dense(g, pre + "vec1"), s1[2]))
        qd, qv = _dense(g, pre + "data2"), _dense(g, pre + "vec2")
        scale = orc.score_scale("V", s1[3], s1[4])
        for angles, key in ((grid, ""), (g[pre + "refine_angles"], "refine_")):
            sel = _spread(len(angles), 8)
            sc, tr = orc.search(ts, "V", qd, qv, angles[sel], s1[2])
            assert np.array_equal(sc.astype(np.float64) * scale, g[pre + key + "score"][sel]), (side, key)
            assert np.array_equal(tr, g[pre + key + "trans"][sel]), (side, key)


@pytest.mark.parametrize("mode", ["V", "O", "C", "P", "L"])
def test_pair200_refined_models_match_reference_prints(golden_dir, mode):
    """At side 75 (the 200^3 / 100^3 pair, s = 2): the oracle's get_score
    and convert_trans over the reference's refined models reproduce its
    printed get_score lines and model translations."""
    import re
    g = _g(golden_dir, "search_pair200.npz")
    txt = open(f"{golden_dir}/search_pair200_{mode}.txt").read()
    printed = re.findall(r"Overlap=(\S+) (\d+)/(\d+) CC=(\S+) PCC=(\S+)\nScore= (\S+)", txt)
    rows = re.findall(r"\n#(\d+) Rotation= \((\S+) (\S+) (\S+)\) Translation= \((\S+) (\S+) (\S+)\)", txt)
    angles, trans = g[f"{mode}_refined_angle"], g[f"{mode}_refined_trans"]
    assert len(printed) == len(rows) == len(angles) > 0
    d1, v1, d2, v2 = _dense(g, "data1"), _dense(g, "vec1"), _dense(g, "data2"), _dense(g, "vec2")
    st1 = g["stats1"]
    d = int(g["dim"])
    for k in range(len(angles)):
        vec, data = orc.rot_mrc(d2, v2, angles[k])
        ov, nm, total, cc, pcc, score, _ = orc.get_score(d1, v1, st1[2], st1[3], st1[4], data, vec, trans[k])
        p_ov, p_nm, p_total, p_cc, p_pcc, p_score = printed[k]
        assert (nm, total) == (int(p_nm), int(p_total))
        assert ov == float(p_ov)
        for got, want in ((cc, p_cc), (pcc, p_pcc), (score, p_score)):
            assert abs(got - float(want)) <= 1e-12 * max(1.0, abs(float(want))), (k, got, want)
        assert int(rows[k][0]) == k and np.allclose([float(v) for v in rows[k][1:4]], angles[k])
        t = orc.convert_trans(g["cent1"], g["cent2"], orc.euler2rot(angles[k]), trans[k], 2.0, d)
        assert ["{:.3f}".format(v) for v in t] == list(rows[k][4:7]), (k, t, rows[k])


def test_uneven_sides_refined_models_match_reference_prints(golden_dir):
    """Every grid side of the uneven batch (s = 4, mode V): the oracle's
    get_score and convert_trans over the reference's refined models
    reproduce its printed lines."""
    import re
    g = _g(golden_dir, "uneven_sides.npz")
    for side in [int(s) for s in g["sides"]]:
        pre = f"d{side}_"
        txt = str(g[pre + "stdout"])
        printed = re.findall(r"Overlap=(\S+) (\d+)/(\d+) CC=(\S+) PCC=(\S+)\nScore= (\S+)", txt)
        rows = re.findall(r"\n#(\d+) Rotation= \((\S+) (\S+) (\S+)\) Translation= \((\S+) (\S+) (\S+)\)", txt)
        angles, trans = g[pre + "refined_angle"], g[pre + "refined_trans"]
        assert len(printed) == len(rows) == len(angles) > 0, side
        d1, v1 = _dense(g, pre + "data1"), _dense(g, pre + "vec1")
        d2, v2 = _dense(g, pre + "data2"), _dense(g, pre + "vec2")
        st1 = g[pre + "stats1"]
        for k in range(len(angles)):
            vec, data = orc.rot_mrc(d2, v2, angles[k])
            ov, nm, total, cc, pcc, score, _ = orc.get_score(d1, v1, st1[2], st1[3], st1[4], data, vec, trans[k])
            p_ov, p_nm, p_total, p_cc, p_pcc, p_score = printed[k]
            assert (nm, total) == (int(p_nm), int(p_total)), (side, k)
            assert ov == float(p_ov), (side, k)
            for got, want in ((cc, p_cc), (pcc, p_pcc), (score, p_score)):
                assert abs(got - float(want)) <= 1e-12 * max(1.0, abs(float(want))), (side, k, got, want)
            t = orc.convert_trans(g[pre + "cent1"], g[pre + "cent2"], orc.euler2rot(angles[k]), trans[k], 4.0, side)
            assert ["{:.3f}".format(v) for v in t] == list(rows[k][4:7]), (side, k, t, rows[k])
