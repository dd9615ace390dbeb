"""GPU parity: the sm_103a kernels against the CPU oracle (itself pinned to the
reference by tests/golden).  Tolerances:

* gather (rot_mrc / rot_mrc_prob): bit-exact;
* fastVEC: float64 density within 1e-12 relative; float32 vectors within
  2e-6 absolute (a few ulp: the GPU sums the separable window in another order,
  in float-float pairs, or in float64 for very narrow windows);
* search: raw scores within 1e-4 relative to the largest |score| (the
  reference-path FFT is single precision); best translations index-exact
  except where the GPU's pick scores within that tolerance of the oracle's
  maximum in the oracle's own volume (a near-tie: Overlap scores are integer
  counts, so exact ties between translations are common there and any FFT
  picks among them by rounding noise); top-N rotations index-exact in mode V,
  and equal up to reordering among near-equal scores in the other modes.
"""
import os

import numpy as np
import pytest
import torch

from oracle import vesper_oracle as orc

pytestmark = pytest.mark.gpu

SCORE_RTOL = 1e-4


def _vg():
    from vesper_python_gb300 import vesper as vg
    return vg


def small_field(rng, d, zero_frac=0.4, dtype=np.float64):
    data = rng.uniform(0.1, 2.0, size=(d, d, d))
    data[rng.random((d, d, d)) < zero_frac] = 0.0
    vec = rng.normal(size=(d, d, d, 3))
    vec /= np.linalg.norm(vec, axis=-1, keepdims=True)
    vec[data == 0] = 0
    return data.astype(dtype), vec.astype(np.float32)


# ---------------------------------------------------------------------------
# gather
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("d", [8, 9, 12, 13, 15, 16, 21])
def test_rot_gather_bit_exact(dev, d):
    vg = _vg()
    rng = np.random.default_rng(100 + d)
    data, vec = small_field(rng, d)
    angles = orc.calc_angle_comb(30.0)
    if d > 13:
        angles = angles[::5]
    mats = vg.rot_matrices(angles)
    dd, vv, _ = vg.rot_gather_device(dev.to_dev(data), dev.to_dev(vec), dev.to_dev(mats), dev=dev)
    dd = dd.cpu().numpy()
    vv = vv.cpu().numpy()
    bad = 0
    for r, a in enumerate(angles):
        ov, od = orc.rot_mrc(data, vec, a, F=mats[r])
        if not (np.array_equal(od, dd[r]) and np.array_equal(ov, vv[r])):
            bad += 1
    assert bad == 0, f"{bad} of {len(angles)} rotations differ at d={d}"


def test_rot_gather_refinement_angles(dev):
    vg = _vg()
    rng = np.random.default_rng(5)
    for d in (12, 13):
        data, vec = small_field(rng, d)
        angles = orc.refine_angles(orc.calc_angle_comb(30.0)[::97])
        mats = vg.rot_matrices(angles)
        dd, vv, _ = vg.rot_gather_device(dev.to_dev(data), dev.to_dev(vec), dev.to_dev(mats), dev=dev)
        for r, a in enumerate(angles):
            ov, od = orc.rot_mrc(data, vec, a, F=mats[r])
            assert np.array_equal(od, dd[r].cpu().numpy()) and np.array_equal(ov, vv[r].cpu().numpy())


@pytest.mark.parametrize("d", [9, 12])
def test_rot_gather_prob_bit_exact(dev, d):
    vg = _vg()
    rng = np.random.default_rng(200 + d)
    data, vec = small_field(rng, d, dtype=np.float32)
    probs = []
    for c in range(4):
        p = rng.dirichlet([0.5] * 4, size=(d, d, d))[..., c].astype(np.float32)
        p[rng.random((d, d, d)) < 0.5] = 0.0
        probs.append(p)
    angles = orc.calc_angle_comb(30.0)[::7]
    mats = vg.rot_matrices(angles)
    dd, vv, pp = vg.rot_gather_device(dev.to_dev(data.astype(np.float64)), dev.to_dev(vec), dev.to_dev(mats),
                                      probs=dev.to_dev(np.stack(probs)), dev=dev)
    for r, a in enumerate(angles):
        ref = orc.rot_mrc_prob(data, vec, *probs, a, F=mats[r])
        assert np.array_equal(ref[0], vv[r].cpu().numpy())
        assert np.array_equal(ref[1], dd[r].cpu().numpy().astype(np.float32))
        for c in range(4):
            assert np.array_equal(ref[2 + c], pp[r, c].cpu().numpy())


# ---------------------------------------------------------------------------
# fastVEC
# ---------------------------------------------------------------------------
def test_fastvec_golden_cases(dev, golden_dir):
    vg = _vg()
    g = np.load(os.path.join(golden_dir, "fastvec_small.npz"))
    for i in range(3):
        S, sw, so0, so1, so2, dd, dw, do0, do1, do2, gg = g[f"c{i}_params"]
        data, d32, vec = vg.fastvec_device(g[f"c{i}_src"], sw, [so0, so1, so2], int(dd), dw, [do0, do1, do2], gg,
                                           dev=dev)
        rd, rv = g[f"c{i}_data"], g[f"c{i}_vec"]
        data = data.cpu().numpy()
        assert np.array_equal(data != 0, rd != 0)
        assert np.max(np.abs(data - rd) / np.maximum(np.abs(rd), 1e-300)) < 1e-12
        assert np.max(np.abs(vec.cpu().numpy() - rv)) < 2e-6
        assert np.array_equal(d32.cpu().numpy(), rd.astype(np.float32)) or \
            np.max(np.abs(d32.cpu().numpy() - rd.astype(np.float32)) / np.maximum(np.abs(rd), 1e-30)) < 1e-6


def test_fastvec_pair128_maps(dev):
    """The 128^3 / 64^3 generator maps at s=7, g=16 (65^3 windows)."""
    vg = _vg()
    from vesper_python_gb300 import synth
    pair = synth.workload_pair("pair128_s7_a30", seed=0)
    for src, orig in ((pair.map1, pair.orig1), (pair.map2, pair.orig2)):
        m = orc.OMap(src, 1.0, orig)
        dim, new_orig, _, _ = orc.set_vox_size(m, 0.1, 7.0)
        ref_d, ref_v = orc.fastvec(m.data, np.float64(m.xwidth), m.orig.astype(np.float64), dim, 7.0, new_orig, 16.0)
        data, _, vec = vg.fastvec_device(m.data, np.float64(m.xwidth), m.orig.astype(np.float64), dim, 7.0, new_orig,
                                         16.0, dev=dev)
        data = data.cpu().numpy()
        assert np.array_equal(data != 0, ref_d != 0)
        assert np.max(np.abs(data - ref_d) / np.maximum(np.abs(ref_d), 1e-300)) < 1e-12
        assert np.max(np.abs(vec.cpu().numpy() - ref_v)) < 2e-6


def test_fastvec_noncubic_sources(dev, golden_dir):
    """Non-cubic sources with windows clipped at both ends (the float-float
    kernels index each source axis by its own extent), against the reference
    loop's outputs."""
    vg = _vg()
    g = np.load(os.path.join(golden_dir, "fastvec_noncubic.npz"))
    for i in range(2):
        sw, so0, so1, so2, dd, dw, do0, do1, do2, gg = g[f"c{i}_params"]
        data, _, vec = vg.fastvec_device(g[f"c{i}_src"], sw, [so0, so1, so2], int(dd), dw, [do0, do1, do2], gg,
                                         dev=dev)
        rd = g[f"c{i}_data"]
        data = data.cpu().numpy()
        assert np.array_equal(data != 0, rd != 0)
        assert np.max(np.abs(data - rd) / np.maximum(np.abs(rd), 1e-300)) < 1e-12
        assert np.max(np.abs(vec.cpu().numpy() - g[f"c{i}_vec"])) < 2e-6


def test_fastvec_narrow_window_float64_path(dev):
    """dreso / src_width = 0.7: the smallest band weight (about 2e-31) is below
    what a float-float pair holds to full precision, so the contractions run in
    float64; same tolerances."""
    vg = _vg()
    rng = np.random.default_rng(11)
    src = rng.uniform(0.2, 1.0, size=(20, 18, 16)).astype(np.float32)
    src[rng.random(src.shape) < 0.4] = 0
    so, do = np.array([0.5, -0.25, 0.0]), np.array([1.0, 0.75, 0.5])
    ref_d, ref_v = orc.fastvec(src, 1.0, so, 9, 2.0, do, 0.7)
    data, _, vec = vg.fastvec_device(src, 1.0, so, 9, 2.0, do, 0.7, dev=dev)
    data = data.cpu().numpy()
    assert np.count_nonzero(ref_d) > 100
    assert np.array_equal(data != 0, ref_d != 0)
    assert np.max(np.abs(data - ref_d) / np.maximum(np.abs(ref_d), 1e-300)) < 1e-12
    assert np.max(np.abs(vec.cpu().numpy() - ref_v)) < 2e-6


# ---------------------------------------------------------------------------
# search
# ---------------------------------------------------------------------------
NEAR_TIE = 1e-5


def _check_search(scores, lins, ref_scores, ref_trans, d, vol_fn=None):
    """Scores within SCORE_RTOL of the largest; with ``vol_fn`` (rotation row
    -> the oracle's correlation volume of that rotation) every translation
    that differs from the oracle's must be a near-tie: within NEAR_TIE of the
    maximum of that volume.  Returns the differing rows."""
    lin_ref = ref_trans[:, 0] * d * d + ref_trans[:, 1] * d + ref_trans[:, 2]
    scale = np.max(np.abs(ref_scores))
    err = np.max(np.abs(scores - ref_scores)) / scale
    assert err < SCORE_RTOL, f"score error {err}"
    mism = np.nonzero(lins != lin_ref)[0]
    if vol_fn is not None:
        for r in mism:
            flat = np.asarray(vol_fn(r), np.float64).reshape(-1)
            gap = (flat.max() - flat[lins[r]]) / np.max(np.abs(flat))
            assert gap <= NEAR_TIE, f"rotation {r}: translation {lins[r]} is {gap:.3g} below the maximum"
    return mism


def _vol_fn(ts, mode, qdata, qvec, angles, ave=0.0):
    """Oracle correlation volume (summed over channels) of rotation row r."""
    def vol(r):
        nv, nd = orc.rot_mrc(qdata, qvec, angles[r])
        return sum(orc.correlate(ts, orc.mode_field(mode, nd, nv, ave)))
    return vol


@pytest.mark.parametrize("mode", ["V", "O", "C", "P", "L"])
def test_search_pair128_golden(dev, golden_dir, mode):
    """Per-rotation raw scores and translations on the golden 13^3 fields."""
    vg = _vg()
    g = np.load(os.path.join(golden_dir, "search_pair128.npz"))
    d = int(g["dim"])
    s1 = g["stats1"]
    angles = g[f"{mode}_angles"]
    name = orc.MODES[mode]
    tdata, tvec = dev.to_dev(g["data1"]), dev.to_dev(g["vec1"])
    spec = vg.target_spectra_device(tdata, tvec, name, s1[2], dev=dev)
    mats = dev.to_dev(vg.rot_matrices(angles))
    sc, ln = vg.search_device(spec, dev.to_dev(g["data2"]), dev.to_dev(g["vec2"]), name, s1[2], mats, dev=dev)
    sc = sc[:, 0].cpu().numpy().astype(np.float64)
    ln = ln[:, 0].cpu().numpy()
    scale = orc.score_scale(mode, s1[3], s1[4])
    ref = g[f"{mode}_score"] / scale
    # any translation mismatch must be a near-tie in the oracle's own volume
    # (Overlap correlates 0/1 masks: its scores are integer counts and exact
    # ties between translations are common; any FFT picks among them by noise)
    ts = orc.target_spectra(orc.mode_field(mode, g["data1"], g["vec1"], s1[2]))
    _check_search(sc, ln, ref, g[f"{mode}_trans"], d, _vol_fn(ts, mode, g["data2"], g["vec2"], angles, s1[2]))
    tol = SCORE_RTOL * np.max(np.abs(ref))
    # top-10 of the global pass and of the refinement: same rotations, allowing
    # reordering only among scores equal within the tolerance
    R = len(orc.calc_angle_comb(30.0))
    for part, sl in (("global", slice(0, R)), ("refine", slice(R, None))):
        top_g = vg.topn_device(torch.as_tensor(sc[sl].astype(np.float32)).to(dev.device).reshape(-1, 1), 10,
                               dev=dev).cpu().numpy()
        top_o = orc.topn(ref[sl], 10)
        assert_topn_equiv(top_g, top_o, ref[sl], tol, f"{mode} {part}")
        if mode == "V":
            assert np.array_equal(top_g, top_o), f"{mode} {part} top-10 differs"
            assert np.array_equal(ln[sl][top_g], (g[f"{mode}_trans"][sl] @ np.array([d * d, d, 1]))[top_o])


def assert_topn_equiv(top_g, top_o, ref_scores, tol, what):
    """Same top-N up to reordering among near-equal scores: the k-th chosen
    score matches the oracle's k-th within tol, and every rotation the two lists
    disagree on scores within tol of the cut-off."""
    assert len(set(top_g.tolist())) == len(top_g), what
    assert np.all(np.abs(ref_scores[top_g] - ref_scores[top_o]) <= tol), what
    cut = ref_scores[top_o[-1]]
    for r in set(top_g.tolist()) ^ set(top_o.tolist()):
        assert abs(ref_scores[r] - cut) <= tol, what


@pytest.mark.parametrize("d", [16, 20, 24, 28, 33, 35, 40, 45, 64])
def test_search_sizes_vs_oracle(dev, d):
    """Odd and even sides with radices 2, 3, 4, 5, 7, 11 against the oracle."""
    vg = _vg()
    rng = np.random.default_rng(d)
    tdata, tvec = small_field(rng, d, zero_frac=0.7)
    qdata, qvec = small_field(rng, d, zero_frac=0.7)
    angles = orc.calc_angle_comb(30.0)[:: max(1, 1008 // 24)]
    spec = vg.target_spectra_device(dev.to_dev(tdata), dev.to_dev(tvec), "VecProduct", 0.0, dev=dev)
    sc, ln = vg.search_device(spec, dev.to_dev(qdata), dev.to_dev(qvec), "VecProduct", 0.0,
                              dev.to_dev(vg.rot_matrices(angles)), dev=dev)
    ts = orc.target_spectra(orc.mode_field("V", tdata, tvec))
    osc, otr = orc.search(ts, "V", qdata, qvec, angles, 0.0)
    _check_search(sc[:, 0].cpu().numpy().astype(np.float64), ln[:, 0].cpu().numpy(), osc.astype(np.float64), otr, d,
                  _vol_fn(ts, "V", qdata, qvec, angles))


@pytest.mark.parametrize("mode", ["O", "C", "P", "L"])
def test_search_scalar_modes_d21(dev, mode):
    vg = _vg()
    d = 21
    rng = np.random.default_rng(77)
    tdata, tvec = small_field(rng, d, zero_frac=0.6)
    qdata, qvec = small_field(rng, d, zero_frac=0.6)
    ave = float(np.mean(tdata[tdata > 0]))
    angles = orc.calc_angle_comb(30.0)[::31]
    name = orc.MODES[mode]
    spec = vg.target_spectra_device(dev.to_dev(tdata), dev.to_dev(tvec), name, ave, dev=dev)
    sc, ln = vg.search_device(spec, dev.to_dev(qdata), dev.to_dev(qvec), name, ave,
                              dev.to_dev(vg.rot_matrices(angles)), dev=dev)
    ts = orc.target_spectra(orc.mode_field(mode, tdata, tvec, ave))
    osc, otr = orc.search(ts, mode, qdata, qvec, angles, ave)
    ln = ln[:, 0].cpu().numpy()
    # only exact ties (common in Overlap, whose scores are integer counts)
    _check_search(sc[:, 0].cpu().numpy().astype(np.float64), ln, osc.astype(np.float64), otr, d,
                  _vol_fn(ts, mode, qdata, qvec, angles, ave))


def test_prob_search_golden(dev, golden_dir):
    vg = _vg()
    g = np.load(os.path.join(golden_dir, "prob_pair128.npz"))
    d = int(g["dim"])
    rd3 = 1.0 / d ** 3
    angles = orc.calc_angle_comb(30.0)
    spec = vg.target_spectra_device(dev.to_dev(g["data1"].astype(np.float64)), dev.to_dev(g["vec1"]), "prob", 0.0,
                                    probs=dev.to_dev(g["probs1"]), dev=dev)
    mats = dev.to_dev(vg.rot_matrices(angles))
    qd, qv, qp = dev.to_dev(g["data2"].astype(np.float64)), dev.to_dev(g["vec2"]), dev.to_dev(g["probs2"])
    s1, l1 = vg.search_device(spec, qd, qv, "prob", 0.0, mats, probs=qp, dev=dev)
    s1 = s1.cpu().numpy().astype(np.float64)
    l1 = l1.cpu().numpy()
    tspec = orc.target_spectra([g["vec1"][..., 0], g["vec1"][..., 1], g["vec1"][..., 2]] + list(g["probs1"]))

    def pvol(part):
        def vol(r):
            res = orc.rot_mrc_prob(g["data2"], g["vec2"], *g["probs2"], angles[r])
            nv = res[0]
            if part == 0:
                return sum(orc.correlate(tspec[:3], [nv[..., 0], nv[..., 1], nv[..., 2]]))
            return sum(orc.correlate(tspec[3:], list(res[2:6])))
        return vol

    _check_search(s1[:, 0], l1[:, 0], g["pass1_vscore"], g["pass1_vtrans"], d, pvol(0))
    _check_search(s1[:, 1], l1[:, 1], g["pass1_pscore"], g["pass1_ptrans"], d, pvol(1))
    st = orc.prob_stats(g["pass1_vscore"], g["pass1_pscore"], rd3)
    mix = (0.5,) + tuple(st)
    s2, l2 = vg.search_device(spec, qd, qv, "prob", 0.0, mats, probs=qp, mix=mix, dev=dev)
    s2 = s2.cpu().numpy().astype(np.float64)
    l2 = l2.cpu().numpy()
    # oracle pass 2 with the pinned numpy 1.21 (float32) arithmetic
    ms = []
    mt = []
    for a in angles:
        r = orc.rot_and_search_prob(tspec, g["data2"], g["vec2"], g["probs2"], a, 0.5, st)
        ms.append(r[4])
        mt.append(r[5])
    ms = np.array(ms, np.float64)
    mt = np.array(mt)
    assert np.max(np.abs(s2[:, 2] - ms)) / np.max(np.abs(ms)) < SCORE_RTOL
    lin_o = mt @ np.array([d * d, d, 1])
    # every differing mixed translation is a near-tie in the oracle's own
    # mixed volume of that rotation
    for r in np.nonzero(l2[:, 2] != lin_o)[0]:
        res = orc.rot_mrc_prob(g["data2"], g["vec2"], *g["probs2"], angles[r])
        nv = res[0]
        cv = orc.correlate(tspec[:3], [nv[..., 0], nv[..., 1], nv[..., 2]])
        cp = orc.correlate(tspec[3:], list(res[2:6]))
        vstd, vave, pstd, pave = st
        m = (np.float32(0.5) * ((sum(cv) - np.float32(vave)) / np.float32(vstd)) +
             np.float32(0.5) * ((sum(cp) - np.float32(pave)) / np.float32(pstd))).reshape(-1).astype(np.float64)
        assert (m.max() - m[l2[r, 2]]) <= 1e-5 * np.max(np.abs(m)), f"rotation {r} not a near-tie"
    top_g = vg.topn_device(torch.as_tensor(s2[:, 2].astype(np.float32)).to(dev.device).reshape(-1, 1), 10,
                           dev=dev).cpu().numpy()
    assert np.array_equal(top_g, orc.topn(ms, 10))


def test_topn_stable_ties(dev):
    vg = _vg()
    s = np.array([1.0, 3.0, 3.0, 2.0, 3.0, -1.0, 2.0], np.float32)
    out = vg.topn_device(torch.as_tensor(s).to(dev.device), 6, dev=dev).cpu().numpy()
    assert list(out) == [1, 2, 4, 3, 6, 0]
    out = vg.topn_device(torch.as_tensor(s).to(dev.device), 9, dev=dev).cpu().numpy()
    assert list(out) == [1, 2, 4, 3, 6, 0, 5, -1, -1]


@pytest.mark.parametrize("d,stride", [(13, 1), (27, 101), (28, 101), (30, 101), (32, 101), (33, 101), (35, 101),
                                      (42, 211), (44, 211), (75, 97)])
def test_register_fft_path_vs_oracle_and_radix_path(dev, d, stride):
    """The register two-step passes (compiled for these sides in mode V)
    against the oracle and against the radix-stage passes."""
    vg = _vg()
    rng = np.random.default_rng(500 + d)
    tdata, tvec = small_field(rng, d, zero_frac=0.7)
    qdata, qvec = small_field(rng, d, zero_frac=0.7)
    angles = orc.calc_angle_comb(30.0)[::stride]
    spec = vg.target_spectra_device(dev.to_dev(tdata), dev.to_dev(tvec), "VecProduct", 0.0, dev=dev)
    mats = dev.to_dev(vg.rot_matrices(angles))
    qd, qv = dev.to_dev(qdata), dev.to_dev(qvec)
    out = {}
    for path in (0, 1):
        sc, ln = vg.search_device(spec, qd, qv, "VecProduct", 0.0, mats, dev=dev, opts=(path, 0, 0))
        out[path] = (sc[:, 0].cpu().numpy().astype(np.float64), ln[:, 0].cpu().numpy())
    ts = orc.target_spectra(orc.mode_field("V", tdata, tvec))
    osc, otr = orc.search(ts, "V", qdata, qvec, angles, 0.0)
    for path in (0, 1):
        _check_search(out[path][0], out[path][1], osc.astype(np.float64), otr, d, _vol_fn(ts, "V", qdata, qvec, angles))
    assert np.max(np.abs(out[0][0] - out[1][0])) <= SCORE_RTOL * np.max(np.abs(osc))


@pytest.mark.parametrize("d,stride", [(8, 7), (9, 7), (11, 7), (12, 3), (13, 1), (16, 5), (21, 11), (24, 13)])
def test_fused_search_vs_oracle_and_pass_path(dev, d, stride):
    """The fused single-kernel search (compiled sides, mode V) against the
    oracle and against the radix-stage passes on the same rotations."""
    vg = _vg()
    assert vg.search_plan(d, "VecProduct", dev=dev)[0] == 2
    rng = np.random.default_rng(700 + d)
    tdata, tvec = small_field(rng, d, zero_frac=0.6)
    qdata, qvec = small_field(rng, d, zero_frac=0.6)
    angles = orc.calc_angle_comb(30.0)[::stride]
    spec = vg.target_spectra_device(dev.to_dev(tdata), dev.to_dev(tvec), "VecProduct", 0.0, dev=dev)
    mats = dev.to_dev(vg.rot_matrices(angles))
    qd, qv = dev.to_dev(qdata), dev.to_dev(qvec)
    out = {}
    for path in (0, 2):
        sc, ln = vg.search_device(spec, qd, qv, "VecProduct", 0.0, mats, dev=dev, opts=(path, 0, 0))
        out[path] = (sc[:, 0].cpu().numpy().astype(np.float64), ln[:, 0].cpu().numpy())
    ts = orc.target_spectra(orc.mode_field("V", tdata, tvec))
    osc, otr = orc.search(ts, "V", qdata, qvec, angles, 0.0)
    _check_search(out[2][0], out[2][1], osc.astype(np.float64), otr, d, _vol_fn(ts, "V", qdata, qvec, angles))
    assert np.max(np.abs(out[0][0] - out[2][0])) <= SCORE_RTOL * np.max(np.abs(osc))


@pytest.mark.parametrize("mode", ["O", "C", "P", "L"])
@pytest.mark.parametrize("d", [12, 15])
def test_fused_scalar_modes_vs_oracle(dev, mode, d):
    """Fused single-kernel search in the scalar modes against the oracle."""
    vg = _vg()
    name = orc.MODES[mode]
    assert vg.search_plan(d, name, dev=dev)[0] == 2
    rng = np.random.default_rng(900 + d)
    tdata, tvec = small_field(rng, d, zero_frac=0.5)
    qdata, qvec = small_field(rng, d, zero_frac=0.5)
    ave = float(np.mean(tdata[tdata > 0]))
    angles = orc.calc_angle_comb(30.0)[::9]
    spec = vg.target_spectra_device(dev.to_dev(tdata), dev.to_dev(tvec), name, ave, dev=dev)
    mats = dev.to_dev(vg.rot_matrices(angles))
    sc, ln = vg.search_device(spec, dev.to_dev(qdata), dev.to_dev(qvec), name, ave, mats, dev=dev)
    ts = orc.target_spectra(orc.mode_field(mode, tdata, tvec, ave))
    osc, otr = orc.search(ts, mode, qdata, qvec, angles, ave)
    got = sc[:, 0].cpu().numpy().astype(np.float64)
    # Overlap scores are integer counts: translations may tie exactly; every
    # differing translation must be such a near-tie in the oracle's volume
    _check_search(got, ln[:, 0].cpu().numpy(), osc.astype(np.float64), otr, d,
                  _vol_fn(ts, mode, qdata, qvec, angles, ave))


def _prob_fields(rng, d):
    data, vec = small_field(rng, d, zero_frac=0.6)
    probs = rng.dirichlet([0.5] * 4, size=(d, d, d)).astype(np.float32).transpose(3, 0, 1, 2).copy()
    probs[:, data == 0] = 0
    return data, vec, probs


@pytest.mark.parametrize("d", [30, 32, 64])
def test_prob_side64_fp32_paths_vs_fp64_oracle(dev, d):
    """Prob mode on the register-pass sides (64: grids padded to 64^3): the
    register passes and the radix-stage passes (float32 FFT) against the
    oracle in float64, vector, probability and mixed scores within 1e-4 of
    the largest."""
    vg = _vg()
    rng = np.random.default_rng(d)
    tdata, tvec, tprobs = _prob_fields(rng, d)
    qdata, qvec, qprobs = _prob_fields(rng, d)
    angles = orc.calc_angle_comb(30.0)[::173]
    spec = vg.target_spectra_device(dev.to_dev(tdata), dev.to_dev(tvec), "prob", 0.0, probs=dev.to_dev(tprobs),
                                    dev=dev)
    mats = dev.to_dev(vg.rot_matrices(angles))
    qd, qv, qp = dev.to_dev(qdata), dev.to_dev(qvec), dev.to_dev(qprobs)
    tspec = orc.target_spectra([tvec[..., 0], tvec[..., 1], tvec[..., 2]] + list(tprobs))
    ref = [orc.rot_and_search_prob(tspec, qdata, qvec, list(qprobs), a, 0.5, None, fp64=True) for a in angles]
    rv = np.array([r[0] for r in ref])
    rp = np.array([r[2] for r in ref])
    rd3 = 1.0 / d ** 3
    st = orc.prob_stats(rv, rp, rd3)
    mix = (0.5,) + tuple(st)
    refm = np.array([orc.rot_and_search_prob(tspec, qdata, qvec, list(qprobs), a, 0.5, st, fp64=True)[4]
                     for a in angles], np.float64)
    assert vg.search_plan(d, "prob", dev=dev)[0] == 1
    for path in (0, 1):
        s1, _ = vg.search_device(spec, qd, qv, "prob", 0.0, mats, probs=qp, dev=dev, opts=(path, 0, 0))
        s2, _ = vg.search_device(spec, qd, qv, "prob", 0.0, mats, probs=qp, mix=mix, dev=dev, opts=(path, 0, 0))
        s1 = s1.cpu().numpy().astype(np.float64)
        s2 = s2.cpu().numpy().astype(np.float64)
        assert np.max(np.abs(s1[:, 0] - rv)) / np.max(np.abs(rv)) < 1e-4, path
        assert np.max(np.abs(s1[:, 1] - rp)) / np.max(np.abs(rp)) < 1e-4, path
        assert np.max(np.abs(s2[:, 2] - refm)) / np.max(np.abs(refm)) < 1e-4, path


@pytest.mark.parametrize("mode", ["O", "C", "P", "L"])
def test_register_passes_scalar_modes_side75(dev, mode):
    """Register passes of the scalar modes at side 75 against the radix-stage
    passes and the oracle on a few rotations."""
    vg = _vg()
    name = orc.MODES[mode]
    d = 75
    assert vg.search_plan(d, name, dev=dev)[0] == 1
    rng = np.random.default_rng(1075)
    tdata, tvec = small_field(rng, d, zero_frac=0.6)
    qdata, qvec = small_field(rng, d, zero_frac=0.6)
    ave = float(np.mean(tdata[tdata > 0]))
    angles = orc.calc_angle_comb(30.0)[::251]
    spec = vg.target_spectra_device(dev.to_dev(tdata), dev.to_dev(tvec), name, ave, dev=dev)
    mats = dev.to_dev(vg.rot_matrices(angles))
    out = {}
    for path in (0, 1):
        sc, ln = vg.search_device(spec, dev.to_dev(qdata), dev.to_dev(qvec), name, ave, mats, dev=dev,
                                  opts=(path, 0, 0))
        out[path] = sc[:, 0].cpu().numpy().astype(np.float64)
    ts = orc.target_spectra(orc.mode_field(mode, tdata, tvec, ave))
    osc, _ = orc.search(ts, mode, qdata, qvec, angles, ave)
    scale = np.max(np.abs(osc))
    for path in (0, 1):
        assert np.max(np.abs(out[path] - osc)) <= SCORE_RTOL * scale, path


def test_all_zero_query_takes_the_first_translation(dev):
    """An all-zero rotated query gives an all-zero correlation volume; numpy's
    argmax (and so the reference) returns translation 0 whatever the signs of
    the zeros, on every kernel family."""
    vg = _vg()
    for d in (13, 30):
        rng = np.random.default_rng(d)
        tdata, tvec = small_field(rng, d, zero_frac=0.5)
        qdata = np.zeros((d, d, d))
        qvec = np.zeros((d, d, d, 3), np.float32)
        spec = vg.target_spectra_device(dev.to_dev(tdata), dev.to_dev(tvec), "VecProduct", 0.0, dev=dev)
        mats = dev.to_dev(vg.rot_matrices(orc.calc_angle_comb(30.0)[:20]))
        paths = [0, vg.search_plan(d, "VecProduct", dev=dev)[0]]
        for path in sorted(set(paths)):
            sc, ln = vg.search_device(spec, dev.to_dev(qdata), dev.to_dev(qvec), "VecProduct", 0.0, mats, dev=dev,
                                      opts=(path, 0, 0))
            assert np.all(sc[:, 0].cpu().numpy() == 0.0), (d, path)
            assert np.all(ln[:, 0].cpu().numpy() == 0), (d, path)
