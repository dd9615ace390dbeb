"""End-to-end GPU path against the reference's recorded output: the float64
rescoring kernel against the oracle's get_score, the device-resident
alignment pipeline and the ``main.py orig`` command line on the golden pair
(128^3 / 64^3 maps at s = 7, A = 30, d = 13)."""
import contextlib
import io
import os
import re

import numpy as np
import torch
import pytest

from oracle import vesper_oracle as orc

pytestmark = pytest.mark.gpu


def _field(rng, d, zero_frac=0.5):
    data = rng.uniform(0.1, 2.0, size=(d, d, d))
    data[rng.random((d, d, d)) < zero_frac] = 0.0
    vec = rng.normal(size=(d, d, d, 3)).astype(np.float32)
    vec[data == 0] = 0
    return data, vec


@pytest.mark.parametrize("trans", [(0, 0, 0), (3, 12, 7), (12, 1, 6), (6, 7, 0)])
def test_rescore_matches_oracle_get_score(dev, trans):
    from vesper_python_gb300 import vesper as vg
    rng = np.random.default_rng(sum(trans) + 3)
    d = 13
    tdata, tvec = _field(rng, d)
    sdata, svec = _field(rng, d)
    pos = tdata[tdata > 0]
    tave, tstd, tpstd = np.mean(pos), np.linalg.norm(pos), np.linalg.norm(pos - np.mean(pos))
    ov, nm, total, cc, pcc, score, sco = orc.get_score(tdata, tvec, tave, tstd, tpstd, sdata, svec, trans)

    class T:
        pass

    t = T()
    t.data, t.vec, t.ave, t.std, t.std_norm_ave = tdata, tvec, tave, tstd, tpstd
    sr = vg.get_score_device(t, dev.to_dev(sdata), dev.to_dev(svec), trans, dev=dev)
    assert (sr.nm, sr.total) == (nm, total)
    assert abs(sr.cc - cc) <= 1e-12 * max(1.0, abs(cc))
    assert abs(sr.pcc - pcc) <= 1e-12 * max(1.0, abs(pcc))
    # the reference's per-voxel dot products are float32; ours are float64
    assert abs(sr.score - score) <= 1e-5 * max(1.0, abs(score))
    assert np.allclose(sr.sco_arr, sco, rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("d", [13, 32, 75])
def test_rescore_batch_matches_oracle_get_score(dev, d):
    """vesper_rescore_batch (many blocks, several models, device
    translations) against the oracle's get_score for each model."""
    import ctypes
    from vesper_python_gb300 import _native
    rng = np.random.default_rng(d)
    tdata, tvec = _field(rng, d)
    pos = tdata[tdata > 0]
    tave, tstd, tpstd = np.mean(pos), np.linalg.norm(pos), np.linalg.norm(pos - np.mean(pos))
    models = [_field(rng, d) for _ in range(3)]
    trans = [(1, 0, d - 1), (0, 0, 0), (d // 2 + 1, 2, 3)]
    wrapped = np.array([[t - d if t > 0.5 * d else t for t in tr] for tr in trans], np.int32)
    sd = dev.to_dev(np.stack([m[0] for m in models]))
    sv = dev.to_dev(np.stack([m[1] for m in models]))
    res = torch.empty((3, 8), dtype=torch.float64, device=dev.device)
    nb = _native.size_query("vesper_rescore_batch_workspace_size", d, 3)
    ws = torch.empty(nb, dtype=torch.uint8, device=dev.device)
    td, tv, trd = dev.to_dev(tdata), dev.to_dev(tvec), dev.to_dev(wrapped)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    _native.check(dev.lib.vesper_rescore_batch(p(td), p(tv), tave, tstd, tpstd, p(sd), p(sv), d, p(trd), 3, p(res),
                                               p(ws), nb, dev.stream))
    r = res.cpu().numpy()
    for k in range(3):
        ov, nm, total, cc, pcc, score, _ = orc.get_score(tdata, tvec, tave, tstd, tpstd, models[k][0], models[k][1],
                                                         trans[k])
        assert (int(r[k, 0]), int(r[k, 1])) == (nm, total)
        assert abs(r[k, 2] - cc) <= 1e-12 * max(1.0, abs(cc))
        assert abs(r[k, 3] - pcc) <= 1e-12 * max(1.0, abs(pcc))
        assert abs(r[k, 4] - score) <= 1e-5 * max(1.0, abs(score))


def _model_lines(text, prefix):
    return [ln for ln in text.splitlines() if re.match(rf"^{re.escape(prefix)}\d+ Rotation=", ln)]


def test_aligner_matches_golden_refined_models(dev, golden_dir):
    from vesper_python_gb300 import align, synth
    g = np.load(os.path.join(golden_dir, "search_pair128.npz"))
    pair = synth.workload_pair("pair128_s7_a30", seed=0)
    al = align.Aligner(dev)
    p = align.AlignParams(t=0.1, T=0.1, g=16.0, s=7.0, A=30.0, N=10, mode="VecProduct")
    res = al.align_device(dev.to_dev(pair.map1), dev.to_dev(pair.map2), 1.0, 1.0, pair.orig1, pair.orig2, p)
    assert res.dim == int(g["dim"])
    ang = np.array([m.angle for m in res.models])
    tr = np.array([m.vec_trans for m in res.models])
    assert np.array_equal(ang, g["V_refined_angle"])
    assert np.array_equal(tr, g["V_refined_trans"])
    assert np.allclose([m.vec_score for m in res.models], g["V_refined_score"], rtol=1e-4)


def test_main_orig_cli_matches_reference_stdout(dev, golden_dir, tmp_path):
    """Rotation/translation lines byte-identical to the reference's stdout;
    the printed scores within 1e-4 relative."""
    from vesper_python_gb300 import main as cli
    from vesper_python_gb300 import mrc, synth
    pair = synth.workload_pair("pair128_s7_a30", seed=0)
    a = tmp_path / "map1.mrc"
    b = tmp_path / "map2.mrc"
    mrc.write_mrc(a, np.swapaxes(pair.map1, 0, 2), 1.0, pair.orig1)
    mrc.write_mrc(b, np.swapaxes(pair.map2, 0, 2), 1.0, pair.orig2)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        cli.main(["orig", "-a", str(a), "-b", str(b), "-t", "0.1", "-T", "0.1", "-s", "7", "-A", "30"])
    out = buf.getvalue()
    ref = open(os.path.join(golden_dir, "search_pair128_V.txt")).read()
    setup = open(os.path.join(golden_dir, "search_pair128_setup.txt")).read()
    for prefix in ("M", "#"):
        assert _model_lines(out, prefix) == _model_lines(ref, prefix)
    for key in ("#dmax=", "Nvox=", "cent=", "ori="):
        assert [ln for ln in out.splitlines() if ln.startswith(key)] == \
            [ln for ln in setup.splitlines() if ln.startswith(key)]

    def nums(text, key):
        return [float(re.search(rf"{key}\s*([-0-9.e+]+)", ln).group(1)) for ln in text.splitlines() if key in ln]

    for key in ("Score=", "CC=", "PCC=", "Overlap="):
        o, r = nums(out, key), nums(ref, key)
        assert len(o) == len(r) == 10
        assert np.allclose(o, r, rtol=1e-4, atol=1e-6), key
    sums_o, sums_r = nums(out, "SUM="), nums(setup, "SUM=")
    assert np.allclose(sums_o, sums_r, rtol=1e-12)


def test_prob_pipeline_top_models(dev, golden_dir, tmp_path):
    """main.py prob on the golden prob pair: the refined models' rotations and
    translations match the reference's stdout."""
    from vesper_python_gb300 import main as cli
    from vesper_python_gb300 import mrc, synth
    pair = synth.make_pair(0, 128, 400, 40.0, with_prob=True, threshold=0.1)
    a, b = tmp_path / "m1.mrc", tmp_path / "m2.mrc"
    mrc.write_mrc(a, np.swapaxes(pair.map1, 0, 2), 1.0, pair.orig1)
    mrc.write_mrc(b, np.swapaxes(pair.map2, 0, 2), 1.0, pair.orig2)
    pa, pb = tmp_path / "p1.npy", tmp_path / "p2.npy"
    # main.py swaps the .npy axes like the MRC data: store them in file order
    np.save(pa, np.swapaxes(pair.prob1, 0, 2))
    np.save(pb, np.swapaxes(pair.prob2, 0, 2))
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        cli.main(["prob", "-a", str(a), "-npa", str(pa), "-b", str(b), "-npb", str(pb), "-t", "0.1", "-T", "0.1",
                  "-s", "7", "-A", "30", "-alpha", "0.5"])
    out = buf.getvalue()
    ref = open(os.path.join(golden_dir, "prob_pair128.txt")).read()
    assert _model_lines(out, "#") == _model_lines(ref, "#")


def test_align_many_equals_one_at_a_time(dev):
    """A batch of uneven pairs through align_many gives, pair by pair, what
    align_device gives for each pair alone."""
    from vesper_python_gb300 import align, synth
    al = align.Aligner(dev)
    p = align.AlignParams(t=0.1, T=0.1, g=16.0, s=7.0, A=30.0, N=5, mode="VecProduct")
    pairs = [synth.uneven_pair(i) for i in range(3)]
    items = [(dev.to_dev(pr.map1), dev.to_dev(pr.map2), pr.width, pr.width, pr.orig1, pr.orig2) for pr in pairs]
    many = al.align_many(items, p)
    for it, r in zip(items, many):
        one = al.align_device(*it, p)
        assert one.dim == r.dim
        assert [m.angle for m in one.models] == [m.angle for m in r.models]
        assert [m.vec_trans for m in one.models] == [m.vec_trans for m in r.models]
        assert [m.dot_score for m in one.models] == [m.dot_score for m in r.models]
        assert one.top == r.top


@pytest.mark.parametrize("d", [13, 30, 75])
def test_map_stats_many_blocks(dev, d):
    """vesper_map_stats_ws (many blocks) against numpy and the one-block form."""
    import ctypes
    from vesper_python_gb300 import _native
    rng = np.random.default_rng(d)
    data = rng.uniform(-0.5, 2.0, size=(d, d, d))
    data[rng.random((d, d, d)) < 0.3] = 0.0
    t = dev.to_dev(data)
    a = torch.empty(5, dtype=torch.float64, device=dev.device)
    b = torch.empty(5, dtype=torch.float64, device=dev.device)
    nb = _native.size_query("vesper_map_stats_workspace_size", d)
    ws = torch.empty(nb, dtype=torch.uint8, device=dev.device)
    p = lambda x: ctypes.c_void_p(x.data_ptr())
    _native.check(dev.lib.vesper_map_stats(p(t), d, p(a), dev.stream))
    _native.check(dev.lib.vesper_map_stats_ws(p(t), d, p(b), p(ws), nb, dev.stream))
    pos = data[data > 0]
    want = np.array([data.sum(), np.count_nonzero(data), pos.mean(), np.linalg.norm(pos),
                     np.linalg.norm(pos - pos.mean())])
    np.testing.assert_allclose(a.cpu().numpy(), want, rtol=1e-12)
    np.testing.assert_allclose(b.cpu().numpy(), want, rtol=1e-12)


def test_align_many_graph_replay_equals_eager(dev):
    """The global stage captured as a CUDA graph: first call captures, the
    second replays; both give exactly the eager results."""
    from vesper_python_gb300 import align, synth
    al = align.Aligner(dev)
    p = align.AlignParams(t=0.1, T=0.1, g=16.0, s=7.0, A=30.0, N=5, mode="VecProduct")
    pairs = [synth.uneven_pair(i) for i in range(3, 6)]
    items = [(dev.to_dev(pr.map1), dev.to_dev(pr.map2), pr.width, pr.width, pr.orig1, pr.orig2) for pr in pairs]
    eager = al.align_many(items, p)
    g1 = al.align_many(items, p, graph=True)
    g2 = al.align_many(items, p, graph=True)
    # two graphs per batch signature: the global stage, then refinement + rescoring
    assert al.graph_captures == 2 and al.graph_replays == 4
    for a, b, c in zip(eager, g1, g2):
        for r in (b, c):
            assert r.top == a.top
            assert [m.angle for m in r.models] == [m.angle for m in a.models]
            assert [m.dot_score for m in r.models] == [m.dot_score for m in a.models]
            assert (r.ave, r.std) == (a.ave, a.std)


def test_prob_interpolate_golden_and_oracle(dev, golden_dir):
    """GPU hole filling against the reference function's outputs (golden) and
    against the oracle on a larger map, bit for bit; a map without a positive
    first channel raises as the reference does."""
    from vesper_python_gb300 import vesper as vg
    g = np.load(os.path.join(golden_dir, "interp_small.npz"))
    for n in range(4):
        a = g[f"in{n}"].copy()
        vg.interpolate(a)
        np.testing.assert_array_equal(a, g[f"out{n}"])
    rng = np.random.default_rng(7)
    a = np.zeros((61, 70, 83, 4), np.float32)
    a[1::2, ::2, 1::2] = rng.random(a[1::2, ::2, 1::2].shape).astype(np.float32)
    a[rng.random(a.shape) < 0.05] = 0.0
    b = a.copy()
    orc.interpolate(b)
    t = dev.to_dev(a)
    vg.interpolate_device(t, dev)
    np.testing.assert_array_equal(t.cpu().numpy(), b)
    with pytest.raises(UnboundLocalError):
        vg.interpolate(np.zeros((4, 4, 4, 4), np.float32))


def test_interpolation_cli(dev, tmp_path, golden_dir):
    """interpolation.py insert/graph: prints, the saved .npy equals the
    reference's output, one MRC per channel."""
    from vesper_python_gb300 import interpolation, mrc
    g = np.load(os.path.join(golden_dir, "interp_small.npz"))
    np.save(tmp_path / "in.npy", g["in0"])
    ref_map = tmp_path / "ref.mrc"
    mrc.write_mrc(ref_map, np.zeros(g["in0"].shape[2::-1], np.float32), voxel_size=1.0, origin=(1.0, 2.0, 3.0))
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        interpolation.main(["graph", "-f", str(tmp_path / "in.npy"), "-s", str(tmp_path / "out"), "-m", str(ref_map)])
    lines = buf.getvalue().splitlines()
    assert lines[0] == "Usage Modes:" and lines[4:8] == [str(v) for v in g["in0"].shape]
    assert lines[8] == "Saved interpolated map as: " + str(tmp_path / "out") + ".npy"
    np.testing.assert_array_equal(np.load(tmp_path / "out.npy"), g["out0"])
    for c in range(4):
        m = mrc.read_mrc(tmp_path / f"out_{c}.mrc")
        nx, ny, nz = g["out0"].shape[:3]
        np.testing.assert_array_equal(m.data[:nz - 2, :ny - 2, :nx - 2],
                                      np.transpose(g["out0"][:nx - 2, :ny - 2, :nz - 2, c], (2, 1, 0)))
        assert tuple(m.origin) == (1.0, 2.0, 3.0)


def test_prepare_maps_equals_per_map(dev):
    """vesper_prepare_maps (one launch per 64 maps) thresholds every map in
    place and gives each map's (radius bits, count) as vesper_prepare_map
    does: uneven shapes, an all-zero map, a negative threshold, and more
    maps than one launch takes."""
    import ctypes
    from vesper_python_gb300 import _native
    from vesper_python_gb300 import vesper as vg
    rng = np.random.default_rng(7)
    shapes = [(17, 20, 23), (64, 64, 64), (5, 1, 9), (8, 8, 8), (33, 2, 40)] + [(6, 7, 5)] * 66
    maps, ths = [], []
    for i, sh in enumerate(shapes):
        a = rng.uniform(-0.5, 1.0, size=sh).astype(np.float32)
        a[rng.random(sh) < 0.4] = 0
        if i == 3:
            a[:] = 0
        maps.append(a)
        ths.append(-1.0 if i == 2 else float(rng.uniform(0.0, 0.6)))
    cents = [np.array([x * 0.5 for x in sh]) + (0.25 if i % 2 else 0.0) for i, sh in enumerate(shapes)]
    # per map
    ref_data, ref_out = [], []
    for a, th, c in zip(maps, ths, cents):
        t = dev.to_dev(a)
        o = torch.empty(2, dtype=torch.int64, device=dev.device)
        _native.check(dev.lib.vesper_prepare_map(ctypes.c_void_p(t.data_ptr()), *a.shape, th, vg._host_d3(c),
                                                 ctypes.c_void_p(o.data_ptr()), dev.stream))
        ref_data.append(t.cpu().numpy())
        ref_out.append(o.cpu().numpy())
    # all at once
    ts = [dev.to_dev(a) for a in maps]
    nm = len(ts)
    out = torch.full((nm, 2), -1, dtype=torch.int64, device=dev.device)
    ptrs = (ctypes.c_void_p * nm)(*[t.data_ptr() for t in ts])
    dims = (ctypes.c_int * (3 * nm))(*[v for a in maps for v in a.shape])
    thr = (ctypes.c_double * nm)(*ths)
    cen = (ctypes.c_double * (3 * nm))(*[float(v) for c in cents for v in c])
    _native.check(dev.lib.vesper_prepare_maps(nm, ptrs, dims, thr, cen, ctypes.c_void_p(out.data_ptr()), dev.stream))
    got = out.cpu().numpy()
    for i in range(nm):
        np.testing.assert_array_equal(got[i], ref_out[i], err_msg=f"map {i}")
        np.testing.assert_array_equal(ts[i].cpu().numpy(), ref_data[i], err_msg=f"map {i}")
    assert got[3, 1] == 0 and got[3, 0] == 0


def test_graph_late_stage_many_pairs_of_one_side(dev):
    """Eight 128^3 / 64^3 pairs whose grids share sides (28 to 32, the
    three-pass search): the graph form runs the pairs' refinement chains on
    concurrent streams, and every pair's results equal the eager form's (no
    scratch is shared between streams)."""
    from vesper_python_gb300 import align, synth
    al = align.Aligner(dev)
    p = align.AlignParams(t=0.1, T=0.1, g=16.0, s=3.0, A=30.0, N=5, mode="VecProduct")
    pairs = [synth.workload_pair("prop128_s3_a10", seed=s) for s in range(8)]
    items = [(dev.to_dev(pr.map1), dev.to_dev(pr.map2), pr.width, pr.width, pr.orig1, pr.orig2) for pr in pairs]
    eager = al.align_many(items, p)
    dims = [r.dim for r in eager]
    assert len(set(dims)) < len(dims) and min(dims) > 24
    for _ in range(2):
        g = al.align_many(items, p, graph=True)
        for a, r in zip(eager, g):
            assert r.top == a.top
            assert [m.angle for m in r.models] == [m.angle for m in a.models]
            assert [m.vec_trans for m in r.models] == [m.vec_trans for m in a.models]
            assert [m.dot_score for m in r.models] == [m.dot_score for m in a.models]
            assert [m.cc for m in r.models] == [m.cc for m in a.models]


def test_refine_slots_and_pick_match_tensor_formulation(dev):
    """vesper_refine_slots and vesper_refine_pick against the same steps in
    torch tensor arithmetic: slots of the 5-degree lattice (filter before the
    wrap, dropped slots row 0), stable masked top-N with ties to the lower
    slot, the picks' rows, scores, translations and wrapped translations."""
    import ctypes
    from vesper_python_gb300 import _native, align
    from vesper_python_gb300 import vesper as vg
    c_ = lambda t: ctypes.c_void_p(t.data_ptr())
    rng = np.random.default_rng(11)
    L = vg.LATTICE_N
    al = align.Aligner(dev)
    lat = vg.lattice_rot_matrices_device(dev)
    grid_rows = al._grid_rows(10.0, vg.calc_angle_comb(10.0))
    off = al._ref_offsets()
    n, N, d, nscore = 5, 10, 30, 1
    ngrid = int(grid_rows.shape[0])
    tg_h = rng.integers(0, ngrid, size=(n, N))
    tg_h[1, 7:] = -1
    tg_h[2, 0] = 0                                  # the grid's first angle: offsets wrap and drop
    tg_h[3, :] = ngrid - 1                          # the last: z = 175 drops z + 5
    tg = dev.to_dev(tg_h.astype(np.int64))
    crow = torch.empty((n, N * 27), dtype=torch.int64, device=dev.device)
    valid = torch.empty((n, N * 27), dtype=torch.bool, device=dev.device)
    rmats = torch.empty((n, N * 27, 3, 3), dtype=torch.float32, device=dev.device)
    _native.check(dev.lib.vesper_refine_slots(c_(tg), n, N, c_(grid_rows), ngrid, c_(off), L, c_(lat), c_(crow),
                                              c_(valid), c_(rmats), dev.stream))
    # the tensor formulation
    rows = grid_rows.index_select(0, tg.clamp(min=0).reshape(-1)).reshape(n, N)
    base = torch.stack([rows // (L * L), (rows // L) % L, rows % L], dim=2)
    cand = base[:, :, None, :] + off[None, None, :, :]
    v_ref = (cand[..., 0] < L) & (cand[..., 1] < L) & (cand[..., 2] < L // 2) & (tg >= 0)[:, :, None]
    cand = torch.where(cand < 0, cand + L, cand)
    c_ref = (cand[..., 0] * L + cand[..., 1]) * L + cand[..., 2]
    v_ref = v_ref.reshape(n, N * 27)
    c_ref = torch.where(v_ref, c_ref.reshape(n, N * 27), torch.zeros_like(v_ref, dtype=torch.int64))
    assert torch.equal(valid, v_ref) and torch.equal(crow, c_ref)
    assert torch.equal(rmats, lat.index_select(0, c_ref.reshape(-1)).reshape(n, N * 27, 3, 3))
    assert bool((~valid[1, 7 * 27:]).all()) and bool((~valid[3]).any())
    # picks, with exact ties among the scores
    RS = dev.to_dev(rng.integers(0, 40, size=(n, N * 27, nscore)).astype(np.float32))
    RL = dev.to_dev(rng.integers(0, d ** 3, size=(n, N * 27, nscore)).astype(np.int32))
    for i in range(n):
        out = [torch.empty(N, dtype=torch.int32, device=dev.device), torch.empty(N, dtype=torch.int64, device=dev.device),
               torch.empty(N, dtype=torch.float32, device=dev.device), torch.empty(N, dtype=torch.int64, device=dev.device),
               torch.empty((N, 3, 3), dtype=torch.float32, device=dev.device),
               torch.empty((N, 3), dtype=torch.int32, device=dev.device)]
        _native.check(dev.lib.vesper_refine_pick(c_(RS[i]), c_(RL[i]), nscore, c_(valid[i]), c_(crow[i]), N * 27, N,
                                                 c_(lat), d, *[c_(t) for t in out], dev.stream))
        masked = torch.where(valid[i], RS[i, :, 0], torch.full_like(RS[i, :, 0], float("-inf")))
        rtop = vg.topn_device(masked.contiguous(), N, dev=dev)
        sel = rtop.to(torch.int64).clamp(min=0)
        r_rows = crow[i].gather(0, sel)
        r_lin = RL[i, :, 0].to(torch.int64).gather(0, sel)
        t = torch.stack([r_lin // (d * d), (r_lin // d) % d, r_lin % d], dim=1)
        trd = torch.where(2 * t > d, t - d, t).to(torch.int32)
        assert torch.equal(out[0], rtop)
        assert torch.equal(out[1], r_rows)
        assert torch.equal(out[2], RS[i, :, 0].gather(0, sel))
        assert torch.equal(out[3], r_lin)
        assert torch.equal(out[4], lat.index_select(0, r_rows))
        assert torch.equal(out[5], trd)
