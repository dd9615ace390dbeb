"""Host-side logic of the package (no GPU): angle grid, rotation matrices,
refinement set, map I/O and set-up, CLI, output geometry, PDB writer and the
rotation sharding helpers."""
import contextlib
import io
import os

import numpy as np
import pytest

from oracle import vesper_oracle as orc
from vesper_python_gb300 import main as cli
from vesper_python_gb300 import mrc, shard, synth
from vesper_python_gb300 import vesper as vg


def test_angle_grid_matches_golden(golden_dir):
    g = np.load(os.path.join(golden_dir, "angles.npz"))
    for key in g.files:
        assert np.array_equal(vg.calc_angle_comb(float(key[1:])), g[key])


def test_rotation_matrices_bitwise():
    angles = vg.calc_angle_comb(30.0)
    mats = vg.rot_matrices(angles)
    for a, m in zip(angles[::5], mats[::5]):
        assert np.array_equal(m, orc.rot_matrix_f32(a))
    ref = orc.refine_angles(angles[[0, 17, 500, 1007]])
    assert np.array_equal(vg.refine_angle_list(angles[[0, 17, 500, 1007]]), ref)
    for a, m in zip(ref, vg.rot_matrices(ref)):
        assert np.array_equal(m, orc.rot_matrix_f32(a))


def test_next_fast_len_agrees():
    for n in range(1, 400):
        assert vg.next_fast_len(n) == orc.next_fast_len(n)


def test_mrc_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    a = rng.normal(size=(7, 5, 6)).astype(np.float32)  # (nz, ny, nx)
    p = tmp_path / "m.mrc"
    mrc.write_mrc(p, a, voxel_size=1.5, origin=(1.0, -2.0, 3.5))
    m = mrc.read_mrc(p)
    assert (m.nx, m.ny, m.nz) == (6, 5, 7)
    assert np.array_equal(m.data, a)
    assert np.array_equal(m.voxel_size, np.float32([1.5, 1.5, 1.5]))
    assert np.array_equal(m.origin, np.float32([1.0, -2.0, 3.5]))
    o = vg.mrc_obj(str(p))
    assert o.data.shape == (6, 5, 7) and np.array_equal(o.data, np.swapaxes(a, 0, 2))
    assert o.xwidth.dtype == np.float32 and o.orig.dtype == np.float32


def test_mrc_bad_files(tmp_path):
    p = tmp_path / "short.mrc"
    p.write_bytes(b"\0" * 100)
    with pytest.raises(mrc.MrcFormatError):
        mrc.read_mrc(p)
    a = np.zeros((4, 4, 4), np.float32)
    q = tmp_path / "trunc.mrc"
    mrc.write_mrc(q, a)
    q.write_bytes(q.read_bytes()[:-10])
    with pytest.raises(mrc.MrcFormatError):
        mrc.read_mrc(q)


def test_set_vox_size_prints_match_reference(golden_dir):
    pair = synth.workload_pair("pair128_s7_a30", seed=0)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        m1 = vg.mrc_obj.from_array(pair.map1, 1.0, pair.orig1)
        m2 = vg.mrc_obj.from_array(pair.map2, 1.0, pair.orig2)
        _, n1 = vg.mrc_set_vox_size(m1, 0.1, 7.0)
        _, n2 = vg.mrc_set_vox_size(m2, 0.1, 7.0)
    ref = open(os.path.join(golden_dir, "search_pair128_setup.txt")).read()
    assert ref.startswith(buf.getvalue())
    g = np.load(os.path.join(golden_dir, "search_pair128.npz"))
    cli._unify(n1, n2, 7.0)
    assert n1.xdim == int(g["dim"]) and np.array_equal(n1.orig, g["orig1"]) and np.array_equal(n2.orig, g["orig2"])


def test_empty_map_raises_like_reference():
    m = vg.mrc_obj.from_array(np.zeros((8, 8, 8), np.float32))
    with pytest.raises(ValueError):
        with contextlib.redirect_stdout(io.StringIO()):
            vg.mrc_set_vox_size(m, 0.1, 7.0)


def test_convert_trans_matches_oracle():
    cen1 = np.array([64.0, 64.0, 64.0])
    cen2 = np.array([60.5, 61.0, 59.0])
    for ang in ([240.0, 90.0, 355.0], [0.0, 0.0, 0.0], [35.0, 125.0, 270.0]):
        for tr in ((0, 0, 0), (12, 1, 7), (6, 7, 12)):
            a = vg.convert_trans(cen1, cen2, vg.euler2rot(ang), tr, 7.0, 13)
            b = orc.convert_trans(cen1, cen2, orc.euler2rot(ang), tr, 7.0, 13)
            assert np.array_equal(a, b)


def test_cli_defaults_and_quirks():
    p = cli.build_parser()
    a = p.parse_args(["orig", "-a", "x.mrc", "-b", "y.mrc"])
    assert (a.t, a.T, a.g, a.s, a.A, a.N, a.S, a.M, a.E, a.o) == (None, None, 16.0, 7.0, 30.0, 10, False, "V", False,
                                                                  None)
    a = p.parse_args(["orig", "-a", "x", "-b", "y", "-S", "False", "-A", "15"])
    assert a.S is True and isinstance(a.A, float)  # type=bool: any non-empty string is True
    b = p.parse_args(["prob", "-a", "x", "-npa", "p", "-b", "y", "-npb", "q"])
    assert (b.alpha, b.P, b.vav, b.vstd, b.pav, b.pstd) == (0.5, 4, None, None, None, None)
    with pytest.raises(SystemExit):
        with contextlib.redirect_stderr(io.StringIO()):
            p.parse_args(["orig", "-a", "x"])


def test_show_vec_format(tmp_path):
    rng = np.random.default_rng(1)
    d = 5
    data = np.where(rng.random((d, d, d)) < 0.3, rng.uniform(0.5, 2, (d, d, d)), 0.0)
    vec = rng.normal(size=(d, d, d, 3)).astype(np.float32)
    sco = rng.normal(size=(d, d, d))
    vg.show_vec(np.array([1.0, 2.0, 3.0]), vec, data, sco, 12.3456, 7.0, (4, 1, 0), (0, 0, 0), tmp_path, 3)
    f = tmp_path / "R_03-S__12.346.pdb"
    lines = f.read_text().splitlines()
    nz = np.argwhere(data != 0)
    assert len(lines) == 2 * len(nz)
    add = np.array([1.0, 2.0, 3.0]) - np.array([-1, 1, 0]) * 7.0
    x, y, z = nz[0]
    tmp = np.array([x, y, z]) * 7.0 + add
    assert lines[0] == "ATOM{:>7d}  CA  ALA{:>6d}    ".format(1, 1) + "{:8.3f}{:8.3f}{:8.3f}{:6.2f}{:6.2f}".format(
        tmp[0], tmp[1], tmp[2], 1.0, sco[x, y, z])
    assert lines[1].startswith("ATOM      2  CB  ALA     1    ")


def test_shard_merge_equals_global_stable_topn():
    rng = np.random.default_rng(2)
    scores = rng.integers(0, 40, 1000).astype(np.float32)  # many exact ties
    ref = orc.topn(scores, 25)
    for world in (1, 2, 3, 4, 7):
        parts = []
        for r in range(world):
            lo, hi = shard.shard_range(len(scores), r, world)
            parts.append(shard.local_topn(scores[lo:hi], 25, lo))
        _, ix = shard.merge_topn(parts, 25)
        assert np.array_equal(ix, ref), world
    assert shard.shard_range(10, 0, 3) == (0, 4) and shard.shard_range(10, 2, 3) == (7, 10)


def test_workload_generator_is_deterministic():
    a = synth.make_pair(5, 32, 20, 10.0)
    b = synth.make_pair(5, 32, 20, 10.0)
    assert np.array_equal(a.map1, b.map1) and np.array_equal(a.map2, b.map2)
    assert a.map1.shape == (32, 32, 32) and a.map2.shape == (16, 16, 16)
    p = synth.make_pair(5, 32, 20, 10.0, with_prob=True)
    assert p.prob1.shape == (32, 32, 32, 4)
    s = p.prob1.sum(-1)
    assert np.allclose(s[p.map1 >= 0.1], 1.0, atol=1e-5) and np.all(s[p.map1 < 0.1] == 0)


def test_refine_angle_list_equals_oracle_loop():
    """The vectorised refinement set equals the reference-order loop (oracle)."""
    from vesper_python_gb300 import vesper as vg
    rng = np.random.default_rng(3)
    for A in (10.0, 15.0, 30.0):
        grid = vg.calc_angle_comb(A)
        for _ in range(50):
            tops = [grid[i] for i in rng.choice(len(grid), 10, replace=False)]
            a = vg.refine_angle_list(tops)
            b = orc.refine_angles(tops)
            assert a.dtype == b.dtype and np.array_equal(a, b)


def test_lattice_rows_equal_rot_matrices():
    """Rows of the 5-degree lattice table are the rotation matrices of the
    refinement angles bit for bit; off-lattice angles are refused."""
    from vesper_python_gb300 import vesper as vg
    rng = np.random.default_rng(4)
    grid = vg.calc_angle_comb(15.0)
    tops = [grid[i] for i in rng.choice(len(grid), 10, replace=False)]
    ref = vg.refine_angle_list(tops)
    idx = vg.lattice_index(ref)
    k = np.arange(vg.LATTICE_N) * vg.LATTICE_STEP
    lat = np.stack(np.meshgrid(k, k, k, indexing="ij"), -1).reshape(-1, 3)
    assert np.array_equal(lat[idx], ref)
    assert np.array_equal(vg.rot_matrices(lat[idx]), vg.rot_matrices(ref))
    assert vg.lattice_index(np.array([[7.0, 0.0, 0.0]])) is None
    assert vg.lattice_index(np.array([[360.0, 0.0, 0.0]])) is None


def test_model_translation_is_convert_trans():
    """Model.translation (computed on first use) is convert_trans of its
    angle and translation, as the reference prints it."""
    from vesper_python_gb300 import align
    m = align.Model((30.0, 60.0, 90.0), 1.0, (3, 20, 1), 0.5, 0.1, 0.2, 3.0,
                    (np.array([10.0, 20.0, 30.0]), np.array([5.0, 6.0, 7.0]), 3.0, 24))
    want = orc.convert_trans(np.array([10.0, 20.0, 30.0]), np.array([5.0, 6.0, 7.0]),
                             orc.euler2rot((30.0, 60.0, 90.0)), (3, 20, 1), 3.0, 24)
    assert np.array_equal(m.translation, want)


def test_distinct_lattice_rows_expand_back():
    """Refinement sets searched once per distinct angle: every entry of every
    pair's list maps back to its own lattice row within its pair's block."""
    from vesper_python_gb300 import align
    from vesper_python_gb300 import vesper as vg
    ac = vg.calc_angle_comb(10.0)
    rng = np.random.default_rng(4)
    sets = []
    for _ in range(5):   # clustered top-N (many overlaps) and scattered ones
        base = int(rng.integers(0, len(ac) - 1300))
        sets.append(vg.refine_angle_list([ac[base + o] for o in (0, 1, 36, 37, 1296, 2, 3, 38, 72, 1297)]))
        sets.append(vg.refine_angle_list([ac[i] for i in rng.integers(0, len(ac), 10)]))
    key = vg.lattice_index(np.concatenate(sets))
    rows, counts, local = align.distinct_lattice_rows(key, [len(s) for s in sets])
    assert counts.sum() == len(rows) and len(local) == len(key)
    off = ioff = 0
    for s, c in zip(sets, counts):
        blk = rows[off:off + c]
        assert np.all(np.diff(blk) > 0)          # distinct within the pair
        assert np.array_equal(blk[local[ioff:ioff + len(s)]], vg.lattice_index(s))
        off += c
        ioff += len(s)
    assert counts[0] < len(sets[0])              # the clustered set repeats angles


def test_pack_bytes_round_trip():
    """The packed device-to-host read-back: mixed dtypes and shapes (odd byte
    counts padded to 8) come back equal."""
    import torch
    from vesper_python_gb300 import align
    ts = [torch.arange(5, dtype=torch.float32), torch.arange(3, dtype=torch.int32),
          torch.arange(6, dtype=torch.int64).reshape(2, 3), torch.ones((2, 2, 2), dtype=torch.float64),
          torch.arange(7, dtype=torch.int16), torch.zeros(0, dtype=torch.float32)]
    packed, layout = align.pack_bytes(ts)
    assert packed.dtype == torch.uint8 and all(off % 8 == 0 for off, _, _ in layout)
    back = align.unpack_bytes(packed.numpy(), layout)
    for t, a in zip(ts, back):
        assert a.shape == tuple(t.shape) and np.array_equal(a, t.numpy())
    assert align.pack_bytes([]) == (None, [])


def test_set_vox_size_cases_match_reference(golden_dir):
    """mrc_set_vox_size of the package against the reference's own results on
    small maps with negative values: thresholds 0, 0.25 and -0.3 (dens shifted,
    data clipped at 0), voxel sizes 2 and 5, a non-cubic map with a non-zero
    origin: identical printed lines, thresholded data and dens (by digest), and
    new grid (xdim, orig, cent)."""
    import contextlib
    import hashlib
    import io
    from vesper_python_gb300 import vesper as vg
    g = np.load(f"{golden_dir}/voxsize_cases.npz")

    def digest(a):
        return hashlib.sha1(np.ascontiguousarray(a).tobytes()).hexdigest()

    for k in range(int(g["ncase"])):
        si, width, o0, o1, o2, th, vs = g[f"c{k}_params"]
        m = vg.mrc_obj.from_array(g[f"src{int(si)}"], float(width), (o0, o1, o2))
        buf = io.StringIO()
        with contextlib.redirect_stdout(buf):
            m, n = vg.mrc_set_vox_size(m, float(th), float(vs))
        assert buf.getvalue() == str(g[f"c{k}_print"]), k
        assert digest(np.asarray(m.data, np.float32)) == str(g[f"c{k}_digest"][0]), k
        assert digest(np.asarray(m.dens, np.float64).reshape(-1)) == str(g[f"c{k}_digest"][1]), k
        assert np.array_equal(np.array([n.xdim, *n.orig, *n.cent], np.float64), g[f"c{k}_grid"]), k


def test_show_vec_writes_the_reference_files(golden_dir, tmp_path):
    """show_vec writes the same file name and the same bytes as the
    reference's writer (two models: a translation past d/2 and a negative
    score)."""
    from vesper_python_gb300 import vesper as vg
    g = np.load(f"{golden_dir}/show_vec_cases.npz")
    for k in range(2):
        p = g[f"c{k}_params"]
        origin, trans, score, rank = p[0:3], tuple(int(v) for v in p[3:6]), float(p[6]), int(p[7])
        out = tmp_path / f"case{k}"
        out.mkdir()
        vg.show_vec(origin, g[f"c{k}_vec"], g[f"c{k}_data"], g[f"c{k}_sco"], score, 7.0, trans, (0, 0, 0), out, rank)
        files = sorted(x.name for x in out.iterdir())
        assert files == [str(g[f"c{k}_name"])]
        assert (out / files[0]).read_text() == str(g[f"c{k}_text"])


def test_size_grids_matches_size_grid():
    """The aligner's batched grid sizing gives every map what the per-map
    mrc_set_vox_size step gives (the same float64 operations): sides, new
    origins and centres bit for bit, the float32 origins, and the empty-map
    error."""
    from vesper_python_gb300 import align
    rng = np.random.default_rng(5)
    for _ in range(50):
        n = int(rng.integers(1, 20))
        r2 = rng.uniform(10, 5000, size=(n, 2))
        prh = np.zeros((n, 4), np.uint64)
        prh[:, 0], prh[:, 2] = r2.view(np.uint64)[:, 0], r2.view(np.uint64)[:, 1]
        prh[:, 1], prh[:, 3] = 5, 7
        cents = [tuple(np.array([x * 0.5 for x in rng.integers(20, 300, 3)]) for _ in range(2)) for _ in range(n)]
        widths = [tuple(float(np.float32(rng.uniform(0.5, 3))) for _ in range(2)) for _ in range(n)]
        origs = [tuple(tuple(rng.uniform(-50, 50, 3)) for _ in range(2)) for _ in range(n)]
        s = float(rng.choice([2.0, 3.0, 4.0, 7.0]))
        dims, norig, ncent, o32 = align._size_grids(prh, cents, widths, origs, s)
        for i in range(n):
            for m in range(2):
                o = np.array([np.float32(v) for v in origs[i][m]])
                d, no, c = align._size_grid(prh[i, 2 * m], prh[i, 2 * m + 1], cents[i][m], widths[i][m], o, s)
                assert d == dims[i][m]
                assert np.array_equal(no, norig[i, m]) and no.dtype == norig.dtype
                assert np.array_equal(c, ncent[i, m]) and c.dtype == ncent.dtype
                assert np.array_equal(o, o32[i, m]) and o.dtype == o32.dtype
    prh[0, 3] = 0
    with pytest.raises(ValueError, match="empty sequence"):
        align._size_grids(prh, cents, widths, origs, s)


def test_lattice_angle_inverts_lattice_index():
    """The aligner's angle of a 5-degree lattice row (the refined models'
    rotations) is the angle whose lattice row it is, as numpy float64
    degrees, and repeated rows return the same tuple."""
    from vesper_python_gb300 import align
    al = align.Aligner.__new__(align.Aligner)     # no device needed for the lattice arithmetic
    rng = np.random.default_rng(3)
    rows = rng.integers(0, vg.LATTICE_N ** 3, size=200).tolist() + [0, vg.LATTICE_N ** 3 - 1]
    angles = [al._lattice_angle(r) for r in rows]
    assert all(type(v) is np.float64 for a in angles for v in a)
    assert vg.lattice_index(np.array(angles)).tolist() == rows
    assert al._lattice_angle(rows[0]) is angles[0]


def test_autotune_candidates():
    """Every side tries batches 8..256 with both channel chunks and both
    column widths; batches above 256 only while one batch's spectra (S + U)
    stay within the L2-sized cap."""
    from vesper_python_gb300 import autotune
    for d, nch, ngrp in ((75, 3, 1), (44, 3, 1), (64, 7, 2), (32, 3, 1), (12, 1, 1)):
        cands = autotune.candidates(nch, d, ngrp)
        per = (nch + ngrp) * d * d * (d // 2 + 1) * 8
        batches = sorted({c["batch"] for c in cands})
        want = [b for b in autotune.BATCHES if b <= 256 or b * per <= autotune.BATCH_BYTES]
        assert batches == want
        assert {8, 16, 32, 64, 128, 256} <= set(batches)
        for b in batches:
            shapes = {(c["cchunk"], c["W"]) for c in cands if c["batch"] == b}
            assert shapes == {(cc, w) for cc in {1, nch} for w in (16, 32)}
    assert max(c["batch"] for c in autotune.candidates(1, 12, 1)) == 2048
    assert max(c["batch"] for c in autotune.candidates(3, 75, 1)) == 256


def test_side_groups_smallest_first_ties_in_order():
    """Pairs grouped by pooled side, the smallest group first and groups of
    equal size in order of their first pair."""
    import types
    from vesper_python_gb300 import align
    p = types.SimpleNamespace(proposal_pool=2)
    P = [types.SimpleNamespace(dim=d, name=i) for i, d in enumerate((28, 30, 32, 30, 28, 30, 27))]
    groups = align.Aligner._side_groups(P, p)
    assert [s for s, _ in groups] == [16, 14, 15]
    assert [[st.name for st in g] for _, g in groups] == [[2], [0, 4, 6], [1, 3, 5]]
    P2 = [types.SimpleNamespace(dim=d) for d in (32, 28)]
    assert [s for s, _ in align.Aligner._side_groups(P2, p)] == [16, 14]


def test_batch_sig_tracks_what_a_captured_stage_reads():
    """The graph cache key changes with any map address or shape, grid
    geometry, parameter or angle grid, and not otherwise."""
    import dataclasses
    import types

    import torch

    from vesper_python_gb300 import align

    def pair(a, b, dim=30, w=1.0):
        return types.SimpleNamespace(src1=a, src2=b, dim=dim, no1=np.array([1.0, 2.0, 3.0]),
                                     no2=np.array([4.0, 5.0, 6.0]), width1=w, width2=w,
                                     o1=np.array([0.0, 0.0, 0.0]), o2=np.array([1.0, 1.0, 1.0]))
    m1, m2, m3 = torch.zeros(8, 8, 8), torch.zeros(4, 4, 4), torch.zeros(4, 4, 4)
    mats, mats2 = torch.zeros(10, 3, 3), torch.zeros(10, 3, 3)
    p = align.AlignParams()
    sig = align.Aligner._batch_sig
    base = sig([pair(m1, m2)], p, mats)
    assert sig([pair(m1, m2)], p, mats) == base
    assert sig([pair(m1, m3)], p, mats) != base                    # another query map buffer
    assert sig([pair(m1, m2, dim=32)], p, mats) != base            # another grid side
    assert sig([pair(m1, m2, w=2.0)], p, mats) != base             # another voxel width
    assert sig([pair(m1, m2), pair(m1, m2)], p, mats) != base      # another pair count
    assert sig([pair(m1, m2)], p, mats2) != base                   # another angle grid
    assert sig([pair(m1, m2)], dataclasses.replace(p, N=p.N + 1), mats) != base
    assert sig([pair(m1, m2)], dataclasses.replace(p, A=p.A + 5), mats) != base
