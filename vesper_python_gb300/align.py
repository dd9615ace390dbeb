"""One full pair alignment on the device, the unit of throughput
("map-pair alignments/s"): the work of ``main.py orig`` (main.py:158-206 and
search_map_fft, VESPER_1_prob_new.py:568-795) minus file I/O and printing:

  1. threshold + radius of both maps        vesper_prepare_map   (:59-118)
  2. grid sizing / unification              host (next_fast_len, main.py:166-185)
  3. fastVEC of both maps                   vesper_fastvec       (:145-257)
  4. target statistics + spectra            vesper_map_stats, vesper_target_spectra (:157-161, :601-628)
  5. rotational search over the angle grid  vesper_search        (:644-655)
  6. top-N, refinement angle set, search    vesper_topn + host + vesper_search (:664, :689-739)
  7. rotated top-N models + float64 scores  vesper_rot_gather + vesper_rescore (:756-781)

``align_device`` takes maps already resident on the GPU; ``align_host``
takes host arrays, copies them in each call and returns host results (the
end-to-end form).
"""
from __future__ import annotations

import ctypes
import dataclasses

import numpy as np
import torch

from . import _native
from . import vesper as vg


@dataclasses.dataclass
class AlignParams:
    t: float = 0.0
    T: float = 0.0
    g: float = 16.0
    s: float = 7.0
    A: float = 30.0
    N: int = 10
    mode: str = "VecProduct"
    batch: int = 0
    # learned rotation proposal (mode V only): a proposal.ProposalNet, the
    # fraction of the grid it hands to the exact search, the pooling of its
    # input fields, and the fallback threshold (exhaustive search when the
    # subset's best exact score is less than fallback_z standard deviations
    # above the subset's mean; None: never)
    proposal: object = None
    proposal_frac: float = 0.05
    proposal_pool: int = 2
    proposal_fallback_z: float | None = 5.0


@dataclasses.dataclass
class Model:
    angle: tuple
    vec_score: float
    vec_trans: tuple
    translation: np.ndarray      # converted translation (A), as printed
    overlap: float
    cc: float
    pcc: float
    dot_score: float             # float64 "Score=" of get_score


@dataclasses.dataclass
class AlignResult:
    dim: int
    std: float
    ave: float
    top: list                    # global-pass top-N (angle, vec_score, vec_trans)
    models: list                 # refined top-N Model
    launches: int = 0


def _size_grid(dmax2_bits, count, cent, width, orig, s):
    """mrc_set_vox_size (VESPER_1_prob_new.py:81-100) from the device radius."""
    if count == 0:
        raise ValueError("max() arg is an empty sequence")
    dmax = float(np.sqrt(np.frombuffer(np.uint64(dmax2_bits).tobytes(), dtype=np.float64)[0]))
    dmax = dmax * np.float64(width)
    new_cent = cent * np.float64(width) + orig
    new_dim = vg.next_fast_len(int(2 * dmax / s))
    new_orig = new_cent - 0.5 * new_dim * s
    return new_dim, new_orig, new_cent


class Aligner:
    """Holds the device, cached angle-grid matrices and scratch buffers."""

    def __init__(self, dev: vg.Device | None = None):
        self.dev = dev or vg.default_device()
        self.lib = self.dev.lib
        self.launches = 0
        self.d2h_bytes = 0
        self.profile = None      # set to a dict to collect per-pass search timings
        self.stages = None       # set to a dict to collect per-stage device milliseconds
        self._marks = []
        self._prep = torch.empty(4, dtype=torch.int64, device=self.dev.device)
        self._stats = torch.empty(5, dtype=torch.float64, device=self.dev.device)

    def _mark(self, name):
        """Event at a stage boundary (only while self.stages is a dict)."""
        if self.stages is not None:
            e = torch.cuda.Event(enable_timing=True)
            e.record()
            self._marks.append((name, e))

    def _close_marks(self):
        if self.stages is None or not self._marks:
            return
        self._marks[-1][1].synchronize()
        for (name, e0), (_, e1) in zip(self._marks[:-1], self._marks[1:]):
            self.stages[name] = self.stages.get(name, 0.0) + e0.elapsed_time(e1)
        self._marks = []

    def _prepare(self, src, th, cent, out):
        sx, sy, sz = src.shape
        _native.check(self.lib.vesper_prepare_map(ctypes.c_void_p(src.data_ptr()), sx, sy, sz, float(th),
                                                  vg._host_d3(cent), ctypes.c_void_p(out.data_ptr()),
                                                  self.dev.stream))
        self.launches += 2

    def align_device(self, src1, src2, width1, width2, orig1, orig2, p: AlignParams) -> AlignResult:
        dev = self.dev
        mode = p.mode
        self.launches = 0
        self.d2h_bytes = 0
        cent1 = np.array([s * 0.5 for s in src1.shape])
        cent2 = np.array([s * 0.5 for s in src2.shape])
        self._mark("prepare")
        self._prepare(src1, p.t, cent1, self._prep[0:2])
        self._prepare(src2, p.T, cent2, self._prep[2:4])
        pr = self._prep.cpu().numpy().view(np.uint64)
        self.d2h_bytes += self._prep.numel() * 8
        o1 = np.array([np.float32(v) for v in orig1])
        o2 = np.array([np.float32(v) for v in orig2])
        d1, no1, c1 = _size_grid(pr[0], pr[1], cent1, width1, o1, p.s)
        d2, no2, c2 = _size_grid(pr[2], pr[3], cent2, width2, o2, p.s)
        if d1 > d2:
            dim = d1
            no2 = c2 - 0.5 * p.s * dim
        else:
            dim = d2
            no1 = c1 - 0.5 * p.s * dim
        self._mark("fastvec")
        tdata, _, tvec = vg.fastvec_device(src1, np.float64(np.float32(width1)), o1.astype(np.float64), dim, p.s,
                                           no1, p.g, dev=dev)
        qdata, _, qvec = vg.fastvec_device(src2, np.float64(np.float32(width2)), o2.astype(np.float64), dim, p.s,
                                           no2, p.g, dev=dev)
        self.launches += 8
        _native.check(self.lib.vesper_map_stats(ctypes.c_void_p(tdata.data_ptr()), dim,
                                                ctypes.c_void_p(self._stats.data_ptr()), dev.stream))
        self.launches += 1
        stats = None
        ave = 0.0
        if mode in ("PCC", "CC"):
            stats = self._stats.cpu().numpy()
            self.d2h_bytes += 40
            ave = float(stats[2])
        self._mark("spectra")
        spec = vg.target_spectra_device(tdata, tvec, mode, ave, dev=dev)
        self.launches += 2
        angle_comb = vg.calc_angle_comb(p.A)
        mats = vg.rot_matrices_device(angle_comb, dev, key=("grid", float(p.A)))
        grid_index = None
        self.proposal_info = None
        if p.proposal is not None:
            scores, lin, grid_index = self._proposal_pass(p, spec, tdata, tvec, qdata, qvec, mats, dim, ave)
        if grid_index is None:
            self._mark("search")
            scores, lin = vg.search_device(spec, qdata, qvec, mode, ave, mats, batch=p.batch, dev=dev,
                                           profile=self.profile, tuned=True)
            self.launches += self._search_launches(dim, mode, len(angle_comb), p.batch)
        top = vg.topn_device(scores, p.N, dev=dev)
        self.launches += 1
        raw = scores[:, 0].cpu().numpy()
        lin_h = lin[:, 0].cpu().numpy()
        top_h = [int(i) for i in top.cpu().numpy() if i >= 0]
        self.d2h_bytes += raw.nbytes + lin_h.nbytes + top.numel() * 4
        raw_grid, lin_grid = raw, lin_h
        if grid_index is not None:
            # subset positions -> grid indices (the subset is in ascending grid order)
            gi = grid_index.cpu().numpy()
            self.d2h_bytes += gi.nbytes
            raw_grid = np.zeros(len(angle_comb), raw.dtype)
            lin_grid = np.zeros(len(angle_comb), lin_h.dtype)
            raw_grid[gi] = raw
            lin_grid[gi] = lin_h
            top_h = [int(gi[i]) for i in top_h]
        if stats is None:
            stats = self._stats.cpu().numpy()
            self.d2h_bytes += 40
        rd3 = 1.0 / dim ** 3
        scale = 1.0
        if mode == "CC":
            scale = 1.0 / stats[3] ** 2
        elif mode == "PCC":
            scale = 1.0 / stats[4] ** 2
        # statistics over the correlated rotations (the whole grid, or the subset)
        score_arr = raw.astype(np.float64) * scale * rd3
        ave_s, std_s = float(np.mean(score_arr)), float(np.std(score_arr))
        score_grid = raw_grid.astype(np.float64) * scale * rd3
        top_list = [(tuple(angle_comb[r]), float(score_grid[r]), vg.unravel(lin_grid[r], dim)) for r in top_h]
        if p.A > 5.0:
            self._mark("refine")
            ref_angles = vg.refine_angle_list([angle_comb[r] for r in top_h])
            rmats = dev.to_dev(vg.rot_matrices(ref_angles))
            rs, rl = vg.search_device(spec, qdata, qvec, mode, ave, rmats, batch=p.batch, dev=dev, tuned=True)
            self.launches += self._search_launches(dim, mode, len(ref_angles), p.batch)
            rtop = vg.topn_device(rs, p.N, dev=dev)
            self.launches += 1
            rraw = rs[:, 0].cpu().numpy()
            rlh = rl[:, 0].cpu().numpy()
            self.d2h_bytes += rraw.nbytes + rlh.nbytes + rtop.numel() * 4
            rtop = [int(i) for i in rtop.cpu().numpy() if i >= 0]
            sel_angles = ref_angles[rtop]
            entries = [(tuple(ref_angles[r]), float(np.float64(rraw[r]) * scale * rd3), vg.unravel(rlh[r], dim))
                       for r in rtop]
        else:
            sel_angles = np.array([e[0] for e in top_list])
            entries = top_list
        models = []
        self._mark("rescore")
        if entries:
            sel = dev.to_dev(vg.rot_matrices(sel_angles))
            gd, gv, _ = vg.rot_gather_device(qdata, qvec, sel, dev=dev)
            self.launches += 1
            nm_ = len(entries)
            res = torch.empty((nm_, 8), dtype=torch.float64, device=dev.device)
            # translations wrapped to (-d/2, d/2] as get_score does (:1323-1329)
            trw = np.array([[t - dim if t > 0.5 * dim else t for t in tr] for (_, _, tr) in entries], np.int32)
            trd = dev.to_dev(trw)
            ws = dev.workspace(("rescore", dim), _native.size_query("vesper_rescore_batch_workspace_size", dim, nm_))
            _native.check(self.lib.vesper_rescore_batch(
                ctypes.c_void_p(tdata.data_ptr()), ctypes.c_void_p(tvec.data_ptr()), float(stats[2]),
                float(stats[3]), float(stats[4]), ctypes.c_void_p(gd.data_ptr()), ctypes.c_void_p(gv.data_ptr()),
                dim, ctypes.c_void_p(trd.data_ptr()), nm_, ctypes.c_void_p(res.data_ptr()),
                ctypes.c_void_p(ws.data_ptr()), ws.numel(), dev.stream))
            self.launches += 4
            rh = res.cpu().numpy()
            self.d2h_bytes += rh.nbytes
            for k, (ang, sc, tr) in enumerate(entries):
                r = vg.euler2rot(ang)
                new_trans = vg.convert_trans(c1, c2, r, tr, p.s, dim)
                nm, total = rh[k, 0], rh[k, 1]
                models.append(Model(ang, sc, tr, new_trans, float(nm / total), float(rh[k, 2]), float(rh[k, 3]),
                                    float(rh[k, 4])))
        self._mark("end")
        self._close_marks()
        return AlignResult(dim, std_s, ave_s, top_list, models, self.launches)

    def _proposal_pass(self, p, spec, tdata, tvec, qdata, qvec, mats, dim, ave):
        """Global pass of the learned proposal: network scores of every
        rotation, exact search of the best fraction.  Returns (scores, lin,
        grid indices of the subset), or (None, None, None) when the fallback
        rule sends the pair to the exhaustive search."""
        from . import proposal as prop
        if p.mode != "VecProduct":
            raise ValueError("the learned proposal ranks rotations for mode VecProduct only")
        dev = self.dev
        self._mark("proposal")
        pool = int(p.proposal_pool)
        dp = (dim + pool - 1) // pool
        fTQ = torch.empty((2, 4, dp, dp, dp), dtype=torch.float32, device=dev.device)
        prop.map_field(tdata, tvec, pool, dev, out=fTQ[0])
        prop.map_field(qdata, qvec, pool, dev, out=fTQ[1])
        s = p.proposal.rotation_scores(fTQ, mats)
        order = prop.subset_from_scores(dev, s, p.proposal_frac).to(torch.int64)
        sub = mats.index_select(0, order)
        self._mark("search")
        scores, lin = vg.search_device(spec, qdata, qvec, p.mode, ave, sub, batch=p.batch, dev=dev,
                                       profile=self.profile, tuned=True)
        self.launches += 2 + 4 + 1 + 1 + 1 + self._search_launches(dim, p.mode, int(order.numel()), p.batch)
        sc0 = scores[:, 0]
        z = float(((sc0.max() - sc0.mean()) / (sc0.std() + 1e-30)).item())
        self.d2h_bytes += 4
        self.proposal_info = {"subset": int(order.numel()), "z": z, "fallback": False}
        if p.proposal_fallback_z is not None and z < p.proposal_fallback_z:
            self.proposal_info["fallback"] = True
            return None, None, None
        return scores, lin, order

    def _search_launches(self, dim, mode, nrot, batch):
        if batch <= 0:
            from . import autotune
            t = autotune.cached(dim, mode, self.dev)
            if t and t.get("batch"):
                batch = int(t["batch"])
        return vg.search_plan(dim, mode, batch, nrot, None, self.dev)[1]

    def align_host(self, map1, map2, width1, width2, orig1, orig2, p: AlignParams, pinned=None):
        """End-to-end: host [x][y][z] float32 maps (pinned if given) -> results."""
        dev = self.dev
        if pinned is None:
            h1 = torch.from_numpy(np.ascontiguousarray(map1, np.float32))
            h2 = torch.from_numpy(np.ascontiguousarray(map2, np.float32))
        else:
            h1, h2 = pinned
        s1 = h1.to(dev.device, non_blocking=True)
        s2 = h2.to(dev.device, non_blocking=True)
        return self.align_device(s1, s2, width1, width2, orig1, orig2, p)
