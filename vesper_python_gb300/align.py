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
import functools

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
    overlap: float
    cc: float
    pcc: float
    dot_score: float             # float64 "Score=" of get_score
    geom: tuple = dataclasses.field(default=None, repr=False)   # (centre 1, centre 2, voxel spacing, side)

    @functools.cached_property
    def translation(self) -> np.ndarray:
        """The converted translation (A) as main.py prints it (convert_trans,
        VESPER_1_prob_new.py:1554-1566), computed when first asked for."""
        c1, c2, s, dim = self.geom
        return vg.convert_trans(c1, c2, vg.euler2rot(self.angle), self.vec_trans, s, dim)


@dataclasses.dataclass
class AlignResult:
    dim: int
    std: float
    ave: float
    top: list                    # global-pass top-N (angle, vec_score, vec_trans)
    models: list                 # refined top-N Model
    launches: int = 0


_NP_DTYPES = {torch.float32: np.dtype(np.float32), torch.float64: np.dtype(np.float64),
              torch.int32: np.dtype(np.int32), torch.int64: np.dtype(np.int64), torch.int16: np.dtype(np.int16),
              torch.uint8: np.dtype(np.uint8)}


def pack_bytes(tensors):
    """The bytes of ``tensors`` (any dtypes in _NP_DTYPES) in one uint8 tensor
    on their device, each piece starting 8-byte aligned, and the layout
    [(offset, dtype, shape)] that unpack_bytes reads back; (None, []) for no
    tensors."""
    pieces, layout, off = [], [], 0
    for t in tensors:
        b = t.contiguous().reshape(-1).view(torch.uint8)
        pad = (-b.numel()) % 8
        pieces.append(b)
        if pad:
            pieces.append(torch.empty(pad, dtype=torch.uint8, device=b.device))   # filler, never read
        layout.append((off, _NP_DTYPES[t.dtype], tuple(t.shape)))
        off += b.numel() + pad
    return (torch.cat(pieces) if pieces else None), layout


def unpack_bytes(buf, layout):
    """numpy copies of the tensors packed by pack_bytes, from its bytes ``buf``."""
    out = []
    for off, dt, shape in layout:
        n = int(np.prod(shape, dtype=np.int64)) * dt.itemsize
        out.append(buf[off:off + n].view(dt).reshape(shape).copy())
    return out


def distinct_lattice_rows(key, lens):
    """Distinct lattice rows of consecutive angle lists (list i has lens[i]
    entries; key = their lattice rows, concatenated): the distinct rows pair by
    pair (ascending within a pair), their count per pair, and for every entry
    its position within its pair's distinct rows."""
    lens = np.asarray(lens, np.int64)
    span = vg.LATTICE_N ** 3
    pid = np.repeat(np.arange(len(lens), dtype=np.int64), lens)
    ukeys, inv = np.unique(pid * span + np.asarray(key, np.int64), return_inverse=True)
    counts = np.bincount(ukeys // span, minlength=len(lens))
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
    return ukeys % span, counts, inv.reshape(-1) - starts[pid]


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


def _size_grids(prh, cents, widths, origs, s):
    """_size_grid of both maps of every pair at once: prh uint64 [n][4] (radius
    bits and count of map 1, then map 2), cents / widths / origs per pair and
    map.  The same float64 operations element by element; returns the sides
    (int [n][2]), new origins and centres (float64 [n][2][3]) and the origins
    as float32 [n][2][3]."""
    n = len(cents)
    q = np.asarray(prh, np.uint64).reshape(n, 2, 2)
    if (q[:, :, 1] == 0).any():
        raise ValueError("max() arg is an empty sequence")
    dmax = np.sqrt(np.ascontiguousarray(q[:, :, 0]).view(np.float64))
    dmax = dmax * np.array(widths, np.float64)
    o32 = np.asarray(origs, np.float64).astype(np.float32)   # each value rounded to float32 (np.float32(v))
    cent = np.array(cents, np.float64) * np.array(widths, np.float64)[:, :, None] + o32
    raw = (2 * dmax / s).astype(np.int64)          # int() of each (positive) value
    dl = [[_fast_len(v) for v in row] for row in raw.tolist()]
    dims = np.array(dl, np.int64)
    norig = cent - 0.5 * dims[:, :, None] * s
    return dl, norig, cent, o32


@functools.lru_cache(maxsize=None)
def _fast_len(n):
    return vg.next_fast_len(n)


class _Pair:
    """Per-pair state of align_many between its stages."""

    def __init__(self, src1, src2, width1, width2, orig1, orig2):
        self.src1, self.src2 = src1, src2
        self.width1, self.width2 = width1, width2
        self.orig1, self.orig2 = orig1, orig2
        self.launches = 0
        self.order = None
        self.sub = None
        self.z = None
        self.fallback = False


class Aligner:
    """Holds the device, cached angle-grid matrices and scratch buffers."""

    def __init__(self, dev: vg.Device | None = None, group=None):
        self.dev = dev or vg.default_device()
        # torch.distributed process group: with one, every search splits its
        # rotations across the group's ranks (one GPU each) and gathers the
        # per-rotation results (vg.search_device_sharded); the CUDA-graph form
        # is then not used (the gather is a host exchange)
        self.group = group
        self.lib = self.dev.lib
        self.launches = 0
        self.d2h_bytes = 0
        self.profile = None      # set to a dict to collect per-pass search timings
        self.stages = None       # set to a dict to collect per-stage device milliseconds
        self._marks = []
        self._graphs = {}        # batch signature -> (CUDA graph, its statistics, per-pair outputs)
        self.graph_captures = 0
        self.graph_replays = 0
        self.pair_events = None  # set to a list to get one event per pair after its last kernel
        self._staging = {}       # (slot, shape) -> device buffer for host inputs

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

    def _prepare_all(self, P, p, prep):
        """vesper_prepare_maps over both maps of every pair: map 2i is pair
        i's first map, 2i + 1 its second; prep [n][4] receives their
        (radius bits, count) pairs in that order."""
        srcs = [t for st in P for t in (st.src1, st.src2)]
        # the argument arrays depend only on the maps' addresses and shapes and
        # the thresholds (the centres are half the shapes): kept for a repeat
        key = (tuple((t.data_ptr(), tuple(t.shape)) for t in srcs), float(p.t), float(p.T))
        args = self.__dict__.get("_prep_args")
        if args is None or args[0] != key:
            maps = [m for st in P for m in ((st.src1, p.t, st.cent1), (st.src2, p.T, st.cent2))]
            nm = len(maps)
            args = self._prep_args = (key, nm, (ctypes.c_void_p * nm)(*[m[0].data_ptr() for m in maps]),
                                      (ctypes.c_int * (3 * nm))(*[int(v) for m in maps for v in m[0].shape]),
                                      (ctypes.c_double * nm)(*[float(m[1]) for m in maps]),
                                      (ctypes.c_double * (3 * nm))(*[float(v) for m in maps for v in m[2]]))
        _, nm, ptrs, dims, ths, cents = args
        _native.check(self.lib.vesper_prepare_maps(nm, ptrs, dims, ths, cents, ctypes.c_void_p(prep.data_ptr()),
                                                   self.dev.stream))

    def align_device(self, src1, src2, width1, width2, orig1, orig2, p: AlignParams) -> AlignResult:
        """One pair: ``align_many`` with a batch of one."""
        return self.align_many([(src1, src2, width1, width2, orig1, orig2)], p)[0]

    def align_many(self, items, p: AlignParams, graph: bool = False) -> list:
        """Align a batch of pairs, items = [(src1, src2, width1, width2, orig1,
        orig2)] with device maps of any (uneven) sizes.  Every stage is launched
        for all pairs before the host waits: one wait for the grid sizes, one
        for the proposal's flatness test (learned proposal only), one for all
        results.  With graph=True the global stage and the refinement +
        rescoring stage each replay as one CUDA graph per batch signature
        (modes other than CC and PCC, whose spectra need a host value)."""
        dev = self.dev
        mode = p.mode
        self.launches = 0
        self.d2h_bytes = 0
        n = len(items)
        if n == 0:
            return []
        P = [_Pair(*it) for it in items]
        # ---- 1. threshold + radius (device), grid sizing (host) ----------------
        self._mark("prepare")
        prep = torch.empty((n, 4), dtype=torch.int64, device=dev.device)
        for st in P:
            st.cent1 = np.array([x * 0.5 for x in st.src1.shape])
            st.cent2 = np.array([x * 0.5 for x in st.src2.shape])
        self._prepare_all(P, p, prep)
        P[0].launches += (2 * n + 63) // 64      # one launch per 64 maps
        prh = prep.cpu().numpy().view(np.uint64)
        self.d2h_bytes += prep.numel() * 8
        # ---- 2. fastVEC, target statistics and spectra -------------------------
        dims, norig, ncent, origs = _size_grids(prh, [(st.cent1, st.cent2) for st in P],
                                                 [(st.width1, st.width2) for st in P],
                                                 [(st.orig1, st.orig2) for st in P], p.s)
        for i, st in enumerate(P):
            st.o1, st.o2 = origs[i, 0], origs[i, 1]
            st.no1, st.no2, st.c1, st.c2 = norig[i, 0], norig[i, 1], ncent[i, 0], ncent[i, 1]
            d1, d2 = dims[i]
            if d1 > d2:
                st.dim = d1
                st.no2 = st.c2 - 0.5 * p.s * st.dim
            else:
                st.dim = d2
                st.no1 = st.c1 - 0.5 * p.s * st.dim
        grids = self.__dict__.setdefault("_angle_grid_cache", {})   # the angle grid per step, read-only
        angle_comb = grids.get(float(p.A))
        if angle_comb is None:
            angle_comb = grids[float(p.A)] = vg.calc_angle_comb(p.A)
            angle_comb.setflags(write=False)
        nang = len(angle_comb)
        mats = vg.rot_matrices_device(angle_comb, dev, key=("grid", float(p.A)))
        if p.proposal is not None and mode != "VecProduct":
            raise ValueError("the learned proposal ranks rotations for mode VecProduct only")
        # ---- 2-3. fastVEC, statistics, spectra, global pass (one CUDA graph per
        # batch signature when graph=True: the stage needs no host value
        # between its launches except in modes CC/PCC) --------------------------
        if graph and mode not in ("PCC", "CC") and self.group is None:
            stats, sh = self._global_stage_graph(P, p, mats, nang), None
        else:
            stats, sh = self._global_stage(P, p, mats, nang)
        device_late = graph and mode not in ("PCC", "CC") and p.A > 5.0 and self.group is None and \
            self._grid_rows(p.A, angle_comb) is not None

        def global_results():
            # the global results go to the host while the refinement runs
            return self._fetch_start([[st.scores[:, 0].contiguous(), st.lin[:, 0].contiguous(), st.top] +
                                      ([st.order] if st.order is not None else []) for st in P], slot=0)

        gh = None
        zs = None
        if p.proposal is not None:
            zdev = torch.stack([st.z for st in P])
            if device_late:
                # the refinement graph is launched before the flatness test is
                # read back, so the device does not wait for the host; a pair
                # that falls back to the exhaustive search (rare) is refined
                # again below
                zh = self._fetch_start([[zdev]], slot=2)
                gh = global_results()
                self._late_stage_graph(P, p, stats, mats)
                zs = self._fetch_finish(zh)[0][0]
            else:
                zs = zdev.cpu().numpy()
                self.d2h_bytes += zs.nbytes
            redo = [st for st, z in zip(P, zs) if p.proposal_fallback_z is not None and z < p.proposal_fallback_z]
            for st in redo:       # the fallback: the whole grid
                st.order = None
                st.fallback = True
                self._global_search(p, st, mats, nang)
                st.tg.copy_(st.top.to(st.tg.dtype))     # top grid indices, read by the device late stage
            if redo and device_late:
                gh = global_results()
                self._late_stage_graph(P, p, stats, mats)
            self.proposal_info = {"subset": int(np.ceil(p.proposal_frac * nang)), "z": [float(z) for z in zs],
                                  "fallback": [bool(st.fallback) for st in P]}
        else:
            self.proposal_info = None
        if device_late:
            # refinement and rescoring on the device from the top indices, no
            # host value in between, replayed as one CUDA graph.  (Eager calls
            # keep the host-driven refinement below, which searches each
            # distinct angle once: fewer rotations, one more host round trip.)
            if gh is None:
                gh = global_results()
                self._late_stage_graph(P, p, stats, mats)
            return self._finish_device_late(P, p, gh, angle_comb)
        if sh is None:
            sh = stats.cpu().numpy()
            self.d2h_bytes += sh.nbytes
        # one wait for every pair's global results, then per pair: host
        # bookkeeping and the refinement launch (the device works on pair i
        # while the host prepares pair i+1)
        glob = self._fetch([[st.scores[:, 0].contiguous(), st.lin[:, 0].contiguous(), st.top] +
                            ([st.order] if st.order is not None else []) for st in P])
        rd3s, scales = [], []
        if p.A > 5.0:
            self._mark("refine")
        for i, st in enumerate(P):
            top_h = [int(t) for t in glob[i][2] if t >= 0]
            if st.order is not None:
                # subset positions -> grid indices (the subset is in ascending grid order)
                top_h = [int(glob[i][3][t]) for t in top_h]
            st.top_h = top_h
            rd3 = 1.0 / st.dim ** 3
            scale = 1.0
            if mode == "CC":
                scale = 1.0 / sh[i, 3] ** 2
            elif mode == "PCC":
                scale = 1.0 / sh[i, 4] ** 2
            rd3s.append(rd3)
            scales.append(scale)

        def global_lists():
            # statistics over the correlated rotations (the whole grid, or the
            # subset) and the global top-N list; run while the refinement
            # searches are on the device
            for i, st in enumerate(P):
                raw, lin_h = glob[i][0], glob[i][1]
                raw_grid, lin_grid = raw, lin_h
                if st.order is not None:
                    gi = glob[i][3]
                    raw_grid = np.zeros(nang, raw.dtype)
                    lin_grid = np.zeros(nang, lin_h.dtype)
                    raw_grid[gi] = raw
                    lin_grid[gi] = lin_h
                score_arr = raw.astype(np.float64) * scales[i] * rd3s[i]
                st.ave_s, st.std_s = float(np.mean(score_arr)), float(np.std(score_arr))
                score_grid = raw_grid.astype(np.float64) * scales[i] * rd3s[i]
                st.top_list = [(tuple(angle_comb[r]), float(score_grid[r]), vg.unravel(lin_grid[r], st.dim))
                               for r in st.top_h]

        # ---- 4. refinement around each pair's top-N: every pair's angle set and
        # matrices at once (one index copy and one gather from the lattice
        # table), then the searches.  The +-5 degree sets of neighbouring top-N
        # angles overlap and the reference keeps the duplicates (:689-713); a
        # rotation's result depends on its angle alone, so each distinct angle
        # is searched once and the results are expanded back to the full list
        # (same scores, same order, same stable top-N).
        if p.A > 5.0:
            sets = [vg.refine_angle_list([angle_comb[r] for r in st.top_h]) for st in P]
            allm, counts, inv_all = self._distinct_rotations(sets)
            off = ioff = 0
            for st, ra, nu in zip(P, sets, counts):
                st.ref_angles = ra
                rmats = allm[off:off + nu]
                sel = inv_all[ioff:ioff + len(ra)]
                off += nu
                ioff += len(ra)
                rs, rl = vg.search_device_sharded(st.spec, st.qdata, st.qvec, mode, st.ave, rmats, self.group,
                                                  batch=p.batch, dev=dev, tuned=True)
                st.launches += self._search_launches(st.dim, mode, nu, p.batch)
                st.rs, st.rl = rs.index_select(0, sel), rl.index_select(0, sel)
                st.rtop = vg.topn_device(st.rs, p.N, dev=dev)
                st.launches += 1
        global_lists()
        # ---- 5. rotated top-N models and their float64 scores -------------------
        if p.A > 5.0:
            ref = self._fetch([[st.rs[:, 0].contiguous(), st.rl[:, 0].contiguous(), st.rtop] for st in P])
        self._mark("rescore")
        for i, st in enumerate(P):
            if p.A > 5.0:
                rraw, rlh, rtoph = ref[i]
                rtop = [int(t) for t in rtoph if t >= 0]
                st.sel_angles = st.ref_angles[rtop]
                st.entries = [(tuple(st.ref_angles[r]), float(np.float64(rraw[r]) * scales[i] * rd3s[i]),
                               vg.unravel(rlh[r], st.dim)) for r in rtop]
            else:
                st.sel_angles = np.array([e[0] for e in st.top_list])
                st.entries = st.top_list
        # every pair's model matrices and wrapped translations in one copy each
        # (translations wrapped to (-d/2, d/2] as get_score does, :1323-1329)
        withm = [st for st in P if st.entries]
        if withm:
            selm = vg.rot_matrices_lattice(np.concatenate([np.asarray(st.sel_angles, np.float64).reshape(-1, 3)
                                                           for st in withm]), dev)
            trd_all = dev.to_dev_async(np.array([[t - st.dim if t > 0.5 * st.dim else t for t in tr]
                                                 for st in withm for (_, _, tr) in st.entries], np.int32))
        off = 0
        for i, st in enumerate(P):
            if not st.entries:
                continue
            dim = st.dim
            nm_ = len(st.entries)
            sel = selm[off:off + nm_]
            trd = trd_all[off:off + nm_]
            off += nm_
            gd, gv, _ = vg.rot_gather_device(st.qdata, st.qvec, sel, dev=dev)
            st.res = torch.empty((nm_, 8), dtype=torch.float64, device=dev.device)
            ws = dev.workspace(("rescore_batch", i, dim, nm_),
                               _native.size_query("vesper_rescore_batch_workspace_size", dim, nm_))
            _native.check(self.lib.vesper_rescore_batch(
                ctypes.c_void_p(st.tdata.data_ptr()), ctypes.c_void_p(st.tvec.data_ptr()), float(sh[i, 2]),
                float(sh[i, 3]), float(sh[i, 4]), ctypes.c_void_p(gd.data_ptr()), ctypes.c_void_p(gv.data_ptr()),
                dim, ctypes.c_void_p(trd.data_ptr()), nm_, ctypes.c_void_p(st.res.data_ptr()),
                ctypes.c_void_p(ws.data_ptr()), ws.numel(), dev.stream))
            st.launches += 5
            if self.pair_events is not None:
                e = torch.cuda.Event(enable_timing=True)
                e.record()
                self.pair_events.append(e)
        resh = self._fetch([[st.res] if st.entries else [] for st in P])
        out = []
        for i, st in enumerate(P):
            models = []
            if st.entries:
                rh = resh[i][0]
                for k, (ang, sc, tr) in enumerate(st.entries):
                    nm, total = rh[k, 0], rh[k, 1]
                    models.append(Model(ang, sc, tr, float(nm / total), float(rh[k, 2]), float(rh[k, 3]),
                                        float(rh[k, 4]), (st.c1, st.c2, p.s, st.dim)))
            self.launches += st.launches
            out.append(AlignResult(st.dim, st.std_s, st.ave_s, st.top_list, models, st.launches))
        # the coarse fields of each pair (device tensors), for callers that
        # score or inspect them further
        self.last_fields = [{"tdata": getattr(st, "tdata", None), "tvec": getattr(st, "tvec", None),
                             "qdata": getattr(st, "qdata", None), "qvec": getattr(st, "qvec", None),
                             "ave": float(getattr(st, "ave", 0.0))} for st in P]
        self._mark("end")
        self._close_marks()
        return out

    def _distinct_rotations(self, sets):
        """Matrices of the distinct angles of every pair's angle list (pair by
        pair, consecutive), their count per pair, and for every entry of the
        concatenated lists its row within its pair's block (device int64):
        entry j of pair i is row inv[j] of that pair's distinct matrices."""
        dev = self.dev
        lens = np.array([len(ra) for ra in sets], np.int64)
        allang = np.concatenate(sets) if len(sets) else np.zeros((0, 3))
        key = vg.lattice_index(allang)
        if key is None:     # off the 5-degree lattice: per pair, on the angles
            uniq = [np.unique(ra, axis=0, return_inverse=True) for ra in sets]
            allm = vg.rot_matrices_lattice(np.concatenate([u for u, _ in uniq]), dev)
            inv = np.concatenate([iv.reshape(-1) for _, iv in uniq]).astype(np.int64)
            return allm, [len(u) for u, _ in uniq], dev.to_dev_async(inv)
        rows, counts, local = distinct_lattice_rows(key, lens)
        allm = vg.lattice_rot_matrices_device(dev).index_select(0, dev.to_dev_async(rows))
        return allm, [int(c) for c in counts], dev.to_dev_async(local)

    FV_STREAMS = 8
    GLOBAL_SIDE = True       # the proposal form's global searches on the side streams too

    def _side_streams(self):
        if getattr(self, "_side", None) is None:
            self._side = [torch.cuda.Stream(self.dev.device) for _ in range(self.FV_STREAMS)]
        return self._side

    def _global_stage(self, P, p, mats, nang):
        """fastVEC of both maps, target statistics and spectra, proposal subset
        and global search of every pair (device work only, except the
        statistics read that modes CC/PCC need before their spectra)."""
        dev = self.dev
        mode = p.mode
        n = len(P)
        for st in P:
            st.tg = None     # made below (each run of the stage, captured or not)
        self._mark("fastvec")
        stats = torch.empty((n, 5), dtype=torch.float64, device=dev.device)
        # fastVEC and statistics of the pairs on FV_STREAMS side streams: one
        # map's kernels fill only part of the GPU (latency-bound, 10^2-10^3
        # blocks), so pairs overlap; the streams fork from and join the current
        # stream (also inside a CUDA-graph capture)
        cur = torch.cuda.current_stream(dev.device)
        capturing = torch.cuda.is_current_stream_capturing()   # the graph's pool keeps its blocks
        side = self._side_streams()
        # with the learned proposal the pairs go to the streams grouped by
        # pooled side, in the order the network scores the sides, and the
        # network waits only for its side's pairs (an event per pair), so the
        # first side is scored while the others' fastVEC still runs
        overlap = p.proposal is not None and self.GLOBAL_SIDE and self.group is None and self.profile is None
        order = list(range(n))
        if overlap:
            index = {id(st): i for i, st in enumerate(P)}
            order = [index[id(st)] for _, sts in self._side_groups(P, p) for st in sts]
        for sd in side:
            sd.wait_stream(cur)
        for slot, i in enumerate(order):
            st = P[i]
            dim = st.dim
            st.sidx = slot % len(side)
            with torch.cuda.stream(side[st.sidx]):
                st.tdata, _, st.tvec = vg.fastvec_device(st.src1, np.float64(np.float32(st.width1)),
                                                         st.o1.astype(np.float64), dim, p.s, st.no1, p.g, dev=dev,
                                                         want_f32=False)
                st.qdata, _, st.qvec = vg.fastvec_device(st.src2, np.float64(np.float32(st.width2)),
                                                         st.o2.astype(np.float64), dim, p.s, st.no2, p.g, dev=dev,
                                                         want_f32=False)
                ws = dev.workspace(("stats", dim), _native.size_query("vesper_map_stats_workspace_size", dim))
                _native.check(self.lib.vesper_map_stats_ws(ctypes.c_void_p(st.tdata.data_ptr()), dim,
                                                           ctypes.c_void_p(stats[i].data_ptr()),
                                                           ctypes.c_void_p(ws.data_ptr()), ws.numel(), dev.stream))
                if mode not in ("PCC", "CC"):     # spectra need no host value: same stream
                    st.ave = 0.0
                    st.spec = vg.target_spectra_device(st.tdata, st.tvec, mode, st.ave, dev=dev)
                    st.launches += 2
                if overlap:
                    st.fv_done = torch.cuda.Event()
                    st.fv_done.record()
            if not capturing:
                for t in (st.tdata, st.tvec, st.qdata, st.qvec) + ((st.spec,) if mode not in ("PCC", "CC") else ()):
                    t.record_stream(cur)    # made on a side stream, used on this one
            st.launches += 12
        if not overlap:
            for sd in side:
                cur.wait_stream(sd)
        sh = None
        if mode in ("PCC", "CC"):
            sh = stats.cpu().numpy()
            self.d2h_bytes += sh.nbytes
        self._mark("spectra")
        if sh is not None:      # CC / PCC: the spectra use the target's mean
            for i, st in enumerate(P):
                st.ave = float(sh[i, 2])
                st.spec = vg.target_spectra_device(st.tdata, st.tvec, mode, st.ave, dev=dev)
                st.launches += 2
        if p.proposal is not None:
            # every pair correlates the subset its pooled side's network scores
            # select (the same size for all): results in one buffer, the
            # z-scores of the subsets' best scores in one reduction
            self._mark("proposal")
            k = max(1, int(np.ceil(p.proposal_frac * nang)))
            nscore = dev.lib.vesper_search_nscore(vg.MODE_CODES[mode], 0)
            S = torch.empty((n, k, nscore), dtype=torch.float32, device=dev.device)
            L = torch.empty((n, k, nscore), dtype=torch.int32, device=dev.device)
            if self.GLOBAL_SIDE and self.group is None and self.profile is None:
                # each pooled side's pairs are searched on the side streams as
                # soon as that side's subsets are selected, while the network
                # scores the next side (capping the searches' batch at 128, 64
                # or 32 to keep the concurrent scratch near the L2 size measured
                # slower)
                cur = torch.cuda.current_stream(dev.device)
                capturing = torch.cuda.is_current_stream_capturing()
                side = self._side_streams()
                index = {id(st): i for i, st in enumerate(P)}

                def launch(sts):
                    for st in sts:
                        i = index[id(st)]
                        sd = side[st.sidx]     # the stream of the pair's fastVEC
                        sd.wait_stream(cur)
                        with torch.cuda.stream(sd):
                            self._global_search(p, st, st.sub, nang, out=(S[i], L[i]), zscore=False)
                            st.tg = self._top_grid(st)
                        if not capturing:
                            st.top.record_stream(cur)
                            st.tg.record_stream(cur)

                self._proposal_subsets(p, P, mats, after_side=launch, wait=True)
                self._mark("search")
                for sd in side:
                    cur.wait_stream(sd)
            else:
                self._proposal_subsets(p, P, mats)
                self._mark("search")
                for i, st in enumerate(P):
                    self._global_search(p, st, st.sub, nang, out=(S[i], L[i]), zscore=False)
            sc0 = S[:, :, 0]
            z = (sc0.max(dim=1).values - sc0.mean(dim=1)) / (sc0.std(dim=1) + 1e-30)
            for i, st in enumerate(P):
                st.z = z[i]
        else:
            self._mark("search")
            for st in P:
                self._global_search(p, st, mats, nang)
        for st in P:   # the global top-N as grid indices (-1: none), where not yet made
            if st.tg is None:
                st.tg = self._top_grid(st)
        return stats, sh

    @staticmethod
    def _top_grid(st):
        """The pair's global top-N as grid indices (int64, -1: none)."""
        if st.order is None:
            return st.top.to(torch.int64)
        t = st.top.to(torch.int64)
        return torch.where(t >= 0, st.order.to(torch.int64).index_select(0, t.clamp(min=0)), torch.full_like(t, -1))

    _STAGE_FIELDS = ("tdata", "tvec", "qdata", "qvec", "ave", "spec", "order", "sub", "scores", "lin", "top", "z",
                     "tg", "launches")

    def _global_stage_graph(self, P, p, mats, nang):
        """_global_stage through a CUDA graph cached by the batch's signature
        (input addresses and shapes, grid geometry, parameters): a repeated
        batch replays one graph instead of its hundreds of launches.  A new
        signature runs the stage once eagerly (autotuning, first launches),
        then captures it."""
        sig = self._batch_sig(P, p, mats)
        ent = self._graphs.get(sig)
        if ent is None:
            base = [st.launches for st in P]
            self._global_stage(P, p, mats, nang)           # warm-up: tunes, loads kernels, fills caches
            marks, self.stages = self.stages, None
            for st, b0 in zip(P, base):
                st.launches = b0
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                stats, _ = self._global_stage(P, p, mats, nang)
            self.stages = marks
            saved = []
            for st, b0 in zip(P, base):
                sv = {k: getattr(st, k) for k in self._STAGE_FIELDS}
                sv["launches"] = st.launches - b0          # launches inside the graph
                st.launches = b0
                saved.append(sv)
            ent = self._graphs[sig] = (g, stats, saved)
            self.graph_captures += 1
        g, stats, saved = ent
        self._mark("global")
        g.replay()
        for st, sv in zip(P, saved):
            for k in self._STAGE_FIELDS:
                if k == "launches":
                    st.launches += sv[k]
                else:
                    setattr(st, k, sv[k])
        self.graph_replays += 1
        return stats

    @staticmethod
    def _batch_sig(P, p, mats):
        """What a captured stage depends on: input addresses and shapes, grid
        geometry, parameters, the angle grid."""
        return (tuple((st.src1.data_ptr(), st.src2.data_ptr(), tuple(st.src1.shape), tuple(st.src2.shape), st.dim,
                       *np.asarray(st.no1, np.float64).tolist(), *np.asarray(st.no2, np.float64).tolist(),
                       float(st.width1), float(st.width2), *np.asarray(st.o1).tolist(), *np.asarray(st.o2).tolist())
                      for st in P),
                (p.t, p.T, p.g, p.s, p.A, p.N, p.mode, p.batch, id(p.proposal), p.proposal_frac, p.proposal_pool),
                mats.data_ptr())

    # ---- refinement and rescoring on the device ---------------------------------
    # The +-5 degree refinement set of a top angle is its 27 neighbours on the
    # 5-degree lattice in the reference's meshgrid order, kept where x < 360,
    # y < 360 and z < 180 and wrapped by +360 where negative (:689-713).  Every
    # pair gets N x 27 slots in that order, the slots the filter drops marked
    # invalid and left out of the top-N (their score reads -inf), so the stable
    # top-N over the slots is the reference's over its list, duplicates
    # included.  The models' rotations are rows of the lattice table, their
    # translations come from the search's linear index, and the float64
    # rescoring reads the target statistics from the device: nothing in the
    # stage needs a host value, so it replays as one CUDA graph.

    def _grid_rows(self, A, angle_comb):
        """Device int64 lattice rows of the angle grid's angles, or None when
        the grid is off the 5-degree lattice."""
        cache = self.__dict__.setdefault("_grid_rows_cache", {})
        if A not in cache:
            idx = vg.lattice_index(angle_comb)
            cache[A] = None if idx is None else self.dev.to_dev(np.asarray(idx, np.int64))
        return cache[A]

    def _ref_offsets(self):
        t = self.__dict__.get("_ref_off")
        if t is None:
            t = self._ref_off = self.dev.to_dev((vg._REFINE_OFFSETS // 5).astype(np.int64))   # [27, 3] lattice steps
        return t

    def _late_stage(self, P, p, stats):
        dev = self.dev
        mode = p.mode
        L = vg.LATTICE_N
        n, N = len(P), p.N
        lat = vg.lattice_rot_matrices_device(dev)
        grid_rows = self._grid_rows(p.A, None)
        off = self._ref_offsets()
        self._mark("refine")
        c_ = ctypes.c_void_p
        tg = torch.stack([st.tg for st in P])                                  # [n, N] grid indices
        # the refinement slots of every pair (vesper_refine_slots)
        crow = torch.empty((n, N * 27), dtype=torch.int64, device=dev.device)
        valid = torch.empty((n, N * 27), dtype=torch.bool, device=dev.device)
        rmats = torch.empty((n, N * 27, 3, 3), dtype=torch.float32, device=dev.device)
        _native.check(self.lib.vesper_refine_slots(c_(tg.data_ptr()), n, N, c_(grid_rows.data_ptr()),
                                                   int(grid_rows.shape[0]), c_(off.data_ptr()), L,
                                                   c_(lat.data_ptr()), c_(crow.data_ptr()), c_(valid.data_ptr()),
                                                   c_(rmats.data_ptr()), dev.stream))
        P[0].launches += 1
        nscore = dev.lib.vesper_search_nscore(vg.MODE_CODES[mode], 0)
        RS = torch.empty((n, N * 27, nscore), dtype=torch.float32, device=dev.device)
        RL = torch.empty((n, N * 27, nscore), dtype=torch.int32, device=dev.device)
        # every pair's chain (search of its slots, top-N and picks, gather and
        # float64 rescoring of the refined models) on one of FV_STREAMS side
        # streams: the chains are short launches that fill little of the GPU,
        # so pairs overlap; the streams fork from and join the current stream
        # (also inside a CUDA-graph capture).  The shared inputs above are
        # freed only after the join.
        cur = torch.cuda.current_stream(dev.device)
        capturing = torch.cuda.is_current_stream_capturing()
        side = self._side_streams()
        for sd in side:
            sd.wait_stream(cur)
        for i, st in enumerate(P):
            d = st.dim
            with torch.cuda.stream(side[i % len(side)]):
                vg.search_device(st.spec, st.qdata, st.qvec, mode, st.ave, rmats[i], batch=p.batch, dev=dev,
                                 tuned=True, out=(RS[i], RL[i]))
                st.rtop = torch.empty(N, dtype=torch.int32, device=dev.device)
                st.r_rows = torch.empty(N, dtype=torch.int64, device=dev.device)
                st.r_score = torch.empty(N, dtype=torch.float32, device=dev.device)
                st.r_lin = torch.empty(N, dtype=torch.int64, device=dev.device)
                mm = torch.empty((N, 3, 3), dtype=torch.float32, device=dev.device)
                trd = torch.empty((N, 3), dtype=torch.int32, device=dev.device)   # wrapped as get_score (:1323-1329)
                _native.check(self.lib.vesper_refine_pick(
                    c_(RS[i].data_ptr()), c_(RL[i].data_ptr()), nscore, c_(valid[i].data_ptr()),
                    c_(crow[i].data_ptr()), N * 27, N, c_(lat.data_ptr()), d, c_(st.rtop.data_ptr()),
                    c_(st.r_rows.data_ptr()), c_(st.r_score.data_ptr()), c_(st.r_lin.data_ptr()), c_(mm.data_ptr()),
                    c_(trd.data_ptr()), dev.stream))
                gd, gv, _ = vg.rot_gather_device(st.qdata, st.qvec, mm, dev=dev)
                st.res = torch.empty((N, 8), dtype=torch.float64, device=dev.device)
                ws = dev.workspace(("rescore_batch", i, d, N),
                                   _native.size_query("vesper_rescore_batch_workspace_size", d, N))
                _native.check(self.lib.vesper_rescore_batch_dev(
                    c_(st.tdata.data_ptr()), c_(st.tvec.data_ptr()), c_(stats[i].data_ptr()), c_(gd.data_ptr()),
                    c_(gv.data_ptr()), d, c_(trd.data_ptr()), N, c_(st.res.data_ptr()), c_(ws.data_ptr()),
                    ws.numel(), dev.stream))
                if self.pair_events is not None and not capturing:
                    e = torch.cuda.Event(enable_timing=True)
                    e.record()
                    self.pair_events.append(e)
            st.launches += self._search_launches(d, mode, N * 27, p.batch) + 7
            if not capturing:
                for tt in (st.rtop, st.r_rows, st.r_score, st.r_lin, st.res):
                    tt.record_stream(cur)    # made on a side stream, read on this one
        for sd in side:
            cur.wait_stream(sd)

    _LATE_FIELDS = ("rtop", "r_rows", "r_score", "r_lin", "res", "launches")

    def _late_stage_graph(self, P, p, stats, mats):
        """_late_stage through a CUDA graph cached by the batch's signature
        (its inputs are the global stage graph's outputs, at fixed addresses)."""
        sig = self._batch_sig(P, p, mats)
        graphs = self.__dict__.setdefault("_late_graphs", {})
        ent = graphs.get(sig)
        if ent is None:
            base = [st.launches for st in P]
            marks, events = self.stages, self.pair_events
            self._late_stage(P, p, stats)                   # warm-up: tunes, loads kernels, sizes workspaces
            self.stages, self.pair_events = None, None
            for st, b0 in zip(P, base):
                st.launches = b0
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self._late_stage(P, p, stats)
            self.stages, self.pair_events = marks, events
            saved = []
            for st, b0 in zip(P, base):
                sv = {k: getattr(st, k) for k in self._LATE_FIELDS}
                sv["launches"] = st.launches - b0
                st.launches = b0
                saved.append(sv)
            ent = graphs[sig] = (g, saved)
            self.graph_captures += 1
        g, saved = ent
        self._mark("refine")
        g.replay()
        for st, sv in zip(P, saved):
            for k in self._LATE_FIELDS:
                if k == "launches":
                    st.launches += sv[k]
                else:
                    setattr(st, k, sv[k])
        if self.pair_events is not None:   # every pair ends with the graph
            e = torch.cuda.Event(enable_timing=True)
            e.record()
            self.pair_events.extend([e] * len(P))
        self.graph_replays += 1

    def _finish_device_late(self, P, p, gh, angle_comb):
        """The host bookkeeping of the device late stage: the global pass's
        statistics and top-N list from the results ``gh`` (copied before the
        late stage was launched, so this part runs while the device refines),
        then one wait for the refined models and their scores.  Modes CC and
        PCC never come here, so every score scale is 1."""
        mode = p.mode
        assert mode not in ("CC", "PCC")
        self._mark("results")
        late = self._fetch_start([[st.rtop, st.r_rows, st.r_score, st.r_lin, st.res] for st in P], slot=1)
        glob = self._fetch_finish(gh)
        angles = self._angle_tuples(p.A, angle_comb)
        scale = 1.0
        head = []
        for i, st in enumerate(P):
            raw, lin_h, top = glob[i][:3]
            order = glob[i][3] if st.order is not None else None
            rd3 = 1.0 / st.dim ** 3
            tpos = [t for t in top.tolist() if t >= 0]      # positions in the searched rotations
            top_h = [int(order[t]) for t in tpos] if order is not None else tpos   # -> grid indices
            score_arr = raw.astype(np.float64) * scale * rd3
            ave_s, std_s = float(np.mean(score_arr)), float(np.std(score_arr))
            # the score of grid index order[t] is that of position t (float32 -> float64, * scale * rd3)
            top_list = [(angles[r], float(np.float64(raw[t]) * scale * rd3), vg.unravel(lin_h[t], st.dim))
                        for t, r in zip(tpos, top_h)]
            head.append((ave_s, std_s, top_list))
        h = self._fetch_finish(late)
        out = []
        for i, st in enumerate(P):
            rtop, r_rows, r_score, r_lin, res = h[i]
            rd3 = 1.0 / st.dim ** 3
            models = []
            rows_l, score_l, lin_l, res_l = r_rows.tolist(), r_score.tolist(), r_lin.tolist(), res.tolist()
            for k, rk in enumerate(rtop.tolist()):
                if rk < 0:
                    continue
                ang = self._lattice_angle(rows_l[k])
                sc = float(score_l[k] * scale * rd3)
                tr = vg.unravel(lin_l[k], st.dim)
                rr = res_l[k]
                # Nm / total (numpy's division where total is 0: inf or nan with its warning)
                ov = rr[0] / rr[1] if rr[1] != 0.0 else float(np.float64(rr[0]) / rr[1])
                models.append(Model(ang, sc, tr, ov, rr[2], rr[3], rr[4], (st.c1, st.c2, p.s, st.dim)))
            self.launches += st.launches
            ave_s, std_s, top_list = head[i]
            out.append(AlignResult(st.dim, std_s, ave_s, top_list, models, st.launches))
        self.last_fields = [{"tdata": st.tdata, "tvec": st.tvec, "qdata": st.qdata, "qvec": st.qvec,
                             "ave": float(st.ave)} for st in P]
        self._mark("end")
        self._close_marks()
        return out

    def _lattice_angle(self, row):
        """The (x, y, z) angle tuple (np.float64 degrees) of a 5-degree lattice
        row, cached per row."""
        cache = self.__dict__.setdefault("_lattice_angle_cache", {})
        a = cache.get(row)
        if a is None:
            L = vg.LATTICE_N
            a = cache[row] = (np.float64(float(row // (L * L)) * vg.LATTICE_STEP),
                              np.float64(float((row // L) % L) * vg.LATTICE_STEP),
                              np.float64(float(row % L) * vg.LATTICE_STEP))
        return a

    def _angle_tuples(self, A, angle_comb):
        """The rows of the angle grid of step A as tuples (cached per step)."""
        cache = self.__dict__.setdefault("_angle_tuple_cache", {})
        t = cache.get(float(A))
        if t is None or len(t) != len(angle_comb):
            t = cache[float(A)] = [tuple(r) for r in angle_comb]
        return t

    def _fetch_start(self, groups, slot):
        """Start the copy of device tensors (a list of lists) to the host: one
        packed transfer into pinned buffer ``slot`` (one per copy that can be
        in flight), ordered on the current stream; _fetch_finish waits for it
        and returns the numpy arrays."""
        packed, layout = pack_bytes([t for g in groups for t in g])
        lens = [len(g) for g in groups]
        if packed is None:
            return None, layout, None, lens
        bufs = self.__dict__.setdefault("_pinned_slots", {})
        host = bufs.get(slot)
        if host is None or host.numel() < packed.numel():
            host = bufs[slot] = torch.empty(max(packed.numel(), 1 << 20), dtype=torch.uint8, pin_memory=True)
        host[:packed.numel()].copy_(packed, non_blocking=True)
        ev = torch.cuda.Event()
        ev.record()
        self.d2h_bytes += packed.numel()
        return host, layout, ev, lens

    @staticmethod
    def _fetch_finish(handle):
        host, layout, ev, lens = handle
        if host is None:
            return [[] for _ in lens]
        ev.synchronize()
        arrays = iter(unpack_bytes(host.numpy(), layout))
        return [[next(arrays) for _ in range(k)] for k in lens]

    def _fetch(self, groups):
        """Device tensors (a list of lists) to numpy with one copy and one
        wait: the tensors' bytes are packed on the device (8-byte aligned
        pieces), copied to pinned memory in one transfer, and split on the
        host."""
        packed, layout = pack_bytes([t for g in groups for t in g])
        if packed is None:
            return [[] for _ in groups]
        host = getattr(self, "_pinned", None)
        if host is None or host.numel() < packed.numel():   # one pinned buffer, grown on demand
            host = self._pinned = torch.empty(max(packed.numel(), 1 << 20), dtype=torch.uint8, pin_memory=True)
        host[:packed.numel()].copy_(packed, non_blocking=True)
        torch.cuda.current_stream(self.dev.device).synchronize()
        arrays = iter(unpack_bytes(host.numpy(), layout))
        self.d2h_bytes += packed.numel()
        return [[next(arrays) for _ in g] for g in groups]

    @staticmethod
    def _side_groups(P, p):
        """The pairs grouped by pooled grid side, smallest group first (its
        searches start soonest), ties in order of first appearance:
        [(pooled side, [pairs])]."""
        pool = int(p.proposal_pool)
        groups = {}
        for st in P:
            groups.setdefault((st.dim + pool - 1) // pool, []).append(st)
        return sorted(groups.items(), key=lambda kv: len(kv[1]))

    def _proposal_subsets(self, p, P, mats, after_side=None, wait=False):
        """Network scores of every rotation and the exact-search subset
        (ascending grid indices) of every pair; all on the device.  Pairs of
        one pooled side share the encoder launches (one per layer for all
        their maps) and one top-k launch; ``after_side(pairs)`` is called once
        a pooled side's subsets are selected; with ``wait`` the current
        stream first waits for each side's pairs' fastVEC (their events)."""
        from . import proposal as prop
        dev = self.dev
        pool = int(p.proposal_pool)
        cur = torch.cuda.current_stream(dev.device)
        for dp, sts in self._side_groups(P, p):
            if wait:
                for st in sts:
                    cur.wait_event(st.fv_done)
            fTQ = torch.empty((2 * len(sts), 4, dp, dp, dp), dtype=torch.float32, device=dev.device)
            for i, st in enumerate(sts):
                prop.map_field(st.tdata, st.tvec, pool, dev, out=fTQ[2 * i])
                prop.map_field(st.qdata, st.qvec, pool, dev, out=fTQ[2 * i + 1])
            s = p.proposal.rotation_scores_many(fTQ, mats)
            orders = prop.subset_from_scores(dev, s, p.proposal_frac).to(torch.int64)
            subs = mats.index_select(0, orders.reshape(-1)).reshape((len(sts), orders.shape[1]) + tuple(mats.shape[1:]))
            for i, st in enumerate(sts):
                st.order = orders[i]
                st.sub = subs[i]
                # 2 fields + (4 layers + vmajor + top-k) shared by the group + scoring
                st.launches += 3 + (6 if i == 0 else 0)
            if after_side is not None:
                after_side(sts)

    def _global_search(self, p, st, mats, nang, out=None, zscore=True):
        """Search of the given rotations, top-N and (subset searches, unless
        the caller batches it) the z-score of the best exact score over the
        subset; all on the device."""
        if self.group is not None:
            sc, ln = vg.search_device_sharded(st.spec, st.qdata, st.qvec, p.mode, st.ave, mats, self.group,
                                              batch=p.batch, dev=self.dev, tuned=True)
            if out is not None:
                out[0].copy_(sc)
                out[1].copy_(ln)
                sc, ln = out
            st.scores, st.lin = sc, ln
        else:
            st.scores, st.lin = vg.search_device(st.spec, st.qdata, st.qvec, p.mode, st.ave, mats, batch=p.batch,
                                                 dev=self.dev, profile=self.profile, tuned=True, out=out)
        st.launches += self._search_launches(st.dim, p.mode, int(mats.shape[0]), p.batch)
        st.top = vg.topn_device(st.scores, p.N, dev=self.dev)
        st.launches += 1
        if not zscore:
            return
        if st.order is not None:
            sc0 = st.scores[:, 0]
            st.z = (sc0.max() - sc0.mean()) / (sc0.std() + 1e-30)
        elif p.proposal is not None:
            st.z = torch.zeros((), dtype=torch.float32, device=self.dev.device)

    def _search_launches(self, dim, mode, nrot, batch):
        if batch <= 0:
            from . import autotune
            t = autotune.cached(dim, mode, self.dev)
            if t and t.get("batch"):
                batch = int(t["batch"])
        return vg.search_plan(dim, mode, batch, nrot, None, self.dev)[1]

    def align_host_many(self, items, p: AlignParams, graph: bool = False):
        """End-to-end batch: items = [(host map1, host map2, width1, width2,
        orig1, orig2)] with float32 [x][y][z] torch tensors (pinned for an
        asynchronous copy) -> results."""
        dev = self.dev
        dev_items = [(self._stage_in(2 * i, h1), self._stage_in(2 * i + 1, h2), w1, w2, o1, o2)
                     for i, (h1, h2, w1, w2, o1, o2) in enumerate(items)]
        return self.align_many(dev_items, p, graph)

    def _stage_in(self, slot, h):
        """Copy a host map into a device staging buffer kept per (slot, shape),
        so repeated batches present the same addresses (and replay their
        CUDA graph)."""
        key = (slot, tuple(h.shape))
        buf = self._staging.get(key)
        if buf is None:
            buf = self._staging[key] = torch.empty(tuple(h.shape), dtype=torch.float32, device=self.dev.device)
        buf.copy_(h, non_blocking=True)
        return buf

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
