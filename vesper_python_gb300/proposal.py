"""Learned rotation proposal for the exhaustive rotational search.

A Siamese 3-D convolutional encoder (4 layers: 4 -> 32 -> 32 -> 32 -> 8
channels, 3x3x3 kernels, ReLU between layers, bfloat16 weights, float32
accumulation) maps each map's coarse field (vx, vy, vz, density mask) to a
feature field.  A rotation is scored by correlating the target's features
with the rotated query's features at zero translation (the reference's
nearest-voxel rotation of the grid).  The top fraction of the angle grid by
that score is then correlated exactly by vesper_search; the exhaustive search
remains the fallback and the measure of recall.

Training labels come from the exhaustive GPU search itself: for each training
pair the per-rotation best scores are turned into a target distribution
q = softmax(beta * z) over rotations (z: z-scored search scores), and the
network's rotation scores are trained with softmax cross-entropy.  Forward,
backward and the Adam update run in this library's kernels
(vesper_prop_* in libvesper_gb300.so).
"""
from __future__ import annotations

import ctypes
import dataclasses
import json
import math
import os
import time

import numpy as np
import torch

from . import _native
from . import vesper as vg

CHANNELS = (4, 32, 32, 32, 8)


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def map_field(data, vec, pool=1, dev=None, out=None):
    """4-channel network input [4][dp][dp][dp] (vx, vy, vz, mask) of a fastVEC
    result, averaged over pool^3 blocks (vesper_prop_field)."""
    dev = dev or vg.default_device()
    d = int(data.shape[0])
    dp = (d + pool - 1) // pool
    f = out if out is not None else torch.empty((4, dp, dp, dp), dtype=torch.float32, device=data.device)
    _native.check(dev.lib.vesper_prop_field(_p(data), _p(vec), d, int(pool), _p(f), dev.stream))
    return f


class ProposalNet:
    def __init__(self, dev: vg.Device, seed: int = 0):
        self.dev = dev
        self.lib = dev.lib
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.W, self.b, self.Wbf = [], [], []
        for cin, cout in zip(CHANNELS[:-1], CHANNELS[1:]):
            std = math.sqrt(2.0 / (cin * 27))
            w = (torch.randn((cout, cin, 27), generator=g) * std).to(dev.device)
            self.W.append(w.contiguous())
            self.b.append(torch.zeros(cout, device=dev.device))
            self.Wbf.append(w.to(torch.bfloat16).contiguous())
        self.relu = [1] * (len(CHANNELS) - 2) + [0]
        self.gW = [torch.zeros_like(w) for w in self.W]
        self.gb = [torch.zeros_like(b) for b in self.b]
        self.mW = [torch.zeros_like(w) for w in self.W]
        self.vW = [torch.zeros_like(w) for w in self.W]
        self.mb = [torch.zeros_like(b) for b in self.b]
        self.vb = [torch.zeros_like(b) for b in self.b]
        self.step_count = 0
        self._ws = None

    # ---- state -------------------------------------------------------------
    def state_dict(self):
        return {"W": [w.cpu() for w in self.W], "b": [b.cpu() for b in self.b],
                "mW": [m.cpu() for m in self.mW], "vW": [v.cpu() for v in self.vW],
                "mb": [m.cpu() for m in self.mb], "vb": [v.cpu() for v in self.vb], "step": self.step_count}

    def load_state_dict(self, s):
        d = self.dev.device
        self.W = [w.to(d).contiguous() for w in s["W"]]
        self.b = [b.to(d).contiguous() for b in s["b"]]
        self.Wbf = [w.to(torch.bfloat16).contiguous() for w in self.W]
        for name in ("mW", "vW", "mb", "vb"):
            if name in s:
                setattr(self, name, [t.to(d).contiguous() for t in s[name]])
        self.step_count = int(s.get("step", 0))

    # ---- forward / backward ------------------------------------------------
    def encode(self, field, nmap=1):
        """Activations of every layer; ``field`` is [4][d][d][d], or
        [nmap][4][d][d][d] for nmap maps encoded in one launch per layer."""
        acts = [field.contiguous()]
        d = int(field.shape[-1])
        lead = (nmap,) if nmap > 1 else ()
        for i, (cin, cout) in enumerate(zip(CHANNELS[:-1], CHANNELS[1:])):
            out = torch.empty(lead + (cout, d, d, d), dtype=torch.float32, device=self.dev.device)
            _native.check(self.lib.vesper_prop_conv_fwd(_p(acts[-1]), cin, _p(self.Wbf[i]), _p(self.b[i]), cout, d,
                                                        self.relu[i], nmap, _p(out), self.dev.stream))
            acts.append(out)
        return acts

    def encode_backward(self, acts, g):
        d = int(acts[0].shape[1])
        for i in range(len(self.W) - 1, -1, -1):
            cin, cout = CHANNELS[i], CHANNELS[i + 1]
            din = torch.empty((cin, d, d, d), dtype=torch.float32, device=self.dev.device) if i > 0 else None
            _native.check(self.lib.vesper_prop_conv_bwd(_p(g), _p(acts[i + 1]), self.relu[i], _p(acts[i]),
                                                        _p(self.Wbf[i]), cin, cout, d, _p(din), _p(self.gW[i]),
                                                        _p(self.gb[i]), self.dev.stream))
            g = din

    def score(self, ET, EQ, mats):
        K, d = int(ET.shape[0]), int(ET.shape[1])
        n = int(mats.shape[0])
        s = torch.empty(n, dtype=torch.float32, device=self.dev.device)
        _native.check(self.lib.vesper_prop_score(_p(ET), _p(EQ), K, d, _p(mats), n, _p(s), self.dev.stream))
        return s

    def score_backward(self, ET, EQ, mats, gs, gET, gEQ):
        K, d = int(ET.shape[0]), int(ET.shape[1])
        nb = _native.size_query("vesper_prop_score_bwd_workspace", K, d)
        if self._ws is None or self._ws.numel() < nb:
            self._ws = torch.empty(nb, dtype=torch.uint8, device=self.dev.device)
        _native.check(self.lib.vesper_prop_score_bwd(_p(ET), _p(EQ), K, d, _p(mats), int(mats.shape[0]), _p(gs),
                                                     _p(gET), _p(gEQ), _p(self._ws), self._ws.numel(),
                                                     self.dev.stream))

    def zero_grad(self):
        for t in self.gW + self.gb:
            t.zero_()

    def loss_and_grad(self, fT, fQ, mats, q, tau):
        """Accumulate the gradients of one pair; returns the loss tensor."""
        aT = self.encode(fT)
        aQ = self.encode(fQ)
        s = self.score(aT[-1], aQ[-1], mats)
        loss = torch.zeros(1, dtype=torch.float32, device=self.dev.device)
        gs = torch.empty_like(s)
        _native.check(self.lib.vesper_prop_softmax_ce(_p(s), _p(q), int(s.numel()), float(tau), _p(loss), _p(gs),
                                                      self.dev.stream))
        gT = torch.zeros_like(aT[-1])
        gQ = torch.zeros_like(aQ[-1])
        self.score_backward(aT[-1], aQ[-1], mats, gs, gT, gQ)
        self.encode_backward(aT, gT)
        self.encode_backward(aQ, gQ)
        return loss

    def adam_step(self, lr, batch, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        for i in range(len(self.W)):
            _native.check(self.lib.vesper_prop_adam(_p(self.W[i]), _p(self.mW[i]), _p(self.vW[i]), _p(self.gW[i]),
                                                    self.W[i].numel(), lr, b1, b2, eps, self.step_count,
                                                    1.0 / batch, _p(self.Wbf[i]), self.dev.stream))
            _native.check(self.lib.vesper_prop_adam(_p(self.b[i]), _p(self.mb[i]), _p(self.vb[i]), _p(self.gb[i]),
                                                    self.b[i].numel(), lr, b1, b2, eps, self.step_count,
                                                    1.0 / batch, None, self.dev.stream))

    def rotation_scores(self, fTQ, mats, half=True):
        """Inference: both maps' fields stacked [2][4][d][d][d] -> score of
        every rotation (one encoder pass over the stack, voxel-major
        features: float16 with vesper_prop_score_f16, else float32 with
        vesper_prop_score_vm)."""
        return self.rotation_scores_many(fTQ, mats, half)[0]

    def rotation_scores_many(self, fTQ, mats, half=True):
        """Inference for P pairs of one pooled side at once: fields
        [2P][4][d][d][d] (target and query of pair i at 2i, 2i + 1) -> scores
        [P][nrot], with one encoder launch per layer and one voxel-major
        conversion for all 2P maps, then one scoring launch for every pair
        (one per pair when the gather map is not cached)."""
        d = int(fTQ.shape[-1])
        nm = int(fTQ.shape[0])
        npair = nm // 2
        K = CHANNELS[-1]
        feat = self.encode(fTQ, nmap=nm)[-1]
        n = int(mats.shape[0])
        s = torch.empty((npair, n), dtype=torch.float32, device=self.dev.device)
        if half:
            vm = torch.empty((nm, d * d * d, K), dtype=torch.float16, device=self.dev.device)
            _native.check(self.lib.vesper_prop_vmajor_f16(_p(feat), K, d, nm, _p(vm), self.dev.stream))
            sm = srcmap(self.dev, d, mats)
            if sm is not None:     # every pair in one launch
                _native.check(self.lib.vesper_prop_score_map_many(_p(vm), npair, K, d, _p(sm), n, _p(s),
                                                                  self.dev.stream))
            else:
                for i in range(npair):
                    _native.check(self.lib.vesper_prop_score_f16(_p(vm[2 * i]), _p(vm[2 * i + 1]), K, d, _p(mats), n,
                                                                 _p(s[i]), self.dev.stream))
        else:
            vm = torch.empty((nm, d * d * d, K), dtype=torch.float32, device=self.dev.device)
            _native.check(self.lib.vesper_prop_vmajor(_p(feat), K, d, nm, _p(vm), self.dev.stream))
            for i in range(npair):
                _native.check(self.lib.vesper_prop_score_vm(_p(vm[2 * i]), _p(vm[2 * i + 1]), K, d, _p(mats), n,
                                                            _p(s[i]), self.dev.stream))
        return s

    def propose(self, fTQ, mats, frac):
        """Grid indices (int32, ascending) of the best ``frac`` of the
        rotations, and the scores of all of them."""
        s = self.rotation_scores(fTQ, mats)
        return subset_from_scores(self.dev, s, frac), s


_SRCMAPS = {}
SRCMAP_BUDGET = 2 << 30      # bytes of cached gather maps (HBM is plentiful; each is nrot * d^3 * 2)


def srcmap(dev, d, mats):
    """Cached int16 gather map [nrot][d^3] of this rotation set on a d^3 grid
    (vesper_prop_srcmap), or None when d^3 exceeds int16 or the cache budget."""
    n = int(mats.shape[0])
    if d ** 3 > 32767:
        return None
    # the entry keeps the rotation tensor alive, so its address names it
    key = (dev.device, d, mats.data_ptr(), n)
    ent = _SRCMAPS.get(key)
    if ent is None:
        need = n * d ** 3 * 2
        if sum(m.numel() * 2 for _, m in _SRCMAPS.values()) + need > SRCMAP_BUDGET:
            return None
        m = torch.empty((n, d ** 3), dtype=torch.int16, device=dev.device)
        _native.check(dev.lib.vesper_prop_srcmap(d, _p(mats), n, _p(m), dev.stream))
        ent = _SRCMAPS[key] = (mats, m)
    return ent[1]


def target_distribution(scores, beta):
    """q = softmax(beta * z) of the exhaustive search's per-rotation scores."""
    s = scores.to(torch.float64)
    z = (s - s.mean()) / (s.std() + 1e-30)
    q = torch.softmax(beta * z, dim=0)
    return q.to(torch.float32)


# ---------------------------------------------------------------------------
# training / evaluation data: config-0-style pairs, generated on the GPU
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class PairFields:
    fTQ: torch.Tensor        # [2][4][dp][dp][dp]: target then query network input
    fT: torch.Tensor         # views of fTQ[0], fTQ[1]
    fQ: torch.Tensor
    tdata: torch.Tensor
    tvec: torch.Tensor
    qdata: torch.Tensor
    qvec: torch.Tensor
    dim: int


def blob_pair_torch(seed, side=128, nblob=400, radius=40.0, sigma=1.5, noise=0.01, device="cuda"):
    """The seeded blob-map generator of synth.make_pair (same distributions)
    evaluated with torch on the GPU: map1 = sum of separable Gaussians + noise,
    map2 = nearest-grid rotated crop (random ZYZ rotation, U[-5, 5] shift) +
    fresh noise."""
    g = torch.Generator(device="cpu").manual_seed(int(seed))
    u = torch.rand(nblob, generator=g, dtype=torch.float64)
    r = radius * u.pow(1.0 / 3.0)
    v = torch.randn(nblob, 3, generator=g, dtype=torch.float64)
    v = v / v.norm(dim=1, keepdim=True)
    pos = (v * r[:, None] + side * 0.5).to(device)
    amp = (0.5 + torch.rand(nblob, generator=g, dtype=torch.float64)).to(device)
    grid = torch.arange(side, dtype=torch.float64, device=device)
    inv = 1.0 / (2.0 * sigma * sigma)
    gx = torch.exp(-(grid[None, :] - pos[:, 0:1]) ** 2 * inv) * amp[:, None]
    gy = torch.exp(-(grid[None, :] - pos[:, 1:2]) ** 2 * inv)
    gz = torch.exp(-(grid[None, :] - pos[:, 2:3]) ** 2 * inv)
    map1 = torch.einsum("bx,by,bz->xyz", gx, gy, gz)
    gn = torch.Generator(device=device).manual_seed(int(seed) * 2 + 1)
    map1 = map1 + noise * torch.randn(map1.shape, generator=gn, dtype=torch.float64, device=device)
    a = float(torch.rand(1, generator=g)) * 2 * math.pi
    bcos = float(torch.rand(1, generator=g)) * 2 - 1
    c = float(torch.rand(1, generator=g)) * 2 * math.pi
    shift = (torch.rand(3, generator=g, dtype=torch.float64) * 10 - 5).to(device)

    def rz(t):
        return torch.tensor([[math.cos(t), -math.sin(t), 0], [math.sin(t), math.cos(t), 0], [0, 0, 1]],
                            dtype=torch.float64)

    b_ang = math.acos(bcos)
    ry = torch.tensor([[math.cos(b_ang), 0, math.sin(b_ang)], [0, 1, 0], [-math.sin(b_ang), 0, math.cos(b_ang)]],
                      dtype=torch.float64)
    m = (rz(a) @ ry @ rz(c)).to(device)
    s2 = side // 2
    q = torch.stack(torch.meshgrid(*(torch.arange(s2, dtype=torch.float64, device=device),) * 3, indexing="ij"),
                    -1).reshape(-1, 3) - s2 * 0.5
    src = q @ m.T + side * 0.5 + shift
    idx = torch.round(src).to(torch.int64)
    ok = ((idx >= 0) & (idx < side)).all(dim=1)
    flat = torch.zeros(q.shape[0], dtype=torch.float64, device=device)
    ii = idx[ok]
    flat[ok] = map1[ii[:, 0], ii[:, 1], ii[:, 2]]
    map2 = flat.reshape(s2, s2, s2) + noise * torch.randn((s2,) * 3, generator=gn, dtype=torch.float64,
                                                           device=device)
    orig2 = np.full(3, (side - s2) * 0.5)
    return map1.to(torch.float32).contiguous(), map2.to(torch.float32).contiguous(), np.zeros(3), orig2


class PairMaker:
    """Fields of config-0-style pairs (128^3 / 64^3 blob maps, g = 16,
    t = T = 0.1) at voxel spacing ``s``; the network input is pooled by
    ``pool``."""

    def __init__(self, dev, s=3.0, g=16.0, t=0.1, pool=2):
        from . import align
        self.dev = dev
        self.al = align.Aligner(dev)
        self.s, self.g, self.t, self.pool = s, g, t, pool

    def fields(self, seed):
        from . import align
        m1, m2, o1, o2 = blob_pair_torch(seed, device=self.dev.device)
        al = self.al
        cent1 = np.array([x * 0.5 for x in m1.shape])
        cent2 = np.array([x * 0.5 for x in m2.shape])
        prep = torch.empty(4, dtype=torch.int64, device=self.dev.device)
        al._prepare(m1, self.t, cent1, prep[0:2])
        al._prepare(m2, self.t, cent2, prep[2:4])
        pr = prep.cpu().numpy().view(np.uint64)
        oo1 = np.array([np.float32(v) for v in o1])
        oo2 = np.array([np.float32(v) for v in o2])
        d1, no1, c1 = align._size_grid(pr[0], pr[1], cent1, 1.0, oo1, self.s)
        d2, no2, c2 = align._size_grid(pr[2], pr[3], cent2, 1.0, oo2, self.s)
        if d1 > d2:
            dim = d1
            no2 = c2 - 0.5 * self.s * dim
        else:
            dim = d2
            no1 = c1 - 0.5 * self.s * dim
        td, _, tv = vg.fastvec_device(m1, 1.0, oo1.astype(np.float64), dim, self.s, no1, self.g, dev=self.dev)
        qd, _, qv = vg.fastvec_device(m2, 1.0, oo2.astype(np.float64), dim, self.s, no2, self.g, dev=self.dev)
        dp = (dim + self.pool - 1) // self.pool
        fTQ = torch.empty((2, 4, dp, dp, dp), dtype=torch.float32, device=self.dev.device)
        map_field(td, tv, self.pool, self.dev, out=fTQ[0])
        map_field(qd, qv, self.pool, self.dev, out=fTQ[1])
        return PairFields(fTQ, fTQ[0], fTQ[1], td, tv, qd, qv, dim)


def exhaustive_scores(dev, pf: PairFields, mats):
    spec = vg.target_spectra_device(pf.tdata, pf.tvec, "VecProduct", 0.0, dev=dev)
    sc, ln = vg.search_device(spec, pf.qdata, pf.qvec, "VecProduct", 0.0, mats, dev=dev, tuned=True)
    return spec, sc[:, 0].contiguous(), ln[:, 0].contiguous()


def label_pairs(dev, maker, seeds, mats, beta, cache, log=None):
    """Fields and target distributions of the given seeds (cached by seed)."""
    t0 = time.time()
    for i, sd in enumerate(seeds):
        sd = int(sd)
        if sd in cache:
            continue
        pf = maker.fields(sd)
        _, sc, _ = exhaustive_scores(dev, pf, mats)
        cache[sd] = (pf.fT, pf.fQ, target_distribution(sc, beta))
        if log and (i + 1) % 500 == 0:
            log(f"labelled {i + 1} pairs ({time.time() - t0:.1f} s)")
    return cache


def train(dev, net, seeds, mats, epochs=1, batch=16, lr=1e-3, tau=0.5, beta=2.0, cache=None, maker=None, log=None):
    """Adam on the softmax cross-entropy between the network's rotation scores
    and the exhaustive search's target distribution, one pair per step of
    gradient accumulation and ``batch`` pairs per update.  ``cache`` (dict)
    keeps each pair's fields and target.  Returns the mean loss per epoch."""
    cache = {} if cache is None else cache
    maker = maker or PairMaker(dev)
    label_pairs(dev, maker, seeds, mats, beta, cache)
    t0 = time.time()
    hist = []
    for ep in range(epochs):
        order = np.random.default_rng(ep).permutation(len(seeds))
        tot = torch.zeros(1, device=dev.device)
        nb = 0
        net.zero_grad()
        for j in order:
            fT, fQ, q = cache[int(seeds[j])]
            tot += net.loss_and_grad(fT, fQ, mats, q, tau)
            nb += 1
            if nb == batch:
                net.adam_step(lr, batch)
                net.zero_grad()
                nb = 0
        if nb:
            net.adam_step(lr, nb)
            net.zero_grad()
        loss = float(tot.item()) / max(1, len(seeds))
        hist.append(loss)
        if log:
            log(f"epoch {ep}: mean loss {loss:.4f} ({time.time() - t0:.1f} s)")
    return hist


# ---------------------------------------------------------------------------
# weights
# ---------------------------------------------------------------------------

WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "proposal_weights.npz")


def save_weights(net, path=WEIGHTS, meta=None):
    arrs = {}
    for i in range(len(net.W)):
        arrs[f"W{i}"] = net.W[i].cpu().numpy()
        arrs[f"b{i}"] = net.b[i].cpu().numpy()
    arrs["meta"] = np.frombuffer(json.dumps(meta or {}).encode(), dtype=np.uint8)
    tmp = path + ".tmp.npz"
    np.savez_compressed(tmp, **arrs)
    os.replace(tmp, path)


def load_weights(dev, path=WEIGHTS):
    z = np.load(path)
    net = ProposalNet(dev)
    net.load_state_dict({"W": [torch.as_tensor(z[f"W{i}"]) for i in range(len(CHANNELS) - 1)],
                         "b": [torch.as_tensor(z[f"b{i}"]) for i in range(len(CHANNELS) - 1)]})
    meta = json.loads(bytes(z["meta"]).decode()) if "meta" in z else {}
    return net, meta


# ---------------------------------------------------------------------------
# proposal rules without the network (what the network is measured against)
# ---------------------------------------------------------------------------

def baseline_scores(dev, pf: PairFields, mats, kind):
    """Rotation scores of a fixed rule: "mask" (zero-shift overlap of the two
    density masks), "raw" (zero-shift correlation of the unrotated 4-channel
    input fields) or "random"."""
    n = int(mats.shape[0])
    if kind == "random":
        g = torch.Generator(device="cpu").manual_seed(n)
        return torch.rand(n, generator=g).to(dev.device)
    sel = slice(3, 4) if kind == "mask" else slice(0, 4)
    ET = pf.fT[sel].contiguous()
    EQ = pf.fQ[sel].contiguous()
    K, d = int(ET.shape[0]), int(ET.shape[1])
    s = torch.empty(n, dtype=torch.float32, device=dev.device)
    _native.check(dev.lib.vesper_prop_score(_p(ET), _p(EQ), K, d, _p(mats), n, _p(s), dev.stream))
    return s


def subset_from_scores(dev, s, frac):
    """Grid indices (int32, ascending) of the best ``frac`` of the scores ``s``
    [n], or, for a score matrix [P][n], of each row ([P][k], one launch)."""
    rows = 1 if s.dim() == 1 else int(s.shape[0])
    n = int(s.shape[-1])
    k = max(1, int(math.ceil(frac * n)))
    idx = torch.empty((rows, k) if s.dim() > 1 else (k,), dtype=torch.int32, device=dev.device)
    _native.check(dev.lib.vesper_topk_subset_batch(_p(s.contiguous()), rows, n, k, _p(idx), dev.stream))
    return idx


# ---------------------------------------------------------------------------
# proposal search with fallback, and its evaluation against the exhaustive one
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class ProposalResult:
    top: np.ndarray          # top-N rotation indices into the full grid
    scores: np.ndarray       # their raw search scores
    lin: np.ndarray          # their best translations (linear index)
    fallback: bool
    winner_rank: int         # network rank of the subset's best rotation
    winner_z: float          # its exact score, z-scored over the subset
    subset: torch.Tensor     # the correlated rotations (grid indices, ascending; device)
    subset_top: np.ndarray   # top-N of the subset alone (before any fallback)


def _top_from(dev, sc, ln, ridx, N):
    top = vg.topn_device(sc.contiguous(), N, dev=dev).cpu().numpy()
    top = top[top >= 0]
    return ridx[top], sc.cpu().numpy()[top], ln.cpu().numpy()[top]


def search_with_proposal(dev, net, pf: PairFields, spec, mats, frac=0.05, N=10, fallback_rank=1.0,
                         fallback_z=None, scores=None):
    """Correlate the best ``frac`` of the grid by the network's ranking.  The
    whole grid is correlated instead (the fallback) when the subset's best
    rotation ranks below ``fallback_rank`` of the subset in the network's own
    order, or when its exact score stands less than ``fallback_z`` standard
    deviations above the subset's mean (a flat landscape).  One device-to-host
    copy when there is no fallback."""
    s = scores if scores is not None else net.rotation_scores(pf.fTQ, mats)
    order = subset_from_scores(dev, s, frac).to(torch.int64)     # ascending grid indices
    k = int(order.numel())
    sub = mats.index_select(0, order)
    sc, ln = vg.search_device(spec, pf.qdata, pf.qvec, "VecProduct", 0.0, sub, dev=dev, tuned=True)
    sc0, ln0 = sc[:, 0].contiguous(), ln[:, 0].contiguous()
    nt = min(N, k)
    top = vg.topn_device(sc0, nt, dev=dev)[:nt].to(torch.int64)   # positions in the subset
    w = top[0]
    sv = s.index_select(0, order)
    rank = (sv > sv[w]).sum().to(torch.float64)
    z = ((sc0[w] - sc0.mean()) / (sc0.std() + 1e-30)).to(torch.float64)
    packed = torch.cat([torch.stack([rank, z]), order[top].to(torch.float64), sc0[top].to(torch.float64),
                        ln0[top].to(torch.float64)]).cpu().numpy()
    rank, z = int(packed[0]), float(packed[1])
    stop = packed[2:2 + nt].astype(np.int64)
    tsc = packed[2 + nt:2 + 2 * nt].astype(np.float32)
    tln = packed[2 + 2 * nt:].astype(np.int64)
    fb = rank > fallback_rank * k or (fallback_z is not None and z < fallback_z)
    if fb:
        fs, fl = vg.search_device(spec, pf.qdata, pf.qvec, "VecProduct", 0.0, mats, dev=dev, tuned=True)
        t, fsc, fln = _top_from(dev, fs[:, 0], fl[:, 0], np.arange(int(mats.shape[0])), N)
        return ProposalResult(t, fsc, fln, True, rank, z, order, stop)
    return ProposalResult(stop, tsc, tln, False, rank, z, order, stop)


def evaluate(dev, net, seeds, mats, frac=0.05, N=10, fallback_rank=1.0, fallback_z=None, maker=None,
             baselines=(), log=None):
    """Top-1 / top-N agreement with the exhaustive search and the search-stage
    time of both forms over the given pair seeds, with per-pair diagnostics
    (network rank and subset z-score of the subset's winner) from which
    other fallback thresholds can be evaluated."""
    maker = maker or PairMaker(dev)
    n = int(mats.shape[0])
    rows = []
    t_ex = t_pr = 0.0
    for i, sd in enumerate(seeds):
        pf = maker.fields(int(sd))
        spec = vg.target_spectra_device(pf.tdata, pf.tvec, "VecProduct", 0.0, dev=dev)
        torch.cuda.synchronize()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record()
        sc, ln = vg.search_device(spec, pf.qdata, pf.qvec, "VecProduct", 0.0, mats, dev=dev, tuned=True)
        ex_top, ex_sc, _ = _top_from(dev, sc[:, 0], ln[:, 0], np.arange(n), N)
        e1.record()
        pr = search_with_proposal(dev, net, pf, spec, mats, frac, N, fallback_rank, fallback_z)
        e2.record()
        torch.cuda.synchronize()
        t_ex += e0.elapsed_time(e1)
        t_pr += e1.elapsed_time(e2)
        win = int(ex_top[0])
        row = {"seed": int(sd), "dim": pf.dim, "top1": bool(pr.top[0] == win),
               "top1_subset": bool(pr.subset_top[0] == win),
               "topN": len(set(pr.top.tolist()) & set(ex_top.tolist())) / max(1, len(ex_top)),
               "fallback": pr.fallback, "rank": pr.winner_rank, "z": pr.winner_z,
               "in_subset_net": bool(win in set(pr.subset.cpu().numpy().tolist())),
               "score_rel_err": float(abs(pr.scores[0] - ex_sc[0]) / max(abs(ex_sc[0]), 1e-30))}
        for kind in baselines:
            sub = subset_from_scores(dev, baseline_scores(dev, pf, mats, kind), frac).cpu().numpy()
            row[f"in_subset_{kind}"] = bool(win in set(sub.tolist()))
        rows.append(row)
        if log and (i + 1) % 100 == 0:
            log(f"evaluated {i + 1} pairs")
    m = len(rows)
    agree = [r for r in rows if r["top1"]]
    out = {"pairs": m, "frac": frac, "fallback_rank": fallback_rank, "fallback_z": fallback_z,
           "top1_agreement": len(agree) / m,
           "top1_agreement_subset_only": sum(r["top1_subset"] for r in rows) / m,
           "topN_recall": sum(r["topN"] for r in rows) / m,
           "fallback_rate": sum(r["fallback"] for r in rows) / m,
           "max_score_rel_err_when_agreeing": max([r["score_rel_err"] for r in agree], default=None),
           "exhaustive_ms_per_pair": t_ex / m, "proposal_ms_per_pair": t_pr / m,
           "search_speedup": t_ex / max(t_pr, 1e-9)}
    for kind in ("net",) + tuple(baselines):
        out[f"winner_in_subset_{kind}"] = sum(r[f"in_subset_{kind}"] for r in rows) / m
    out["curve_z"] = fallback_curve(rows, "z")
    return out, rows


def fallback_curve(rows, key, thresholds=(0.0, 2.0, 3.0, 4.0, 5.0, 6.0, 8.0, 10.0)):
    """Top-1 agreement and fallback rate of the rule "fall back when the
    subset winner's ``key`` is below t" for each threshold t (from the
    subset-only results of evaluate)."""
    out = []
    m = max(1, len(rows))
    for t in thresholds:
        fb = [r[key] < t for r in rows]
        agree = sum(1 if f else int(r["top1_subset"]) for f, r in zip(fb, rows)) / m
        out.append({"t": t, "top1_agreement": agree, "fallback_rate": sum(fb) / m})
    return out


# ---------------------------------------------------------------------------
# command line: train / evaluate on seeded config-0-style pairs
# ---------------------------------------------------------------------------

def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(prog="python -m vesper_python_gb300.proposal")
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--pairs", type=int, default=20000)
    t.add_argument("--epochs", type=int, default=4)
    t.add_argument("--batch", type=int, default=32)
    t.add_argument("--lr", type=float, default=2e-3)
    t.add_argument("--tau", type=float, default=0.5)
    t.add_argument("--beta", type=float, default=2.0)
    t.add_argument("--A", type=float, default=10.0)
    t.add_argument("--s", type=float, default=3.0)
    t.add_argument("--pool", type=int, default=2)
    t.add_argument("--out", default=WEIGHTS)
    t.add_argument("--seed0", type=int, default=0)
    e = sub.add_parser("eval")
    e.add_argument("--pairs", type=int, default=1000)
    e.add_argument("--seed0", type=int, default=10_000_000)
    e.add_argument("--frac", type=float, default=0.05)
    e.add_argument("--fallback-rank", type=float, default=1.0)
    e.add_argument("--fallback-z", type=float, default=None)
    e.add_argument("--weights", default=WEIGHTS)
    e.add_argument("--json", default=None)
    a = ap.parse_args(argv)
    dev = vg.default_device()
    log = lambda m: print(m, flush=True)
    if a.cmd == "train":
        mats = vg.rot_matrices_device(vg.calc_angle_comb(a.A), dev, key=("grid", float(a.A)))
        net = ProposalNet(dev, seed=a.seed0)
        maker = PairMaker(dev, s=a.s, pool=a.pool)
        t0 = time.time()
        seeds = list(range(a.seed0, a.seed0 + a.pairs))
        cache = {}
        label_pairs(dev, maker, seeds, mats, a.beta, cache, log=log)
        torch.cuda.synchronize()
        log(f"labelled {a.pairs} pairs in {time.time() - t0:.1f} s")
        hist = train(dev, net, seeds, mats, epochs=a.epochs, batch=a.batch, lr=a.lr, tau=a.tau, beta=a.beta,
                     cache=cache, maker=maker, log=log)
        save_weights(net, a.out, {"pairs": a.pairs, "epochs": a.epochs, "lr": a.lr, "tau": a.tau, "beta": a.beta,
                                  "A": a.A, "s": a.s, "pool": a.pool, "loss": hist,
                                  "seconds": time.time() - t0})
        log(f"saved {a.out}")
    else:
        net, meta = load_weights(dev, a.weights)
        A = float(meta.get("A", 10.0))
        mats = vg.rot_matrices_device(vg.calc_angle_comb(A), dev, key=("grid", A))
        maker = PairMaker(dev, s=float(meta.get("s", 3.0)), pool=int(meta.get("pool", 2)))
        seeds = list(range(a.seed0, a.seed0 + a.pairs))
        res, _ = evaluate(dev, net, seeds, mats, a.frac, 10, a.fallback_rank, a.fallback_z, maker=maker,
                          baselines=("mask", "raw", "random"), log=log)
        res["training"] = {k: meta.get(k) for k in ("pairs", "epochs", "s", "pool", "A")}
        print(json.dumps(res), flush=True)
        if a.json:
            with open(a.json, "w") as f:
                json.dump(res, f, indent=1)


if __name__ == "__main__":
    main()
