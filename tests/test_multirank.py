"""Rotation sharding across ranks, on CPU ranks over gloo (world size 2 and 3):
each rank searches its block of the angle grid with the CPU oracle, then the
gathered top-N and prob statistics must equal the single-process ones."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _problem():
    from oracle import vesper_oracle as orc
    rng = np.random.default_rng(4)
    d = 9
    tdata = np.where(rng.random((d, d, d)) < 0.5, rng.uniform(0.1, 2, (d, d, d)), 0.0)
    tvec = rng.normal(size=(d, d, d, 3)).astype(np.float32)
    qdata = np.roll(tdata, 1, axis=1)
    qvec = np.roll(tvec, 1, axis=1)
    probs_t = rng.random((4, d, d, d)).astype(np.float32)
    probs_q = np.roll(probs_t, 1, axis=2)
    angles = orc.calc_angle_comb(60.0)
    return orc, d, tdata, tvec, qdata, qvec, probs_t, probs_q, angles


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from vesper_python_gb300 import shard
        orc, d, tdata, tvec, qdata, qvec, pt, pq, angles = _problem()
        lo, hi = shard.shard_range(len(angles), rank, world)
        ts = orc.target_spectra(orc.mode_field("V", tdata, tvec))
        sc, _ = orc.search(ts, "V", qdata, qvec, angles[lo:hi], 0.0)
        top_sc, top_ix = shard.gather_topn(sc.astype(np.float64), 10, lo)
        t7 = orc.target_spectra([tvec[..., 0], tvec[..., 1], tvec[..., 2]] + list(pt))
        vs = [orc.rot_and_search_prob(t7, qdata, qvec, pq, a, 0.5)[0] for a in angles[lo:hi]]
        ps = [orc.rot_and_search_prob(t7, qdata, qvec, pq, a, 0.5)[2] for a in angles[lo:hi]]
        rd3 = 1.0 / d ** 3
        allv = shard.gather_scores(np.asarray(vs, np.float64) * rd3)
        allp = shard.gather_scores(np.asarray(ps, np.float64) * rd3)
        stats = shard.prob_stats(allv, allp)
        if rank == 0:
            out.put((top_ix.tolist(), [float(s) for s in stats]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_search_equals_single_process(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    top_ix, stats = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    orc, d, tdata, tvec, qdata, qvec, pt, pq, angles = _problem()
    ts = orc.target_spectra(orc.mode_field("V", tdata, tvec))
    sc, _ = orc.search(ts, "V", qdata, qvec, angles, 0.0)
    assert top_ix == list(orc.topn(sc, 10))
    t7 = orc.target_spectra([tvec[..., 0], tvec[..., 1], tvec[..., 2]] + list(pt))
    res = [orc.rot_and_search_prob(t7, qdata, qvec, pq, a, 0.5) for a in angles]
    ref = orc.prob_stats([r[0] for r in res], [r[2] for r in res], 1.0 / d ** 3)
    assert stats == [float(s) for s in ref]


# ---------------------------------------------------------------------------
# the product's sharded search (vesper.search_device_sharded, the call
# search_map_fft / search_map_fft_prob / Aligner.align_many make when given a
# process group), with the per-rank GPU search stubbed to the oracle
# ---------------------------------------------------------------------------

class _FakeLib:
    @staticmethod
    def vesper_search_nscore(code, with_mix):
        return (3 if with_mix else 2) if code == 5 else 1


class _FakeDev:
    device = "cpu"
    lib = _FakeLib()

    @staticmethod
    def to_dev(a, dtype=None):
        import torch
        return torch.as_tensor(a)


def _oracle_search_device(problem):
    """search_device stand-in for CPU ranks: rotmats rows are angle rows; the
    oracle computes the raw scores and linear translations."""
    import torch
    orc, d, tdata, tvec, qdata, qvec, pt, pq, angles = problem

    def search_device(spec, data, vec, mode, ave, rotmats, probs=None, mix=None, dev=None, **kw):
        rows = rotmats.numpy()
        if mode == "prob":
            t7 = orc.target_spectra([tvec[..., 0], tvec[..., 1], tvec[..., 2]] + list(pt))
            out = [orc.rot_and_search_prob(t7, qdata, qvec, pq, a, 0.5) for a in rows]
            sc = np.array([[o[0], o[2]] for o in out], np.float32)
            tr = [[o[1], o[3]] for o in out]
        else:
            ts = orc.target_spectra(orc.mode_field("V", tdata, tvec))
            s, t = orc.search(ts, "V", qdata, qvec, rows, 0.0)
            sc = s.reshape(-1, 1).astype(np.float32)
            tr = [[tuple(x)] for x in t]
        ln = np.array([[(a * d + b) * d + c for (a, b, c) in r] for r in tr], np.int32).reshape(sc.shape)
        return torch.as_tensor(sc), torch.as_tensor(ln)
    return search_device


def _product_worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import torch
        from vesper_python_gb300 import vesper as vg
        prob = _problem()
        orc, d, *_rest, angles = prob
        vg.search_device = _oracle_search_device(prob)
        rot = torch.as_tensor(np.asarray(angles, np.float64))
        sc, ln = vg.search_device_sharded(None, None, None, "VecProduct", 0.0, rot, dist.group.WORLD, dev=_FakeDev())
        s1, _ = vg.search_device_sharded(None, None, None, "prob", 0.0, rot, dist.group.WORLD, dev=_FakeDev())
        rd3 = 1.0 / d ** 3
        s1 = s1.numpy().astype(np.float64) * rd3
        stats = (np.std(s1[:, 0]), np.mean(s1[:, 0]), np.std(s1[:, 1]), np.mean(s1[:, 1]))
        if rank == 0:
            out.put((sc.numpy()[:, 0].tolist(), ln.numpy()[:, 0].tolist(), [float(v) for v in stats]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_product_sharded_search_equals_single_process(world):
    """search_device_sharded across gloo ranks: every rotation's score and
    translation, the stable top-10 and the prob statistics equal the
    single-process results."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_product_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    sc, ln, stats = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    orc, d, tdata, tvec, qdata, qvec, pt, pq, angles = _problem()
    ts = orc.target_spectra(orc.mode_field("V", tdata, tvec))
    osc, otr = orc.search(ts, "V", qdata, qvec, angles, 0.0)
    assert np.array_equal(np.asarray(sc, np.float32), osc.astype(np.float32))
    assert ln == [int((a * d + b) * d + c) for a, b, c in otr]
    assert list(orc.topn(np.asarray(sc), 10)) == list(orc.topn(osc, 10))
    t7 = orc.target_spectra([tvec[..., 0], tvec[..., 1], tvec[..., 2]] + list(pt))
    res = [orc.rot_and_search_prob(t7, qdata, qvec, pq, a, 0.5) for a in angles]
    ref = orc.prob_stats([r[0] for r in res], [r[2] for r in res], 1.0 / d ** 3)
    assert stats == [float(s) for s in ref]
