"""The proposal network's float64 oracle checked by central finite differences
(CPU only): the oracle is what the GPU gradients are compared with."""
import numpy as np
import pytest

from oracle import proposal_oracle as po
from oracle import vesper_oracle as orc


def _fd(f, x, idx, eps=1e-6):
    xp = x.copy()
    xm = x.copy()
    xp[idx] += eps
    xm[idx] -= eps
    return (f(xp) - f(xm)) / (2 * eps)


@pytest.fixture(scope="module")
def small_net():
    rng = np.random.default_rng(0)
    ch = (4, 5, 3)
    layers = []
    for cin, cout in zip(ch[:-1], ch[1:]):
        layers.append((rng.normal(size=(cout, cin, 27)) * 0.3, rng.normal(size=cout) * 0.1, 1))
    layers[-1] = (layers[-1][0], layers[-1][1], 0)
    return layers


def test_conv_bwd_finite_differences(small_net):
    rng = np.random.default_rng(1)
    d = 4
    x = rng.normal(size=(4, d, d, d))
    g = rng.normal(size=(3, d, d, d))

    def loss(layers, xx):
        return float(np.sum(po.encoder_fwd(xx, layers)[-1] * g))

    acts = po.encoder_fwd(x, small_net)
    grads = po.encoder_bwd(acts, small_net, g)
    for li in range(len(small_net)):
        W, b, relu = small_net[li]
        for idx in [(0, 0, 0), (1, 2, 13), (2, 3, 26)]:
            if idx[0] >= W.shape[0] or idx[1] >= W.shape[1]:
                continue

            def f(Wm, li=li):
                ls = list(small_net)
                ls[li] = (Wm, ls[li][1], ls[li][2])
                return loss(ls, x)
            assert abs(_fd(f, W, idx) - grads[li][0][idx]) < 1e-5 * max(1.0, abs(grads[li][0][idx]))

        def fb(bm, li=li):
            ls = list(small_net)
            ls[li] = (ls[li][0], bm, ls[li][2])
            return loss(ls, x)
        assert abs(_fd(fb, b, (1,)) - grads[li][1][1]) < 1e-5 * max(1.0, abs(grads[li][1][1]))


@pytest.mark.parametrize("d", [5, 6])
def test_score_bwd_finite_differences(d):
    rng = np.random.default_rng(d)
    K = 3
    ET = rng.normal(size=(K, d ** 3))
    EQ = rng.normal(size=(K, d ** 3))
    from vesper_python_gb300 import vesper as vg
    mats = vg.rot_matrices(orc.calc_angle_comb(30.0)[::211])
    maps = [po.src_map(d, m) for m in mats]
    g = rng.normal(size=len(maps))
    gT, gQ = po.score_bwd(ET, EQ, maps, g)
    f_t = lambda e: float(np.dot(po.score_fwd(e, EQ, maps), g))
    f_q = lambda e: float(np.dot(po.score_fwd(ET, e, maps), g))
    for idx in [(0, 0), (1, d ** 3 // 2), (2, d ** 3 - 1)]:
        assert abs(_fd(f_t, ET, idx) - gT[idx]) < 1e-6 * max(1.0, abs(gT[idx]))
        assert abs(_fd(f_q, EQ, idx) - gQ[idx]) < 1e-6 * max(1.0, abs(gQ[idx]))


def test_softmax_ce_finite_differences():
    rng = np.random.default_rng(3)
    s = rng.normal(size=40) * 5
    q = rng.random(40) ** 4
    q /= q.sum()
    loss, g = po.softmax_ce(s, q, 0.4)
    assert loss > 0
    for i in (0, 7, 39):
        assert abs(_fd(lambda v: po.softmax_ce(v, q, 0.4)[0], s, (i,)) - g[i]) < 1e-6


def test_src_map_is_reference_gather():
    """src_map agrees with the oracle's rot_mrc gather (every voxel nonzero,
    so the reference's gather takes every in-bounds voxel)."""
    d = 7
    rng = np.random.default_rng(4)
    data = rng.uniform(0.5, 1.0, size=(d, d, d))
    vec = np.zeros((d, d, d, 3), np.float32)
    ang = orc.calc_angle_comb(30.0)[100]
    F = orc.rot_matrix_f32(ang)
    _, od = orc.rot_mrc(data, vec, ang, F)
    m = po.src_map(d, F)
    want = np.where(m >= 0, data.reshape(-1)[np.maximum(m, 0)], 0.0)
    np.testing.assert_array_equal(od.reshape(-1), want)
