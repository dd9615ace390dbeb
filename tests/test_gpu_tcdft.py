"""Split-BF16 tensor-core pass B (vesper_tc_pass_b) against the same pass in
float64 numpy: U[b][g] = IDFT_x( sum_{c in g} T_c * DFT_x(S_c) ), unnormalised.
The split keeps about 16 significant bits per operand, so the tolerance is
1e-4 of the largest |U| (the float32 FFT path holds about 1e-6)."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _run(dev, S, T, ngrp, split):
    from vesper_python_gb300 import _native
    nb, nch, d = S.shape[0], S.shape[1], S.shape[2]
    St = dev.to_dev(S.astype(np.complex64))
    Tt = dev.to_dev(T.astype(np.complex64))
    U = torch.zeros((nb, ngrp) + S.shape[2:], dtype=torch.complex64, device=dev.device)
    err = torch.zeros(1, dtype=torch.int32, device=dev.device)
    _native.check(dev.lib.vesper_tc_pass_b(ctypes.c_void_p(St.data_ptr()), ctypes.c_void_p(Tt.data_ptr()),
                                           ctypes.c_void_p(U.data_ptr()), d, nch, ngrp, split, nb,
                                           ctypes.c_void_p(err.data_ptr()), dev.stream))
    torch.cuda.synchronize()
    return U.cpu().numpy(), int(err.item())


def _want(S, T, ngrp, split):
    X = np.fft.fft(S.astype(np.complex128), axis=2)
    d = S.shape[2]
    groups = [(0, split), (split, S.shape[1])] if ngrp == 2 else [(0, S.shape[1])]
    out = []
    for cb, ce in groups:
        P = np.sum(T[None, cb:ce] * X[:, cb:ce], axis=1)
        out.append(np.fft.ifft(P, axis=1) * d)
    return np.stack(out, axis=1)


@pytest.mark.parametrize("d,nch,ngrp,split", [(32, 3, 1, 3), (32, 7, 2, 3), (64, 7, 2, 3), (64, 3, 1, 3)])
def test_tc_pass_b_matches_float64(dev, d, nch, ngrp, split):
    rng = np.random.default_rng(d + nch)
    H = d // 2 + 1
    nb = 3
    S = rng.normal(size=(nb, nch, d, d, H)) + 1j * rng.normal(size=(nb, nch, d, d, H))
    T = rng.normal(size=(nch, d, d, H)) + 1j * rng.normal(size=(nch, d, d, H))
    got, err = _run(dev, S, T, ngrp, split)
    assert err == 0
    want = _want(S, T, ngrp, split)
    scale = np.max(np.abs(want))
    rel = np.max(np.abs(got - want)) / scale
    assert rel < 1e-4, rel


def _fields(rng, d, zero_frac=0.6):
    data = rng.uniform(0.1, 2.0, size=(d, d, d))
    data[rng.random((d, d, d)) < zero_frac] = 0
    vec = rng.normal(size=(d, d, d, 3))
    vec /= np.linalg.norm(vec, axis=-1, keepdims=True)
    vec[data == 0] = 0
    probs = rng.dirichlet([0.5] * 4, size=(d, d, d)).astype(np.float32).transpose(3, 0, 1, 2).copy()
    probs[:, data == 0] = 0
    return data, vec.astype(np.float32), probs


@pytest.mark.parametrize("d", [32, 64])
def test_prob_search_tensor_pass_b_vs_fp64_oracle(dev, d):
    """Prob-mode search with pass B on the tensor cores (path 3) and with the
    float32 register passes (path 1), both against the float64 oracle: vector
    and probability scores, and the mixed score.  Bars: path 1 as its own
    test (1e-4, 1e-3); path 3 at 5e-4 and 5e-3 of the largest score (the
    split-BF16 operands keep about 16 bits).  The measured errors are
    printed."""
    from oracle import vesper_oracle as orc
    from vesper_python_gb300 import vesper as vg
    rng = np.random.default_rng(100 + d)
    tdata, tvec, tprobs = _fields(rng, d)
    qdata, qvec, qprobs = _fields(rng, d)
    angles = orc.calc_angle_comb(30.0)[::173]
    spec = vg.target_spectra_device(dev.to_dev(tdata), dev.to_dev(tvec), "prob", 0.0, probs=dev.to_dev(tprobs),
                                    dev=dev)
    mats = dev.to_dev(vg.rot_matrices(angles))
    qd, qv, qp = dev.to_dev(qdata), dev.to_dev(qvec), dev.to_dev(qprobs)
    tspec = orc.target_spectra([tvec[..., 0], tvec[..., 1], tvec[..., 2]] + list(tprobs))
    ref = [orc.rot_and_search_prob(tspec, qdata, qvec, list(qprobs), a, 0.5, None, fp64=True) for a in angles]
    rv = np.array([r[0] for r in ref])
    rp = np.array([r[2] for r in ref])
    st = orc.prob_stats(rv, rp, 1.0 / d ** 3)
    mix = (0.5,) + tuple(st)
    refm = np.array([orc.rot_and_search_prob(tspec, qdata, qvec, list(qprobs), a, 0.5, st, fp64=True)[4]
                     for a in angles], np.float64)
    assert vg.search_plan(d, "prob", opts=(3, 0, 0), dev=dev)[0] == 3
    errs = {}
    for path in (1, 3):
        s1, _ = vg.search_device(spec, qd, qv, "prob", 0.0, mats, probs=qp, dev=dev, opts=(path, 0, 0))
        s2, _ = vg.search_device(spec, qd, qv, "prob", 0.0, mats, probs=qp, mix=mix, dev=dev, opts=(path, 0, 0))
        s1 = s1.cpu().numpy().astype(np.float64)
        s2 = s2.cpu().numpy().astype(np.float64)
        errs[path] = (np.max(np.abs(s1[:, 0] - rv)) / np.max(np.abs(rv)),
                      np.max(np.abs(s1[:, 1] - rp)) / np.max(np.abs(rp)),
                      np.max(np.abs(s2[:, 2] - refm)) / np.max(np.abs(refm)))
    print(f"side {d}: relative errors (vec, prob, mixed) float32 path {errs[1]}, split-BF16 path {errs[3]}")
    assert max(errs[1][:2]) < 1e-4 and errs[1][2] < 1e-3
    assert max(errs[3][:2]) < 5e-4 and errs[3][2] < 5e-3


def test_vec_search_tensor_pass_b_side32(dev):
    """Mode V at side 32 with pass B on the tensor cores: scores against the
    float32 path within 5e-4 of the largest, best translations equal except
    where the two scores are that close."""
    from oracle import vesper_oracle as orc
    from vesper_python_gb300 import vesper as vg
    d = 32
    rng = np.random.default_rng(7)
    tdata, tvec, _ = _fields(rng, d, 0.5)
    qdata, qvec, _ = _fields(rng, d, 0.5)
    spec = vg.target_spectra_device(dev.to_dev(tdata), dev.to_dev(tvec), "VecProduct", 0.0, dev=dev)
    mats = dev.to_dev(vg.rot_matrices(orc.calc_angle_comb(30.0)[::7]))
    qd, qv = dev.to_dev(qdata), dev.to_dev(qvec)
    sa, la = vg.search_device(spec, qd, qv, "VecProduct", 0.0, mats, dev=dev, opts=(1, 0, 0))
    sb, lb = vg.search_device(spec, qd, qv, "VecProduct", 0.0, mats, dev=dev, opts=(3, 0, 0))
    sa, sb = sa.cpu().numpy()[:, 0], sb.cpu().numpy()[:, 0]
    scale = np.max(np.abs(sa))
    assert np.max(np.abs(sa - sb)) < 5e-4 * scale
    diff = la.cpu().numpy()[:, 0] != lb.cpu().numpy()[:, 0]
    assert np.all(np.abs(sa - sb)[diff] < 5e-4 * scale)
    assert int(diff.sum()) <= max(1, len(sa) // 50)


def test_tc_wait_timeout_is_reported_and_context_survives(dev):
    """Failure detection without a fault: the stall self-test makes every CTA
    wait on a barrier that nothing completes; the bounded wait gives up after
    20 ms, the status word reads 1, and the same context then runs the pass
    correctly."""
    from vesper_python_gb300 import _native
    d, nch, ngrp, split = 32, 7, 2, 3
    rng = np.random.default_rng(9)
    H = d // 2 + 1
    S = rng.normal(size=(1, nch, d, d, H)) + 1j * rng.normal(size=(1, nch, d, d, H))
    T = rng.normal(size=(nch, d, d, H)) + 1j * rng.normal(size=(nch, d, d, H))
    St, Tt = dev.to_dev(S.astype(np.complex64)), dev.to_dev(T.astype(np.complex64))
    U = torch.zeros((1, ngrp) + S.shape[2:], dtype=torch.complex64, device=dev.device)
    err = torch.zeros(1, dtype=torch.int32, device=dev.device)
    _native.check(dev.lib.vesper_tc_pass_b_stall_test(ctypes.c_void_p(St.data_ptr()), ctypes.c_void_p(Tt.data_ptr()),
                                                      ctypes.c_void_p(U.data_ptr()), d, nch, ngrp, split, 20,
                                                      ctypes.c_void_p(err.data_ptr()), dev.stream))
    torch.cuda.synchronize()
    assert int(err.item()) == 1
    assert float(U.abs().max().item()) == 0.0        # nothing written
    got, err2 = _run(dev, S, T, ngrp, split)
    assert err2 == 0
    want = _want(S, T, ngrp, split)
    assert np.max(np.abs(got - want)) / np.max(np.abs(want)) < 1e-4


def test_search_is_deterministic(dev):
    """The same search twice gives the same bits (float32 path and the
    tensor-core path): the argmax keys are atomic maxima and every reduction
    has a fixed order."""
    from oracle import vesper_oracle as orc
    from vesper_python_gb300 import vesper as vg
    d = 32
    rng = np.random.default_rng(21)
    tdata, tvec, _ = _fields(rng, d, 0.5)
    qdata, qvec, _ = _fields(rng, d, 0.5)
    spec = vg.target_spectra_device(dev.to_dev(tdata), dev.to_dev(tvec), "VecProduct", 0.0, dev=dev)
    mats = dev.to_dev(vg.rot_matrices(orc.calc_angle_comb(30.0)[::5]))
    qd, qv = dev.to_dev(qdata), dev.to_dev(qvec)
    for path in (-1, 3):
        a = vg.search_device(spec, qd, qv, "VecProduct", 0.0, mats, dev=dev, opts=(path, 0, 0))
        b = vg.search_device(spec, qd, qv, "VecProduct", 0.0, mats, dev=dev, opts=(path, 0, 0))
        assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1]), path
