"""vesper_search_static: the search for callers that cannot allocate device
memory (code that runs while another thread holds a global-mode stream
capture, where cudaMalloc fails, or a host application that hands over only
pre-allocated buffers under a fixed device-memory budget).  It uses a fixed
scratch array inside the library instead of a caller-provided workspace.
Called through the C ABI and compared with vesper_search on the same inputs,
bit for bit (every pipeline batch computes the same results), on two calls in
a row: the second call finds the first call's leftovers in the shared
scratch.  The cases cover the fused kernel (keys only), the register passes
(the S/U regions), the radix-stage passes in prob mode and the Laplacian
mode's rotated-density region.  The device's free memory is the same before
and after a call, and a call records into a CUDA graph captured in global
mode."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import vesper_oracle as orc

pytestmark = pytest.mark.gpu


def _field(rng, d, zero_frac=0.6):
    data = rng.uniform(0.1, 2.0, size=(d, d, d))
    data[rng.random((d, d, d)) < zero_frac] = 0.0
    vec = rng.normal(size=(d, d, d, 3))
    vec /= np.linalg.norm(vec, axis=-1, keepdims=True)
    vec[data == 0] = 0
    return data, vec.astype(np.float32)


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _static_search(lib, dev, spec, qd, qv, qp, d, mode, mats, mix, sc, ln):
    """One vesper_search_static call into the preallocated outputs sc, ln;
    returns the device's free memory just before and just after the call."""
    n = int(mats.shape[0])
    sc.fill_(float("nan"))
    ln.fill_(-7)
    mixarr = (ctypes.c_double * 5)(*mix) if mix is not None else None
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(dev.device)[0]
    rc = lib.vesper_search_static(_p(spec), _p(qd), _p(qv), _p(qp), d, mode, 0.0, _p(mats), n, mixarr, _p(sc),
                                  _p(ln), dev.stream)
    assert rc == 0, lib.vesper_last_error()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info(dev.device)[0]
    return free0, free1


@pytest.mark.parametrize("mode_name,d", [("VecProduct", 24), ("VecProduct", 15), ("VecProduct", 30), ("prob", 16),
                                         ("Laplacian", 18)])
def test_static_search_matches_workspace_search(dev, mode_name, d):
    from vesper_python_gb300 import vesper as vg
    lib = dev.lib
    rng = np.random.default_rng(31 + d)
    tdata, tvec = _field(rng, d)
    qdata, qvec = _field(rng, d)
    probs_t = probs_q = None
    mix = None
    if mode_name == "prob":
        probs_t = dev.to_dev(rng.random((4, d, d, d)).astype(np.float32))
        probs_q = dev.to_dev(np.where(rng.random((4, d, d, d)) < 0.5, rng.random((4, d, d, d)), 0)
                             .astype(np.float32))
        mix = (0.5, 2.0, 1.0, 3.0, 4.0)
    spec = vg.target_spectra_device(dev.to_dev(tdata), dev.to_dev(tvec), mode_name, 0.0, probs=probs_t, dev=dev)
    mats = dev.to_dev(vg.rot_matrices(orc.calc_angle_comb(30.0)[::9]))
    qd, qv = dev.to_dev(qdata), dev.to_dev(qvec)
    ref_sc, ref_ln = vg.search_device(spec, qd, qv, mode_name, 0.0, mats, probs=probs_q, mix=mix, dev=dev)
    ref_sc = ref_sc.cpu().numpy()
    ref_ln = ref_ln.cpu().numpy()
    code = vg.MODE_CODES[mode_name]
    nscore = lib.vesper_search_nscore(code, 1 if mix is not None else 0)
    sc = torch.empty((int(mats.shape[0]), nscore), dtype=torch.float32, device=dev.device)
    ln = torch.empty((int(mats.shape[0]), nscore), dtype=torch.int32, device=dev.device)
    for call in range(2):
        free0, free1 = _static_search(lib, dev, spec, qd, qv, probs_q, d, code, mats, mix, sc, ln)
        if call == 1:   # after the first call's per-device and per-side set-up
            assert free1 == free0, "device memory changed across the call"
        np.testing.assert_array_equal(sc.cpu().numpy(), ref_sc, err_msg=f"call {call}")
        np.testing.assert_array_equal(ln.cpu().numpy(), ref_ln, err_msg=f"call {call}")


@pytest.mark.parametrize("mode_name,d", [("VecProduct", 30), ("prob", 16)])
def test_static_search_under_global_capture(dev, mode_name, d):
    """After a first call, vesper_search_static records into a CUDA graph
    captured in global mode (where an allocation or a synchronizing call would
    invalidate the capture), and the replayed graph gives the workspace
    search's results bit for bit."""
    from vesper_python_gb300 import vesper as vg
    lib = dev.lib
    rng = np.random.default_rng(57 + d)
    tdata, tvec = _field(rng, d)
    qdata, qvec = _field(rng, d)
    probs_t = probs_q = None
    mix = None
    if mode_name == "prob":
        probs_t = dev.to_dev(rng.random((4, d, d, d)).astype(np.float32))
        probs_q = dev.to_dev(np.where(rng.random((4, d, d, d)) < 0.5, rng.random((4, d, d, d)), 0)
                             .astype(np.float32))
        mix = (0.5, 2.0, 1.0, 3.0, 4.0)
    spec = vg.target_spectra_device(dev.to_dev(tdata), dev.to_dev(tvec), mode_name, 0.0, probs=probs_t, dev=dev)
    mats = dev.to_dev(vg.rot_matrices(orc.calc_angle_comb(30.0)[::7]))
    qd, qv = dev.to_dev(qdata), dev.to_dev(qvec)
    ref_sc, ref_ln = vg.search_device(spec, qd, qv, mode_name, 0.0, mats, probs=probs_q, mix=mix, dev=dev)
    ref_sc = ref_sc.cpu().numpy()
    ref_ln = ref_ln.cpu().numpy()
    code = vg.MODE_CODES[mode_name]
    nscore = lib.vesper_search_nscore(code, 1 if mix is not None else 0)
    n = int(mats.shape[0])
    sc = torch.empty((n, nscore), dtype=torch.float32, device=dev.device)
    ln = torch.empty((n, nscore), dtype=torch.int32, device=dev.device)
    _static_search(lib, dev, spec, qd, qv, probs_q, d, code, mats, mix, sc, ln)   # per-device and per-side set-up
    mixarr = (ctypes.c_double * 5)(*mix) if mix is not None else None
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, capture_error_mode="global"):
        rc = lib.vesper_search_static(_p(spec), _p(qd), _p(qv), _p(probs_q), d, code, 0.0, _p(mats), n, mixarr,
                                      _p(sc), _p(ln), dev.stream)
    assert rc == 0, lib.vesper_last_error()
    for replay in range(2):
        sc.fill_(float("nan"))
        ln.fill_(-7)
        g.replay()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(sc.cpu().numpy(), ref_sc, err_msg=f"replay {replay}")
        np.testing.assert_array_equal(ln.cpu().numpy(), ref_ln, err_msg=f"replay {replay}")


def test_static_search_rejects_oversize(dev):
    """Spectra, fields and 600,000 rotations' outputs at d=75 need more than
    the fixed scratch: the call is refused before any launch."""
    lib = dev.lib
    d = 75
    nrot = 600000
    small = torch.zeros(16, dtype=torch.float64, device=dev.device)
    out = torch.zeros(16, dtype=torch.float32, device=dev.device)
    rc = lib.vesper_search_static(_p(small), _p(small), _p(out), None, d, 0, 0.0, _p(out), nrot, None, _p(out),
                                  _p(out), dev.stream)
    assert rc == 2
    assert b"scratch" in lib.vesper_last_error()
    torch.cuda.synchronize()
