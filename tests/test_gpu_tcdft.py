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
