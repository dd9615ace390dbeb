"""Small, self-contained cases for profiler captures of single kernels, run
through ``python bench.py --case <name> [arg]``:

  search<d> [nrot [batch]]
      three register/fused-path searches of seeded random side-d fields over
      the first nrot (default 1008) rotations of the 30-degree grid, with the
      autotuned launch shape or the given batch
  prop
      learned-proposal scorings (committed weights) of one held-out
      128^3 / 64^3 pair at s = 3 over the 10-degree grid, timed
  cufft<d> [nrot]
      comparison only: the FFT work of a mode-V search through cuFFT
      (torch.fft, no gather) next to this library's whole search, per rotation
  tcb<d>
      the split-BF16 tensor-core pass B alone on random side-d spectra
      (prob layout, 16 rotations), timed
  fastvec
      fastVEC of both maps of the seed-0 128^3 / 64^3 generator pair at s = 3,
      g = 16 (the learned-proposal workload's maps), timed per map
  prob<d>
      prob-mode searches (both passes) of seeded random side-d fields with
      four probability channels over the 15-degree grid, timed per kernel
      family (at sides 32 and 64 also with pass B on the tensor cores)

Each run is a few GPU milliseconds, so a capture of one of its launches ends
in seconds.
"""
from __future__ import annotations

import sys

import numpy as np
import torch

from vesper_python_gb300 import proposal as P
from vesper_python_gb300 import vesper as vg


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    dev = vg.default_device()
    what = argv[0]
    if what.startswith("search"):
        d = int(what[6:])
        nrot = int(argv[1]) if len(argv) > 1 else 1008
        rng = np.random.default_rng(d)
        data = rng.uniform(0.1, 2, size=(d, d, d))
        data[rng.random((d, d, d)) < 0.5] = 0
        vec = rng.normal(size=(d, d, d, 3))
        vec /= np.linalg.norm(vec, axis=-1, keepdims=True)
        vec[data == 0] = 0
        td, tv = dev.to_dev(data), dev.to_dev(vec.astype(np.float32))
        spec = vg.target_spectra_device(td, tv, "VecProduct", 0.0, dev=dev)
        mats = dev.to_dev(vg.rot_matrices(vg.calc_angle_comb(30.0)[:nrot]))
        batch = int(argv[2]) if len(argv) > 2 else 0     # a fixed batch: no autotuning launches
        for _ in range(3):
            vg.search_device(spec, td, tv, "VecProduct", 0.0, mats, dev=dev, tuned=batch == 0, batch=batch)
    elif what.startswith("prob"):
        # prob mode: both passes (statistics pass, mixed pass) over the 15-degree
        # grid on seeded random side-d fields with four probability channels;
        # prints the device time per rotation of each pass and kernel family
        d = int(what[4:])
        rng = np.random.default_rng(d)

        def fields():
            data = rng.uniform(0.1, 2, size=(d, d, d))
            data[rng.random((d, d, d)) < 0.6] = 0
            vec = rng.normal(size=(d, d, d, 3))
            vec /= np.linalg.norm(vec, axis=-1, keepdims=True)
            vec[data == 0] = 0
            probs = rng.dirichlet([0.5] * 4, size=(d, d, d)).astype(np.float32).transpose(3, 0, 1, 2).copy()
            probs[:, data == 0] = 0
            return dev.to_dev(data), dev.to_dev(vec.astype(np.float32)), dev.to_dev(probs)
        td, tv, tp = fields()
        qd, qv, qp = fields()
        spec = vg.target_spectra_device(td, tv, "prob", 0.0, probs=tp, dev=dev)
        mats = vg.rot_matrices_device(vg.calc_angle_comb(15.0), dev, key=("grid", 15.0))
        n = int(mats.shape[0])
        mix = (0.5, 1.0, 0.0, 1.0, 0.0)
        paths = [0, 1] if vg.search_plan(d, "prob", dev=dev)[0] == 1 else [0]
        if d in (32, 64):
            paths.append(3)       # pass B on the tensor cores (split-BF16)
        for path in paths:
            for label, mx in (("pass1", None), ("pass2", mix)):
                vg.search_device(spec, qd, qv, "prob", 0.0, mats, probs=qp, mix=mx, dev=dev, opts=(path, 0, 0))
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(3):
                    vg.search_device(spec, qd, qv, "prob", 0.0, mats, probs=qp, mix=mx, dev=dev, opts=(path, 0, 0))
                e1.record()
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / 3
                prof = {}
                vg.search_device(spec, qd, qv, "prob", 0.0, mats, probs=qp, mix=mx, dev=dev, opts=(path, 0, 0),
                                 profile=prof)
                passes = " / ".join(f"{1000 * t / n:.3f}" for t in prof["pass_ms"][:3])
                print(f"prob side {d} path {path} {label}: {ms:.2f} ms for {n} rotations, "
                      f"{1000 * ms / n:.3f} us per rotation (passes A / B / C {passes} us)")
    elif what.startswith("cufft"):
        # comparison only: the FFT work of a mode-V search done by cuFFT
        # (torch.fft), in batches of 64 rotations of already rotated fields (no
        # gather): 3 forward real transforms, product with the conjugate target
        # spectra, channel sum, inverse transform, argmax; next to this
        # library's whole search (gather included) on the same side
        d = int(what[5:])
        nrot = int(argv[1]) if len(argv) > 1 else 1024
        B = 64
        g = torch.Generator(device=dev.device).manual_seed(d)
        x = torch.randn((B, 3, d, d, d), device=dev.device, generator=g)
        T = torch.fft.rfftn(torch.randn((3, d, d, d), device=dev.device, generator=g), dim=(-3, -2, -1)).conj()

        def cufft_search():
            for _ in range(0, nrot, B):
                X = torch.fft.rfftn(x, dim=(-3, -2, -1))
                r = torch.fft.irfftn((X * T).sum(dim=1), s=(d, d, d), dim=(-3, -2, -1))
                r.reshape(B, -1).argmax(dim=1)

        rng = np.random.default_rng(d)
        data = rng.uniform(0.1, 2, size=(d, d, d))
        data[rng.random((d, d, d)) < 0.5] = 0
        vec = rng.normal(size=(d, d, d, 3))
        vec /= np.linalg.norm(vec, axis=-1, keepdims=True)
        vec[data == 0] = 0
        td, tv = dev.to_dev(data), dev.to_dev(vec.astype(np.float32))
        spec = vg.target_spectra_device(td, tv, "VecProduct", 0.0, dev=dev)
        ang = vg.calc_angle_comb(10.0)[:nrot]
        mats = dev.to_dev(vg.rot_matrices(ang))

        def ours():
            vg.search_device(spec, td, tv, "VecProduct", 0.0, mats, dev=dev, tuned=True)

        for name, fn, n in (("cuFFT (torch.fft), no gather", cufft_search, (nrot + B - 1) // B * B),
                            ("this library's search", ours, len(ang))):
            fn()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            for _ in range(3):
                fn()
            e1.record()
            torch.cuda.synchronize()
            print(f"side {d} {name}: {1000 * e0.elapsed_time(e1) / 3 / n:.3f} us per rotation")
    elif what.startswith("tcb"):
        # the tensor-core pass B alone (vesper_tc_pass_b) on random spectra of
        # side d, prob-mode layout (7 channels, 2 groups), 16 rotations, 3 calls
        import ctypes

        from vesper_python_gb300 import _native
        d = int(what[3:])
        H = d // 2 + 1
        nb = 16
        g = torch.Generator(device=dev.device).manual_seed(d)
        S = torch.randn((nb, 7, d, d, H), dtype=torch.complex64, device=dev.device, generator=g)
        T = torch.randn((7, d, d, H), dtype=torch.complex64, device=dev.device, generator=g)
        U = torch.empty((nb, 2, d, d, H), dtype=torch.complex64, device=dev.device)
        err = torch.zeros(1, dtype=torch.int32, device=dev.device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for i in range(4):
            if i == 1:
                e0.record()
            _native.check(dev.lib.vesper_tc_pass_b(ctypes.c_void_p(S.data_ptr()), ctypes.c_void_p(T.data_ptr()),
                                                   ctypes.c_void_p(U.data_ptr()), d, 7, 2, 3, nb,
                                                   ctypes.c_void_p(err.data_ptr()), dev.stream))
        e1.record()
        torch.cuda.synchronize()
        print(f"tensor pass B side {d}: {1000 * e0.elapsed_time(e1) / 3 / nb:.3f} us per rotation, "
              f"status {int(err.item())}")
    elif what == "fastvec":
        import contextlib
        import io

        from vesper_python_gb300 import synth
        pair = synth.workload_pair("prop128_s3_a10", seed=0)
        for name, (src, orig) in (("map1", (pair.map1, pair.orig1)), ("map2", (pair.map2, pair.orig2))):
            m = vg.mrc_obj.from_array(src, 1.0, orig)
            with contextlib.redirect_stdout(io.StringIO()):
                _, mn = vg.mrc_set_vox_size(m, 0.1, 3.0)
            sd = dev.to_dev(m.data)
            args = (sd, np.float64(m.xwidth), m.orig.astype(np.float64), mn.xdim, 3.0, mn.orig, 16.0)
            vg.fastvec_device(*args, dev=dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            for _ in range(10):
                vg.fastvec_device(*args, dev=dev)
            e1.record()
            torch.cuda.synchronize()
            print(f"fastvec {name} {m.data.shape} -> {mn.xdim}^3: {1000 * e0.elapsed_time(e1) / 10:.1f} us per map")
    elif what == "prop":
        net = P.load_weights(dev)[0]
        maker = P.PairMaker(dev)
        mats = vg.rot_matrices_device(vg.calc_angle_comb(10.0), dev, key=("grid", 10.0))
        pf = maker.fields(30_000_000)
        net.rotation_scores(pf.fTQ, mats)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(3):
            net.rotation_scores(pf.fTQ, mats)
        e1.record()
        torch.cuda.synchronize()
        print(f"proposal scores of one pair, {int(mats.shape[0])} rotations: {e0.elapsed_time(e1) / 3:.3f} ms "
              f"(encoder and scoring)")
    else:
        raise SystemExit(f"unknown case {what!r}")
    torch.cuda.synchronize()
    print("ok", what)


