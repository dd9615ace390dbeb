"""Autotuner for the rotational search launch shape.

For a (grid side, mode) pair it times vesper_search_tuned over a sample of
rotations for every candidate of

  batch      rotations per pipeline step (8 to 256, and up to 2048 while S + U of
             a step stay within 160 MB)
  cchunk     channels gathered and transformed per pass-A block
  W          spectrum columns per pass-B block

and keeps the fastest.  The kernel family (register two-step FFT where it is
compiled for the side, radix-stage otherwise) is fixed by the side, so every
candidate computes bit-identical results and the choice only changes speed.
Results are cached per process and, unless VESPER_AUTOTUNE_CACHE is set to
an empty string, in a JSON file (default ~/.cache/vesper_gb300/autotune.json).
"""
from __future__ import annotations

import json
import os
import threading

import torch

_lock = threading.Lock()
_mem: dict = {}


def _cache_path():
    p = os.environ.get("VESPER_AUTOTUNE_CACHE")
    if p is None:
        p = os.path.join(os.path.expanduser("~"), ".cache", "vesper_gb300", "autotune.json")
    return p or None


_NAMES: dict = {}


def _key(dim, mode, dev):
    name = _NAMES.get(dev.device)
    if name is None:
        name = _NAMES[dev.device] = torch.cuda.get_device_name(dev.device) if torch.cuda.is_available() else "cpu"
    return f"{name}|d={dim}|mode={mode}"


def _load_disk():
    p = _cache_path()
    if not p or not os.path.exists(p):
        return {}
    try:
        with open(p) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save_disk(entries):
    p = _cache_path()
    if not p:
        return
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + f".{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(entries, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass


BATCHES = (8, 16, 32, 64, 128, 256, 512, 1024, 2048)
# S + U of one batch above 256 rotations: about the L2 size.  Up to 256 every
# side tries the batch whatever its size: at side 75 (5.1 MB of S per
# rotation, mode V) 256 rotations ran 8.7 us per rotation against 8.9 with
# 128 and 11.5 with 16, the largest batch whose S stays in L2, since the S
# round trip through DRAM costs less than the CTAs a smaller batch leaves idle.
BATCH_BYTES = 160 << 20


def candidates(nch, dim=None, ngrp=1):
    per = None if dim is None else (nch + ngrp) * dim * dim * (dim // 2 + 1) * 8
    out = []
    for batch in BATCHES:
        if batch > 256 and (per is None or batch * per > BATCH_BYTES):
            continue
        for cc in sorted({1, nch}):
            for W in (16, 32):
                out.append({"batch": batch, "cchunk": cc, "W": W})
    return out


def tune(dev, spec, data, vec, mode, ave, rotmats, probs=None, mix=None, sample=256, reps=2):
    """Time every candidate on the first ``sample`` rotations; return the best
    {"batch", "cchunk", "W", "ms_per_rot"}."""
    from . import vesper as vg
    dim = int(data.shape[0])
    key = _key(dim, mode, dev)
    with _lock:
        if key in _mem:
            return _mem[key]
        disk = _load_disk()
        if key in disk:
            _mem[key] = disk[key]
            return disk[key]
    if vg.search_plan(dim, mode, 0, 1, None, dev)[0] == 2:
        # the fused single-kernel search has no launch shape to choose
        best = {"batch": 0, "cchunk": 0, "W": 0, "ms_per_rot": None, "path": 2}
        with _lock:
            _mem[key] = best
        return best
    nch = {"VecProduct": 3, "prob": 7}.get(mode, 1)
    ngrp = 2 if mode == "prob" else 1
    cands = candidates(nch, dim, ngrp)
    # the sample covers two steps of the largest batch tried
    sample = max(sample, 2 * max(c["batch"] for c in cands))
    mats = rotmats[: min(sample, rotmats.shape[0])]
    best = None
    for c in cands:
        try:
            ms = None
            for _ in range(reps):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                vg.search_device(spec, data, vec, mode, ave, mats, probs=probs, mix=mix, batch=c["batch"], dev=dev,
                                 opts=(-1, c["cchunk"], c["W"]))
                e1.record()
                torch.cuda.synchronize()
                t = e0.elapsed_time(e1)
                ms = t if ms is None else min(ms, t)
        except Exception:   # a candidate that does not fit is skipped
            continue
        per = ms / mats.shape[0]
        if best is None or per < best["ms_per_rot"]:
            best = dict(c, ms_per_rot=per)
    if best is None:
        best = {"batch": 0, "cchunk": 0, "W": 0, "ms_per_rot": None}
    with _lock:
        _mem[key] = best
        disk = _load_disk()
        disk[key] = best
        _save_disk(disk)
    return best


def cached(dim, mode, dev):
    with _lock:
        return _mem.get(_key(dim, mode, dev))
