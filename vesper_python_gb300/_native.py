"""Build and load the sm_103a C-ABI library ``libvesper_gb300.so``.

The library is compiled in-tree with nvcc (one translation unit per .cu file,
compiled in parallel, one ``-gencode`` for sm_103a) and loaded with ctypes.
There is no fallback: every compute entry of the package calls through this
library and raises if it cannot be loaded.
"""
from __future__ import annotations

import ctypes
import glob
import os
import shutil
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "libvesper_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I" + INCLUDE]

_lock = threading.Lock()
_lib = None


class VesperError(RuntimeError):
    """A C-ABI call returned a non-zero vesper_status."""

    def __init__(self, code, msg):
        super().__init__(f"vesper error {code}: {msg}")
        self.code = code


def _nvcc():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvesper_gb300.so")
    return nvcc


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + [os.path.join(INCLUDE, "vesper_gb300.h")]


def needs_build() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(p) > t for p in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA source for sm_103a and link the shared library."""
    with _lock:
        if not force and not needs_build():
            return LIB_PATH
        os.makedirs(os.path.join(BUILD, "obj"), exist_ok=True)
        nvcc = _nvcc()
        srcs = _sources()

        def compile_one(src):
            obj = os.path.join(BUILD, "obj", os.path.basename(src)[:-3] + ".o")
            cmd = [nvcc, "-c", src, "-o", obj] + ARCH + NVCC_FLAGS
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr)
            return obj

        with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
            objs = list(ex.map(compile_one, srcs))
        tmp = LIB_PATH + f".{os.getpid()}.tmp"
        cmd = [nvcc, "-shared", "-o", tmp] + objs + ARCH
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
        return LIB_PATH


_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double
_sz = ctypes.c_size_t
_psz = ctypes.POINTER(ctypes.c_size_t)

# name -> argtypes (restype int for all)
SIGNATURES = {
    "vesper_version": [],
    "vesper_last_error": [],
    "vesper_max_dim": [_i],
    "vesper_fast_len_ok": [_i],
    "vesper_fp32_peak_probe": [_i, _i, _i, _vp, _vp, _vp],
    "vesper_prepare_map": [_vp, _i, _i, _i, _d, _vp, _vp, _vp],
    "vesper_prepare_maps": [_i, _vp, _vp, _vp, _vp, _vp, _vp],
    "vesper_map_stats": [_vp, _i, _vp, _vp],
    "vesper_map_stats_workspace_size": [_i, _psz],
    "vesper_map_stats_ws": [_vp, _i, _vp, _vp, _sz, _vp],
    "vesper_fastvec_workspace_size": [_i, _i, _i, _i, _psz],
    "vesper_fastvec": [_vp, _i, _i, _i, _d, _vp, _i, _d, _vp, _d, _vp, _vp, _vp, _vp, _sz, _vp],
    "vesper_rot_gather": [_vp, _vp, _vp, _i, _vp, _i, _vp, _vp, _vp, _vp],
    "vesper_spectra_bytes": [_i, _i, _psz],
    "vesper_target_workspace_size": [_i, _i, _psz],
    "vesper_target_spectra": [_vp, _vp, _vp, _i, _i, _d, _vp, _vp, _sz, _vp],
    "vesper_search_nscore": [_i, _i],
    "vesper_search_workspace_size": [_i, _i, _i, _i, _psz],
    "vesper_search": [_vp, _vp, _vp, _vp, _i, _i, _d, _vp, _i, _vp, _vp, _vp, _i, _vp, _sz, _vp],
    "vesper_search_profile": [_vp, _vp, _vp, _vp, _i, _i, _d, _vp, _i, _vp, _vp, _vp, _i, _vp, _sz, _vp, _vp, _vp,
                              _vp],
    "vesper_search_tuned": [_vp, _vp, _vp, _vp, _i, _i, _d, _vp, _i, _vp, _vp, _vp, _i, _vp, _sz, _vp, _vp],
    "vesper_search_plan": [_i, _i, _i, _i, _vp, _vp, _vp],
    "vesper_search_static": [_vp, _vp, _vp, _vp, _i, _i, _d, _vp, _i, _vp, _vp, _vp, _vp],
    "vesper_topn": [_vp, _i, _i, _i, _vp, _vp],
    "vesper_rescore_workspace_size": [_i, _psz],
    "vesper_rescore": [_vp, _vp, _d, _d, _d, _vp, _vp, _i, _vp, _vp, _vp, _vp, _sz, _vp],
    "vesper_rescore_batch_workspace_size": [_i, _i, _psz],
    "vesper_rescore_batch": [_vp, _vp, _d, _d, _d, _vp, _vp, _i, _vp, _i, _vp, _vp, _sz, _vp],
    "vesper_rescore_batch_dev": [_vp, _vp, _vp, _vp, _vp, _i, _vp, _i, _vp, _vp, _sz, _vp],
    "vesper_refine_slots": [_vp, _i, _i, _vp, _i, _vp, _i, _vp, _vp, _vp, _vp, _vp],
    "vesper_refine_pick": [_vp, _vp, _i, _vp, _vp, _i, _i, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "vesper_prob_interpolate": [_vp, _i, _i, _i, _i, _vp, _sz, _vp],
    "vesper_prob_interpolate_found": [_vp, _vp, _vp],
    "vesper_prop_field": [_vp, _vp, _i, _i, _vp, _vp],
    "vesper_prop_conv_fwd": [_vp, _i, _vp, _vp, _i, _i, _i, _i, _vp, _vp],
    "vesper_prop_vmajor": [_vp, _i, _i, _i, _vp, _vp],
    "vesper_prop_score_vm": [_vp, _vp, _i, _i, _vp, _i, _vp, _vp],
    "vesper_prop_vmajor_f16": [_vp, _i, _i, _i, _vp, _vp],
    "vesper_prop_score_f16": [_vp, _vp, _i, _i, _vp, _i, _vp, _vp],
    "vesper_prop_srcmap": [_i, _vp, _i, _vp, _vp],
    "vesper_prop_score_map": [_vp, _vp, _i, _i, _vp, _i, _vp, _vp],
    "vesper_prop_score_map_many": [_vp, _i, _i, _i, _vp, _i, _vp, _vp],
    "vesper_prop_conv_bwd": [_vp, _vp, _i, _vp, _vp, _i, _i, _i, _vp, _vp, _vp, _vp],
    "vesper_prop_score": [_vp, _vp, _i, _i, _vp, _i, _vp, _vp],
    "vesper_prop_score_bwd_workspace": [_i, _i, _psz],
    "vesper_prop_score_bwd": [_vp, _vp, _i, _i, _vp, _i, _vp, _vp, _vp, _vp, _sz, _vp],
    "vesper_prop_softmax_ce": [_vp, _vp, _i, ctypes.c_float, _vp, _vp, _vp],
    "vesper_prop_adam": [_vp, _vp, _vp, _vp, _i, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, _i,
                         ctypes.c_float, _vp, _vp],
    "vesper_topk_subset": [_vp, _i, _i, _vp, _vp],
    "vesper_topk_subset_batch": [_vp, _i, _i, _i, _vp, _vp],
    "vesper_tc_pass_b": [_vp, _vp, _vp, _i, _i, _i, _i, _i, _vp, _vp],
    "vesper_tc_pass_b_stall_test": [_vp, _vp, _vp, _i, _i, _i, _i, _i, _vp, _vp],
    "vesper_search_status": [_vp, _sz, _vp, _vp],
}


def load(build_if_needed: bool = True):
    """Load libvesper_gb300.so (building it first if sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_needed and needs_build():
        build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run vesper_python_gb300.build()")
    lib = ctypes.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_char_p if name == "vesper_last_error" else ctypes.c_int
    _lib = lib
    return lib


def check(rc: int):
    if rc != 0:
        msg = load().vesper_last_error().decode(errors="replace")
        raise VesperError(rc, msg)


_SIZES: dict = {}


def size_query(fn_name, *args) -> int:
    """A ``*_size``/``*_bytes`` query of the library (a pure function of its
    integer arguments, so answers are memoised)."""
    key = (fn_name,) + args
    v = _SIZES.get(key)
    if v is None:
        out = ctypes.c_size_t(0)
        check(getattr(load(), fn_name)(*args, ctypes.byref(out)))
        v = _SIZES[key] = int(out.value)
    return v
