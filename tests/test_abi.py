"""The C-ABI library: it builds, loads, exports every symbol the header
declares, and its host-only entry points answer without a GPU."""
import ctypes
import os
import re

import pytest

from vesper_python_gb300 import _native

HEADER = os.path.join(_native.INCLUDE, "vesper_gb300.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(?:int|const char \*)\s*\*?\s*(vesper_\w+)\s*\(", txt)))


def test_header_lists_entry_points():
    syms = declared_symbols()
    for s in ("vesper_fastvec", "vesper_rot_gather", "vesper_target_spectra", "vesper_search", "vesper_topn",
              "vesper_rescore"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    lib = _native.load()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    # the Python binding covers every declared symbol
    assert set(declared_symbols()) <= set(_native.SIGNATURES)


def test_host_queries_without_gpu():
    lib = _native.load()
    assert lib.vesper_version() >= 100
    for n, ok in ((12, 1), (13, 1), (75, 1), (143, 0), (169, 0), (17, 0), (64, 1), (1, 0)):
        assert lib.vesper_fast_len_ok(n) == ok, n
    assert lib.vesper_search_nscore(0, 0) == 1 and lib.vesper_search_nscore(5, 0) == 2
    assert lib.vesper_search_nscore(5, 1) == 3
    b = _native.size_query("vesper_search_workspace_size", 75, 0, 8, 24624)
    # S (8 x 3 channels) + U (8 x 1 group) complex64 spectra + keys
    assert b >= 8 * 4 * 75 * 75 * 38 * 8 + 24624 * 3 * 8
    assert _native.size_query("vesper_spectra_bytes", 75, 0) == 3 * 75 * 75 * 38 * 8
    assert _native.size_query("vesper_fastvec_workspace_size", 200, 200, 200, 75) > 0


def test_invalid_arguments_return_status():
    lib = _native.load()
    rc = lib.vesper_search(None, None, None, None, 12, 0, 0.0, None, 4, None, None, None, 0, None, 0, None)
    assert rc == 1
    assert b"missing" in lib.vesper_last_error()
    rc = lib.vesper_search(None, None, None, None, 17, 0, 0.0, None, 4, None, None, None, 0, None, 0, None)
    assert rc == 2  # 17 is not a supported FFT length
    rc = lib.vesper_topn(None, 10, 1, 3, None, None)
    assert rc == 1
    with pytest.raises(_native.VesperError):
        _native.check(lib.vesper_rot_gather(None, None, None, 12, None, 1, None, None, None, None))
    rc = lib.vesper_fastvec(None, 1, 1, 1, 1.0, None, 4, 1.0, None, 16.0, None, None, None, None, 0, None)
    assert rc == 1
    assert lib.vesper_search_workspace_size(12, 0, 0, 10, ctypes.POINTER(ctypes.c_size_t)()) == 1


def test_tensor_core_path_host_checks():
    """Search path 3 (split-BF16 pass B): the plan reports it at sides 32 and
    64 and refuses other sides; the pass-B entry validates its arguments
    before touching the GPU."""
    lib = _native.load()
    path, nl = ctypes.c_int(-9), ctypes.c_int(-9)
    opts = (ctypes.c_int * 3)(3, 0, 0)
    for d in (32, 64):
        assert lib.vesper_search_plan(d, 5, 8, 100, opts, ctypes.byref(path), ctypes.byref(nl)) == 0
        assert path.value == 3 and nl.value == 2 + 3 * 13
    assert lib.vesper_search_plan(30, 5, 8, 100, opts, ctypes.byref(path), ctypes.byref(nl)) == 2
    # bad channel split, empty second group, unsupported side
    assert lib.vesper_tc_pass_b(None, None, None, 64, 7, 2, 3, 1, None, None) == 1
    assert lib.vesper_tc_pass_b(1, 1, 1, 64, 3, 2, 3, 1, 1, None) == 1
    assert lib.vesper_tc_pass_b(1, 1, 1, 30, 3, 1, 3, 1, 1, None) == 2
    assert lib.vesper_search_status(None, 0, None, None) == 1


def test_topk_subset_batch_rejects_bad_args():
    lib = _native.load()
    assert lib.vesper_topk_subset_batch(None, 2, 100, 5, None, None) == 1
    assert lib.vesper_topk_subset_batch(1, 0, 100, 5, 1, None) == 1
    assert lib.vesper_topk_subset_batch(1, 2, 100, 101, 1, None) == 1


def _header_params():
    """{name: [parameter kind]} from the header: p pointer, z size_t,
    d double, l 64-bit integer, i int."""
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for name, params in re.findall(r"\b(?:int|const char \*)\s*\*?\s*(vesper_\w+)\s*\(([^)]*)\)\s*;", txt):
        kinds = []
        for prm in [p.strip() for p in params.split(",") if p.strip() and p.strip() != "void"]:
            if "*" in prm:
                kinds.append("p")
            elif prm.startswith("size_t"):
                kinds.append("z")
            elif prm.startswith("double"):
                kinds.append("d")
            elif re.match(r"(u?int64_t|long long)\b", prm):
                kinds.append("l")
            else:
                kinds.append("i")
        out[name] = kinds
    return out


def _ctypes_kind(t):
    if t in (ctypes.c_void_p, ctypes.c_char_p) or (isinstance(t, type) and issubclass(t, ctypes._Pointer)):
        return "p"
    if t is ctypes.c_size_t:
        return "z"
    if t is ctypes.c_double:
        return "d"
    if t in (ctypes.c_int64, ctypes.c_longlong, ctypes.c_uint64) and ctypes.sizeof(t) == 8 and t is not ctypes.c_int:
        return "l"
    return "i"


def test_python_binding_matches_header_parameters():
    """Every ctypes signature the package binds has the header's parameter
    count and kinds (pointer, size_t, double, 64-bit or plain int)."""
    hdr = _header_params()
    assert set(hdr) == set(declared_symbols())
    for name, kinds in hdr.items():
        got = [_ctypes_kind(t) for t in _native.SIGNATURES[name]]
        assert got == kinds, (name, got, kinds)


def test_integration_stub_matches_header_parameters():
    """The ctypes stub a maintainer of the reference would add (the binding
    shown in INTEGRATION.md) declares each function with the header's
    parameter count and kinds."""
    path = os.path.join(os.path.dirname(_native.INCLUDE), "INTEGRATION.md")
    if not os.path.exists(path):
        pytest.skip("integration guide not present")
    hdr = _header_params()
    lines = re.findall(r"lib\.(vesper_\w+)\.argtypes = \[(.*)\]", open(path).read())
    assert lines
    names = {"vp": "p", "i32": "i", "f64": "d", "sz": "z", "ctypes.POINTER(sz)": "p"}
    for name, args in lines:
        got = [names[a.strip()] for a in args.split(",") if a.strip()]
        assert got == hdr[name], (name, got, hdr[name])
