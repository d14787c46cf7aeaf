"""The C-ABI library builds for sm_103a, loads, and exports every entry
point include/hashdag_gb300.h declares (no device calls; CPU only)."""
import ctypes as C
import os
import re

from hashdag_gb300 import _capi, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "hashdag_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:hd_status|void|const char\*|uint32_t)\s+(hd_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    build.build()
    names = declared_functions()
    assert len(names) >= 25
    lib = C.CDLL(_capi.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    bound = {n for n, _, _ in _capi.SIGNATURES}
    assert set(names) <= bound, set(names) - bound


def test_abi_version_and_default_config():
    build.build()
    L = _capi.lib()
    assert L.hd_abi_version() == 8
    cfg = _capi.Config()
    L.hd_default_config(15, C.byref(cfg))
    assert (cfg.depth, cfg.color_tree_levels, cfg.top_levels) == (15, 10, 9)
    assert (cfg.top_bucket_size, cfg.low_bucket_size, cfg.low_bucket_bits) == (1024, 4096, 16)
    L.hd_default_config(10, C.byref(cfg))
    assert (cfg.color_tree_levels, cfg.top_bucket_bits) == (5, 10)


def test_invalid_config_is_rejected_without_device():
    build.build()
    L = _capi.lib()
    cfg = _capi.Config()
    L.hd_default_config(10, C.byref(cfg))
    cfg.depth = 40
    h = C.c_void_p()
    assert L.hd_create(C.byref(cfg), C.byref(h)) == _capi.HD_ERR_INVALID
    assert not h.value
