"""Locates and loads the in-tree shared libraries with ctypes."""
import ctypes
import os

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(PKG_DIR, "lib")
CORE_LIB = os.path.join(LIB_DIR, "libtal_bsw.so")
SYNTH_LIB = os.path.join(LIB_DIR, "libtal_bsw_synth.so")

_cache = {}


def _load(path: str, what: str):
    if path in _cache:
        return _cache[path]
    if not os.path.exists(path):
        raise RuntimeError(
            f"{what} not built: {path} is missing (run __graft_entry__.build())")
    lib = ctypes.CDLL(path)
    _cache[path] = lib
    return lib


def load_synth():
    lib = _load(SYNTH_LIB, "synthetic workload generator")
    if not getattr(lib, "_typed", False):
        lib.tal_synth_plan.restype = ctypes.c_int
        lib.tal_synth_fill.restype = ctypes.c_int
        lib._typed = True
    return lib


def load_core():
    return _load(CORE_LIB, "CUDA BSW library")
