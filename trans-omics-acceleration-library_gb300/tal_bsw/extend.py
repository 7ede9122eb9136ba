"""Python front end of the caller-side seed extension (include/tal_extend.h)."""
from __future__ import annotations

import ctypes

import numpy as np

from .api import BandedPairWiseSW, _buf_ptr
from .seeddata import REGION_DTYPE, SEED_DTYPE


class _ExtParams(ctypes.Structure):
    _fields_ = [("w", ctypes.c_int32), ("pen_clip5", ctypes.c_int32), ("pen_clip3", ctypes.c_int32),
                ("band_tries", ctypes.c_int32)]


def _typed(lib):
    if not getattr(lib, "_tal_extend_typed", False):
        fn = lib.tal_bsw_extend_seeds
        fn.restype = ctypes.c_int
        fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                       ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(_ExtParams),
                       ctypes.c_void_p]
        lib._tal_extend_typed = True
    return lib


def extend_seeds(bsw: BandedPairWiseSW, ref, reads, read_off, seeds: np.ndarray, w: int = 100,
                 pen_clip5: int = 5, pen_clip3: int = 5, band_tries: int = 1) -> np.ndarray:
    """Left and right extension of every seed with the handle's scoring;
    returns one REGION_DTYPE record per seed.  band_tries > 1 runs an
    extension again with the doubled band while its score changed and its
    max_off reached 3/4 of the band's half (BWA-MEM's loop uses 2)."""
    lib = _typed(bsw._lib)
    sd = np.ascontiguousarray(seeds, SEED_DTYPE)
    ro = np.ascontiguousarray(read_off, np.int64)
    ref = np.ascontiguousarray(ref, np.uint8)
    reads = np.ascontiguousarray(reads, np.uint8)
    out = np.zeros(sd.shape[0], REGION_DTYPE)
    xp = _ExtParams(int(w), int(pen_clip5), int(pen_clip3), int(band_tries))
    rc = lib.tal_bsw_extend_seeds(bsw._h, _buf_ptr(ref), int(ref.shape[0]), _buf_ptr(reads), ro.ctypes.data,
                                  int(ro.shape[0] - 1), sd.ctypes.data, int(sd.shape[0]), ctypes.byref(xp),
                                  out.ctypes.data)
    bsw._check(rc)
    return out
