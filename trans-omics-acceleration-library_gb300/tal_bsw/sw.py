"""Python front end of the unbanded Smith-Waterman scorer (include/tal_sw.h),
with the reference's class names and getScores signature
(src/alignment/Smith-Waterman/PairWiseSW_{8,16,32}.h)."""
from __future__ import annotations

import ctypes

import numpy as np

from .api import TAL_OK, TalBswError, _buf_ptr, core_lib
from .swdata import SW_DTYPE


class _SwParams(ctypes.Structure):
    _fields_ = [("w_match", ctypes.c_int32), ("w_mismatch", ctypes.c_int32),
                ("w_open", ctypes.c_int32), ("w_extend", ctypes.c_int32)]


_SIGS = {
    "tal_sw_create": (ctypes.c_int, [ctypes.POINTER(_SwParams), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "tal_sw_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "tal_sw_scores": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                     ctypes.c_int]),
    "tal_sw_scores_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_size_t, ctypes.c_int32, ctypes.c_int]),
    "tal_sw_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "tal_sw_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "tal_sw_last_bad_pair": (ctypes.c_int64, [ctypes.c_void_p]),
    "tal_sw_last_cells": (ctypes.c_uint64, [ctypes.c_void_p]),
}


def _lib():
    lib = core_lib()
    if not getattr(lib, "_tal_sw_typed", False):
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._tal_sw_typed = True
    return lib


class PairWiseSW:
    """GB300 drop-in for the reference's PairWiseSW_<bits> classes:
    ``PairWiseSW_16(w_match, w_mismatch, w_open, w_extend).getScores(pairArray,
    seqBuf, numPairs, numThreads)`` writes each pair's local alignment score."""

    bits = 16

    def __init__(self, w_match: int, w_mismatch: int, w_open: int, w_extend: int, device: int = -1):
        self._lib = _lib()
        p = _SwParams(int(w_match), int(w_mismatch), int(w_open), int(w_extend))
        h = ctypes.c_void_p()
        rc = self._lib.tal_sw_create(ctypes.byref(p), int(device), ctypes.byref(h))
        if rc != TAL_OK:
            raise TalBswError(rc, "tal_sw_create failed (positive gap/mismatch weight or no GB300)")
        self._h = h

    def getScores(self, pairArray: np.ndarray, seqBuf, numPairs: int, numThreads: int = 1) -> None:
        if not isinstance(pairArray, np.ndarray) or pairArray.dtype != SW_DTYPE or \
                not pairArray.flags["C_CONTIGUOUS"]:
            raise TypeError("pairArray must be a contiguous array of SW_DTYPE records")
        n = int(numPairs)
        if n < 0 or n > pairArray.shape[0]:
            raise ValueError("numPairs out of range for pairArray")
        self._check(self._lib.tal_sw_scores(self._h, pairArray.ctypes.data, _buf_ptr(seqBuf), n,
                                            self.bits))

    def scores_device(self, d_pairs: int, d_seqbuf: int, seq_bytes: int, numPairs: int) -> None:
        self._check(self._lib.tal_sw_scores_device(self._h, d_pairs, d_seqbuf, int(seq_bytes),
                                                   int(numPairs), self.bits))

    @property
    def stream(self) -> int:
        return int(self._lib.tal_sw_stream(self._h) or 0)

    @property
    def last_cells(self) -> int:
        return int(self._lib.tal_sw_last_cells(self._h))

    def _check(self, rc: int) -> None:
        if rc != TAL_OK:
            msg = self._lib.tal_sw_last_error(self._h)
            raise TalBswError(rc, (msg or b"").decode(), int(self._lib.tal_sw_last_bad_pair(self._h)))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.tal_sw_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class PairWiseSW_8(PairWiseSW):
    bits = 8


class PairWiseSW_16(PairWiseSW):
    bits = 16


class PairWiseSW_32(PairWiseSW):
    bits = 32
