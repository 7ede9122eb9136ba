"""Python front end of the anchor chaining DP (include/tal_chain.h), with the
reference's class name, constructor and mm_dp_vectorized call
(src/chaining/parallel_chaining_32_bit.h:104-118, :216)."""
from __future__ import annotations

import ctypes

import numpy as np

from .api import TAL_OK, TalBswError, core_lib
from .chaindata import ANCHOR_DTYPE


class _ChainParams(ctypes.Structure):
    _fields_ = [("max_dist_x", ctypes.c_int32), ("max_dist_y", ctypes.c_int32),
                ("bw", ctypes.c_int32), ("max_skip", ctypes.c_int32), ("max_iter", ctypes.c_int32),
                ("gap_scale", ctypes.c_float), ("is_cdna", ctypes.c_int32), ("n_segs", ctypes.c_int32)]


_P = ctypes.c_void_p
_SIGS = {
    "tal_chain_create": (ctypes.c_int, [ctypes.POINTER(_ChainParams), ctypes.c_int, ctypes.POINTER(_P)]),
    "tal_chain_destroy": (ctypes.c_int, [_P]),
    "tal_chain_dp": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _P, _P, _P]),
    "tal_chain_dp_device": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                           _P, _P, _P]),
    "tal_chain_stream": (_P, [_P]),
    "tal_chain_last_error": (ctypes.c_char_p, [_P]),
    "tal_chain_last_bad_read": (ctypes.c_int64, [_P]),
    "tal_chain_last_evals": (ctypes.c_uint64, [_P]),
}


def _lib():
    lib = core_lib()
    if not getattr(lib, "_tal_chain_typed", False):
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._tal_chain_typed = True
    return lib


def _check_array(a, dtype, n, name):
    if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags["C_CONTIGUOUS"] or \
            a.shape[0] < n:
        raise TypeError(f"{name} must be a contiguous {dtype} array of at least {n} entries")


class dp_chain:  # noqa: N801 -- the reference's class name
    """GB300 drop-in for the reference's ``dp_chain(max_dist_x, max_dist_y, bw,
    max_skip, max_iter, gap_scale, is_cdna, n_segs)``: ``mm_dp_vectorized(n,
    anchors, f, p, v, dr, dq)`` fills one read's f, p, v; ``mm_dp_batch``
    scores many reads in one launch (one warp per read)."""

    def __init__(self, max_dist_x: int, max_dist_y: int, bw: int, max_skip: int, max_iter: int,
                 gap_scale: float, is_cdna: int, n_segs: int, device: int = -1):
        self._lib = _lib()
        p = _ChainParams(int(max_dist_x), int(max_dist_y), int(bw), int(max_skip), int(max_iter),
                         float(gap_scale), int(is_cdna), int(n_segs))
        h = ctypes.c_void_p()
        rc = self._lib.tal_chain_create(ctypes.byref(p), int(device), ctypes.byref(h))
        if rc != TAL_OK:
            raise TalBswError(rc, "tal_chain_create failed (negative bw/max_iter or no GB300)")
        self._h = h

    def mm_dp_vectorized(self, n: int, anchors: np.ndarray, f: np.ndarray, p: np.ndarray,
                         v: np.ndarray, dr: int, dq: int) -> None:
        n = int(n)
        _check_array(anchors, ANCHOR_DTYPE, n, "anchors")
        for a, dt, nm in ((f, np.uint32, "f"), (p, np.int32, "p"), (v, np.int32, "v")):
            _check_array(a, np.dtype(dt), n, nm)
        offs = np.array([0, n], np.int64)
        self._check(self._lib.tal_chain_dp(self._h, anchors.ctypes.data, offs.ctypes.data, 1, int(dr),
                                           int(dq), f.ctypes.data, p.ctypes.data, v.ctypes.data))

    def mm_dp_batch(self, anchors: np.ndarray, offsets: np.ndarray, dr: int, dq: int, out=None):
        """Reads anchors[offsets[k], offsets[k+1]); returns (f, p, v) for all
        anchors -- written into `out` = (f, p, v) when given (e.g. pinned
        host arrays, which the device copies into directly)."""
        offsets = np.ascontiguousarray(offsets, np.int64)
        n = int(offsets[-1]) if offsets.shape[0] else 0
        _check_array(anchors, ANCHOR_DTYPE, n, "anchors")
        if out is None:
            f = np.zeros(anchors.shape[0], np.uint32)
            p = np.zeros(anchors.shape[0], np.int32)
            v = np.zeros(anchors.shape[0], np.int32)
        else:
            f, p, v = out
            for a, dt, nm in ((f, np.uint32, "f"), (p, np.int32, "p"), (v, np.int32, "v")):
                _check_array(a, np.dtype(dt), n, nm)
        self._check(self._lib.tal_chain_dp(self._h, anchors.ctypes.data, offsets.ctypes.data,
                                           offsets.shape[0] - 1, int(dr), int(dq), f.ctypes.data,
                                           p.ctypes.data, v.ctypes.data))
        return f, p, v

    def mm_dp_device(self, d_anchors: int, d_offsets: int, n_reads: int, dr: int, dq: int,
                     d_f: int, d_p: int, d_v: int) -> None:
        """The same on device buffers (pointers); synchronous."""
        self._check(self._lib.tal_chain_dp_device(self._h, d_anchors, d_offsets, int(n_reads), int(dr),
                                                  int(dq), d_f, d_p, d_v))

    @property
    def stream(self) -> int:
        return int(self._lib.tal_chain_stream(self._h) or 0)

    @property
    def last_evals(self) -> int:
        return int(self._lib.tal_chain_last_evals(self._h))

    def _check(self, rc: int) -> None:
        if rc != TAL_OK:
            msg = self._lib.tal_chain_last_error(self._h)
            raise TalBswError(rc, (msg or b"").decode(), int(self._lib.tal_chain_last_bad_read(self._h)))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.tal_chain_destroy(self._h)
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
