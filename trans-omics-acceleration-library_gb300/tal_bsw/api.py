"""Python mirror of the reference's BandedPairWiseSW (src/alignment/BSW/bandedSWA.h:113-336)
over the C ABI in include/tal_bsw.h.

    bsw = BandedPairWiseSW(o_del, e_del, o_ins, e_ins, zdrop, end_bonus, mat, w_match,
                           w_mismatch, numThreads)
    bsw.getScores16(pairArray, seqBufRef, seqBufQer, numPairs, numThreads, w)

Same names, argument order and meaning as the reference; ``pairArray`` is a numpy
array of SeqPair records (tal_bsw.seqpair.SEQPAIR_DTYPE) updated in place.  Where
the reference exits the process on failure (bandedSWA.cpp:88-93), this raises
TalBswError.  There is no CPU fallback: without the CUDA library or a GB300 the
constructor raises.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from ._lib import load_core
from .seqpair import SEQPAIR_DTYPE

TAL_OK, TAL_EINVAL, TAL_EDOMAIN, TAL_ENOMEM, TAL_ECUDA, TAL_ETIMEOUT, TAL_ENODEV, TAL_EBUSY = range(8)
STATUS_NAMES = {0: "TAL_OK", 1: "TAL_EINVAL", 2: "TAL_EDOMAIN", 3: "TAL_ENOMEM", 4: "TAL_ECUDA",
                5: "TAL_ETIMEOUT", 6: "TAL_ENODEV", 7: "TAL_EBUSY"}
AUTO, BITS8, BITS16 = 0, 8, 16
GROUPED = 0x100  # OR into BITS8 / BITS16: every pair in the reference's SIMD groups (same outputs, slower)
PER_PAIR = 0x200  # OR in: every pair alone in its group (scalarBandedSWAWrapper's semantics)


class TalBswError(RuntimeError):
    def __init__(self, status: int, message: str, bad_pair: int = -1):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
        self.bad_pair = bad_pair


class _Params(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in
                ("o_del", "e_del", "o_ins", "e_ins", "zdrop", "end_bonus", "w_match", "w_mismatch")]


_SIGS = {
    "tal_bsw_create": (ctypes.c_int, [ctypes.POINTER(_Params), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "tal_bsw_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "tal_bsw_scores": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_int32, ctypes.c_int32, ctypes.c_int]),
    "tal_bsw_scores_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                             ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int32, ctypes.c_int32,
                                             ctypes.c_void_p, ctypes.c_int]),
    "tal_bsw_sync": (ctypes.c_int, [ctypes.c_void_p]),
    "tal_bsw_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "tal_bsw_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "tal_bsw_last_bad_pair": (ctypes.c_int64, [ctypes.c_void_p]),
    "tal_bsw_launch_count": (ctypes.c_uint64, [ctypes.c_void_p]),
    "tal_bsw_last_kernel_ms": (ctypes.c_float, [ctypes.c_void_p]),
    "tal_bsw_last_cells": (ctypes.c_uint64, [ctypes.c_void_p]),
    "tal_bsw_last_regroup": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64),
                                            ctypes.POINTER(ctypes.c_int64)]),
    "tal_bsw_scores_batched_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                     ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                                                     ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                                     ctypes.c_int]),
    "tal_bsw_scores_batched": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                              ctypes.c_void_p, ctypes.c_int]),
    "tal_bsw_autotune_reset": (ctypes.c_int, [ctypes.c_void_p]),
    "tal_bsw_bin_config": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "tal_bsw_segment_config": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                              ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                              ctypes.POINTER(ctypes.c_int)]),
    "tal_bsw_probe_int_peak": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_double)]),
    "tal_bsw_now_ns": (ctypes.c_int64, []),
    "tal_bsw_server_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "tal_bsw_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "tal_bsw_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_uint64)]),
    "tal_bsw_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int64, ctypes.c_void_p]),
    "tal_bsw_server_get_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
}


class ServerConfig(ctypes.Structure):
    """tal_bsw_server_config; zero fields take the library's defaults."""
    _fields_ = [("pool_bytes", ctypes.c_size_t), ("staging_bytes", ctypes.c_size_t),
                ("max_tick_pairs", ctypes.c_int32), ("slots", ctypes.c_int32),
                ("latency_pairs", ctypes.c_int32), ("pad_", ctypes.c_int32)]


class RequestInfo(ctypes.Structure):
    """tal_bsw_request_info: a completed request's status and steady-clock times."""
    _fields_ = [("status", ctypes.c_int32), ("tick_requests", ctypes.c_int32),
                ("bad_pair", ctypes.c_int64), ("tick_pairs", ctypes.c_int64),
                ("submit_ns", ctypes.c_int64), ("admit_ns", ctypes.c_int64),
                ("launch_ns", ctypes.c_int64), ("done_ns", ctypes.c_int64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("ticks", ctypes.c_uint64), ("pairs", ctypes.c_uint64),
                ("launches", ctypes.c_uint64), ("pool_bytes", ctypes.c_uint64),
                ("pool_used_bytes", ctypes.c_uint64), ("pool_peak_bytes", ctypes.c_uint64),
                ("queued", ctypes.c_int32), ("admitted", ctypes.c_int32), ("running", ctypes.c_int32),
                ("max_tick_requests", ctypes.c_int32), ("max_ticks_in_flight", ctypes.c_int32),
                ("pad_", ctypes.c_int32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "pad_"}


def core_lib():
    lib = load_core()
    if not getattr(lib, "_tal_typed", False):
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._tal_typed = True
    return lib


def _as_pairs(pairArray: np.ndarray) -> np.ndarray:
    if not isinstance(pairArray, np.ndarray) or pairArray.dtype != SEQPAIR_DTYPE:
        raise TypeError("pairArray must be a numpy array of SEQPAIR_DTYPE records")
    if not pairArray.flags["C_CONTIGUOUS"] or not pairArray.flags["WRITEABLE"]:
        raise TypeError("pairArray must be C-contiguous and writeable (updated in place)")
    return pairArray


def _buf_ptr(buf) -> int:
    if isinstance(buf, np.ndarray):
        if buf.dtype != np.uint8 or not buf.flags["C_CONTIGUOUS"]:
            raise TypeError("sequence buffers must be contiguous uint8 arrays")
        return buf.ctypes.data
    if isinstance(buf, int):
        return buf
    raise TypeError("sequence buffer must be a uint8 numpy array or an address")


class BandedPairWiseSW:
    """GB300 drop-in for the reference class.  ``mat`` is accepted and ignored,
    as by the reference's vector kernels (bandedSWA.cpp:1883-1892)."""

    def __init__(self, o_del: int, e_del: int, o_ins: int, e_ins: int, zdrop: int,
                 end_bonus: int, mat=None, w_match: int = 1, w_mismatch: int = 4,
                 numThreads: int = 1, device: int = -1):
        self._lib = core_lib()
        self.params = dict(o_del=o_del, e_del=e_del, o_ins=o_ins, e_ins=e_ins, zdrop=zdrop,
                           end_bonus=end_bonus, a=w_match, b=w_mismatch)
        p = _Params(o_del, e_del, o_ins, e_ins, zdrop, end_bonus, w_match, w_mismatch)
        h = ctypes.c_void_p()
        rc = self._lib.tal_bsw_create(ctypes.byref(p), int(device), ctypes.byref(h))
        if rc != TAL_OK:
            raise TalBswError(rc, "tal_bsw_create failed (parameters out of range or no GB300)")
        self._h = h
        self.SW_cells = 0

    # -- reference entry points -------------------------------------------------
    def getScores8(self, pairArray, seqBufRef, seqBufQer, numPairs: int, numThreads: int = 1,
                   w: int = 100, grouped: bool = False) -> None:
        """Outputs equal the reference's on any input (pairs whose outputs
        depend on their SIMD group are re-scored in it).  grouped: compute
        every pair in the reference's groups of 64 (same outputs, slower)."""
        self._scores(pairArray, seqBufRef, seqBufQer, numPairs, w, BITS8 | (GROUPED if grouped else 0))

    def getScores16(self, pairArray, seqBufRef, seqBufQer, numPairs: int, numThreads: int = 1,
                    w: int = 100, grouped: bool = False) -> None:
        """Outputs equal the reference's on any input (pairs whose outputs
        depend on their SIMD group are re-scored in it).  grouped: compute
        every pair in the reference's groups of 32 (same outputs, slower)."""
        self._scores(pairArray, seqBufRef, seqBufQer, numPairs, w, BITS16 | (GROUPED if grouped else 0))

    def getScoresAuto(self, pairArray, seqBufRef, seqBufQer, numPairs: int,
                      numThreads: int = 1, w: int = 100) -> None:
        """Each pair to the 8-bit kernel when it is inside the 8-bit range,
        else to the 16-bit kernel."""
        self._scores(pairArray, seqBufRef, seqBufQer, numPairs, w, AUTO)

    def scalarBandedSWAWrapper(self, seqPairArray, seqBufRef, seqBufQer, numPairs: int,
                               nthreads: int = 1, w: int = 100) -> None:
        """bandedSWA.cpp:242-260: every pair scored on its own.  Runs on the GPU
        where the scalar path equals the vector kernels for a pair alone
        (e_del = e_ins = 1; the scoring matrix of bench-bsw, which this class
        assumes), else raises."""
        if self.params["e_del"] != 1 or self.params["e_ins"] != 1:
            raise TalBswError(TAL_EINVAL, "the scalar path runs on the GPU only with e_del = e_ins = 1")
        self._scores(seqPairArray, seqBufRef, seqBufQer, numPairs, w, BITS16 | PER_PAIR)

    def scalarBandedSWA(self, qlen: int, query, tlen: int, target, w: int, h0: int):
        """bandedSWA.cpp:116-237 for one pair: returns (score, qle, tle, gtle,
        gscore, max_off)."""
        from .seqpair import new_pairs
        p = new_pairs(1)
        p["len1"], p["len2"], p["h0"] = tlen, qlen, h0
        self.scalarBandedSWAWrapper(p, np.ascontiguousarray(target, np.uint8),
                                    np.ascontiguousarray(query, np.uint8), 1, 1, w)
        r = p[0]
        return int(r["score"]), int(r["qle"]), int(r["tle"]), int(r["gtle"]), int(r["gscore"]), int(r["max_off"])

    # -- device-resident form -------------------------------------------------------
    def scores_device(self, d_pairs: int, d_ref: int, ref_bytes: int, d_qer: int, qer_bytes: int,
                      numPairs: int, w: int, bits: int = BITS16, d_w: Optional[int] = None,
                      sync: bool = True) -> None:
        rc = self._lib.tal_bsw_scores_device(self._h, d_pairs, d_ref, ref_bytes, d_qer, qer_bytes,
                                             int(numPairs), int(w), d_w, int(bits))
        self._check(rc)
        if sync:
            self.sync()

    # -- batched form --------------------------------------------------------------
    def scores_batched(self, pairArray, seqBufRef, seqBufQer, numPairs: int, w: int = 100,
                       wpair: Optional[np.ndarray] = None, bits: int = AUTO) -> None:
        """Length-binned, autotuned, graph-captured scoring of a mixed batch on
        host buffers (pairs updated in place); wpair: optional band per pair."""
        pa = _as_pairs(pairArray)
        n = int(numPairs)
        if n < 0 or n > pa.shape[0]:
            raise ValueError("numPairs out of range for pairArray")
        wp = None
        if wpair is not None:
            wpair = np.ascontiguousarray(wpair, np.int32)
            if wpair.shape[0] < n:
                raise ValueError("wpair shorter than numPairs")
            wp = wpair.ctypes.data
        self._check(self._lib.tal_bsw_scores_batched(self._h, pa.ctypes.data, _buf_ptr(seqBufRef),
                                                     _buf_ptr(seqBufQer), n, int(w), wp, int(bits)))
        self.SW_cells += self.last_cells

    def scores_batched_device(self, d_pairs: int, d_ref: int, ref_bytes: int, d_qer: int,
                              qer_bytes: int, numPairs: int, w: int, bits: int = AUTO,
                              d_w: Optional[int] = None) -> None:
        self._check(self._lib.tal_bsw_scores_batched_device(self._h, d_pairs, d_ref, ref_bytes, d_qer,
                                                            qer_bytes, int(numPairs), int(w), d_w,
                                                            int(bits)))

    def autotune_reset(self) -> None:
        self._check(self._lib.tal_bsw_autotune_reset(self._h))

    def bin_config(self, b: int):
        g, k, m = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(self._lib.tal_bsw_bin_config(self._h, int(b), ctypes.byref(g), ctypes.byref(k),
                                                 ctypes.byref(m)))
        return g.value, k.value, m.value

    def segment_config(self, seg: int):
        """(lanes per pair, columns per lane, largest query length, row ring)
        of segment seg (length bin seg // 5, band class seg % 5)."""
        g, k, m, w = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(self._lib.tal_bsw_segment_config(self._h, int(seg), ctypes.byref(g), ctypes.byref(k),
                                                     ctypes.byref(m), ctypes.byref(w)))
        return g.value, k.value, m.value, w.value

    def sync(self) -> None:
        self._check(self._lib.tal_bsw_sync(self._h))

    @property
    def stream(self) -> int:
        return int(self._lib.tal_bsw_stream(self._h) or 0)

    @property
    def launch_count(self) -> int:
        return int(self._lib.tal_bsw_launch_count(self._h))

    @property
    def last_kernel_ms(self) -> float:
        """Device time of the last plain call's scoring kernel (CUDA events)."""
        return float(self._lib.tal_bsw_last_kernel_ms(self._h))

    @property
    def last_cells(self) -> int:
        """DP cells computed by the last collected call."""
        return int(self._lib.tal_bsw_last_cells(self._h))

    def last_regroup(self):
        """(pairs flagged, SIMD groups re-scored) by the last collected call:
        the pairs whose outputs could depend on their group in the reference,
        and the groups scored again with the reference's grouping for them."""
        f, g = ctypes.c_int64(0), ctypes.c_int64(0)
        self._check(self._lib.tal_bsw_last_regroup(self._h, ctypes.byref(f), ctypes.byref(g)))
        return int(f.value), int(g.value)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.tal_bsw_destroy(self._h)
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

    # -- internals ------------------------------------------------------------------
    def _check(self, rc: int) -> None:
        if rc != TAL_OK:
            msg = self._lib.tal_bsw_last_error(self._h)
            bad = int(self._lib.tal_bsw_last_bad_pair(self._h))
            raise TalBswError(rc, (msg or b"").decode(), bad)

    def _scores(self, pairArray, seqBufRef, seqBufQer, numPairs, w, bits) -> None:
        pa = _as_pairs(pairArray)
        n = int(numPairs)
        if n < 0 or n > pa.shape[0]:
            raise ValueError("numPairs out of range for pairArray")
        rc = self._lib.tal_bsw_scores(self._h, pa.ctypes.data, _buf_ptr(seqBufRef),
                                      _buf_ptr(seqBufQer), n, int(w), int(bits))
        self._check(rc)
        # the reference's counter of DP cells (bandedSWA.h:116, never
        # incremented there): kept here from the library's own count
        self.SW_cells += self.last_cells


def now_ns() -> int:
    """The serving loop's steady clock, in nanoseconds."""
    return int(core_lib().tal_bsw_now_ns())


class BswServer:
    """Serving loop over the C ABI (tal_bsw_server_create / tal_bsw_submit /
    tal_bsw_poll): requests of any size are admitted into a device pool as
    memory allows and run with continuous batching.  The server keeps a
    reference to each request's arrays until the request is polled complete
    (the library reads and writes them until then)."""

    def __init__(self, bsw: BandedPairWiseSW, pool_bytes: int = 0, staging_bytes: int = 0,
                 max_tick_pairs: int = 0, slots: int = 0, latency_pairs: int = 0):
        self._lib = core_lib()
        cfg = ServerConfig(int(pool_bytes), int(staging_bytes), int(max_tick_pairs), int(slots),
                           int(latency_pairs), 0)
        s = ctypes.c_void_p()
        rc = self._lib.tal_bsw_server_create(bsw._h, ctypes.byref(cfg), ctypes.byref(s))
        if rc != TAL_OK:
            raise TalBswError(rc, "tal_bsw_server_create failed")
        self._s = s
        self._keep = {}

    def submit(self, pairArray, seqBufRef, seqBufQer, numPairs: Optional[int] = None, w: int = 100,
               wpair: Optional[np.ndarray] = None, bits: int = AUTO) -> int:
        """Queues a request (pairs updated in place when it completes); returns its ticket."""
        pa = _as_pairs(pairArray) if isinstance(pairArray, np.ndarray) else None
        if pa is not None:
            n = pa.shape[0] if numPairs is None else int(numPairs)
            if n < 0 or n > pa.shape[0]:
                raise ValueError("numPairs out of range for pairArray")
            pptr = pa.ctypes.data
        else:
            n, pptr = int(numPairs), int(pairArray)
        wp = None
        if wpair is not None:
            if isinstance(wpair, np.ndarray):
                wpair = np.ascontiguousarray(wpair, np.int32)
                if wpair.shape[0] < n:
                    raise ValueError("wpair shorter than numPairs")
                wp = wpair.ctypes.data
            else:
                wp = int(wpair)
        t = ctypes.c_uint64()
        rc = self._lib.tal_bsw_submit(self._s, pptr, _buf_ptr(seqBufRef), _buf_ptr(seqBufQer), n,
                                      int(w), wp, int(bits), ctypes.byref(t))
        if rc != TAL_OK:
            raise TalBswError(rc, "tal_bsw_submit refused the request")
        self._keep[t.value] = (pairArray, seqBufRef, seqBufQer, wpair)
        return t.value

    def poll(self, ticket: int, timeout_us: int = -1) -> Optional[RequestInfo]:
        """The request's RequestInfo once complete (the ticket is then
        released), or None if it is not complete within timeout_us."""
        info = RequestInfo()
        rc = self._lib.tal_bsw_poll(self._s, ctypes.c_uint64(ticket), int(timeout_us), ctypes.byref(info))
        if rc == TAL_ETIMEOUT:
            return None
        if rc != TAL_OK:
            raise TalBswError(rc, "tal_bsw_poll: unknown ticket")
        self._keep.pop(ticket, None)
        return info

    def stats(self) -> dict:
        st = ServerStats()
        rc = self._lib.tal_bsw_server_get_stats(self._s, ctypes.byref(st))
        if rc != TAL_OK:
            raise TalBswError(rc, "tal_bsw_server_get_stats failed")
        return st.as_dict()

    def close(self) -> None:
        if getattr(self, "_s", None):
            self._lib.tal_bsw_server_destroy(self._s)
            self._s = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def probe_int_peak(device: int = 0):
    """(DPX 16x2 add-max, int32) thread-instructions per second on `device`."""
    lib = core_lib()
    a, b = ctypes.c_double(), ctypes.c_double()
    rc = lib.tal_bsw_probe_int_peak(int(device), ctypes.byref(a), ctypes.byref(b))
    if rc != TAL_OK:
        raise TalBswError(rc, "tal_bsw_probe_int_peak failed")
    return a.value, b.value
