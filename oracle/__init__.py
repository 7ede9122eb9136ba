"""ORACLE — test infrastructure only.

ctypes front end for the CPU restatement of the reference's banded
Smith-Waterman (oracle/bsw_oracle.cpp, built into oracle/_build/) and, where it
was built on this machine, for the reference itself (oracle/_ref/, built from
the reference sources by oracle/build_ref.sh).  Only tests/, the smoke check
and bench.py's CPU legs import this package; the product library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle_bsw.so")
REF_DIR = os.path.join(HERE, "_ref")

_PARAM_KEYS = ("o_del", "e_del", "o_ins", "e_ins", "zdrop", "end_bonus", "a", "b")
_libs: Dict[str, ctypes.CDLL] = {}


ORACLE_SRCS = ("bsw_oracle.cpp", "sw_oracle.cpp", "chain_oracle.cpp")


def build(force: bool = False) -> str:
    """Compile the restatements (g++, host only)."""
    srcs = [os.path.join(HERE, f) for f in ORACLE_SRCS]
    if force or not os.path.exists(ORACLE_SO) or \
            os.path.getmtime(ORACLE_SO) < max(os.path.getmtime(f) for f in srcs):
        os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
        subprocess.check_call(["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                               "-pthread", "-o", ORACLE_SO, *srcs])
    return ORACLE_SO


def build_ref() -> None:
    """Compile the reference from its own sources into oracle/_ref (x86 only;
    a no-op where the reference tree is absent)."""
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh")])


def _oracle():
    if "oracle" not in _libs:
        if not os.path.exists(ORACLE_SO):
            build()
        lib = ctypes.CDLL(ORACLE_SO)
        lib.oracle_bsw_vector.restype = ctypes.c_int
        lib.oracle_bsw_vector.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_int32, ctypes.c_int]
        lib.oracle_sw.restype = ctypes.c_int
        lib.oracle_sw.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                  ctypes.c_int64, ctypes.c_int]
        lib.oracle_bsw_detect.restype = ctypes.c_int
        lib.oracle_bsw_detect.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                          ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_int32, ctypes.c_void_p, ctypes.c_int]
        lib.oracle_bsw_scalar.restype = ctypes.c_int
        lib.oracle_bsw_scalar.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                          ctypes.c_void_p, ctypes.c_int]
        _libs["oracle"] = lib
    return _libs["oracle"]


def _params(p: Dict[str, int]) -> np.ndarray:
    return np.array([int(p[k]) for k in _PARAM_KEYS], np.int32)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def vector(pairs: np.ndarray, ref: np.ndarray, qer: np.ndarray, w: int,
           params: Dict[str, int], bits: int = 16, lanes: Optional[int] = None,
           nthreads: int = 1) -> np.ndarray:
    """getScores16 / getScores8 restated; returns a scored copy of ``pairs``.
    lanes: group width (default 32 for 16-bit, 64 for 8-bit, as the reference)."""
    out = np.ascontiguousarray(pairs).copy()
    lanes = lanes or (32 if bits == 16 else 64)
    pv = _params(params)
    rc = _oracle().oracle_bsw_vector(_ptr(pv), bits, lanes, _ptr(out), out.shape[0],
                                     _ptr(ref), _ptr(qer), int(w), nthreads)
    if rc != 0:
        raise ValueError("oracle_bsw_vector rejected its arguments")
    return out


def detect(pairs: np.ndarray, ref: np.ndarray, qer: np.ndarray, w: int,
           params: Dict[str, int], bits: int = 16, nthreads: int = 1):
    """The library's group-coupling detector restated: every pair scored alone
    (the per-pair kernels' outputs) and a flag per pair, non-zero where its
    outputs may depend on the other pairs of its SIMD group.  Returns
    (scored copy, flags)."""
    out = np.ascontiguousarray(pairs).copy()
    flags = np.zeros(out.shape[0], np.int32)
    pv = _params(params)
    rc = _oracle().oracle_bsw_detect(_ptr(pv), bits, _ptr(out), out.shape[0], _ptr(ref),
                                     _ptr(qer), int(w), _ptr(flags), nthreads)
    if rc != 0:
        raise ValueError("oracle_bsw_detect rejected its arguments")
    return out, flags


def scalar(pairs: np.ndarray, ref: np.ndarray, qer: np.ndarray, w: int,
           params: Dict[str, int], nthreads: int = 1):
    """scalarBandedSWAWrapper restated; returns (scored copy, ref-cells)."""
    out = np.ascontiguousarray(pairs).copy()
    pv = _params(params)
    cells = np.zeros(1, np.uint64)
    rc = _oracle().oracle_bsw_scalar(_ptr(pv), _ptr(out), out.shape[0], _ptr(ref), _ptr(qer),
                                     int(w), _ptr(cells), nthreads)
    if rc != 0:
        raise ValueError("oracle_bsw_scalar rejected its arguments")
    return out, int(cells[0])


def ref_available(isa: str = "avx512") -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libbsw_ref_{isa}.so"))


def reference(pairs: np.ndarray, ref: np.ndarray, qer: np.ndarray, w: int,
              params: Dict[str, int], mode: int = 16, isa: str = "avx512",
              pristine: bool = True) -> np.ndarray:
    """The reference's own getScores16 (mode 16) / getScores8 (8) /
    scalarBandedSWAWrapper (0), compiled from its sources.

    pristine: run the vector kernels one SIMD group at a time on zeroed
    scratch rows, which makes them deterministic (the reference reads one
    scratch cell per group that it may not have written; see ref_shim.cpp)."""
    key = "ref_" + isa
    if key not in _libs:
        path = os.path.join(REF_DIR, f"libbsw_ref_{isa}.so")
        if not os.path.exists(path):
            raise RuntimeError(f"reference build missing: {path}")
        lib = ctypes.CDLL(path)
        lib.ref_bsw_run.restype = ctypes.c_int
        lib.ref_bsw_run.argtypes = [ctypes.c_int] * 9 + [ctypes.c_void_p, ctypes.c_void_p,
                                                         ctypes.c_void_p, ctypes.c_int32,
                                                         ctypes.c_int32, ctypes.c_int]
        _libs[key] = lib
    lib = _libs[key]
    out = np.ascontiguousarray(pairs).copy()
    p = params
    rc = lib.ref_bsw_run(p["o_del"], p["e_del"], p["o_ins"], p["e_ins"], p["zdrop"],
                         p["end_bonus"], p["a"], p["b"], mode, _ptr(out), _ptr(ref), _ptr(qer),
                         out.shape[0], int(w), 1 if pristine else 0)
    if rc != 0:
        raise RuntimeError("ref_bsw_run failed")
    return out


def eligible8(pairs: np.ndarray, w, params: Dict[str, int]) -> np.ndarray:
    """Per-pair 8-bit eligibility: the reference's own 8-bit limits
    (len1, len2 < MAX_SEQ_LEN8 = 128, bandedSWA.h:82; h0 + a*min(len1, len2) in
    int8 range) plus the no-wrap conditions under which getScores8 and an
    exact-integer evaluation agree (gap scores and the first column in int8)."""
    p = params
    l1 = pairs["len1"].astype(np.int64)
    l2 = pairs["len2"].astype(np.int64)
    h0 = pairs["h0"].astype(np.int64)
    w = np.broadcast_to(np.asarray(w, np.int64), l1.shape)
    ok = (l1 >= 0) & (l2 >= 0) & (l1 <= 127) & (l2 <= 127) & (h0 >= 0)
    ok &= h0 + p["a"] * np.minimum(l1, l2) <= 127
    oe = max(p["o_del"] + p["e_del"], p["o_ins"] + p["e_ins"])
    if oe > 127 or 1 - max(p["b"], 1) - oe < -128:
        return np.zeros(l1.shape, bool)
    kmax = np.minimum(l1 - 1, np.maximum(w, 0) + 1)
    ok &= (kmax < 1) | (h0 - p["o_del"] - kmax * p["e_del"] >= -128)
    return ok


def routed(pairs: np.ndarray, ref: np.ndarray, qer: np.ndarray, w, params: Dict[str, int],
           bits: int = 0, nthreads: int = 1, lanes: Optional[int] = None) -> np.ndarray:
    """Scores every pair with getScores8 or getScores16 semantics: bits 8/16
    forces one; bits 0 routes each pair by eligible8().  w may be a scalar or
    a per-pair array (the pairs of each band and precision, in order, form
    one call).  lanes: SIMD group width (default: the reference's 32 / 64;
    1 scores every pair alone in its group)."""
    out = np.ascontiguousarray(pairs).copy()
    n = out.shape[0]
    if n == 0:
        return out
    warr = np.broadcast_to(np.asarray(w, np.int64), (n,))
    if bits == 8:
        is8 = np.ones(n, bool)
    elif bits == 16:
        is8 = np.zeros(n, bool)
    else:
        is8 = eligible8(out, warr, params)
    for wv in np.unique(warr):
        for b in (8, 16):
            sel = np.nonzero((warr == wv) & (is8 == (b == 8)))[0]
            if sel.size:
                out[sel] = vector(out[sel], ref, qer, int(wv), params, bits=b, lanes=lanes,
                                  nthreads=nthreads)
    return out


# ---------------------------------------------------------------- unbanded SW
SW_KEYS = ("match", "mismatch", "open", "extend")


def sw(pairs: np.ndarray, seqbuf: np.ndarray, stride: int, params: Dict[str, int],
       nthreads: int = 1) -> np.ndarray:
    """The reference's unbanded Smith-Waterman scores restated
    (oracle/sw_oracle.cpp); returns a scored copy of the 12-byte pairs."""
    out = np.ascontiguousarray(pairs).copy()
    pv = np.array([int(params[k]) for k in SW_KEYS], np.int32)
    rc = _oracle().oracle_sw(_ptr(pv), _ptr(out), out.shape[0], _ptr(seqbuf), int(stride),
                             int(nthreads))
    if rc != 0:
        raise ValueError("oracle_sw rejected its arguments")
    return out


def sw_ref_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libsw_ref_avx512.so"))


def _sw_ref_lib():
    if "sw_ref" not in _libs:
        lib = ctypes.CDLL(os.path.join(REF_DIR, "libsw_ref_avx512.so"))
        lib.ref_sw_run.restype = ctypes.c_int
        lib.ref_sw_run.argtypes = [ctypes.c_int] * 5 + [ctypes.c_void_p, ctypes.c_void_p,
                                                        ctypes.c_int32]
        lib.ref_sw_max_len.restype = ctypes.c_int
        _libs["sw_ref"] = lib
    return _libs["sw_ref"]


def sw_reference(pairs: np.ndarray, seqbuf: np.ndarray, params: Dict[str, int],
                 bits: int = 16) -> np.ndarray:
    """The reference's own PairWiseSW_8/_16/_32::getScores (bits 8, 16, 32) or
    its scalar smithWatermanOnePairWrapper (bits 0) on a copy of pairs."""
    out = np.ascontiguousarray(pairs).copy()
    rc = _sw_ref_lib().ref_sw_run(int(bits), *[int(params[k]) for k in SW_KEYS], _ptr(out),
                                  _ptr(seqbuf), out.shape[0])
    if rc != 0:
        raise RuntimeError("ref_sw_run failed")
    return out


def sw_ref_max_len(bits: int) -> int:
    """The reference's MAX_SEQ_LEN for a precision (its sequence stride)."""
    return int(_sw_ref_lib().ref_sw_max_len(int(bits)))


# ---------------------------------------------------------------- DP chaining
ANCHOR_DTYPE = np.dtype([("r", "<u8"), ("q", "<i4"), ("l", "<i4")])
CHAIN_REF_VARIANTS = ("avx512", "avx512_ofast", "avx2")


def chain(anchors: np.ndarray, offsets: np.ndarray, bw: int, max_iter: int, dr: int, dq: int,
          nthreads: int = 1):
    """The reference's DP chaining (dp_chain::mm_dp_vectorized) restated
    (oracle/chain_oracle.cpp); returns (f uint32, p int32, v int32)."""
    a = np.ascontiguousarray(anchors, ANCHOR_DTYPE)
    o = np.ascontiguousarray(offsets, np.int64)
    n = a.shape[0]
    f = np.zeros(n, np.uint32)
    p = np.zeros(n, np.int32)
    v = np.zeros(n, np.int32)
    lib = _oracle()
    lib.oracle_chain.restype = ctypes.c_int
    lib.oracle_chain.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32] + \
        [ctypes.c_int32] * 4 + [ctypes.c_void_p] * 3 + [ctypes.c_int]
    rc = lib.oracle_chain(_ptr(a), _ptr(o), o.shape[0] - 1, int(bw), int(max_iter), int(dr), int(dq),
                          _ptr(f), _ptr(p), _ptr(v), int(nthreads))
    if rc != 0:
        raise ValueError("oracle_chain rejected its offsets")
    return f, p, v


def chain_ref_available(variant: str = "avx512") -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libchain_ref_{variant}.so"))


def chain_reference(anchors: np.ndarray, offsets: np.ndarray, params, dr: int, dq: int,
                    variant: str = "avx512"):
    """The reference's own dp_chain (built from its header by build_ref.sh;
    variant: avx512, avx512_ofast or avx2); params: the constructor's eight
    tunables in order.  Returns (f, p, v)."""
    key = "chain_" + variant
    if key not in _libs:
        lib = ctypes.CDLL(os.path.join(REF_DIR, f"libchain_ref_{variant}.so"))
        lib.ref_chain_run.restype = ctypes.c_int
        lib.ref_chain_run.argtypes = [ctypes.c_int] * 5 + [ctypes.c_float, ctypes.c_int, ctypes.c_int,
                                                           ctypes.c_void_p, ctypes.c_void_p,
                                                           ctypes.c_int32, ctypes.c_int32,
                                                           ctypes.c_int32] + [ctypes.c_void_p] * 3
        _libs[key] = lib
    a = np.ascontiguousarray(anchors, ANCHOR_DTYPE)
    o = np.ascontiguousarray(offsets, np.int64)
    n = a.shape[0]
    f = np.zeros(n, np.uint32)
    p = np.zeros(n, np.int32)
    v = np.zeros(n, np.int32)
    mdx, mdy, bw, msk, mit, gs, cdna, nseg = params
    rc = _libs[key].ref_chain_run(int(mdx), int(mdy), int(bw), int(msk), int(mit), float(gs),
                                  int(cdna), int(nseg), _ptr(a), _ptr(o), o.shape[0] - 1, int(dr),
                                  int(dq), _ptr(f), _ptr(p), _ptr(v))
    if rc != 0:
        raise RuntimeError("ref_chain_run failed")
    return f, p, v


# ---------------------------------------------------------------- seed extension
def _max_gap(params, n, w):
    """clamp(max((n*a - o_del) // e_del + 1, (n*a - o_ins) // e_ins + 1), 1, 2w),
    C integer division (truncation)."""
    def cdiv(x, y):
        q = abs(x) // y
        return q if x >= 0 else -q
    a = params["a"]
    d = cdiv(n * a - params["o_del"], params["e_del"]) + 1
    i = cdiv(n * a - params["o_ins"], params["e_ins"]) + 1
    return min(max(d, i, 1), 2 * w)


def _scored_with_tries(P: np.ndarray, T: np.ndarray, Q: np.ndarray, w: int, params: Dict[str, int],
                       tries: int) -> np.ndarray:
    """Scores the batch P at band w, then, per pair, again at band w << i
    while its last attempt changed the score (the first always counts) and
    reached max_off >= (band >> 1) + (band >> 2); the last attempt stands."""
    R = routed(P, T, Q, w, params, bits=0)
    prev = np.full(P.shape[0], -1, np.int64)
    active = np.ones(P.shape[0], bool)
    for i in range(1, max(1, tries)):
        wp = w << (i - 1)
        go = active & (R["score"] != prev) & (R["max_off"] >= (wp >> 1) + (wp >> 2))
        active = go
        if not go.any():
            break
        prev[go] = R["score"][go]
        sub = R[go].copy()
        for f in ("score", "tle", "gtle", "qle", "gscore", "max_off"):
            sub[f] = -1
        R[go] = routed(sub, T, Q, w << i, params, bits=0)
    return R


def extend(ref: np.ndarray, reads: np.ndarray, read_off: np.ndarray, seeds: np.ndarray,
           params: Dict[str, int], w: int, pen_clip5: int, pen_clip3: int,
           band_tries: int = 1) -> np.ndarray:
    """The caller-side seed extension of include/tal_extend.h restated: left
    pairs (reversed sequences before the seed, h0 = len * a), their clipping
    choice, right pairs (after the seed, h0 = the left result), the region,
    with BWA-MEM's band-doubling retries when band_tries > 1.
    Parity unpinned: this stage (BWA-MEM2's mem_chain2aln) is not in the
    reference; the specification is the header's, the pairs are scored by
    the pinned BSW oracle (`routed`) in the reference's SIMD groups: each
    batch (left, right, every retry) is one getScores call per precision,
    pairs in batch order, as the library's extension layer issues them."""
    from tal_bsw.seqpair import SEQPAIR_DTYPE
    from tal_bsw.seeddata import REGION_DTYPE
    a = params["a"]
    n = seeds.shape[0]
    tparts, qparts, lp, rp = [], [], [], []
    tpos = qpos = 0
    left_of = np.full(n, -1, np.int64)
    right_of = np.full(n, -1, np.int64)
    for s in range(n):
        r, qb, rb, ln = int(seeds["read"][s]), int(seeds["qbeg"][s]), int(seeds["rbeg"][s]), int(seeds["len"][s])
        r0 = int(read_off[r])
        L = int(read_off[r + 1]) - r0
        if qb > 0:
            rs = max(0, rb - qb - _max_gap(params, qb, w))
            t = ref[rs:rb][::-1]
            q = reads[r0:r0 + qb][::-1]
            left_of[s] = len(lp)
            lp.append((tpos, qpos, s, t.shape[0], q.shape[0], ln * a))
            tparts.append(t); qparts.append(q)
            tpos += t.shape[0]; qpos += q.shape[0]
        qe0, re0 = qb + ln, rb + ln
        if qe0 < L:
            ql = L - qe0
            re = min(ref.shape[0], re0 + ql + _max_gap(params, ql, w))
            t = ref[re0:re]
            q = reads[r0 + qe0:r0 + L]
            right_of[s] = len(rp)
            rp.append((tpos, qpos, s, t.shape[0], q.shape[0], 0))
            tparts.append(t); qparts.append(q)
            tpos += t.shape[0]; qpos += q.shape[0]
    T = np.concatenate(tparts + [np.zeros(16, np.uint8)]).astype(np.uint8)
    Q = np.concatenate(qparts + [np.zeros(16, np.uint8)]).astype(np.uint8)

    def mk(rows):
        p = np.zeros(len(rows), SEQPAIR_DTYPE)
        for k, (idr, idq, sid, l1, l2, h0) in enumerate(rows):
            p[k]["idr"], p[k]["idq"], p[k]["id"] = idr, idq, sid
            p[k]["len1"], p[k]["len2"], p[k]["h0"] = l1, l2, h0
        for f in ("score", "tle", "gtle", "qle", "gscore", "max_off"):
            p[f] = -1
        return p

    L_ = _scored_with_tries(mk(lp), T, Q, w, params, band_tries) if lp else mk([])

    def left_outcome(s):
        qb, rb, ln = int(seeds["qbeg"][s]), int(seeds["rbeg"][s]), int(seeds["len"][s])
        k = left_of[s]
        if k < 0:
            return qb, rb, ln * a
        p = L_[k]
        if p["gscore"] <= 0 or p["gscore"] <= p["score"] - pen_clip5:
            return qb - int(p["qle"]), rb - int(p["tle"]), int(p["score"])
        return 0, rb - int(p["gtle"]), int(p["gscore"])

    R = mk(rp)
    for s in range(n):
        if right_of[s] >= 0:
            R[right_of[s]]["h0"] = left_outcome(s)[2]
    R_ = _scored_with_tries(R, T, Q, w, params, band_tries) if rp else R
    out = np.zeros(n, REGION_DTYPE)
    for s in range(n):
        qb, rb, sc = left_outcome(s)
        out[s]["qb"], out[s]["rb"], out[s]["left_score"] = qb, rb, sc
        r = int(seeds["read"][s])
        L = int(read_off[r + 1] - read_off[r])
        qe0 = int(seeds["qbeg"][s] + seeds["len"][s])
        re0 = int(seeds["rbeg"][s] + seeds["len"][s])
        k = right_of[s]
        if k < 0:
            out[s]["qe"], out[s]["re"] = qe0, re0
        else:
            p = R_[k]
            if p["gscore"] <= 0 or p["gscore"] <= p["score"] - pen_clip3:
                out[s]["qe"], out[s]["re"], sc = qe0 + int(p["qle"]), re0 + int(p["tle"]), int(p["score"])
            else:
                out[s]["qe"], out[s]["re"], sc = L, re0 + int(p["gtle"]), int(p["gscore"])
        out[s]["score"] = sc
    return out
