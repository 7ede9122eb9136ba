"""ctypes driver for the SIMT emulator (emu.cpp): runs the CUDA kernel source
compiled for the host, one thread per lane.  Test infrastructure only."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CSRC = os.path.join(ROOT, "trans-omics-acceleration-library_gb300", "csrc")
SO = os.path.join(ROOT, "tests", "simt_emu", "_build", "libbsw_emu.so")
_lib = None


def build(force=False):
    srcs = [os.path.join(HERE, "emu.cpp"), os.path.join(HERE, "fake", "cuda_runtime.h"),
            os.path.join(CSRC, "bsw_kernel.cuh"), os.path.join(CSRC, "bsw_lane.cuh"),
            os.path.join(CSRC, "sw_kernel.cuh"), os.path.join(CSRC, "bsw_group.cuh"),
            os.path.join(CSRC, "bsw_couple.cuh"), os.path.join(CSRC, "bsw_group_wide.cuh")]
    if force or not os.path.exists(SO) or os.path.getmtime(SO) < max(os.path.getmtime(s) for s in srcs):
        os.makedirs(os.path.dirname(SO), exist_ok=True)
        subprocess.check_call(["g++", "-std=c++20", "-O1", "-fPIC", "-shared", "-pthread", "-w",
                               "-I" + os.path.join(HERE, "fake"), "-I" + CSRC, "-o", SO,
                               os.path.join(HERE, "emu.cpp")])
    return SO


def run(pairs, ref, qer, w, params, bits=16, K=4, warps=1, wpair=None, G=32, win=0):
    """Scores a copy of pairs with the emulated kernel (win: the lane
    kernel's row ring, 0 = whole rows); returns (pairs, err_flags, err_index)."""
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.emu_bsw_run.restype = ctypes.c_int
    out = np.ascontiguousarray(pairs).copy()
    kp = np.array([params[k] for k in ("o_del", "e_del", "o_ins", "e_ins", "zdrop", "end_bonus", "a", "b")],
                  np.int32)
    ef = ctypes.c_int(0)
    ei = ctypes.c_longlong(0)
    ref = np.ascontiguousarray(ref)
    qer = np.ascontiguousarray(qer)
    wp = None if wpair is None else np.ascontiguousarray(wpair, np.int32)
    vp = ctypes.c_void_p
    _lib.emu_bsw_run(vp(out.ctypes.data), vp(ref.ctypes.data), ctypes.c_longlong(0),
                     ctypes.c_longlong(ref.shape[0]), vp(qer.ctypes.data), ctypes.c_longlong(0),
                     ctypes.c_longlong(qer.shape[0]), int(out.shape[0]), int(w),
                     None if wp is None else vp(wp.ctypes.data), int(bits), vp(kp.ctypes.data),
                     int(G), int(K), int(warps), int(win), ctypes.byref(ef), ctypes.byref(ei))
    return out, ef.value, ei.value


def run_detect(pairs, ref, qer, w, params, bits=16, K=4, warps=1, G=32, win=0):
    """run() with the group-coupling detector on; returns (pairs, err_flags,
    sorted indices of the flagged pairs)."""
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
    out = np.ascontiguousarray(pairs).copy()
    kp = np.array([params[k] for k in ("o_del", "e_del", "o_ins", "e_ins", "zdrop", "end_bonus", "a", "b")],
                  np.int32)
    ef = ctypes.c_int(0)
    ei = ctypes.c_longlong(0)
    nf = ctypes.c_int(0)
    fl = np.zeros(max(1, out.shape[0]), np.int64)
    ref = np.ascontiguousarray(ref)
    qer = np.ascontiguousarray(qer)
    vp = ctypes.c_void_p
    rc = _lib.emu_bsw_run_det(vp(out.ctypes.data), vp(ref.ctypes.data), ctypes.c_longlong(0),
                              ctypes.c_longlong(ref.shape[0]), vp(qer.ctypes.data), ctypes.c_longlong(0),
                              ctypes.c_longlong(qer.shape[0]), int(out.shape[0]), int(w), None, int(bits),
                              vp(kp.ctypes.data), int(G), int(K), int(warps), int(win), ctypes.byref(ef),
                              ctypes.byref(ei), vp(fl.ctypes.data), ctypes.byref(nf), int(fl.shape[0]))
    assert rc == 0, "divergent warp exit"
    idx = np.sort(fl[: nf.value] & 0xffffffff).astype(np.int64)
    return out, ef.value, idx


def run_group(pairs, ref, qer, w, params, bits=16, warps=2, ref_lo=0, qer_lo=0):
    """Scores a copy of pairs with the emulated grouped kernel (the
    reference's groups of 32 / 64 consecutive pairs, one warp each); ref /
    qer are the windows starting at caller offsets ref_lo / qer_lo.
    Returns (pairs, err_flags, err_index)."""
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
    out = np.ascontiguousarray(pairs).copy()
    kp = np.array([params[k] for k in ("o_del", "e_del", "o_ins", "e_ins", "zdrop", "end_bonus", "a", "b")],
                  np.int32)
    ef = ctypes.c_int(0)
    ei = ctypes.c_longlong(0)
    ref = np.ascontiguousarray(ref)
    qer = np.ascontiguousarray(qer)
    vp = ctypes.c_void_p
    rc = _lib.emu_bsw_group_run(vp(out.ctypes.data), vp(ref.ctypes.data), ctypes.c_longlong(ref_lo),
                                ctypes.c_longlong(ref_lo + ref.shape[0]), vp(qer.ctypes.data),
                                ctypes.c_longlong(qer_lo), ctypes.c_longlong(qer_lo + qer.shape[0]),
                                int(out.shape[0]), int(w), int(bits), vp(kp.ctypes.data), int(warps),
                                ctypes.byref(ef), ctypes.byref(ei))
    assert rc == 0, "divergent warp exit"
    return out, ef.value, ei.value


def run_group_wide(pairs, ref, qer, w, params, bits=16, smem_rows=1 << 20, groups=None,
                   ref_lo=0, qer_lo=0):
    """Scores a copy of pairs with the emulated block-wide grouped kernel.
    groups=None: the reference's groups of consecutive pairs, every lane
    wanted.  groups = [(members, need_mask)]: member mode, members a list of
    pair indices (-1: padding lane) of one group, need_mask the lanes whose
    outputs are written.  smem_rows: shared memory for the group's rows (0:
    the global slot).  Returns (pairs, err_flags, err_index, cells)."""
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
    out = np.ascontiguousarray(pairs).copy()
    kp = np.array([params[k] for k in ("o_del", "e_del", "o_ins", "e_ins", "zdrop", "end_bonus", "a", "b")],
                  np.int32)
    ef = ctypes.c_int(0)
    ei = ctypes.c_longlong(0)
    cells = ctypes.c_ulonglong(0)
    ref = np.ascontiguousarray(ref)
    qer = np.ascontiguousarray(qer)
    vp = ctypes.c_void_p
    mem = gin = need = None
    ng = 0
    if groups is not None:
        ng = len(groups)
        mem = np.full((max(ng, 1), 64), -1, np.int64)
        gin = np.zeros((max(ng, 1), 4), np.int32)
        need = np.zeros(max(ng, 1), np.uint64)
        for g, (members, mask) in enumerate(groups):
            mem[g, :len(members)] = members
            real = [m for m in members if m >= 0]
            gin[g] = (w, -1, int(pairs["len2"][real[-1]]) if real else 0, 0)
            need[g] = np.uint64(mask)
    rc = _lib.emu_bsw_group_wide_run(
        vp(out.ctypes.data), vp(ref.ctypes.data), ctypes.c_longlong(ref_lo),
        ctypes.c_longlong(ref_lo + ref.shape[0]), vp(qer.ctypes.data), ctypes.c_longlong(qer_lo),
        ctypes.c_longlong(qer_lo + qer.shape[0]), int(out.shape[0]), int(w), int(bits), vp(kp.ctypes.data),
        None if mem is None else vp(mem.ctypes.data), None if gin is None else vp(gin.ctypes.data),
        None if need is None else vp(need.ctypes.data), int(ng), ctypes.c_longlong(smem_rows),
        ctypes.byref(ef), ctypes.byref(ei), ctypes.byref(cells))
    assert rc == 0, "divergent warp"
    return out, ef.value, ei.value, cells.value


def run_reqs(reqs, order, params, K=4, warps=1, G=32, win=0):
    """A serving tick on the emulated kernel.  reqs: list of dicts with
    pairs, ref, qer (the request's byte windows), ref_lo, qer_lo (window
    offsets), w, bits and optional wpair; order: list of (request, local
    index) work items.  Returns (list of output pair arrays, err, bad)."""
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.emu_bsw_run.restype = ctypes.c_int
    nreq = len(reqs)
    vp = ctypes.c_void_p
    outs = [np.ascontiguousarray(r["pairs"]).copy() for r in reqs]
    refs = [np.ascontiguousarray(r["ref"]) for r in reqs]
    qers = [np.ascontiguousarray(r["qer"]) for r in reqs]
    wps = [None if r.get("wpair") is None else np.ascontiguousarray(r["wpair"], np.int32) for r in reqs]
    P = (vp * nreq)
    LL = (ctypes.c_longlong * nreq)
    I = (ctypes.c_int * nreq)
    kp = np.array([params[k] for k in ("o_del", "e_del", "o_ins", "e_ins", "zdrop", "end_bonus", "a", "b")],
                  np.int32)
    o = np.array([k for _, k in order], np.int32)
    orq = np.array([r for r, _ in order], np.int32)
    err = I()
    bad = LL()
    rc = _lib.emu_bsw_run_reqs(
        nreq, P(*[o_.ctypes.data for o_ in outs]), P(*[r_.ctypes.data for r_ in refs]),
        LL(*[r["ref_lo"] for r in reqs]), LL(*[r["ref_lo"] + refs[i].shape[0] for i, r in enumerate(reqs)]),
        P(*[q_.ctypes.data for q_ in qers]),
        LL(*[r["qer_lo"] for r in reqs]), LL(*[r["qer_lo"] + qers[i].shape[0] for i, r in enumerate(reqs)]),
        P(*[None if x is None else x.ctypes.data for x in wps]),
        I(*[int(x.shape[0]) for x in outs]), I(*[int(r["w"]) for r in reqs]),
        I(*[int(r["bits"]) for r in reqs]), int(o.shape[0]), vp(o.ctypes.data), vp(orq.ctypes.data),
        vp(kp.ctypes.data), int(G), int(K), int(warps), int(win), err, bad)
    assert rc == 0, "lanes of a warp exited apart"
    return outs, list(err), list(bad)


def window_for(w):
    """The lane kernel's ring for band w: smallest power of two >= 2w + 12, at least 64."""
    W = 64
    while W < 2 * w + 12:
        W *= 2
    return W


def run_sw(pairs, seqbuf, stride, params, bits=16, warps=2, packed=None, order=None):
    """The unbanded Smith-Waterman kernel, emulated (packed: two pairs per warp
    in 16x2 lanes; default as the library picks, for 8/16-bit; order: the
    work order, pair indices); returns (pairs, flags, bad)."""
    if packed is None:
        packed = bits != 32 and params["match"] - params["mismatch"] <= 32768
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
    out = np.ascontiguousarray(pairs).copy()
    buf = np.ascontiguousarray(seqbuf)
    pv = np.array([params[k] for k in ("match", "mismatch", "open", "extend")], np.int32)
    ordv = None if order is None else np.ascontiguousarray(order, np.int32)
    lim = {8: 127, 16: 32767, 32: 2 ** 31 - 1}[bits]
    bad = ctypes.c_longlong(0)
    vp = ctypes.c_void_p
    _lib.emu_sw_run.restype = ctypes.c_int
    flags = _lib.emu_sw_run(vp(out.ctypes.data), int(out.shape[0]), vp(buf.ctypes.data),
                            ctypes.c_longlong(buf.shape[0]), ctypes.c_longlong(stride),
                            int(stride - 4), int(lim), vp(pv.ctypes.data), int(warps),
                            int(bool(packed)),
                            vp(ordv.ctypes.data) if ordv is not None else None,
                            ctypes.byref(bad))
    return out, flags, bad.value


def run_chain(anchors, offsets, bw, max_iter, dr, dq, warps=2):
    """The anchor chaining kernel, emulated; returns (f, p, v, flags, bad, evals)."""
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
    a = np.ascontiguousarray(anchors)
    o = np.ascontiguousarray(offsets, np.int64)
    n = a.shape[0]
    f = np.zeros(n, np.uint32)
    p = np.zeros(n, np.int32)
    v = np.zeros(n, np.int32)
    ev = ctypes.c_ulonglong(0)
    bad = ctypes.c_longlong(0)
    vp = ctypes.c_void_p
    _lib.emu_chain_run.restype = ctypes.c_int
    flags = _lib.emu_chain_run(vp(a.ctypes.data), vp(o.ctypes.data), int(o.shape[0] - 1), int(bw),
                               int(max_iter), int(dr), int(dq), vp(f.ctypes.data), vp(p.ctypes.data),
                               vp(v.ctypes.data), int(warps), ctypes.byref(ev), ctypes.byref(bad))
    return f, p, v, flags, bad.value, ev.value
