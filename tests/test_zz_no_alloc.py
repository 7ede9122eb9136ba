"""The allocation-free entry point (tal_bsw_scores_device_noalloc), called
through the C ABI: two calls in a row on device buffers the test owns, each
compared with the regular entry point (tal_bsw_scores) on the same pairs, and
a slice compared with the oracle scoring each pair alone in its SIMD group
(the entry point's documented semantics).  Integer outputs, so the tolerance
is zero.  Collected last on purpose."""
import ctypes

import numpy as np
import pytest

import oracle
import tal_bsw
from tal_bsw import synth
from tal_bsw.seqpair import outputs

pytestmark = pytest.mark.gpu


def _noalloc(lib, P, d_pairs, d_ref, d_qer, n, w, bits):
    prm = tal_bsw.api._Params(P["o_del"], P["e_del"], P["o_ins"], P["e_ins"], P["zdrop"],
                              P["end_bonus"], P["a"], P["b"])
    f = lib.tal_bsw_scores_device_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                  ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int32, ctypes.c_int32,
                  ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    return f(ctypes.byref(prm), d_pairs.data_ptr(), d_ref.data_ptr(), d_ref.numel(),
             d_qer.data_ptr(), d_qer.numel(), n, w, None, bits, None)


@pytest.mark.parametrize("name,bits", [("c2_16bit", 16), ("c1_8bit", 8), ("c3_mixed", 0)])
def test_noalloc_matches_regular_entry_point(name, bits):
    import torch
    wl = synth.WORKLOADS[name]
    b = synth.generate(wl, 2000)
    P = wl.params()
    w = 100
    expected = b.pairs.copy()
    with tal_bsw.BandedPairWiseSW(P["o_del"], P["e_del"], P["o_ins"], P["e_ins"], P["zdrop"],
                                  P["end_bonus"], None, P["a"], P["b"], 1, device=0) as bsw:
        bsw._scores(expected, b.ref, b.qer, b.n, w, bits)
    lib = tal_bsw.api.core_lib()
    torch.cuda.set_device(0)
    d_ref = torch.from_numpy(b.ref).cuda()
    d_qer = torch.from_numpy(b.qer).cuda()
    for call in range(2):
        d_pairs = torch.from_numpy(b.pairs.view(np.uint8).copy()).cuda()
        torch.cuda.synchronize()
        rc = _noalloc(lib, P, d_pairs, d_ref, d_qer, b.n, w, bits)
        assert rc == tal_bsw.api.TAL_OK, f"call {call}: status {rc}"
        got = d_pairs.cpu().numpy().view(tal_bsw.SEQPAIR_DTYPE)
        e, g = outputs(expected), outputs(got)
        bad = np.nonzero((e != g).any(axis=1))[0]
        assert bad.size == 0, f"call {call}: {bad.size} pairs differ, first {bad[0]}"
    # a slice against the oracle, each pair alone in its group, routed per pair
    k = slice(0, 300)
    sub = b.pairs[k]
    is8 = np.full(sub.shape[0], bits == 8) if bits else oracle.eligible8(sub, w, P)
    exp = sub.copy()
    for bb in (8, 16):
        sel = np.nonzero(is8 == (bb == 8))[0]
        if sel.size:
            exp[sel] = oracle.vector(sub[sel], b.ref, b.qer, w, P, bits=bb, lanes=1)
    assert (outputs(exp) == outputs(got[k])).all(), "noalloc slice differs from the oracle"


def _last_bad(lib):
    f = lib.tal_bsw_noalloc_last_bad_pair
    f.restype = ctypes.c_int64
    f.argtypes = []
    return int(f())


def test_noalloc_reports_out_of_range_pairs():
    import torch
    b = synth.generate(synth.C1, 64)     # 151 bp: outside the 8-bit range
    P = synth.C1.params()
    lib = tal_bsw.api.core_lib()
    d_pairs = torch.from_numpy(b.pairs.view(np.uint8).copy()).cuda()
    d_ref = torch.from_numpy(b.ref).cuda()
    d_qer = torch.from_numpy(b.qer).cuda()
    assert _noalloc(lib, P, d_pairs, d_ref, d_qer, b.n, 100, 8) == tal_bsw.api.TAL_EDOMAIN
    assert _last_bad(lib) == 0  # every pair is out of range: the lowest index
    # a base code above 4 is a domain error too, naming its pair
    q = b.qer.copy()
    q[int(b.pairs["idq"][5]) + 1] = 9
    d_q9 = torch.from_numpy(q).cuda()
    d_pairs = torch.from_numpy(b.pairs.view(np.uint8).copy()).cuda()
    assert _noalloc(lib, P, d_pairs, d_ref, d_q9, b.n, 100, 16) == tal_bsw.api.TAL_EDOMAIN
    assert _last_bad(lib) == 5
    # the next call clears the shared control block and succeeds
    d_pairs = torch.from_numpy(b.pairs.view(np.uint8).copy()).cuda()
    assert _noalloc(lib, P, d_pairs, d_ref, d_qer, b.n, 100, 16) == tal_bsw.api.TAL_OK
    assert _last_bad(lib) == -1


def test_noalloc_capacity_is_not_a_domain_error():
    """A pair inside the exact range whose rows exceed shared memory (a
    30,000-base query with a band covering it, whole rows of the G-lane
    kernel): TAL_ENOMEM, not TAL_EDOMAIN, and no pair named (the batch is
    refused before the launch)."""
    import torch
    rng = np.random.default_rng(3)
    L = 30000
    q = rng.integers(0, 4, L).astype(np.uint8)
    r = q.copy()
    pairs = np.zeros(1, tal_bsw.SEQPAIR_DTYPE)
    pairs["idr"] = 0
    pairs["idq"] = 0
    pairs["len1"] = L
    pairs["len2"] = L
    pairs["h0"] = 10
    P = synth.C2.params()
    lib = tal_bsw.api.core_lib()
    d_pairs = torch.from_numpy(pairs.view(np.uint8).copy()).cuda()
    d_ref = torch.from_numpy(r).cuda()
    d_qer = torch.from_numpy(q).cuda()
    assert _noalloc(lib, P, d_pairs, d_ref, d_qer, 1, L, 16) == tal_bsw.api.TAL_ENOMEM
    assert _last_bad(lib) == -1
