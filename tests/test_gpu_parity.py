"""GPU parity: the CUDA path (through the C ABI) against the oracle on the same
seeded inputs -- every workload shape at test size, the edge cases, and the
golden fixtures the reference itself produced.  Integer outputs: bit-exact."""
import glob
import os

import numpy as np
import pytest

import oracle
import tal_bsw
from tal_bsw import synth
from tal_bsw.seqpair import outputs

from _cases import DEFAULT, edge_cases, extension_pairs, workload_slices

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _bsw(P):
    return tal_bsw.BandedPairWiseSW(P["o_del"], P["e_del"], P["o_ins"], P["e_ins"], P["zdrop"],
                                    P["end_bonus"], None, P["a"], P["b"], 1, device=0)


def _gpu(pairs, ref, qer, w, P, bits):
    got = pairs.copy()
    with _bsw(P) as bsw:
        if np.ndim(w) == 0:
            bsw._scores(got, ref, qer, got.shape[0], int(w), bits)
        else:  # per-pair band: one call per band value (the reference's w is per call)
            for wv in np.unique(w):
                sel = np.nonzero(w == wv)[0]
                sub = got[sel].copy()
                bsw._scores(sub, ref, qer, sub.shape[0], int(wv), bits)
                got[sel] = sub
    return got


def _assert_same(exp, got, what):
    e, g = outputs(exp), outputs(got)
    bad = np.nonzero((e != g).any(axis=1))[0]
    if bad.size:
        k = int(bad[0])
        raise AssertionError(
            f"{what}: {bad.size}/{len(e)} pairs differ; first #{k} "
            f"(len1={exp['len1'][k]} len2={exp['len2'][k]} h0={exp['h0'][k]}): "
            f"gpu {g[k].tolist()} oracle {e[k].tolist()} "
            "(score, tle, gtle, qle, gscore, max_off)")


@pytest.mark.parametrize("case", workload_slices(), ids=lambda c: c[0])
def test_workload_shapes(case):
    name, b, bits = case
    P = b.workload.params()
    w = b.w if b.workload.w_choices else b.workload.w
    exp = oracle.routed(b.pairs, b.ref, b.qer, w, P, bits=bits)
    got = _gpu(b.pairs, b.ref, b.qer, w, P, bits)
    _assert_same(exp, got, name)


@pytest.mark.parametrize("bits", [16, 8])
def test_edge_cases(bits):
    for name, p, r, q, w, P in edge_cases(bits=bits):
        if bits == 8:
            keep = oracle.eligible8(p, w, P)
            p = p[keep]
            if p.shape[0] == 0:
                continue
        exp = oracle.vector(p, r, q, w, P, bits=bits)
        got = _gpu(p, r, q, w, P, bits)
        _assert_same(exp, got, f"{name}/{bits}")


def test_golden_fixtures():
    files = sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))
    assert files, "no golden fixtures"
    for f in files:
        d = np.load(f)
        P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
        got = _gpu(d["inputs"], d["ref"], d["qer"], d["w"], P, int(d["bits"]))
        _assert_same(d["expected"], got, os.path.basename(f))


def test_auto_routing_matches_forced():
    b = synth.generate(synth.C1_8, 500)
    P = b.workload.params()
    a = _gpu(b.pairs, b.ref, b.qer, 100, P, 0)
    e8 = _gpu(b.pairs, b.ref, b.qer, 100, P, 8)
    _assert_same(e8, a, "auto vs 8-bit on 8-bit-eligible pairs")


def test_out_of_range_rejected():
    b = synth.generate(synth.C1, 64)   # 151 bp: outside the 8-bit range
    P = b.workload.params()
    got = b.pairs.copy()
    with _bsw(P) as bsw:
        with pytest.raises(tal_bsw.TalBswError) as ei:
            bsw.getScores8(got, b.ref, b.qer, b.n, 1, 100)
        assert ei.value.status == tal_bsw.api.TAL_EDOMAIN
        assert ei.value.bad_pair == 0
    assert (outputs(got) == -1).all(), "no outputs are written on a range error"


@pytest.mark.parametrize("wl,bits", [(synth.C2, 16), (synth.C1_8, 8), (synth.C3, 0)])
def test_plain_launch_length_order(wl, bits):
    """Batches from 2,048 pairs run in target-length order (a device counting
    sort before the scoring launch): the outputs equal the oracle's and those
    of the caller's order (TAL_BSW_NO_ORDER), pair by pair."""
    b = synth.generate(wl, 6000)
    P = b.workload.params()
    w = 100
    exp = oracle.routed(b.pairs, b.ref, b.qer, w, P, bits=bits)
    got = _gpu(b.pairs, b.ref, b.qer, w, P, bits)
    _assert_same(exp, got, f"{wl.name} ordered")
    os.environ["TAL_BSW_NO_ORDER"] = "1"
    try:
        unordered = _gpu(b.pairs, b.ref, b.qer, w, P, bits)
    finally:
        del os.environ["TAL_BSW_NO_ORDER"]
    _assert_same(unordered, got, f"{wl.name} ordered vs caller's order")


def test_plain_launch_length_order_reports_the_callers_index():
    """A bad pair inside a length-ordered launch is reported by its index in
    the caller's array."""
    b = synth.generate(synth.C2, 5000)
    P = b.workload.params()
    q = b.qer.copy()
    k = 3001
    q[int(b.pairs["idq"][k]) + 3] = 9   # a query base code above 4
    got = b.pairs.copy()
    with _bsw(P) as bsw:
        with pytest.raises(tal_bsw.TalBswError) as ei:
            bsw.getScores16(got, b.ref, q, b.n, 1, 100)
    assert ei.value.bad_pair == k


def test_host_call_in_chunks():
    """Host-buffer calls of 262,144+ pairs copy and score in four chunks (the
    next chunk's copies overlap this chunk's scoring): outputs equal the
    device-resident call's and, on a sample, the oracle's; a bad pair in a
    later chunk is reported by its index in the caller's array."""
    import torch
    b = synth.generate(synth.C2, 300000)
    P = b.workload.params()
    got = b.pairs.copy()
    with _bsw(P) as bsw:
        bsw.getScores16(got, b.ref, b.qer, b.n, 1, 100)
        dp = torch.from_numpy(b.pairs.view(np.uint8).reshape(-1).copy()).cuda()
        dr = torch.from_numpy(b.ref).cuda()
        dq = torch.from_numpy(b.qer).cuda()
        bsw.scores_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(), b.n,
                          100, 16)
        bsw.sync()
        dev = dp.cpu().numpy().view(tal_bsw.SEQPAIR_DTYPE)
        _assert_same(dev, got, "chunked host call vs device-resident call")
        k = np.arange(0, b.n, 150)
        exp = oracle.vector(b.pairs[k], b.ref, b.qer, 100, P, bits=16)
        _assert_same(exp, got[k], "chunked host call vs oracle (sample)")
        q = b.qer.copy()
        bad = 250001
        q[int(b.pairs["idq"][bad]) + 2] = 7
        g2 = b.pairs.copy()
        with pytest.raises(tal_bsw.TalBswError) as ei:
            bsw.getScores16(g2, b.ref, q, b.n, 1, 100)
        assert ei.value.bad_pair == bad
        assert (outputs(g2) == -1).all(), "no outputs are written on an error"


def test_long_queries_near_the_16_bit_limit():
    """Queries of 20,000-32,700 bases: narrow bands in rings (lane kernel),
    a band of 8,000 in a 16,384-column ring (G lanes per pair), a band of
    10,000 in whole rows of 22,000 columns, and each in the grouped kernel; a
    query of 30,000 with a band of 20,000 needs more shared memory than a
    block has for the per-pair kernels: the regroup pass scores it exactly
    (TAL_EDOMAIN with per-pair semantics)."""
    from _cases import DEFAULT, pack
    rng = np.random.default_rng(77)

    def pair(L, extra):
        q = rng.integers(0, 4, L).astype(np.uint8)
        r = q.copy()
        m = rng.random(L) < 0.03
        r[m] = (r[m] + 1) % 4
        return np.concatenate([r, rng.integers(0, 4, extra).astype(np.uint8)]), q

    for lens, w in (((30000, 32700, 20000), 50), ((20000,), 8000), ((22000,), 10000)):
        refs, qers = zip(*[pair(L, 40) for L in lens])  # h0 + min length stays below 2^15
        p, r, q = pack(list(refs), list(qers), [50] * len(lens))
        exp = oracle.vector(p, r, q, w, DEFAULT, bits=16)
        got = _gpu(p, r, q, w, DEFAULT, 16)
        _assert_same(exp, got, f"long queries, w={w}")
        # the grouped kernel keeps its rows in global scratch: same outputs
        got = _gpu(p, r, q, w, DEFAULT, 16 | tal_bsw.api.GROUPED)
        _assert_same(exp, got, f"long queries, w={w}, grouped")
    # rows too long for shared memory: exact through the regroup pass (rows in
    # global scratch); with per-pair semantics a refusal.  The target follows the
    # query for 3,000 bases and then diverges, so the alignment ends by z-drop
    # and the re-scored group stops early
    r0, q0 = pair(30000, 0)
    r0[3000:] = rng.integers(0, 4, r0.shape[0] - 3000).astype(np.uint8)
    refs, qers = zip(*[(r0, q0), pair(600, 20)])
    p, r, q = pack(list(refs), list(qers), [50, 50])
    exp = oracle.vector(p, r, q, 20000, DEFAULT, bits=16)
    got = _gpu(p, r, q, 20000, DEFAULT, 16)
    _assert_same(exp, got, "a query of 30,000 with a band of 20,000")
    with _bsw(DEFAULT) as bsw:
        with pytest.raises(tal_bsw.TalBswError) as ei:
            bsw._scores(p.copy(), r, q, 2, 20000, 16 | tal_bsw.api.PER_PAIR)
        assert ei.value.status == tal_bsw.api.TAL_EDOMAIN


# ---------------------------------------------------------------- grouped scoring
GROUPED = tal_bsw.api.GROUPED


def _grouped_files():
    out = []
    for f in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        d = np.load(f)
        if int(d["bits"]) in (8, 16) and np.ndim(d["w"]) == 0:
            out.append(f)
    return out


@pytest.mark.parametrize("f", _grouped_files(), ids=os.path.basename)
def test_grouped_matches_golden(f):
    """TAL_BSW_GROUPED: the reference's SIMD groups on the GPU give its
    outputs on every fixture, the coupled ones (where a pair's outputs depend
    on its group) included."""
    d = np.load(f)
    P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
    bits = int(d["bits"])
    got = _gpu(d["inputs"], d["ref"], d["qer"], d["w"], P, bits | GROUPED)
    _assert_same(d["expected"], got, os.path.basename(f) + " grouped")


def test_default_path_is_exact_on_coupled_and_wrapping_fixtures():
    """Without any flag the plain call equals the reference on the fixtures
    where a pair's outputs depend on its SIMD group (the per-pair kernels
    flag those pairs and their groups are re-scored in the reference's
    grouping) and on those whose int8 / int16 values wrap (outside the
    per-pair kernels' exact range, scored by the grouped kernel)."""
    files = sorted(glob.glob(os.path.join(GOLDEN, "coupled*.npz")) + glob.glob(os.path.join(GOLDEN, "wrap*.npz")))
    assert len(files) >= 6
    for f in files:
        d = np.load(f)
        P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
        bits = int(d["bits"])
        with _bsw(P) as bsw:
            got = d["inputs"].copy()
            bsw._scores(got, d["ref"], d["qer"], got.shape[0], int(d["w"]), bits)
            flagged, groups = bsw.last_regroup()
        _assert_same(d["expected"], got, os.path.basename(f) + " default path")
        if "coupled" in f:
            alone = oracle.vector(d["inputs"], d["ref"], d["qer"], int(d["w"]), P, bits=bits, lanes=1)
            assert (outputs(alone) != outputs(d["expected"])).any(1).sum() >= 1
            assert flagged >= 1 and groups >= 1


def _coupled_mix():
    """Pairs of the 16- and 8-bit coupled fixtures (same scoring) as one
    batch: interleaved in runs of 7, bands 4 and 8 per pair.  The expected
    outputs are the reference's for that batch split as its caller would --
    one call per (band, precision) class, pairs in array order."""
    parts = []
    for name in ("coupled16_band_4.npz", "coupled16_band_8.npz", "coupled8_band_8.npz"):
        d = np.load(os.path.join(GOLDEN, name))
        parts.append((d["inputs"], d["ref"], d["qer"], int(d["w"])))
    P = {k: int(v) for k, v in zip(np.load(os.path.join(GOLDEN, "coupled16_band_4.npz"))["param_keys"],
                                   np.load(os.path.join(GOLDEN, "coupled16_band_4.npz"))["param_vals"])}
    refs, qers, rows, ws = [], [], [], []
    roff = qoff = 0
    for p, r, q, w in parts:
        p = p.copy()
        p["idr"] += roff
        p["idq"] += qoff
        refs.append(r); qers.append(q); rows.append(p); ws.append(np.full(p.shape[0], w, np.int32))
        roff += r.shape[0]; qoff += q.shape[0]
    pairs = np.concatenate(rows)
    wpair = np.concatenate(ws)
    ref, qer = np.concatenate(refs), np.concatenate(qers)
    rng = np.random.default_rng(17)
    runs = np.array_split(np.arange(pairs.shape[0]), pairs.shape[0] // 7)
    order = np.concatenate([runs[k] for k in rng.permutation(len(runs))])
    pairs, wpair = pairs[order], wpair[order]
    exp = oracle.routed(pairs, ref, qer, wpair, P, bits=0)
    return pairs, ref, qer, wpair, P, exp


def test_batched_and_device_calls_are_exact_on_coupled_pairs():
    """The batched form (per-pair bands, 8/16-bit routing) and the
    device-resident plain call re-score flagged pairs' groups in the grouping
    the reference's caller would use, so they equal the reference on a
    batch mixing coupled pairs of both precisions and two bands."""
    import torch
    pairs, ref, qer, wpair, P, exp = _coupled_mix()
    with _bsw(P) as bsw:
        got = pairs.copy()
        bsw.scores_batched(got, ref, qer, got.shape[0], w=100, wpair=wpair, bits=0)
        _assert_same(exp, got, "batched, coupled mix")
        assert bsw.last_regroup()[1] >= 1
        dp = torch.from_numpy(pairs.view(np.uint8).reshape(-1).copy()).cuda()
        dr = torch.from_numpy(ref).cuda()
        dq = torch.from_numpy(qer).cuda()
        dw = torch.from_numpy(wpair).cuda()
        bsw.scores_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(),
                          pairs.shape[0], 100, 0, d_w=dw.data_ptr())
        bsw.sync()
        dev = dp.cpu().numpy().view(tal_bsw.SEQPAIR_DTYPE)
        _assert_same(exp, dev, "device call, coupled mix")
        # the same again: the pass leaves its tables empty for the next call
        got2 = pairs.copy()
        bsw.scores_batched(got2, ref, qer, got2.shape[0], w=100, wpair=wpair, bits=0)
        _assert_same(exp, got2, "batched, coupled mix, second call")


def test_server_is_exact_on_coupled_requests():
    """Serving: coupled fixtures as requests in one tick, each request its
    own caller array -- every output equals the reference's."""
    reqs = []
    for name in ("coupled16_band_4.npz", "coupled8_band_8.npz", "coupled16_band_8.npz", "wrap16_h0_near_limit_band_100.npz"):
        d = np.load(os.path.join(GOLDEN, name))
        reqs.append((d["inputs"].copy(), d["ref"], d["qer"], int(d["w"]), int(d["bits"]), d["expected"]))
    P = {k: int(v) for k, v in zip(np.load(os.path.join(GOLDEN, "coupled16_band_4.npz"))["param_keys"],
                                   np.load(os.path.join(GOLDEN, "coupled16_band_4.npz"))["param_vals"])}
    with _bsw(P) as bsw, tal_bsw.BswServer(bsw, pool_bytes=256 << 20) as srv:
        tickets = [srv.submit(p, r, q, w=w, bits=b) for p, r, q, w, b, _ in reqs]
        infos = [srv.poll(t, timeout_us=60_000_000) for t in tickets]
    for (p, _, _, _, _, e), info, name in zip(reqs, infos, range(len(reqs))):
        assert info is not None and info.status == tal_bsw.api.TAL_OK
        _assert_same(e, p, f"server request {name}")


def _extension_batch(w):
    """About 14,000 right-extension pairs of 6,000 reads (queries 100-250 bp
    after the seed), in seed order, band w."""
    return extension_pairs(6000, w, 100, 250, 1000 + w, DEFAULT)


@pytest.mark.parametrize("w", [4, 8, 16])
def test_default_path_is_exact_on_extension_batches(w):
    """Stress of the default (exact) path at scale: whole seed-extension
    batches with narrow bands, where tens of pairs per batch have outputs
    that depend on their SIMD group.  The plain call equals the reference's
    grouped outputs on every pair, 16-bit on the whole batch and 8-bit on
    its int8-eligible pairs."""
    pairs, ref, qer = _extension_batch(w)
    for bits, sel in ((16, np.arange(pairs.shape[0])),
                      (8, np.nonzero(oracle.eligible8(pairs, w, DEFAULT))[0])):
        p = pairs[sel]
        exp = oracle.vector(p, ref, qer, w, DEFAULT, bits=bits, nthreads=8)
        alone = oracle.vector(p, ref, qer, w, DEFAULT, bits=bits, lanes=1, nthreads=8)
        coupled = int((outputs(alone) != outputs(exp)).any(1).sum())
        assert coupled >= 1, "the batch should hold group-dependent pairs"
        with _bsw(DEFAULT) as bsw:
            got = p.copy()
            bsw._scores(got, ref, qer, got.shape[0], w, bits)
            flagged, groups = bsw.last_regroup()
        _assert_same(exp, got, f"extension batch w={w} bits={bits} ({coupled} group-dependent pairs)")
        assert flagged >= 1 and groups >= 1


def test_batched_form_is_exact_on_mixed_extension_batches():
    """The batched form on the three extension batches mixed (bands 4, 8 and
    16 per pair, 8/16-bit routing per pair, interleaved in runs of 11): equal
    to the reference's caller splitting the batch into one call per (band,
    precision) class, pairs in array order."""
    rows, refs, qers, ws = [], [], [], []
    roff = qoff = 0
    for w in (4, 8, 16):
        p, r, q = _extension_batch(w)
        p = p.copy()
        p["idr"] += roff
        p["idq"] += qoff
        rows.append(p); refs.append(r); qers.append(q); ws.append(np.full(p.shape[0], w, np.int32))
        roff += r.shape[0]; qoff += q.shape[0]
    pairs, wpair = np.concatenate(rows), np.concatenate(ws)
    ref, qer = np.concatenate(refs), np.concatenate(qers)
    runs = np.array_split(np.arange(pairs.shape[0]), pairs.shape[0] // 11)
    order = np.concatenate([runs[k] for k in np.random.default_rng(23).permutation(len(runs))])
    pairs, wpair = pairs[order], wpair[order]
    exp = oracle.routed(pairs, ref, qer, wpair, DEFAULT, bits=0, nthreads=8)
    with _bsw(DEFAULT) as bsw:
        got = pairs.copy()
        bsw.scores_batched(got, ref, qer, got.shape[0], w=16, wpair=wpair, bits=0)
        flagged, groups = bsw.last_regroup()
    _assert_same(exp, got, "batched form, mixed extension batches")
    assert flagged >= 1 and groups >= 1


@pytest.mark.parametrize("wl,bits,n", [(synth.C2, 16, 3000), (synth.C1_8, 8, 5001), (synth.C4, 16, 70)])
def test_grouped_workloads_match_oracle(wl, bits, n):
    b = synth.generate(wl.scaled(n, seed=wl.seed + 77))
    P = b.workload.params()
    exp = oracle.vector(b.pairs, b.ref, b.qer, b.workload.w, P, bits=bits, nthreads=8)
    got = _gpu(b.pairs, b.ref, b.qer, b.workload.w, P, bits | GROUPED)
    _assert_same(exp, got, wl.name + " grouped")


def test_grouped_device_path_and_chunked_host_call_agree():
    """The device-resident call and the host call (copied and scored in
    chunks that end on group boundaries) give the same grouped outputs."""
    import torch
    b = synth.generate(synth.C1_8.scaled(300_001, seed=91))
    P = b.workload.params()
    host = _gpu(b.pairs, b.ref, b.qer, 100, P, 8 | GROUPED)
    with _bsw(P) as bsw:
        dp = torch.from_numpy(b.pairs.view(np.uint8).reshape(-1).copy()).cuda()
        dr = torch.from_numpy(b.ref).cuda()
        dq = torch.from_numpy(b.qer).cuda()
        bsw.scores_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(), b.n,
                          100, bits=8 | GROUPED)
        dev = dp.cpu().numpy().view(b.pairs.dtype)
    _assert_same(host, dev, "grouped host vs device")
    exp = oracle.vector(b.pairs[:640], b.ref, b.qer, 100, P, bits=8)
    _assert_same(exp, host[:640], "grouped chunk 0 head")


def test_grouped_bad_pair_in_a_later_chunk():
    """A grouped host call of 262,144+ pairs (chunks ending on group
    boundaries) names a bad pair in its third chunk by its index in the
    caller's array; a device call with per-pair bands is refused."""
    import torch
    b = synth.generate(synth.C1_8.scaled(270_000, seed=93))
    P = b.workload.params()
    p = b.pairs.copy()
    bad = 201_000
    p["h0"][bad] = -3
    with _bsw(P) as bsw:
        with pytest.raises(tal_bsw.TalBswError) as ei:
            bsw._scores(p, b.ref, b.qer, b.n, 100, 8 | GROUPED)
        assert ei.value.status == tal_bsw.api.TAL_EDOMAIN and ei.value.bad_pair == bad
        dp = torch.from_numpy(b.pairs[:64].view(np.uint8).reshape(-1).copy()).cuda()
        dr = torch.from_numpy(b.ref).cuda()
        dq = torch.from_numpy(b.qer).cuda()
        dw = torch.full((64,), 100, dtype=torch.int32, device="cuda")
        with pytest.raises(tal_bsw.TalBswError) as ei:
            bsw.scores_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(), 64,
                              100, bits=8 | GROUPED, d_w=dw.data_ptr())
        assert ei.value.status == tal_bsw.api.TAL_EINVAL


def test_grouped_refusals():
    b = synth.generate(synth.C2.scaled(64, seed=5))
    P = b.workload.params()
    with _bsw(P) as bsw:
        for bits in (GROUPED, GROUPED | 32):
            with pytest.raises(tal_bsw.TalBswError) as ei:
                bsw._scores(b.pairs.copy(), b.ref, b.qer, b.n, 100, bits)
            assert ei.value.status == tal_bsw.api.TAL_EINVAL
        p = b.pairs.copy()
        p["h0"][40] = -5                 # outside the range
        with pytest.raises(tal_bsw.TalBswError) as ei:
            bsw._scores(p, b.ref, b.qer, b.n, 100, 16 | GROUPED)
        assert ei.value.status == tal_bsw.api.TAL_EDOMAIN and ei.value.bad_pair == 40


@pytest.mark.parametrize("wl,n", [(synth.C1, 100_000), (synth.C1_8, 100_000), (synth.C3, 2_000_000),
                                  (synth.C4, 4_000)])
def test_per_pair_equals_grouped_on_workloads(wl, n):
    """At workload sizes no oracle finishes quickly: the per-pair kernels and
    the grouped kernel (the reference's own grouping) give the same outputs
    on every pair, per (band, precision) call as the reference's caller
    would split a mixed batch."""
    b = synth.generate(wl, n)
    P = wl.params()
    warr = b.w if wl.w_choices else np.full(b.n, wl.w, np.int32)
    is8 = oracle.eligible8(b.pairs, warr, P) if wl.bits == 0 else np.full(b.n, wl.bits == 8)
    with _bsw(P) as bsw:
        for wv in np.unique(warr):
            for bits in (8, 16):
                sel = np.nonzero((warr == wv) & (is8 == (bits == 8)))[0]
                if not sel.size:
                    continue
                a = b.pairs[sel].copy()
                g = b.pairs[sel].copy()
                bsw._scores(a, b.ref, b.qer, a.shape[0], int(wv), bits)
                bsw._scores(g, b.ref, b.qer, g.shape[0], int(wv), bits | GROUPED)
                _assert_same(g, a, f"{wl.name} w={wv} bits={bits}: per pair vs grouped")


def test_scalar_wrapper_matches_the_scalar_path():
    """scalarBandedSWAWrapper / scalarBandedSWA (bandedSWA.cpp:116-260) run on
    the GPU with every pair alone in its group: equal to the oracle's port of
    the reference's scalar code at e_del = e_ins = 1; other gap extensions
    are refused."""
    b = synth.generate(synth.C2.scaled(2000, seed=31))
    P = b.workload.params()
    exp, _ = oracle.scalar(b.pairs, b.ref, b.qer, 100, P)
    with _bsw(P) as bsw:
        got = b.pairs.copy()
        bsw.scalarBandedSWAWrapper(got, b.ref, b.qer, b.n, 1, 100)
        _assert_same(exp, got, "scalarBandedSWAWrapper")
        p0 = b.pairs[7]
        q = b.qer[p0["idq"]:p0["idq"] + p0["len2"]]
        t = b.ref[p0["idr"]:p0["idr"] + p0["len1"]]
        r = bsw.scalarBandedSWA(int(p0["len2"]), q, int(p0["len1"]), t, 100, int(p0["h0"]))
        e = exp[7]
        assert r == (e["score"], e["qle"], e["tle"], e["gtle"], e["gscore"], e["max_off"])
    P2 = dict(P, e_del=2, e_ins=2)
    with _bsw(P2) as bsw:
        with pytest.raises(tal_bsw.TalBswError):
            bsw.scalarBandedSWAWrapper(b.pairs.copy(), b.ref, b.qer, b.n, 1, 100)
