"""The CUDA kernel's source, compiled for the host and run one fiber per lane
(tests/simt_emu), against the reference's golden outputs: checks the kernel's
logic on a machine without a GPU.  The GPU tests run the real thing."""
import glob
import os

import numpy as np
import pytest

import oracle
import simt_emu
from tal_bsw.seqpair import outputs

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
ALL_FILES = sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))
# fixtures whose reference outputs depend on the SIMD grouping: the per-pair
# kernels are checked on them against pair-at-a-time scoring instead
COUPLED = [f for f in ALL_FILES if os.path.basename(f).startswith("coupled")]
# fixtures outside the per-pair kernels' exact range (int8 gap sums or int16
# scores that wrap): grouped kernel only
WRAPPING = [f for f in ALL_FILES if os.path.basename(f).startswith("wrap")]
FILES = [f for f in ALL_FILES if f not in COUPLED and f not in WRAPPING]
CONFIGS = [(1, 4), (4, 4), (8, 4), (8, 2), (16, 4), (32, 4), (32, 2), (4, 2), (16, 2)]


@pytest.mark.parametrize("f", FILES, ids=os.path.basename)
def test_emulated_kernel_matches_golden(f):
    d = np.load(f)
    P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
    n = min(d["inputs"].shape[0], 6 if "c4" in f else 16)
    p = d["inputs"][:n]
    w = d["w"]
    bits = int(d["bits"])
    G, K = CONFIGS[sum(os.path.basename(f).encode()) % len(CONFIGS)]
    if np.ndim(w):
        got, ef, _ = simt_emu.run(p, d["ref"], d["qer"], 0, P, bits=bits, K=K, G=G, warps=2,
                                  wpair=w[:n])
    else:
        got, ef, _ = simt_emu.run(p, d["ref"], d["qer"], int(w), P, bits=bits, K=K, G=G, warps=2)
    assert ef == 0
    e, g = outputs(d["expected"][:n]), outputs(got)
    bad = np.nonzero((e != g).any(1))[0]
    assert bad.size == 0, f"G={G} K={K}: pair {bad[0]}: emu {g[bad[0]].tolist()} ref {e[bad[0]].tolist()}"


def _request(name, lo, hi, **over):
    """Pairs [lo, hi) of a golden fixture as one serving request: its own
    copies of the byte windows its pairs reference, its band and precision."""
    d = np.load(os.path.join(GOLDEN, name))
    p = d["inputs"][lo:hi].copy()
    rlo = int(p["idr"].min()) & ~15
    qlo = int(p["idq"].min()) & ~15
    rhi = int((p["idr"] + p["len1"]).max())
    qhi = int((p["idq"] + p["len2"]).max())
    w = d["w"]
    req = dict(pairs=p, ref=d["ref"][rlo:rhi].copy(), qer=d["qer"][qlo:qhi].copy(), ref_lo=rlo,
               qer_lo=qlo, bits=int(d["bits"]), expected=d["expected"][lo:hi])
    if np.ndim(w):
        req.update(w=0, wpair=w[lo:hi].astype(np.int32))
    else:
        req.update(w=int(w))
    req.update(over)
    return req


@pytest.mark.parametrize("G,K", [(1, 4), (8, 4)])
def test_emulated_request_table(G, K):
    """A serving tick: pairs of five requests (8-bit, 16-bit, per-pair band
    with routing, narrow bands) interleaved in one work list, each request with
    its own buffers; one more request holds a bad pair.  Every good request
    gets the reference's outputs and no error; only the bad request is flagged,
    with its own local index."""
    reqs = [_request("wl_c1_8bit.npz", 0, 9), _request("wl_c2_16bit.npz", 5, 13),
            _request("wl_c3_mixed.npz", 40, 52), _request("edge16_band_3.npz", 0, 7),
            _request("edge8_band_17.npz", 3, 10)]
    bad = _request("wl_c2_16bit.npz", 20, 26)
    bad["pairs"]["len1"][3] = -1           # outside the exact range: TAL_EDOMAIN
    reqs.append(bad)
    P = dict(o_del=6, e_del=1, o_ins=6, e_ins=1, zdrop=100, end_bonus=5, a=1, b=4)
    items = [(r, k) for r, q in enumerate(reqs) for k in range(q["pairs"].shape[0])]
    rng = np.random.default_rng(11)
    order = [items[i] for i in rng.permutation(len(items))]
    outs, err, badidx = simt_emu.run_reqs(reqs, order, P, K=K, warps=2, G=G)
    for r, q in enumerate(reqs[:-1]):
        assert err[r] == 0
        e, g = outputs(q["expected"]), outputs(outs[r])
        diff = np.nonzero((e != g).any(1))[0]
        assert diff.size == 0, f"request {r} pair {diff[0]}: {g[diff[0]].tolist()} vs {e[diff[0]].tolist()}"
    assert err[-1] != 0 and badidx[-1] == 3
    keep = [k for k in range(6) if k != 3]
    assert (outputs(outs[-1])[keep] == outputs(bad["expected"])[keep]).all()


@pytest.mark.parametrize("f", FILES, ids=os.path.basename)
def test_emulated_lane_kernel_with_row_ring(f):
    """The lane kernel keeping a ring of the smallest window its band allows
    (columns wrap around it for every query longer than the ring) gives the
    reference's outputs: the live band never reaches a reused slot and the
    head re-derivation's reads of columns that left the band are answered
    from what was recorded as they left."""
    d = np.load(f)
    P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
    n = min(d["inputs"].shape[0], 6 if "c4" in f else 24)
    p = d["inputs"][:n]
    w = d["w"]
    bits = int(d["bits"])
    wmax = int(np.max(w[:n])) if np.ndim(w) else int(w)
    win = simt_emu.window_for(max(wmax, 0))
    if np.ndim(w):
        got, ef, _ = simt_emu.run(p, d["ref"], d["qer"], 0, P, bits=bits, K=4, G=1, warps=1,
                                  wpair=w[:n], win=win)
    else:
        got, ef, _ = simt_emu.run(p, d["ref"], d["qer"], int(w), P, bits=bits, K=4, G=1, warps=1,
                                  win=win)
    assert ef == 0
    e, g = outputs(d["expected"][:n]), outputs(got)
    bad = np.nonzero((e != g).any(1))[0]
    assert bad.size == 0, f"win={win}: pair {bad[0]}: emu {g[bad[0]].tolist()} ref {e[bad[0]].tolist()}"


def test_emulated_row_ring_wraps_on_long_queries():
    """Many C2-shaped pairs (queries up to 300 columns, band 100) through a
    256-column ring, and band 20 through a 64-column ring, against the oracle."""
    from tal_bsw import synth
    b = synth.generate(synth.C2, 64)
    P = synth.C2.params()
    for w, win in ((100, 256), (20, 64), (3, 64)):
        exp = oracle.vector(b.pairs, b.ref, b.qer, w, P, bits=16, lanes=1)
        got, ef, _ = simt_emu.run(b.pairs, b.ref, b.qer, w, P, bits=16, K=4, G=1, warps=2, win=win)
        assert ef == 0
        e, g = outputs(exp), outputs(got)
        bad = np.nonzero((e != g).any(1))[0]
        assert bad.size == 0, f"w={w} win={win}: pair {bad[0]}: emu {g[bad[0]].tolist()} oracle {e[bad[0]].tolist()}"


@pytest.mark.parametrize("f", FILES, ids=os.path.basename)
def test_emulated_group_kernel_with_row_ring(f):
    """G lanes per pair with power-of-two rings as small as the band allows
    (strips read and write column chunks through the ring; the head
    re-derivation's reads below the band come from the frozen-column record)."""
    d = np.load(f)
    P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
    n = min(d["inputs"].shape[0], 6 if "c4" in f else 16)
    p = d["inputs"][:n]
    w = d["w"]
    bits = int(d["bits"])
    G, K = [(4, 4), (8, 4), (16, 4), (32, 4), (8, 2)][sum(os.path.basename(f).encode()) % 5]
    wmax = int(np.max(w[:n])) if np.ndim(w) else int(w)
    win = simt_emu.window_for(max(wmax, 0))
    kw = dict(bits=bits, K=K, G=G, warps=2, win=win)
    if np.ndim(w):
        got, ef, _ = simt_emu.run(p, d["ref"], d["qer"], 0, P, wpair=w[:n], **kw)
    else:
        got, ef, _ = simt_emu.run(p, d["ref"], d["qer"], int(w), P, **kw)
    assert ef == 0
    e, g = outputs(d["expected"][:n]), outputs(got)
    bad = np.nonzero((e != g).any(1))[0]
    assert bad.size == 0, f"G={G} win={win}: pair {bad[0]}: emu {g[bad[0]].tolist()} ref {e[bad[0]].tolist()}"


@pytest.mark.parametrize("G", [4, 8, 32])
def test_emulated_group_ring_wraps_on_long_queries(G):
    from tal_bsw import synth
    b = synth.generate(synth.C2, 32)
    P = synth.C2.params()
    for w, win in ((100, 256), (20, 64)):
        exp = oracle.vector(b.pairs, b.ref, b.qer, w, P, bits=16, lanes=1)
        got, ef, _ = simt_emu.run(b.pairs, b.ref, b.qer, w, P, bits=16, K=4, G=G, warps=2, win=win)
        assert ef == 0
        e, g = outputs(exp), outputs(got)
        bad = np.nonzero((e != g).any(1))[0]
        assert bad.size == 0, f"G={G} w={w} win={win}: pair {bad[0]}: emu {g[bad[0]].tolist()} oracle {e[bad[0]].tolist()}"


@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLDEN, "sw", "*.npz"))), ids=os.path.basename)
def test_emulated_sw_kernel_matches_golden(f):
    """The unbanded Smith-Waterman wavefront kernel (one warp per pair, rows
    in bands of 32, shuffles between rows) against the reference's scores."""
    d = np.load(f)
    P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
    n = min(d["inputs"].shape[0], 12)
    bits = int(d["bits"])
    for packed in ((False, True) if bits != 32 else (False,)):
        got, flags, _ = simt_emu.run_sw(d["inputs"][:n], d["seqbuf"], int(d["stride"]), P,
                                        bits=bits, warps=2, packed=packed)
        assert flags == 0
        assert (got["score"] == d["expected"]["score"][:n]).all(), \
            (packed, got["score"].tolist(), d["expected"]["score"][:n].tolist())


@pytest.mark.parametrize("bits,params", [
    (16, dict(match=2, mismatch=-3, open=-5, extend=-1)),
    (16, dict(match=300, mismatch=-32000, open=-30000, extend=-2768)),
    (16, dict(match=300, mismatch=-32468, open=-32000, extend=-768)),
    (8, dict(match=1, mismatch=-128, open=-100, extend=-28)),
])
def test_emulated_sw_two_pairs_per_warp_ragged(bits, params):
    """Two pairs per warp in 16x2 lanes: neighbouring pairs of very different
    lengths (empty ones too), an odd pair count, byte codes over the whole
    0..255 range and weights at the element type's limits, against the
    oracle; the 32-bit-lane kernel gives the same scores."""
    from tal_bsw import swdata
    rng = np.random.default_rng(7 + bits)
    n = 13
    hi = {8: 60, 16: 100}[bits]
    b = swdata.generate(n, 0, hi, bits=bits, seed=bits)
    b.seqbuf[:] = rng.integers(0, 256, b.seqbuf.size, dtype=np.uint8)
    b.pairs["len1"] = rng.integers(0, hi + 1, n)
    b.pairs["len2"] = rng.integers(0, hi + 1, n)
    b.pairs["len1"][[0, 5]] = 0
    b.pairs["len2"][[3, 8]] = 0
    # seq2 a mutated copy of seq1 for pairs with high scores
    for k in range(0, n, 2):
        s = b.seqbuf.reshape(2 * n, -1)
        s[2 * k + 1] = s[2 * k]
        s[2 * k + 1, ::7] ^= 1
    exp = oracle.sw(b.pairs, b.seqbuf, b.stride, params)
    # the library's work order: longer sequence first, in buckets of 8
    key = np.maximum(b.pairs["len1"], b.pairs["len2"]) >> 3
    for packed in (True, False):
        for order in (None, np.argsort(-key, kind="stable").astype(np.int32)):
            got, flags, _ = simt_emu.run_sw(b.pairs, b.seqbuf, b.stride, params, bits=bits, warps=2,
                                            packed=packed, order=order)
            assert flags == 0
            assert (got["score"] == exp["score"]).all(), (packed, got["score"].tolist(), exp["score"].tolist())


def test_emulated_sw_two_pairs_per_warp_bad_pair():
    """A pair outside the precision's range sits beside a good one in the
    same warp: it raises the domain flag with its index, and its neighbour
    is still scored."""
    from tal_bsw import swdata
    b = swdata.generate(6, 20, 40, bits=8, seed=3)
    P = dict(match=1, mismatch=-1, open=-2, extend=-1)
    b.pairs["len1"][3] = 100   # (min length + 1) * match above int8 is fine only below 127
    b.pairs["len2"][3] = 130   # past the 8-bit kernel's longest sequence
    exp = oracle.sw(b.pairs[[0, 1, 2, 4, 5]], b.seqbuf, b.stride, P)
    got, flags, bad = simt_emu.run_sw(b.pairs, b.seqbuf, b.stride, P, bits=8, warps=2, packed=True,
                                      order=np.array([5, 3, 0, 1, 2, 4], np.int32))
    assert flags != 0 and bad == 3
    assert (got["score"][[0, 1, 2, 4, 5]] == exp["score"]).all()


@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLDEN, "chain", "*.npz"))), ids=os.path.basename)
def test_emulated_chain_kernel_matches_golden(f):
    """The anchor chaining kernel (one warp per read, lanes over the
    predecessors, two warp reductions per anchor) against the reference's
    outputs; reads cut to keep the emulation short."""
    d = np.load(f)
    P = [float(x) for x in d["params"]]
    offs = d["offsets"]
    keep = min(offs.shape[0] - 1, 6)
    end = int(offs[keep])
    # at most 600 anchors per read: the first anchors of a read do not depend on later ones
    a_parts, o_new, idx = [], [0], []
    for k in range(keep):
        lo, hi = int(offs[k]), int(min(offs[k + 1], offs[k] + 600))
        idx.extend(range(lo, hi))
        o_new.append(o_new[-1] + hi - lo)
    idx = np.array(idx, np.int64)
    anchors = d["anchors"][idx]
    offsets = np.array(o_new, np.int64)
    # the cut changes avg_l, so the expectation is the oracle's on the cut reads,
    # itself pinned to the reference on the full fixtures
    ef, ep, ev = oracle.chain(anchors, offsets, int(P[2]), int(P[4]), int(d["dr"]), int(d["dq"]))
    gf, gp, gv, flags, _, evals = simt_emu.run_chain(anchors, offsets, int(P[2]), int(P[4]),
                                                     int(d["dr"]), int(d["dq"]), warps=2)
    assert flags == 0
    assert (gf == ef).all() and (gp == ep).all() and (gv == ev).all()
    assert end >= 0 and evals > 0


def test_emulated_chain_kernel_full_fixture_short_reads():
    """Whole fixture (no cut) where it is small: the reference's own outputs."""
    d = np.load(os.path.join(GOLDEN, "chain", "short_reads.npz"))
    P = [float(x) for x in d["params"]]
    gf, gp, gv, flags, _, _ = simt_emu.run_chain(d["anchors"], d["offsets"], int(P[2]), int(P[4]),
                                                 int(d["dr"]), int(d["dq"]), warps=2)
    assert flags == 0
    assert (gf == d["f"]).all() and (gp == d["p"]).all() and (gv == d["v"]).all()


def test_emulated_chain_kernel_rejects_negative_length():
    from tal_bsw import chaindata
    a = np.zeros(5, chaindata.ANCHOR_DTYPE)
    a["r"] = np.arange(5) * 10
    a["q"] = np.arange(5) * 10
    a["l"] = [15, 15, -1, 15, 15]
    offs = np.array([0, 2, 5], np.int64)
    gf, gp, gv, flags, bad, _ = simt_emu.run_chain(a, offs, 500, 5000, 5000, 5000)
    assert flags != 0 and bad == 1
    assert gf[:2].tolist() == [15, 25]


def test_emulated_chain_kernel_windows_past_the_ring():
    """Dense anchors (one per base or two): predecessor windows of over a
    thousand anchors, so part of each window comes from global memory instead
    of the warp's shared-memory ring of the newest 1,024."""
    from tal_bsw import chaindata
    b = chaindata.generate(2, 2600, 2800, seed=21, spacing=2, noise=0.0, repeat=0.0)
    n0 = int(b.offsets[1] - b.offsets[0])
    P = chaindata.DRIVER_PARAMS
    ef, ep, ev = oracle.chain(b.anchors, b.offsets, P[2], P[4], 5000, 5000)
    gf, gp, gv, flags, _, evals = simt_emu.run_chain(b.anchors, b.offsets, P[2], P[4], 5000, 5000, warps=2)
    assert flags == 0 and n0 > 2000
    assert evals > 1100 * n0  # windows wider than the ring
    assert (gf == ef).all() and (gp == ep).all() and (gv == ev).all()


@pytest.mark.parametrize("win", [224, 96, 320])
def test_emulated_lane_kernel_exact_rings(win):
    """Lane-kernel rings of any multiple of 32 columns (column j in slot j mod
    W by a multiply-high; the group loop's slot advances by four and wraps),
    e.g. the plain launch's 224 columns for band 100, against the oracle."""
    from tal_bsw import synth
    b = synth.generate(synth.C2, 48)
    P = synth.C2.params()
    w = (win - 12) // 2
    exp = oracle.vector(b.pairs, b.ref, b.qer, w, P, bits=16, lanes=1)
    got, ef, _ = simt_emu.run(b.pairs, b.ref, b.qer, w, P, bits=16, K=4, G=1, warps=1, win=win)
    assert ef == 0
    e, g = outputs(exp), outputs(got)
    bad = np.nonzero((e != g).any(1))[0]
    assert bad.size == 0, f"win={win}: pair {bad[0]}: emu {g[bad[0]].tolist()} oracle {e[bad[0]].tolist()}"


GROUPED_FILES = [f for f in ALL_FILES if "c4" not in f and "c3" not in f and "c1_151" not in f]


@pytest.mark.parametrize("f", GROUPED_FILES, ids=os.path.basename)
def test_emulated_group_kernel_matches_golden(f):
    """The grouped kernel (one warp per SIMD group of the reference, the
    group's shared band, wrapping int16 / int8 values) gives the reference's
    outputs, including on the fixtures where the grouping changes them."""
    d = np.load(f)
    P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
    bits = int(d["bits"])
    lanes = 64 if bits == 8 else 32
    n = d["inputs"].shape[0] if "coupled" in f else min(d["inputs"].shape[0], 3 * lanes + 5)
    p = d["inputs"][:n]
    got, ef, _ = simt_emu.run_group(p, d["ref"], d["qer"], int(d["w"]), P, bits=bits, warps=2)
    assert ef == 0
    # a cut fixture's last group is partial: the reference's own outputs for it
    exp = d["expected"][:n] if n == d["inputs"].shape[0] else oracle.vector(p, d["ref"], d["qer"], int(d["w"]), P, bits=bits)
    e, g = outputs(exp), outputs(got)
    bad = np.nonzero((e != g).any(1))[0]
    assert bad.size == 0, f"pair {bad[0]}: emu {g[bad[0]].tolist()} ref {e[bad[0]].tolist()}"


@pytest.mark.parametrize("f", GROUPED_FILES, ids=os.path.basename)
def test_emulated_wide_group_kernel_matches_golden(f):
    """The block-wide grouped kernel (bsw_group_wide.cuh: four warps share a
    group's columns, E carried across their chunks) gives the reference's
    outputs, with the group's rows in shared memory and, on a few fixtures,
    in the global slot."""
    d = np.load(f)
    P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
    bits = int(d["bits"])
    lanes = 64 if bits == 8 else 32
    n = d["inputs"].shape[0] if "coupled" in f else min(d["inputs"].shape[0], 3 * lanes + 5)
    p = d["inputs"][:n]
    exp = d["expected"][:n] if n == d["inputs"].shape[0] else oracle.vector(p, d["ref"], d["qer"], int(d["w"]), P, bits=bits)
    name = os.path.basename(f)
    for rows in ((1 << 20, 0) if name in ("coupled16_band_4.npz", "wrap8_gap_open_130_band_5.npz",
                                         "edge16_band_3.npz") else (1 << 20,)):
        got, ef, _, _ = simt_emu.run_group_wide(p, d["ref"], d["qer"], int(d["w"]), P, bits=bits, smem_rows=rows)
        assert ef == 0
        e, g = outputs(exp), outputs(got)
        bad = np.nonzero((e != g).any(1))[0]
        assert bad.size == 0, f"rows {rows}: pair {bad[0]}: emu {g[bad[0]].tolist()} ref {e[bad[0]].tolist()}"


@pytest.mark.parametrize("f", COUPLED + [os.path.join(GOLDEN, "wrap8_gap_open_130_band_5.npz"),
                                         os.path.join(GOLDEN, "edge16_zdrop_1.npz")], ids=os.path.basename)
def test_emulated_wide_group_kernel_member_mode(f):
    """Member mode (the regroup pass): groups given as member lists with the
    lanes whose outputs are wanted; those lanes get the reference's outputs
    (the group stops once they have exited), every other pair is untouched."""
    d = np.load(f)
    P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
    bits = int(d["bits"])
    lanes = 64 if bits == 8 else 32
    p = d["inputs"][:3 * lanes + 7]
    n = p.shape[0]
    w = int(d["w"])
    exp = oracle.vector(p, d["ref"], d["qer"], w, P, bits=bits)
    rng = np.random.default_rng(7)
    groups, wanted = [], np.zeros(n, bool)
    for g in range(0, n, lanes):
        members = list(range(g, min(g + lanes, n)))
        k = len(members)
        mask = 0
        for l in rng.choice(k, size=min(k, 1 + g // lanes), replace=False):
            mask |= 1 << int(l)
            wanted[g + int(l)] = True
        groups.append((members + [-1] * (lanes - k), mask))
    got, ef, _, _ = simt_emu.run_group_wide(p, d["ref"], d["qer"], w, P, bits=bits, groups=groups[::-1])
    assert ef == 0
    assert (outputs(got)[wanted] == outputs(exp)[wanted]).all()
    assert (outputs(got)[~wanted] == outputs(p)[~wanted]).all()


@pytest.mark.parametrize("f", COUPLED, ids=os.path.basename)
def test_emulated_lane_kernel_on_coupled_fixtures_scores_pairs_alone(f):
    """On the fixtures where the grouping matters, the per-pair lane kernel
    gives each pair's outputs alone in its group (the oracle at one lane)."""
    d = np.load(f)
    P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
    bits = int(d["bits"])
    p = d["inputs"][:96]
    w = int(d["w"])
    got, ef, _ = simt_emu.run(p, d["ref"], d["qer"], w, P, bits=bits, K=4, G=1, warps=2,
                              win=simt_emu.window_for(w))
    assert ef == 0
    alone = oracle.vector(p, d["ref"], d["qer"], w, P, bits=bits, lanes=1)
    assert (outputs(got) == outputs(alone)).all()


def _detector_cases():
    from test_coupling_detector import _adversarial
    cases = []
    for seed in range(6):
        p, ref, qer, w, P, bits = _adversarial(9100 + seed)
        if p.shape[0]:
            cases.append((f"adv{seed}", p[:90], ref, qer, w, P, bits))
    for f in COUPLED + [os.path.join(GOLDEN, n) for n in ("wl_c2_16bit.npz", "edge16_band_3.npz",
                                                            "edge8_band_17.npz", "edge16_zdrop_1.npz")]:
        d = np.load(f)
        P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
        cases.append((os.path.basename(f), d["inputs"][:90], d["ref"], d["qer"], int(d["w"]), P,
                      int(d["bits"])))
    return cases


@pytest.mark.parametrize("G,K,ring", [(1, 4, False), (1, 4, True), (8, 4, False), (8, 4, True), (32, 2, False)])
@pytest.mark.parametrize("case", _detector_cases(), ids=lambda c: c[0])
def test_emulated_detector_flags_equal_oracle(case, G, K, ring):
    """The kernels' group-coupling detector (bsw_couple.cuh inside the lane
    and G-lane kernels) flags exactly the pairs its CPU restatement flags,
    and scores every other pair as the oracle does alone."""
    name, p, ref, qer, w, P, bits = case
    win = 0
    if ring:  # row rings as the launches size them: a multiple of 32 (lane) / a power of two
        win = (2 * w + 12 + 31) & ~31 if G == 1 else 1 << max(6, (2 * w + 11).bit_length())
        if win >= int(p["len2"].max()) + 4:
            pytest.skip("whole rows are smaller than the ring")
    got, ef, idx = simt_emu.run_detect(p, ref, qer, w, P, bits=bits, K=K, G=G, warps=2, win=win)
    assert ef == 0
    one, flags = oracle.detect(p, ref, qer, w, P, bits=bits)
    want = np.nonzero(flags)[0]
    assert idx.tolist() == want.tolist()
    keep = np.setdiff1d(np.arange(p.shape[0]), want)
    assert (outputs(got)[keep] == outputs(one)[keep]).all()
