"""Seeded pair sets shared by the CPU and GPU tests: the workload shapes at
test sizes, and edge cases of the kinds the reference's code paths branch on
(empty and one-base sequences, N-rich input, h0 at the range limits, z-drop
firing mid-band, end_bonus moving the band, zero rows, narrow bands, the 8-bit
envelope edges, gap extension != 1)."""
import numpy as np

from tal_bsw import synth
from tal_bsw.seqpair import new_pairs

DEFAULT = dict(o_del=6, e_del=1, o_ins=6, e_ins=1, zdrop=100, end_bonus=5, a=1, b=4)


def pack(seqs_ref, seqs_qer, h0s, slack=64):
    n = len(seqs_ref)
    p = new_pairs(n)
    l1 = np.array([len(s) for s in seqs_ref], np.int64)
    l2 = np.array([len(s) for s in seqs_qer], np.int64)
    ro = np.concatenate([[0], np.cumsum(l1)[:-1]]) if n else np.zeros(0, np.int64)
    qo = np.concatenate([[0], np.cumsum(l2)[:-1]]) if n else np.zeros(0, np.int64)
    p["len1"], p["len2"], p["h0"] = l1, l2, np.asarray(h0s, np.int64)
    p["idr"], p["idq"] = ro, qo
    p["id"] = np.arange(n)
    ref = np.concatenate([np.asarray(s, np.uint8) for s in seqs_ref] + [np.zeros(slack, np.uint8)])
    qer = np.concatenate([np.asarray(s, np.uint8) for s in seqs_qer] + [np.zeros(slack, np.uint8)])
    return p, ref, qer


def mutate(rng, q, div, nrate=0.0):
    r = q.copy()
    m = rng.random(len(r)) < div
    r[m] = rng.integers(0, 4, int(m.sum()))
    if nrate:
        r[rng.random(len(r)) < nrate] = 4
    return r


def edge_cases(seed=7, bits=16):
    """(name, pairs, ref, qer, w, params) tuples."""
    rng = np.random.default_rng(seed)
    lmax = 127 if bits == 8 else 400
    out = []

    def add(name, refs, qers, h0s, w=100, **kw):
        P = dict(DEFAULT)
        P.update(kw)
        p, r, q = pack(refs, qers, h0s)
        out.append((name, p, r, q, w, P))

    # empty and one-base sequences
    refs, qers, h0s = [], [], []
    for l1 in (0, 1, 2):
        for l2 in (0, 1, 2):
            for h0 in (0, 1, 7, 30):
                refs.append(rng.integers(0, 4, l1)); qers.append(rng.integers(0, 4, l2)); h0s.append(h0)
    add("tiny", refs, qers, h0s)
    # N-rich sequences
    refs, qers, h0s = [], [], []
    for _ in range(64):
        l2 = int(rng.integers(1, min(lmax, 120)))
        q = rng.integers(0, 4, l2).astype(np.uint8)
        q[rng.random(l2) < 0.3] = 4
        r = mutate(rng, q, 0.05, nrate=0.2)[: min(lmax, l2 + int(rng.integers(0, 8)))]
        refs.append(r); qers.append(q); h0s.append(int(rng.integers(0, 40)))
    add("n_rich", refs, qers, h0s)
    # h0 at range limits (8-bit: h0 + min(len) = 127)
    refs, qers, h0s = [], [], []
    for _ in range(64):
        l2 = int(rng.integers(1, 100)); l1 = min(lmax, l2 + int(rng.integers(0, 20)))
        q = rng.integers(0, 4, l2).astype(np.uint8)
        r = np.concatenate([mutate(rng, q, 0.02), rng.integers(0, 4, max(0, l1 - l2))])[:l1]
        h0 = 127 - min(l1, l2) if bits == 8 else int(rng.choice([0, 1, 200, 1000]))
        refs.append(r); qers.append(q); h0s.append(max(h0, 0))
    add("h0_limits", refs, qers, h0s)
    # random (unrelated) sequences: zero rows early, z-drop
    refs, qers, h0s = [], [], []
    for _ in range(96):
        l1 = int(rng.integers(1, lmax)); l2 = int(rng.integers(1, lmax))
        refs.append(rng.integers(0, 4, l1)); qers.append(rng.integers(0, 4, l2)); h0s.append(int(rng.integers(0, 25)))
    add("unrelated", refs, qers, h0s)
    # similar then diverging: z-drop mid-band
    refs, qers, h0s = [], [], []
    for _ in range(96):
        l2 = int(rng.integers(30, lmax)); cut = int(rng.integers(5, l2))
        q = rng.integers(0, 4, l2).astype(np.uint8)
        r = np.concatenate([q[:cut], rng.integers(0, 4, l2 - cut)]).astype(np.uint8)[:lmax]
        refs.append(r); qers.append(q); h0s.append(int(rng.integers(5, 60)) if bits == 16 else 5)
    for zd in (0, 1, 5, 20):
        add(f"zdrop_{zd}", refs, qers, h0s, zdrop=zd)
    # narrow and tiny bands, band wider than the sequences
    refs, qers, h0s = [], [], []
    for _ in range(64):
        l2 = int(rng.integers(5, lmax)); l1 = int(rng.integers(5, lmax))
        q = rng.integers(0, 4, l2).astype(np.uint8)
        r = np.concatenate([mutate(rng, q, 0.05), rng.integers(0, 4, 200)])[:l1]
        refs.append(r); qers.append(q); h0s.append(int(rng.integers(0, 30)))
    for w in (0, 1, 3, 17, 500):
        add(f"band_{w}", refs, qers, h0s, w=w)
    # end_bonus moving the band clamp, gap extension != 1, other scores
    add("end_bonus_0", refs, qers, h0s, w=50, end_bonus=0)
    add("end_bonus_40", refs, qers, h0s, w=50, end_bonus=40)
    add("gap_e2", refs, qers, h0s, w=30, e_del=2, e_ins=2, o_del=4, o_ins=3)
    add("gap_asym", refs, qers, h0s, w=30, e_del=1, e_ins=3, o_del=9, o_ins=2)
    add("match2", refs, qers, [min(h, 10) for h in h0s], w=40, a=2, b=3) if bits == 16 else None
    return [c for c in out if c is not None]


def workload_slices(n_scale=1.0):
    """(name, Batch, bits) for every workload shape at test size."""
    sizes = {"c1_151bp": 600, "c1_8bit": 600, "c2_16bit": 600, "c3_mixed": 1200, "c4_long": 24}
    res = []
    for name, n in sizes.items():
        wl = synth.WORKLOADS[name]
        res.append((name, synth.generate(wl, max(1, int(n * n_scale))), wl.bits))
    return res


def extension_pairs(n_reads, w, len_lo, len_hi, seed, P=DEFAULT):
    """The right-extension SeqPair batch of a seed-extension call (targets:
    the reference after each seed plus the gap allowance, queries: the read
    after the seed, h0 = the seed length), in seed order: the kind of batch
    where a narrow band makes a lane's outputs depend on its SIMD group."""
    from tal_bsw import seeddata
    b = seeddata.generate(n_reads, len_lo=len_lo, len_hi=len_hi, junk=0.2, indel=0.02, seed=seed)

    def gap(n):
        d = (n * P["a"] - P["o_del"]) // P["e_del"] + 1
        i = (n * P["a"] - P["o_ins"]) // P["e_ins"] + 1
        return min(max(d, i, 1), 2 * w)

    ts, qs, h0s = [], [], []
    for sd in b.seeds:
        r = int(sd["read"])
        r0, L = int(b.read_off[r]), int(b.read_off[r + 1] - b.read_off[r])
        qe0, re0 = int(sd["qbeg"] + sd["len"]), int(sd["rbeg"] + sd["len"])
        if qe0 >= L:
            continue
        ql = L - qe0
        ts.append(b.ref[re0:min(b.ref.shape[0], re0 + ql + gap(ql))])
        qs.append(b.reads[r0 + qe0:r0 + L])
        h0s.append(int(sd["len"]) * P["a"])
    return pack(ts, qs, h0s)


def coupled_cases():
    """Pair sets, in SIMD-group order, whose reference outputs depend on the
    grouping: for each configuration, the 32- (16-bit) or 64-pair (8-bit)
    groups of an extension batch that hold a pair whose grouped outputs
    differ from its outputs alone, plus the two groups after each.  Yields
    (name, pairs, ref, qer, w, bits); the grouping to keep is consecutive
    groups from the first pair."""
    import oracle
    from tal_bsw.seqpair import outputs
    for name, bits, w, lo, hi, seed in (("coupled16_band_4", 16, 4, 60, 300, 6),
                                        ("coupled16_band_8", 16, 8, 60, 300, 1),
                                        ("coupled8_band_8", 8, 8, 40, 127, 8)):
        p, ref, qer = extension_pairs(1500, w, lo, hi, seed)
        if bits == 8:
            keep = (p["len1"] <= 127) & (p["len2"] <= 127) & (p["h0"] + np.minimum(p["len1"], p["len2"]) <= 127)
            p = p[keep]
        lanes = 64 if bits == 8 else 32
        grp = oracle.vector(p, ref, qer, w, DEFAULT, bits=bits)
        one = oracle.vector(p, ref, qer, w, DEFAULT, bits=bits, lanes=1)
        hit = np.nonzero((outputs(grp) != outputs(one)).any(1))[0] // lanes
        gs = sorted({int(g + d) for g in hit for d in (0, 1, 2) if (g + d) * lanes < p.shape[0]})
        sel = np.concatenate([np.arange(g * lanes, min((g + 1) * lanes, p.shape[0])) for g in gs])
        sub = p[sel]
        ts = [ref[int(x["idr"]):int(x["idr"]) + int(x["len1"])] for x in sub]
        qs = [qer[int(x["idq"]):int(x["idq"]) + int(x["len2"])] for x in sub]
        cp, cr, cq = pack(ts, qs, sub["h0"])
        yield name, cp, cr, cq, w, bits


def wrapping_cases():
    """8-bit pair sets with gap opens whose int8 sums wrap (o + e = 130 > 127):
    outside the per-pair kernels' exact range (TAL_EDOMAIN there), scored by
    the grouped kernel, whose values wrap as the reference's do; a third to a
    half of these pairs get other outputs in their group than alone.  70
    pairs: one full group of 64 and a partial one (the padding lanes read the
    query bytes at offset 0).  Then 16-bit pairs whose h0 is within 270 of the
    int16 limit, so their DP values wrap.  Yields (name, pairs, ref, qer, w,
    P, bits)."""
    rng = np.random.default_rng(3)
    P = dict(o_del=120, e_del=10, o_ins=120, e_ins=10, zdrop=100, end_bonus=5, a=1, b=4)
    refs, qers, h0s = [], [], []
    for _ in range(70):
        L = int(rng.integers(5, 120))
        q = rng.integers(0, 4, L).astype(np.uint8)
        r = q.copy()
        m = rng.random(L) < 0.1
        r[m] = (r[m] + 1) % 4
        refs.append(np.concatenate([r, rng.integers(0, 4, int(rng.integers(0, 8))).astype(np.uint8)]))
        qers.append(q)
        h0s.append(int(rng.integers(0, 20)))
    p, ref, qer = pack(refs, qers, h0s)
    for w in (5, 126):
        yield f"wrap8_gap_open_130_band_{w}", p, ref, qer, w, P, 8
    # 16-bit: h0 within 270 of the int16 limit, so the DP values wrap
    refs, qers, h0s = [], [], []
    for _ in range(40):
        L = int(rng.integers(50, 300))
        q = rng.integers(0, 4, L).astype(np.uint8)
        r = q.copy()
        m = rng.random(L) < 0.05
        r[m] = (r[m] + 1) % 4
        refs.append(np.concatenate([r, rng.integers(0, 4, int(rng.integers(0, 30))).astype(np.uint8)]))
        qers.append(q)
        h0s.append(int(rng.integers(32500, 32768)))
    p, ref, qer = pack(refs, qers, h0s)
    yield "wrap16_h0_near_limit_band_100", p, ref, qer, 100, DEFAULT, 16
