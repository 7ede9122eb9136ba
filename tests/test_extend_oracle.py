"""The seed-extension layer's restatement (oracle.extend, include/tal_extend.h's
specification; its BWA-MEM2 counterpart is not in the reference, so parity
for this layer is unpinned): properties any extension must have, on CPU."""
import numpy as np

import oracle
from tal_bsw import seeddata
from tal_bsw.seeddata import SEED_DTYPE

P = dict(o_del=6, e_del=1, o_ins=6, e_ins=1, zdrop=100, end_bonus=5, a=1, b=4)


def test_error_free_reads_extend_to_the_whole_read():
    rng = np.random.default_rng(1)
    ref = rng.integers(0, 4, 20000, dtype=np.uint8)
    reads, offs, seeds = [], [0], []
    for r in range(20):
        L = int(rng.integers(80, 200))
        pos = int(rng.integers(500, 19000 - L))
        reads.append(ref[pos:pos + L])
        offs.append(offs[-1] + L)
        qb = int(rng.integers(0, L - 20))
        seeds.append((r, qb, pos + qb, 20, 0))
    sd = np.array(seeds, SEED_DTYPE)
    out = oracle.extend(ref, np.concatenate(reads), np.array(offs, np.int64), sd, P, 100, 5, 5)
    L = np.diff(offs)
    assert (out["qb"] == 0).all() and (out["qe"] == L).all()
    assert (out["re"] - out["rb"] == L).all() and (out["rb"] == sd["rbeg"] - sd["qbeg"]).all()
    assert (out["score"] == L * P["a"]).all()


def test_regions_contain_their_seed_and_agree_within_a_read():
    b = seeddata.generate(200, seed=8)
    out = oracle.extend(b.ref, b.reads, b.read_off, b.seeds, P, 100, 5, 5)
    s = b.seeds
    assert (out["qb"] <= s["qbeg"]).all() and (out["qe"] >= s["qbeg"] + s["len"]).all()
    assert (out["rb"] <= s["rbeg"]).all() and (out["re"] >= s["rbeg"] + s["len"]).all()
    # reaching a read end may cost up to the clipping penalty below the local best
    assert (out["left_score"] >= s["len"] * P["a"] - 5).all()
    assert (out["score"] >= s["len"] * P["a"] - 10).all()
    # seeds of one read on the same diagonal stretch mostly find the same region
    same = 0
    for r in np.unique(s["read"]):
        k = np.nonzero(s["read"] == r)[0]
        same += len({(int(out["qb"][i]), int(out["qe"][i]), int(out["rb"][i])) for i in k}) == 1
    assert same >= 0.8 * np.unique(s["read"]).size


def test_junk_tail_is_clipped():
    rng = np.random.default_rng(4)
    ref = rng.integers(0, 4, 20000, dtype=np.uint8)
    L, pos = 150, 3000
    read = ref[pos:pos + L].copy()
    read[100:] = (read[100:] + 1) % 4            # the last 50 bases never match
    sd = np.array([(0, 10, pos + 10, 30, 0)], SEED_DTYPE)
    out = oracle.extend(ref, read, np.array([0, L], np.int64), sd, P, 100, 5, 5)
    assert out["qb"][0] == 0 and 100 <= out["qe"][0] < L


def _two_deletion_read(rng, ref, pos):
    # read = ref[pos, pos+60) ref[pos+66, pos+106) ref[pos+112, pos+202): two
    # 6-base deletions, cumulative diagonal offset 12
    return np.concatenate([ref[pos:pos + 60], ref[pos + 66:pos + 106], ref[pos + 112:pos + 202]])


def test_band_retry_follows_a_drift_past_the_band():
    rng = np.random.default_rng(9)
    ref = rng.integers(0, 4, 20000, dtype=np.uint8)
    pos = 5000
    read = _two_deletion_read(rng, ref, pos)
    L = read.shape[0]
    sd = np.array([(0, 10, pos + 10, 30, 0)], SEED_DTYPE)
    offs = np.array([0, L], np.int64)
    one = oracle.extend(ref, read, offs, sd, P, 8, 5, 5)
    two = oracle.extend(ref, read, offs, sd, P, 8, 5, 5, band_tries=2)
    wide = oracle.extend(ref, read, offs, sd, P, 16, 5, 5)
    # band 8 reaches the first deletion (offset 6 = 3/4 of its half: a retry)
    # but not the second; band 16 reaches both, as the wider band alone does
    assert two["score"][0] > one["score"][0]
    assert two["qe"][0] == L and two["re"][0] == pos + 112 + 90
    assert (two[["score", "qe", "re"]] == wide[["score", "qe", "re"]]).all()
    # one try is the default
    assert (oracle.extend(ref, read, offs, sd, P, 8, 5, 5, band_tries=1) == one).all()


def test_band_retry_bookkeeping_matches_a_per_pair_loop():
    """oracle._scored_with_tries against BWA-MEM's extension loop written
    per pair: for i in 0..tries-1: prev = score; score = extend(band w << i);
    stop when score == prev or max_off < (band >> 1) + (band >> 2)."""
    from tal_bsw.seqpair import SEQPAIR_DTYPE
    rng = np.random.default_rng(12)
    n, w, tries = 300, 4, 4
    T = rng.integers(0, 4, n * 200 + 16, dtype=np.uint8)
    Q = T.copy()
    pairs = np.zeros(n, SEQPAIR_DTYPE)
    for k in range(n):
        l1, l2 = int(rng.integers(20, 150)), int(rng.integers(20, 150))
        idr = k * 200
        # the query follows the target with a drift of -12..12 bases
        d = int(rng.integers(-12, 13))
        src = np.clip(np.arange(l2) + np.linspace(0, d, l2).astype(int), 0, l1 - 1)
        Q[idr:idr + l2] = T[idr + src]
        mut = rng.random(l2) < 0.05
        Q[idr:idr + l2][mut] = rng.integers(0, 4, int(mut.sum()))
        pairs[k]["idr"], pairs[k]["idq"], pairs[k]["id"] = idr, idr, k
        pairs[k]["len1"], pairs[k]["len2"], pairs[k]["h0"] = l1, l2, int(rng.integers(10, 40))
    for f in ("score", "tle", "gtle", "qle", "gscore", "max_off"):
        pairs[f] = -1
    got = oracle._scored_with_tries(pairs, T, Q, w, P, tries)
    retried = 0
    for k in range(n):
        score = -1
        for i in range(tries):
            prev = score
            r = oracle.routed(pairs[k:k + 1], T, Q, w << i, P)[0]
            score = int(r["score"])
            retried += i > 0
            if score == prev or r["max_off"] < ((w << i) >> 1) + ((w << i) >> 2):
                break
        assert got[k] == r, k
    assert retried > 50
