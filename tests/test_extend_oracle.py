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
