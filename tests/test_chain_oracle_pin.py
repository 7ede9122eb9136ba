"""The chaining oracle (oracle/chain_oracle.cpp) against the reference's own
dp_chain::mm_dp_vectorized: the golden fixtures made from its AVX-512 build
(tests/golden/chain/), and, where the reference builds on this host, fresh
seeded inputs scored by it directly."""
import glob
import os

import numpy as np
import pytest

import oracle
from tal_bsw import chaindata

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "chain", "*.npz")))


def _params(d):
    P = [float(x) for x in d["params"]]
    return tuple(int(x) if k != 5 else x for k, x in enumerate(P))


def test_fixtures_present():
    names = {os.path.basename(f)[:-4] for f in GOLDEN}
    assert {"driver_like", "short_reads", "unsorted_contigs", "ties", "rounding_paths",
            "jitter_maxiter20_bw50"} <= names


@pytest.mark.parametrize("f", GOLDEN, ids=os.path.basename)
def test_oracle_matches_reference_fixture(f):
    d = np.load(f)
    P = _params(d)
    got_f, got_p, got_v = oracle.chain(d["anchors"], d["offsets"], P[2], P[4], int(d["dr"]),
                                       int(d["dq"]), nthreads=4)
    for name, g, e in (("f", got_f, d["f"]), ("p", got_p, d["p"]), ("v", got_v, d["v"])):
        bad = np.nonzero(g != e)[0]
        assert bad.size == 0, f"{name}: {bad.size} differ, first at {bad[0]}: {g[bad[0]]} vs {e[bad[0]]}"


def test_rounding_fixture_exercises_both_gap_paths():
    """The rounding fixture holds predecessors scored in the scalar loop (at
    most six) and in the vector loop at distances where the float and double
    gap costs differ, so a wrong path choice fails the fixture test."""
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "chain", "rounding_paths.npz"))
    a, offs = d["anchors"], d["offsets"]
    avg = np.float32(105.0)
    aq = np.float32(0.01 * float(avg))
    hits = {"scalar": 0, "vector": 0}
    for k in range(offs.shape[0] - 1):
        r = a["r"][offs[k]:offs[k + 1]].astype(np.int64)
        q = a["q"][offs[k]:offs[k + 1]].astype(np.int64)
        for i in range(r.shape[0]):
            for j in range(i):
                dd = abs((r[i] - r[j]) - (q[i] - q[j]))
                if dd == 0 or dd > 500 or r[i] == r[j] or not 0 < q[i] - q[j] <= 5000:
                    continue
                fl = np.floor(np.float32(dd) * aq)
                db = np.trunc(dd * 0.01 * float(avg))
                if fl != db:
                    hits["scalar" if i <= 6 else "vector"] += 1
    assert hits["scalar"] > 0 and hits["vector"] > 0, hits


@pytest.mark.skipif(not oracle.chain_ref_available("avx512"), reason="reference build absent")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_matches_reference_fresh(seed):
    rng = np.random.default_rng(seed)
    b = chaindata.generate(30, 100, 4000, seed=100 + seed, l_jitter=int(rng.integers(0, 120)),
                           spacing=int(rng.integers(3, 15)))
    P = list(chaindata.DRIVER_PARAMS)
    P[2] = int(rng.integers(20, 600))
    P[4] = int(rng.integers(5, 5000))
    dr, dq = int(rng.integers(500, 6000)), int(rng.integers(500, 6000))
    ef, ep, ev = oracle.chain_reference(b.anchors, b.offsets, tuple(P), dr, dq)
    gf, gp, gv = oracle.chain(b.anchors, b.offsets, P[2], P[4], dr, dq, nthreads=4)
    assert (gf == ef).all() and (gp == ep).all() and (gv == ev).all()


def test_oracle_edge_cases():
    """An empty read, one anchor, a negative-free chain of equal anchors."""
    D = chaindata.ANCHOR_DTYPE
    a = np.zeros(4, D)
    a["r"] = [10, 20, 30, 40]
    a["q"] = [10, 20, 30, 40]
    a["l"] = 15
    offs = np.array([0, 0, 1, 4], np.int64)
    f, p, v = oracle.chain(a, offs, 500, 5000, 5000, 5000)
    assert f[0] == 15 and p[0] == -1
    # anchors 1..3 of the last read: each extends the previous by min(10, 10, 15) = 10
    assert f[1:].tolist() == [15, 25, 35] and p[1:].tolist() == [-1, 0, 1]  # p: index in its read
    assert v[1:].tolist() == [15, 25, 35]
