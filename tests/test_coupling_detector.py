"""The group-coupling detector the per-pair kernels run (its CPU restatement,
oracle.detect): a pair is flagged unless its outputs provably equal its
outputs in any SIMD group of the reference.  Soundness: on seeded adversarial
batches -- narrow bands, seeds longer than the rest of the read, z-drop 0-40,
odd gap and score weights, both precisions -- every pair whose grouped
outputs (the reference's 32 / 64 consecutive pairs, oracle.vector) differ from
its outputs alone is flagged, and so is every such pair of the reference's
own coupled fixtures.  Precision: the benchmark workloads flag almost
nothing, so the exact path costs them little."""
import glob
import os

import numpy as np
import pytest

import oracle
from tal_bsw import synth
from tal_bsw.seqpair import outputs

from _cases import DEFAULT, extension_pairs, mutate, pack

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _adversarial(seed):
    rng = np.random.default_rng(seed)
    P = dict(DEFAULT)
    if rng.random() < 0.6:
        P.update(o_del=int(rng.integers(0, 12)), o_ins=int(rng.integers(0, 12)),
                 e_del=int(rng.integers(1, 4)), e_ins=int(rng.integers(1, 4)),
                 zdrop=int(rng.choice([0, 1, 5, 20, 40, 100])), end_bonus=int(rng.choice([0, 5, 40])),
                 a=int(rng.choice([1, 1, 2])), b=int(rng.integers(1, 7)))
    bits = 16 if rng.random() < 0.7 else 8
    w = int(rng.choice([0, 1, 2, 3, 4, 5, 6, 8, 10, 12, 16, 20, 24, 32, 50, 100]))
    if rng.random() < 0.35 and bits == 16:
        p, ref, qer = extension_pairs(int(rng.integers(150, 400)), w, int(rng.integers(20, 80)),
                                      int(rng.integers(100, 300)), int(rng.integers(1, 10**6)), P)
        return p, ref, qer, w, P, bits
    n = int(rng.integers(400, 1500))
    lmax = 127 if bits == 8 else 300
    refs, qers, h0s = [], [], []
    for _ in range(n):
        l2 = int(rng.integers(0, lmax + 1)) if rng.random() < 0.3 else int(rng.integers(1, min(lmax, 80) + 1))
        q = rng.integers(0, 4, l2).astype(np.uint8)
        if rng.random() < 0.1:
            q[rng.random(l2) < 0.2] = 4
        if rng.random() < 0.5:
            r = mutate(rng, q, float(rng.choice([0.0, 0.02, 0.05, 0.15])))
            if rng.random() < 0.5:
                cut = int(rng.integers(0, l2 + 1))
                r = np.concatenate([r[:cut], rng.integers(0, 4, l2 - cut).astype(np.uint8)])
            r = np.concatenate([r, rng.integers(0, 4, int(rng.integers(0, 40))).astype(np.uint8)])
            r = r[: max(0, l2 + int(rng.integers(-20, 40)))]
        else:
            r = rng.integers(0, 4, int(rng.integers(0, lmax + 1))).astype(np.uint8)
        refs.append(r[:lmax])
        qers.append(q)
        h0s.append(int(rng.integers(0, 250)) if bits == 16 else int(rng.integers(0, 60)))
    p, ref, qer = pack(refs, qers, h0s)
    if bits == 8:
        p = p[oracle.eligible8(p, w, P)]
    return p, ref, qer, w, P, bits


def _check(p, ref, qer, w, P, bits):
    grp = oracle.vector(p, ref, qer, w, P, bits=bits)
    one, flags = oracle.detect(p, ref, qer, w, P, bits=bits)
    alone = oracle.vector(p, ref, qer, w, P, bits=bits, lanes=1)
    assert (outputs(one) == outputs(alone)).all(), "detector's own scoring differs from the oracle alone"
    coupled = (outputs(grp) != outputs(one)).any(1)
    missed = np.nonzero(coupled & (flags == 0))[0]
    assert missed.size == 0, f"{missed.size} coupled pairs not flagged, first {missed[:5]}"
    return int(coupled.sum()), int((flags != 0).sum())


@pytest.mark.parametrize("seed", list(range(24)))
def test_detector_flags_every_coupled_pair(seed):
    p, ref, qer, w, P, bits = _adversarial(9000 + seed)
    if p.shape[0] == 0:
        pytest.skip("no pair in range")
    _check(p, ref, qer, w, P, bits)


def test_detector_sees_coupling():
    """The adversarial sets do hold coupled pairs (so the test has teeth)."""
    total = 0
    for seed in range(24):
        p, ref, qer, w, P, bits = _adversarial(9000 + seed)
        if p.shape[0]:
            total += _check(p, ref, qer, w, P, bits)[0]
    assert total >= 20


@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLDEN, "coupled*.npz"))), ids=os.path.basename)
def test_detector_flags_reference_coupled_fixtures(f):
    d = np.load(f)
    P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
    one, flags = oracle.detect(d["inputs"], d["ref"], d["qer"], int(d["w"]), P, bits=int(d["bits"]))
    coupled = (outputs(one) != outputs(d["expected"])).any(1)
    assert coupled.any()
    assert (flags[coupled] != 0).all()


@pytest.mark.parametrize("name", ["c1_151bp", "c1_8bit", "c2_16bit", "c3_mixed", "c4_long"])
def test_detector_rarely_flags_workloads(name):
    wl = synth.WORKLOADS[name]
    b = synth.generate(wl, 3000 if name != "c4_long" else 150)
    P = wl.params()
    warr = b.w if wl.w_choices else np.full(b.pairs.shape[0], wl.w)
    is8 = (np.ones(warr.shape, bool) if wl.bits == 8 else np.zeros(warr.shape, bool) if wl.bits == 16
           else oracle.eligible8(b.pairs, warr, P))
    nflag = 0
    for wv in np.unique(warr):
        for bits in (8, 16):
            sel = np.nonzero((warr == wv) & (is8 == (bits == 8)))[0]
            if sel.size:
                nflag += _check(b.pairs[sel], b.ref, b.qer, int(wv), P, bits)[1]
    assert nflag <= max(2, b.pairs.shape[0] // 500)
