"""The batched form (device-side length binning, per-bin autotuned kernels,
CUDA graph) against the oracle and against the plain form on the same pairs."""
import numpy as np
import pytest

import oracle
import tal_bsw
from tal_bsw import synth
from tal_bsw.seqpair import outputs

pytestmark = pytest.mark.gpu


def _bsw(P):
    return tal_bsw.BandedPairWiseSW(P["o_del"], P["e_del"], P["o_ins"], P["e_ins"], P["zdrop"],
                                    P["end_bonus"], None, P["a"], P["b"], 1, device=0)


def _same(exp, got, what):
    e, g = outputs(exp), outputs(got)
    bad = np.nonzero((e != g).any(axis=1))[0]
    assert bad.size == 0, (f"{what}: {bad.size}/{len(e)} differ; first #{bad[0]}: "
                           f"gpu {g[bad[0]].tolist()} oracle {e[bad[0]].tolist()}")


def test_batched_mixed_workload_matches_oracle():
    wl = synth.C3
    b = synth.generate(wl, 6000)
    P = wl.params()
    exp = oracle.routed(b.pairs, b.ref, b.qer, b.w, P, bits=0, nthreads=4)
    got = b.pairs.copy()
    with _bsw(P) as bsw:
        bsw.scores_batched(got, b.ref, b.qer, b.n, 100, wpair=b.w, bits=tal_bsw.AUTO)
        _same(exp, got, "batched c3")
        again = b.pairs.copy()
        bsw.scores_batched(again, b.ref, b.qer, b.n, 100, wpair=b.w, bits=tal_bsw.AUTO)
        _same(exp, again, "batched c3, second call (graph replay)")
        cfgs = [bsw.bin_config(k) for k in range(21)]
    assert all(g in (1, 4, 8, 16, 32) for g, _, _ in cfgs)


@pytest.mark.parametrize("name", ["c2_16bit", "c1_8bit", "c4_long"])
def test_batched_equals_plain(name):
    wl = synth.WORKLOADS[name]
    b = synth.generate(wl, 40 if name == "c4_long" else 3000)
    P = wl.params()
    bits = 8 if wl.bits == 8 else 16
    plain = b.pairs.copy()
    batched = b.pairs.copy()
    with _bsw(P) as bsw:
        bsw._scores(plain, b.ref, b.qer, b.n, wl.w, bits)
        bsw.scores_batched(batched, b.ref, b.qer, b.n, wl.w, bits=bits)
    _same(plain, batched, name)


def test_batched_golden_edges():
    """Edge-case fixtures the reference produced, through the batched form."""
    import glob
    import os
    for f in sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "edge16_*.npz"))):
        d = np.load(f)
        P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
        got = d["inputs"].copy()
        with _bsw(P) as bsw:
            bsw.scores_batched(got, d["ref"], d["qer"], got.shape[0], int(d["w"]), bits=16)
        _same(d["expected"], got, os.path.basename(f))


@pytest.mark.parametrize("field,k", [("len2", 0), ("idr", 777), ("len1", 1998)])
def test_batched_host_call_refuses_negative_lengths_and_offsets(field, k):
    """The host call reduces its sequence extents on the device and refuses a
    pair with a negative length or offset: TAL_EDOMAIN naming the first such
    pair; the same handle then scores a good batch."""
    wl = synth.C3
    b = synth.generate(wl, 2000)
    P = wl.params()
    bad = b.pairs.copy()
    bad[field][k] = -3
    bad["idq"][k + 1] = -1  # a later one: the first is reported
    with _bsw(P) as bsw:
        with pytest.raises(tal_bsw.TalBswError) as ei:
            bsw.scores_batched(bad, b.ref, b.qer, b.n, 100, wpair=b.w, bits=tal_bsw.AUTO)
        assert ei.value.status == tal_bsw.api.TAL_EDOMAIN and ei.value.bad_pair == k
        got = b.pairs.copy()
        bsw.scores_batched(got, b.ref, b.qer, b.n, 100, wpair=b.w, bits=tal_bsw.AUTO)
    exp = oracle.routed(b.pairs, b.ref, b.qer, b.w, P, bits=0, nthreads=4)
    _same(exp, got, "batched c3 after a refusal")
