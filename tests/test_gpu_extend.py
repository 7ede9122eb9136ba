"""Caller-side seed extension on the GPU (left batch, right batch with h0 from
the left results, regions) against the layer's restatement (oracle.extend),
whose BSW calls are the pinned oracle; refusals."""
import numpy as np
import pytest

import oracle
import tal_bsw
from tal_bsw import seeddata
from tal_bsw.extend import extend_seeds

pytestmark = pytest.mark.gpu

P = dict(o_del=6, e_del=1, o_ins=6, e_ins=1, zdrop=100, end_bonus=5, a=1, b=4)


def _bsw():
    return tal_bsw.BandedPairWiseSW(P["o_del"], P["e_del"], P["o_ins"], P["e_ins"], P["zdrop"],
                                    P["end_bonus"], None, P["a"], P["b"], 1, device=0)


@pytest.mark.parametrize("seed,w,clip,tries", [(1, 100, 5, 1), (2, 20, 0, 1), (3, 50, 100, 1),
                                                (5, 100, 5, 2), (6, 4, 5, 4)])
def test_gpu_extension_matches_the_restatement(seed, w, clip, tries):
    b = seeddata.generate(1500, len_lo=60, len_hi=300, junk=0.2, indel=0.02 if w < 10 else 0.004,
                          seed=seed)
    exp = oracle.extend(b.ref, b.reads, b.read_off, b.seeds, P, w, clip, clip, band_tries=tries)
    with _bsw() as bsw:
        got = extend_seeds(bsw, b.ref, b.reads, b.read_off, b.seeds, w, clip, clip, band_tries=tries)
    for f in ("rb", "re", "qb", "qe", "score", "left_score"):
        bad = np.nonzero(got[f] != exp[f])[0]
        assert bad.size == 0, f"{f}: {bad.size} differ, first seed {bad[0]}: gpu {got[bad[0]]} oracle {exp[bad[0]]}"


def test_gpu_extension_refusals():
    b = seeddata.generate(20, seed=4)
    with _bsw() as bsw:
        sd = b.seeds.copy()
        sd["qbeg"][5] = 10_000          # outside its read
        with pytest.raises(tal_bsw.TalBswError) as ei:
            extend_seeds(bsw, b.ref, b.reads, b.read_off, sd)
        assert ei.value.status == tal_bsw.api.TAL_EDOMAIN and ei.value.bad_pair == 5
        sd = b.seeds.copy()
        sd["read"][2] = b.n_reads       # no such read
        with pytest.raises(tal_bsw.TalBswError) as ei:
            extend_seeds(bsw, b.ref, b.reads, b.read_off, sd)
        assert ei.value.bad_pair == 2
        out = extend_seeds(bsw, b.ref, b.reads, b.read_off, b.seeds[:0])
        assert out.shape == (0,)
        for tries in (-1, 9):
            with pytest.raises(tal_bsw.TalBswError) as ei:
                extend_seeds(bsw, b.ref, b.reads, b.read_off, b.seeds, band_tries=tries)
            assert ei.value.status == tal_bsw.api.TAL_EINVAL
