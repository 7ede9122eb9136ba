"""The unbanded Smith-Waterman oracle (oracle/sw_oracle.cpp) against the
reference's own PairWiseSW_8/_16/_32 (AVX-512BW) and scalar kernel, compiled
here from the reference sources, and against the golden fixtures they
produced.  CPU only."""
import glob
import os

import numpy as np
import pytest

import oracle
from tal_bsw import swdata

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
PARAMS = [dict(match=1, mismatch=-4, open=-6, extend=-1),
          dict(match=2, mismatch=-3, open=-5, extend=-2),
          dict(match=1, mismatch=-1, open=-1, extend=-1)]


def _edges(bits):
    """Short, empty, unequal and identical sequences, N-rich ones."""
    b = swdata.generate(24, 0, min(40, swdata.MAX_SEQ_LEN[bits]), bits=bits, seed=3)
    p = b.pairs.copy()
    p["len1"][:4] = [0, 1, 0, 5]
    p["len2"][:4] = [0, 0, 1, 5]
    s = b.seqbuf.reshape(-1, b.stride)
    s[2 * 5 + 1] = s[2 * 5]        # pair 5: identical sequences
    s[2 * 6, :40] = 4              # pair 6: N everywhere in seq1 (N matches N)
    s[2 * 6 + 1, :40] = 4
    return p, b.seqbuf, b.stride


@pytest.mark.skipif(not oracle.sw_ref_available(), reason="reference not built here")
@pytest.mark.parametrize("bits", [8, 16, 32])
@pytest.mark.parametrize("pi", range(len(PARAMS)))
def test_oracle_equals_reference(bits, pi):
    P = PARAMS[pi]
    assert oracle.sw_ref_max_len(bits) == swdata.MAX_SEQ_LEN[bits]
    hi = 100 if bits == 8 else 400
    b = swdata.generate(200, 0, hi, bits=bits, seed=11 + pi)
    if bits == 8:   # keep every score inside int8: min(len) * match < 127
        lim = 126 // P["match"] - 1
        b.pairs["len1"] = np.minimum(b.pairs["len1"], lim)
    for pairs, buf, stride in ((b.pairs, b.seqbuf, b.stride), _edges(bits)):
        exp = oracle.sw_reference(pairs, buf, P, bits=bits)
        got = oracle.sw(pairs, buf, stride, P)
        assert (exp["score"] == got["score"]).all(), (bits, P)


@pytest.mark.skipif(not oracle.sw_ref_available(), reason="reference not built here")
def test_scalar_reference_equals_vector():
    """PairWiseSW::smithWatermanOnePair (LOW_INIT start, E before H) and the
    vector kernels' initialisation give the same scores."""
    P = PARAMS[0]
    b = swdata.generate(100, 0, 300, bits=32, seed=5)
    assert (oracle.sw_reference(b.pairs, b.seqbuf, P, bits=0)["score"] ==
            oracle.sw_reference(b.pairs, b.seqbuf, P, bits=32)["score"]).all()


@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLDEN, "sw", "*.npz"))),
                         ids=os.path.basename)
def test_oracle_equals_golden(f):
    d = np.load(f)
    P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
    got = oracle.sw(d["inputs"], d["seqbuf"], int(d["stride"]), P)
    assert (got["score"] == d["expected"]["score"]).all()
