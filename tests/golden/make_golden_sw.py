"""Regenerates the unbanded Smith-Waterman golden fixtures (sw/*.npz) from the
reference itself: PairWiseSW_8 / _16 / _32::getScores, AVX-512BW build made by
oracle/build_ref.sh from the reference sources.  Each fixture holds seeded
12-byte SeqPair records, the sequence buffer (stride = the precision's
MAX_SEQ_LEN), the scoring parameters and the reference's scores.
Run:  python tests/golden/make_golden_sw.py"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "trans-omics-acceleration-library_gb300")]

import oracle  # noqa: E402
from tal_bsw import swdata  # noqa: E402

KEYS = ["match", "mismatch", "open", "extend"]
PARAMS = {"bwa": dict(match=1, mismatch=-4, open=-6, extend=-1),
          "m2": dict(match=2, mismatch=-3, open=-5, extend=-2)}


def save(name, b, P, bits):
    exp = oracle.sw_reference(b.pairs, b.seqbuf, P, bits=bits)
    os.makedirs(os.path.join(HERE, "sw"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "sw", name + ".npz"), inputs=b.pairs, seqbuf=b.seqbuf,
                        stride=np.int32(b.stride), bits=np.int32(bits),
                        param_keys=np.array(KEYS), param_vals=np.array([P[k] for k in KEYS], np.int32),
                        expected=exp)
    print(name, b.n, "pairs")


def main():
    oracle.build_ref()
    assert oracle.sw_ref_available(), "reference build missing"
    for pname, P in PARAMS.items():
        for bits, (lo, hi, n) in {8: (0, 60, 96), 16: (0, 1020, 40), 32: (100, 700, 40)}.items():
            b = swdata.generate(n, lo, hi, bits=bits, seed=77 + bits)
            save(f"sw{bits}_{pname}", b, P, bits)
        # edge lengths: empty, one base, one side empty, identical, all-N
        b = swdata.generate(16, 0, 32, bits=16, seed=5)
        b.pairs["len1"][:4] = [0, 1, 0, 7]
        b.pairs["len2"][:4] = [0, 0, 1, 7]
        s = b.seqbuf.reshape(-1, b.stride)
        s[2 * 5 + 1] = s[2 * 5]
        s[2 * 6, :32] = 4
        s[2 * 6 + 1, :32] = 4
        save(f"sw16_edges_{pname}", b, P, 16)


if __name__ == "__main__":
    main()
