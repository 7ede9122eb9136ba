"""The SeqPair record (bandedSWA.h:90-99) as a numpy dtype: 14 x int32, 56 bytes,
fields in declared order.  Inputs: idr, idq, id, len1, len2, h0, seqid, regid.
Outputs written by the scorer: score, tle, gtle, qle, gscore, max_off."""
import numpy as np

SEQPAIR_FIELDS = ("idr", "idq", "id", "len1", "len2", "h0", "seqid", "regid",
                  "score", "tle", "gtle", "qle", "gscore", "max_off")
OUTPUT_FIELDS = ("score", "tle", "gtle", "qle", "gscore", "max_off")
SEQPAIR_DTYPE = np.dtype([(f, np.int32) for f in SEQPAIR_FIELDS])
assert SEQPAIR_DTYPE.itemsize == 56


def new_pairs(n: int) -> np.ndarray:
    """A SeqPair array with outputs and caller ids set to -1, as the reference's
    loader does (benchmarks/bench-bsw.cpp:160-161)."""
    p = np.zeros(int(n), SEQPAIR_DTYPE)
    for f in ("seqid", "regid") + OUTPUT_FIELDS:
        p[f] = -1
    return p


def outputs(p: np.ndarray) -> np.ndarray:
    """(n, 6) int32 view-copy of the output fields, in OUTPUT_FIELDS order."""
    return np.stack([p[f] for f in OUTPUT_FIELDS], axis=1)
