"""Seeded synthetic inputs for the unbanded Smith-Waterman scorer, in the
reference's layout (src/alignment/Smith-Waterman): 12-byte SeqPair records
{id, len1, len2, score} and one sequence buffer holding pair k's seq1 at
2*id*stride and seq2 at (2*id+1)*stride (stride = the precision's MAX_SEQ_LEN:
128 for 8-bit, 1024 for 16- and 32-bit)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SW_DTYPE = np.dtype([("id", "<i4"), ("len1", "<i2"), ("len2", "<i2"), ("score", "<i4")])
MAX_SEQ_LEN = {8: 128, 16: 1024, 32: 1024}
# Longest sequence the reference scores safely: it rounds lengths up to a
# multiple of 4 and initialises one column past them (PairWiseSW_16.cpp:170-174,
# :303-311), inside buffers of MAX_SEQ_LEN columns.
MAX_LEN = {b: m - 4 for b, m in MAX_SEQ_LEN.items()}


@dataclass
class SwBatch:
    pairs: np.ndarray   # SW_DTYPE
    seqbuf: np.ndarray  # uint8, 2 * n * stride
    stride: int

    @property
    def n(self) -> int:
        return int(self.pairs.shape[0])

    @property
    def cells(self) -> int:
        """The reference driver's cell count: sum of len1 * len2."""
        return int((self.pairs["len1"].astype(np.int64) * self.pairs["len2"]).sum())


def generate(n: int, len_lo: int, len_hi: int, bits: int = 16, seed: int = 20240,
             sub: float = 0.04, nrate: float = 0.001) -> SwBatch:
    """n pairs: seq1 of uniform bases (0..3, N = 4 at rate nrate) and length
    U[len_lo, len_hi]; seq2 = seq1 with substitutions at rate sub, its length
    len1 + U[-10, 10] clipped to [len_lo, len_hi]."""
    stride = MAX_SEQ_LEN[bits]
    if not 0 <= len_lo <= len_hi <= MAX_LEN[bits]:
        raise ValueError("lengths outside the precision's limit")
    rng = np.random.default_rng(seed)
    len1 = rng.integers(len_lo, len_hi + 1, n)
    len2 = np.clip(len1 + rng.integers(-10, 11, n), len_lo, len_hi)
    buf = np.zeros((2 * n, stride), np.uint8)
    s1 = rng.integers(0, 4, (n, stride), dtype=np.uint8)
    s1[rng.random((n, stride)) < nrate] = 4
    s2 = s1.copy()
    mut = rng.random((n, stride)) < sub
    s2[mut] = rng.integers(0, 4, int(mut.sum()), dtype=np.uint8)
    buf[0::2] = s1
    buf[1::2] = s2
    pairs = np.zeros(n, SW_DTYPE)
    pairs["id"] = np.arange(n, dtype=np.int32)
    pairs["len1"] = len1
    pairs["len2"] = len2
    return SwBatch(pairs=pairs, seqbuf=buf.reshape(-1), stride=stride)
