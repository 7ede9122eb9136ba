"""Anchors for the DP chaining kernel: the 16-byte anchor_t records
(src/chaining/parallel_chaining_32_bit.h:58-67) and a seeded generator of
minimap2-like anchor sets, standing in for the anchor files the reference's
driver (benchmarks/bench-dp-chaining.cpp) reads, none of which ship with it."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

ANCHOR_DTYPE = np.dtype([("r", "<u8"), ("q", "<i4"), ("l", "<i4")])

# dp_chain obj(5000, 5000, 500, 25, 5000, 1.0, 0, 1) and mm_dp_vectorized(...,
# 5000, 5000, ...) in the reference driver
DRIVER_PARAMS = (5000, 5000, 500, 25, 5000, 1.0, 0, 1)
DRIVER_DR = 5000
DRIVER_DQ = 5000


@dataclass
class AnchorBatch:
    anchors: np.ndarray   # ANCHOR_DTYPE, reads back to back, each sorted by (r, q)
    offsets: np.ndarray   # int64, n_reads + 1

    @property
    def n_reads(self) -> int:
        return self.offsets.shape[0] - 1

    @property
    def n(self) -> int:
        return self.anchors.shape[0]


def generate(n_reads: int, len_lo: int = 1000, len_hi: int = 10000, seed: int = 77,
             k: int = 15, spacing: int = 11, noise: float = 0.2, repeat: float = 0.3,
             indel: float = 0.05, l_jitter: int = 0) -> AnchorBatch:
    """n_reads reads of length U[len_lo, len_hi] mapped to random loci: an anchor
    (span k, plus U[0, l_jitter]) every U[1, spacing - 1] query bases along the
    true diagonal, which drifts by +-1..3 at a rate `indel` per anchor; with
    probability `repeat` a second copy of half the read's anchors a few kb away
    (a competing chain inside the window); `noise` x as many random anchors near
    the locus.  r = contig << 32 | position.  Sorted by (r, q) per read."""
    rng = np.random.default_rng(seed)
    parts, offs = [], [0]
    for _ in range(n_reads):
        L = int(rng.integers(len_lo, len_hi + 1))
        rid = int(rng.integers(0, 24))
        start = int(rng.integers(1_000_000, 200_000_000))
        steps = rng.integers(1, max(spacing, 2), L // max(spacing // 2, 1) + 8)
        q = np.cumsum(steps)
        q = q[q < L - k]
        m = q.shape[0]
        drift = np.cumsum(np.where(rng.random(m) < indel, rng.integers(-3, 4, m), 0))
        r = start + q + drift
        qs, rs = [q], [r]
        if m > 8 and rng.random() < repeat:
            h = m // 2
            a0 = int(rng.integers(0, m - h))
            rs.append(r[a0:a0 + h] + int(rng.integers(-4000, 4000)))
            qs.append(q[a0:a0 + h])
        nn = int(noise * m)
        if nn:
            rs.append(rng.integers(start - 10_000, start + L + 10_000, nn))
            qs.append(rng.integers(0, L, nn))
        rr = np.concatenate(rs).astype(np.int64)
        qq = np.concatenate(qs).astype(np.int64)
        keep = rr >= 0
        rr, qq = rr[keep], qq[keep]
        a = np.zeros(rr.shape[0], ANCHOR_DTYPE)
        a["r"] = (np.uint64(rid) << np.uint64(32)) | rr.astype(np.uint64)
        a["q"] = qq.astype(np.int32)
        a["l"] = k + (rng.integers(0, l_jitter + 1, rr.shape[0]) if l_jitter else 0)
        a = a[np.lexsort((a["q"], a["r"]))]
        parts.append(a)
        offs.append(offs[-1] + a.shape[0])
    anchors = np.concatenate(parts) if parts else np.zeros(0, ANCHOR_DTYPE)
    return AnchorBatch(anchors=anchors, offsets=np.array(offs, np.int64))
