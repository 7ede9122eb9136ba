"""Seeds for the caller-side extension layer (include/tal_extend.h): record
layouts and a seeded generator of reads sampled from a random reference with
substitutions and indels, each with one to three exact-match seeds taken from
its error-free stretches (the job an SMEM/seed stage does before extension)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SEED_DTYPE = np.dtype([("read", "<i4"), ("qbeg", "<i4"), ("rbeg", "<i8"), ("len", "<i4"),
                       ("pad_", "<i4")])
REGION_DTYPE = np.dtype([("rb", "<i8"), ("re", "<i8"), ("qb", "<i4"), ("qe", "<i4"),
                         ("score", "<i4"), ("left_score", "<i4")])


@dataclass
class SeedBatch:
    ref: np.ndarray        # uint8 bases 0..4
    reads: np.ndarray      # uint8, reads back to back
    read_off: np.ndarray   # int64, n_reads + 1
    seeds: np.ndarray      # SEED_DTYPE

    @property
    def n_reads(self) -> int:
        return self.read_off.shape[0] - 1


def generate(n_reads: int, ref_len: int = 2_000_000, len_lo: int = 100, len_hi: int = 250,
             sub: float = 0.03, indel: float = 0.004, kmin: int = 19, kmax: int = 60,
             max_seeds: int = 3, junk: float = 0.1, seed: int = 55) -> SeedBatch:
    """Reads of length U[len_lo, len_hi] copied from random reference
    positions with substitutions (rate sub), 1-3 base indels (rate indel) and,
    for a fraction `junk`, a random tail of up to a third of the read (so the
    right extension stops short of the read's end).  Seeds: up to max_seeds
    error-free stretches of at least kmin bases (cut to kmax)."""
    rng = np.random.default_rng(seed)
    ref = rng.integers(0, 4, ref_len, dtype=np.uint8)
    ref[rng.random(ref_len) < 0.0005] = 4
    reads, offs, seeds = [], [0], []
    for r in range(n_reads):
        L = int(rng.integers(len_lo, len_hi + 1))
        pos = int(rng.integers(2000, ref_len - 2 * L - 2000))
        # the reference stretch, then indels (1-3 bases each) at random read
        # positions, then substitutions; rp: each read base's reference
        # position (-1: inserted)
        span = L + 64
        q = ref[pos:pos + span].copy()
        rp = np.arange(pos, pos + span, dtype=np.int64)
        for _ in range(int(rng.poisson(indel * L))):
            at = int(rng.integers(1, L - 1))
            k = int(rng.integers(1, 4))
            if rng.random() < 0.5:   # deletion from the read
                q = np.delete(q, np.s_[at:at + k])
                rp = np.delete(rp, np.s_[at:at + k])
            else:                    # insertion into the read
                q = np.insert(q, at, rng.integers(0, 4, k).astype(np.uint8))
                rp = np.insert(rp, at, np.full(k, -1, np.int64))
        q = q[:L].copy()
        rp = rp[:L].copy()
        m = rng.random(L) < sub
        q[m] = (q[m] % 4 + rng.integers(1, 4, int(m.sum())).astype(np.uint8)) % 4
        if rng.random() < junk:
            t = int(rng.integers(1, L // 3 + 1))
            q[L - t:] = rng.integers(0, 4, t)
            rp[L - t:] = -1
        ok = (rp >= 0) & (q == ref[np.maximum(rp, 0)])
        # error-free stretches: matching bases whose reference positions run on
        brk = np.ones(L, bool)
        brk[1:] = ~(ok[1:] & ok[:-1] & (rp[1:] == rp[:-1] + 1))
        starts = np.nonzero(brk & ok)[0]
        ends = np.append(np.nonzero(brk)[0][1:], L)
        runs = []
        for st in starts:
            en = ends[np.searchsorted(ends, st, side="right")]
            if en - st >= kmin:
                runs.append((int(st), int(en - st)))
        rng.shuffle(runs)
        for qb, ln in runs[:max_seeds]:
            ln = min(ln, kmax)
            seeds.append((r, qb, int(rp[qb]), ln, 0))
        reads.append(q)
        offs.append(offs[-1] + L)
    sd = np.array(seeds, SEED_DTYPE) if seeds else np.zeros(0, SEED_DTYPE)
    return SeedBatch(ref=ref, reads=np.concatenate(reads) if reads else np.zeros(0, np.uint8),
                     read_off=np.array(offs, np.int64), seeds=sd)
