"""Generates the golden fixtures of the DP chaining kernel by running the
reference's own dp_chain::mm_dp_vectorized (parallel_chaining_32_bit.h, built
from the reference tree by oracle/build_ref.sh: the AVX-512 path, -O2) on seeded
inputs.  Each fixture also records whether the reference's -Ofast and AVX2
builds gave the same outputs.  Run on an x86 AVX-512 host with the reference
tree present:  python tests/golden/chain/make_golden_chain.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
sys.path[:0] = [ROOT, os.path.join(ROOT, "trans-omics-acceleration-library_gb300")]

import oracle  # noqa: E402
from tal_bsw import chaindata  # noqa: E402

D = chaindata.ANCHOR_DTYPE


def pack(parts):
    offs = [0]
    for a in parts:
        offs.append(offs[-1] + a.shape[0])
    return np.concatenate(parts), np.array(offs, np.int64)


def cases():
    rng = np.random.default_rng(2024)
    P = chaindata.DRIVER_PARAMS
    b = chaindata.generate(16, 1000, 4000, seed=11)
    yield "driver_like", b.anchors, b.offsets, P, 5000, 5000
    b = chaindata.generate(12, 200, 3000, seed=12, l_jitter=40, spacing=4)
    yield "jitter_maxiter20_bw50", b.anchors, b.offsets, (5000, 5000, 50, 25, 20, 1.0, 0, 1), 5000, 5000
    parts = []
    for _ in range(300):  # 0..12 anchors: the scalar loop (<= 6 predecessors) and its edge
        n = int(rng.integers(0, 13))
        a = np.zeros(n, D)
        a["r"] = np.sort(rng.integers(0, 3000, n)).astype(np.uint64)
        a["q"] = rng.integers(0, 3000, n)
        a["l"] = rng.integers(0, 60, n)
        parts.append(a)
    yield ("short_reads",) + pack(parts) + (P, 5000, 5000)
    parts = []
    for _ in range(60):  # unsorted positions, three contigs, q near r: windows with r_j > r_i
        n = int(rng.integers(1, 300))
        a = np.zeros(n, D)
        pos = rng.integers(0, 6000, n)
        a["r"] = (rng.integers(0, 3, n).astype(np.uint64) << np.uint64(32)) | pos.astype(np.uint64)
        a["q"] = pos + rng.integers(-50, 50, n)
        a["l"] = rng.integers(0, 2 ** 20, n)
        parts.append(a)
    yield ("unsorted_contigs",) + pack(parts) + (P, 5000, 5000)
    parts = []
    for _ in range(60):  # every anchor twice: equal scores, the larger j wins
        n = int(rng.integers(1, 150))
        base = np.sort(rng.integers(0, 2000, n)).astype(np.uint64)
        a = np.zeros(n, D)
        a["r"] = base
        a["q"] = (base.astype(np.int64) + rng.integers(0, 3, n)).astype(np.int32)
        a["l"] = 100
        a = np.concatenate([a, a])
        parts.append(a[np.argsort(a["r"], kind="stable")])
    yield ("ties",) + pack(parts) + (P, 5000, 5000)
    parts = []
    for _ in range(200):  # l = 105: float and double gap costs differ at dd = 60, 100, 120 ...
        n = int(rng.integers(2, 20))
        a = np.zeros(n, D)
        r = np.cumsum(rng.integers(150, 400, n))
        a["r"] = r.astype(np.uint64)
        a["q"] = (r - rng.choice([0, 60, 100, 120, 180, 200], n) * rng.choice([-1, 1], n)).astype(np.int32)
        a["l"] = 105
        parts.append(a[np.argsort(a["r"], kind="stable")])
    yield ("rounding_paths",) + pack(parts) + (P, 5000, 5000)


def main():
    for v in oracle.CHAIN_REF_VARIANTS:
        if not oracle.chain_ref_available(v):
            raise SystemExit(f"reference build {v} missing: run oracle/build_ref.sh on an AVX-512 host")
    for name, anchors, offsets, P, dr, dq in cases():
        f, p, v = oracle.chain_reference(anchors, offsets, P, dr, dq, variant="avx512")
        same = {}
        for var in ("avx512_ofast", "avx2"):
            f2, p2, v2 = oracle.chain_reference(anchors, offsets, P, dr, dq, variant=var)
            same[var] = bool((f2 == f).all() and (p2 == p).all() and (v2 == v).all())
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), anchors=anchors, offsets=offsets,
                            params=np.array(P, np.float64), dr=dr, dq=dq, f=f, p=p, v=v,
                            same_ofast=same["avx512_ofast"], same_avx2=same["avx2"])
        print(name, anchors.shape[0], "anchors,", offsets.shape[0] - 1, "reads,", same)


if __name__ == "__main__":
    main()
