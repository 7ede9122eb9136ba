"""Counts the work unit of every benchmark workload: "ref-cells", the
iterations of the reference's scalar inner loop (bandedSWA.cpp:175-200, where
the reference's own disabled SW_cells counter sits, :199), summed over the
workload's pairs, with the band each pair is run with.  Writes
trans-omics-acceleration-library_gb300/tal_bsw/workload_cells.json, which
the benchmark reads to turn time into GCUPS.  Test-side tool (runs the
oracle); the workloads are seeded, so the counts are fixed numbers.

    python oracle/count_cells.py [name ...]
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [ROOT, os.path.join(ROOT, "trans-omics-acceleration-library_gb300")]

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from tal_bsw import synth  # noqa: E402

OUT = os.path.join(ROOT, "trans-omics-acceleration-library_gb300", "tal_bsw", "workload_cells.json")
SLICE = 500_000


def count(wl):
    total_cells = 0
    total_bytes = 0
    for first in range(0, wl.n_pairs, SLICE):
        n = min(SLICE, wl.n_pairs - first)
        b = synth.generate(wl, n, first=first)
        P = wl.params()
        if wl.w_choices:
            for wv in np.unique(b.w):
                sel = b.pairs[b.w == wv]
                total_cells += oracle.scalar(sel, b.ref, b.qer, int(wv), P, nthreads=os.cpu_count())[1]
        else:
            total_cells += oracle.scalar(b.pairs, b.ref, b.qer, wl.w, P, nthreads=os.cpu_count())[1]
        total_bytes += int(b.pairs["len1"].sum() + b.pairs["len2"].sum())
    return total_cells, total_bytes


def main(names):
    data = json.load(open(OUT)) if os.path.exists(OUT) else {}
    for name in names or list(synth.WORKLOADS):
        wl = synth.WORKLOADS[name]
        t = time.time()
        cells, nbytes = count(wl)
        data[name] = {"n_pairs": wl.n_pairs, "seed": wl.seed, "ref_cells": cells,
                      "sequence_bytes": nbytes}
        print(name, cells, f"{time.time() - t:.1f}s", flush=True)
        json.dump(data, open(OUT, "w"), indent=1, sort_keys=True)


if __name__ == "__main__":
    main(sys.argv[1:])
