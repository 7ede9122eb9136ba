"""Regenerates the golden fixtures in this directory from the reference itself.

Run in a container that has the reference sources (it compiles them with
oracle/build_ref.sh):  python tests/golden/make_golden.py
Each fixture holds seeded inputs (SeqPair records, reference and query bytes,
band, precision, scoring parameters) and the outputs of the reference's own
getScores16 / getScores8 (AVX-512BW build, one SIMD group at a time on zeroed
scratch rows -- see oracle/ref_shim.cpp).  The GPU tests replay them without
the reference."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "trans-omics-acceleration-library_gb300"),
                os.path.dirname(HERE)]

import oracle  # noqa: E402
from _cases import DEFAULT, coupled_cases, edge_cases, workload_slices, wrapping_cases  # noqa: E402

KEYS = ["o_del", "e_del", "o_ins", "e_ins", "zdrop", "end_bonus", "a", "b"]


def ref_routed(pairs, ref, qer, w, P, bits):
    out = pairs.copy()
    n = out.shape[0]
    warr = np.broadcast_to(np.asarray(w, np.int64), (n,))
    is8 = (np.ones(n, bool) if bits == 8 else np.zeros(n, bool) if bits == 16
           else oracle.eligible8(out, warr, P))
    for wv in np.unique(warr):
        for b in (8, 16):
            sel = np.nonzero((warr == wv) & (is8 == (b == 8)))[0]
            if sel.size:
                out[sel] = oracle.reference(out[sel], ref, qer, int(wv), P, mode=b)
    return out


def save(name, pairs, ref, qer, w, P, bits):
    exp = ref_routed(pairs, ref, qer, w, P, bits)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), inputs=pairs, ref=ref, qer=qer,
                        w=np.asarray(w, np.int32), bits=np.int32(bits),
                        param_keys=np.array(KEYS), param_vals=np.array([P[k] for k in KEYS], np.int32),
                        expected=exp)
    print(name, pairs.shape[0], "pairs")


def main():
    oracle.build_ref()
    assert oracle.ref_available(), "reference build missing"
    for name, b, bits in workload_slices():
        w = b.w if b.workload.w_choices else b.workload.w
        save("wl_" + name, b.pairs, b.ref, b.qer, w, b.workload.params(), bits)
    for bits in (16, 8):
        for name, p, r, q, w, P in edge_cases(bits=bits):
            if bits == 8:
                p = p[oracle.eligible8(p, w, P)]
                if p.shape[0] == 0:
                    continue
            save(f"edge{bits}_{name}", p, r, q, w, P, bits)
    for name, p, r, q, w, bits in coupled_cases():
        save(name, p, r, q, w, DEFAULT, bits)
    for name, p, r, q, w, P, bits in wrapping_cases():
        save(name, p, r, q, w, P, bits)


if __name__ == "__main__":
    main()
