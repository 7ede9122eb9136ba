"""Builds and runs the C++ caller of the drop-in header (main.cpp).  Test
infrastructure only."""
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIBDIR = os.path.join(ROOT, "trans-omics-acceleration-library_gb300", "lib")
KEYS = ("o_del", "e_del", "o_ins", "e_ins", "zdrop", "end_bonus", "a", "b")


def build(out_dir):
    exe = os.path.join(out_dir, "dropin_main")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                           os.path.join(HERE, "main.cpp"), "-L", LIBDIR, "-ltal_bsw",
                           "-Wl,-rpath," + LIBDIR, "-o", exe])
    return exe


def run(exe, pairs, ref, qer, w, params, mode):
    """mode 8 / 16: getScores8 / getScores16; 0: scalarBandedSWAWrapper.
    Returns (scored pairs, SW_cells)."""
    with tempfile.TemporaryDirectory() as d:
        fi, fo = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(fi, "wb") as f:
            f.write(np.int64(pairs.shape[0]).tobytes())
            f.write(np.int32(w).tobytes())
            f.write(np.int32(mode).tobytes())
            f.write(np.array([params[k] for k in KEYS], np.int32).tobytes())
            f.write(np.ascontiguousarray(pairs).tobytes())
            f.write(np.int64(ref.shape[0]).tobytes())
            f.write(np.ascontiguousarray(ref, np.uint8).tobytes())
            f.write(np.int64(qer.shape[0]).tobytes())
            f.write(np.ascontiguousarray(qer, np.uint8).tobytes())
        subprocess.check_call([exe, fi, fo])
        raw = open(fo, "rb").read()
    n = pairs.shape[0]
    out = np.frombuffer(raw[: n * 56], dtype=pairs.dtype).copy()
    cells = int(np.frombuffer(raw[n * 56: n * 56 + 8], np.uint64)[0])
    return out, cells
