"""The CUDA kernel's source, compiled for the host and run one fiber per lane
(tests/simt_emu), against the reference's golden outputs: checks the kernel's
logic on a machine without a GPU.  The GPU tests run the real thing."""
import glob
import os

import numpy as np
import pytest

import oracle
import simt_emu
from tal_bsw.seqpair import outputs

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FILES = sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))
CONFIGS = [(1, 4), (4, 4), (8, 4), (8, 2), (16, 4), (32, 4), (32, 2), (4, 2), (16, 2)]


@pytest.mark.parametrize("f", FILES, ids=os.path.basename)
def test_emulated_kernel_matches_golden(f):
    d = np.load(f)
    P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
    n = min(d["inputs"].shape[0], 6 if "c4" in f else 16)
    p = d["inputs"][:n]
    w = d["w"]
    bits = int(d["bits"])
    G, K = CONFIGS[sum(os.path.basename(f).encode()) % len(CONFIGS)]
    if np.ndim(w):
        got, ef, _ = simt_emu.run(p, d["ref"], d["qer"], 0, P, bits=bits, K=K, G=G, warps=2,
                                  wpair=w[:n])
    else:
        got, ef, _ = simt_emu.run(p, d["ref"], d["qer"], int(w), P, bits=bits, K=K, G=G, warps=2)
    assert ef == 0
    e, g = outputs(d["expected"][:n]), outputs(got)
    bad = np.nonzero((e != g).any(1))[0]
    assert bad.size == 0, f"G={G} K={K}: pair {bad[0]}: emu {g[bad[0]].tolist()} ref {e[bad[0]].tolist()}"
