"""The C++ drop-in (include/bandedSWA_gb300.h): a program written against
the reference's BandedPairWiseSW interface, compiled with g++ against the
header and libtal_bsw.so, scores the reference's golden batches -- getScores16
on the 16-bit workload slice, getScores8 on the 8-bit one, and
scalarBandedSWAWrapper (e_del = e_ins = 1, bench-bsw's matrix) -- and gets the
reference's outputs, with SW_cells counted."""
import os
import tempfile

import numpy as np
import pytest

from tal_bsw.seqpair import outputs

import cpp_dropin

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def exe():
    d = tempfile.mkdtemp()
    return cpp_dropin.build(d)


@pytest.mark.parametrize("name,mode", [("wl_c2_16bit.npz", 16), ("wl_c1_8bit.npz", 8),
                                       ("coupled16_band_4.npz", 16), ("wl_c2_16bit.npz", 0)])
def test_cpp_caller_gets_reference_outputs(exe, name, mode):
    d = np.load(os.path.join(GOLDEN, name))
    P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
    got, cells = cpp_dropin.run(exe, d["inputs"], d["ref"], d["qer"], int(d["w"]), P, mode)
    e, g = outputs(d["expected"]), outputs(got)
    bad = np.nonzero((e != g).any(1))[0]
    assert bad.size == 0, f"{bad.size} pairs differ, first {bad[0]}: {g[bad[0]]} vs {e[bad[0]]}"
    assert cells > 0
