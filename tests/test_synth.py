"""The seeded workload generator: deterministic, slice-consistent, and shaped
like the workloads it stands in for."""
import numpy as np

from tal_bsw import synth


def test_deterministic_and_slice_consistent():
    a = synth.generate(synth.C2, 40)
    b = synth.generate(synth.C2, 40)
    assert (a.pairs == b.pairs).all() and (a.ref == b.ref).all() and (a.qer == b.qer).all()
    s = synth.generate(synth.C2, 10, first=25)
    for k in range(10):
        pa, ps = a.pairs[25 + k], s.pairs[k]
        assert pa["len1"] == ps["len1"] and pa["len2"] == ps["len2"] and pa["h0"] == ps["h0"]
        assert (a.qer[pa["idq"]:pa["idq"] + pa["len2"]] == s.qer[ps["idq"]:ps["idq"] + ps["len2"]]).all()
        assert (a.ref[pa["idr"]:pa["idr"] + pa["len1"]] == s.ref[ps["idr"]:ps["idr"] + ps["len1"]]).all()


def test_shapes():
    c1 = synth.generate(synth.C1, 2000)
    assert (c1.pairs["len2"] == 151).all()
    d = c1.pairs["len1"] - c1.pairs["len2"]
    assert d.min() >= 0 and d.max() <= 20
    assert c1.pairs["h0"].min() >= 19 and c1.pairs["h0"].max() <= 60
    c18 = synth.generate(synth.C1_8, 2000)
    assert c18.pairs["len1"].max() <= 127
    assert (c18.pairs["h0"] + np.minimum(c18.pairs["len1"], c18.pairs["len2"]) <= 127).all()
    c3 = synth.generate(synth.C3, 20000)
    l2 = c3.pairs["len2"]
    assert l2.min() >= 20 and l2.max() <= 2000 and 100 < np.median(l2) < 140
    assert set(np.unique(c3.w)) == {20, 50, 100}
    c4 = synth.generate(synth.C4, 50)
    assert c4.pairs["len2"].min() >= 1000 and c4.pairs["len2"].max() <= 5000


def test_bases_and_error_rates():
    b = synth.generate(synth.C2, 3000)
    assert b.qer.max() <= 4 and b.ref.max() <= 4
    nfrac = (b.qer[: int(b.pairs["len2"].sum())] == 4).mean()
    assert 0.0003 < nfrac < 0.003
