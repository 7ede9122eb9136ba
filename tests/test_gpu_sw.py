"""The unbanded Smith-Waterman scorer (PairWiseSW_8/16/32 drop-in) on the GPU
against the reference's golden scores and the oracle; out-of-range pairs are
refused."""
import glob
import os

import numpy as np
import pytest

import oracle
from tal_bsw import swdata
from tal_bsw.api import TAL_EDOMAIN, TAL_EINVAL, TalBswError
from tal_bsw.sw import PairWiseSW_8, PairWiseSW_16, PairWiseSW_32

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CLASSES = {8: PairWiseSW_8, 16: PairWiseSW_16, 32: PairWiseSW_32}


def _sw(P, bits):
    return CLASSES[bits](P["match"], P["mismatch"], P["open"], P["extend"], device=0)


@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLDEN, "sw", "*.npz"))), ids=os.path.basename)
def test_gpu_matches_golden(f):
    d = np.load(f)
    P = {k: int(v) for k, v in zip(d["param_keys"], d["param_vals"])}
    bits = int(d["bits"])
    got = d["inputs"].copy()
    with _sw(P, bits) as sw:
        sw.getScores(got, d["seqbuf"], got.shape[0], 1)
        assert sw.last_cells == int((d["inputs"]["len1"].astype(np.int64) * d["inputs"]["len2"]).sum())
    assert (got["score"] == d["expected"]["score"]).all()


@pytest.mark.parametrize("bits,lo,hi", [(16, 0, 1020), (32, 200, 1020), (8, 0, 100)])
def test_gpu_matches_oracle(bits, lo, hi):
    P = dict(match=1, mismatch=-4, open=-6, extend=-1)
    b = swdata.generate(3000 if bits != 16 else 6000, lo, hi, bits=bits, seed=9 + bits)
    exp = oracle.sw(b.pairs, b.seqbuf, b.stride, P, nthreads=8)
    got = b.pairs.copy()
    with _sw(P, bits) as sw:
        sw.getScores(got, b.seqbuf, b.n, 1)
    bad = np.nonzero(got["score"] != exp["score"])[0]
    assert bad.size == 0, f"{bad.size} differ; first #{bad[0]}: gpu {got['score'][bad[0]]} oracle {exp['score'][bad[0]]}"


def test_gpu_device_resident_and_refusals():
    import torch
    P = dict(match=1, mismatch=-4, open=-6, extend=-1)
    b = swdata.generate(500, 0, 600, bits=16, seed=4)
    exp = oracle.sw(b.pairs, b.seqbuf, b.stride, P)
    with _sw(P, 16) as sw:
        dp = torch.from_numpy(b.pairs.view(np.uint8).reshape(-1).copy()).cuda()
        ds = torch.from_numpy(b.seqbuf).cuda()
        sw.scores_device(dp.data_ptr(), ds.data_ptr(), ds.numel(), b.n)
        got = dp.cpu().numpy().view(swdata.SW_DTYPE)
        assert (got["score"] == exp["score"]).all()
        # a sequence longer than the reference's buffers allow
        p = b.pairs.copy()
        p["len1"][3] = 1021
        with pytest.raises(TalBswError) as ei:
            sw.getScores(p, b.seqbuf, b.n, 1)
        assert ei.value.status == TAL_EDOMAIN and ei.value.bad_pair == 3
    # 8-bit: a score that would leave int8
    with _sw(dict(match=2, mismatch=-4, open=-6, extend=-1), 8) as sw8:
        q = swdata.generate(4, 100, 100, bits=8, seed=1)
        s = q.seqbuf.reshape(-1, q.stride)
        s[1] = s[0]                      # pair 0: identical 100-base sequences, score 200
        with pytest.raises(TalBswError) as ei:
            sw8.getScores(q.pairs, q.seqbuf, q.n, 1)
        assert ei.value.status == TAL_EDOMAIN
    with pytest.raises(TalBswError) as ei:
        PairWiseSW_16(1, -4, 6, -1, device=0)   # a positive gap weight
    assert ei.value.status == TAL_EINVAL


@pytest.mark.parametrize("bits,P", [
    (16, dict(match=300, mismatch=-32468, open=-32000, extend=-768)),   # match - mismatch = 2^15
    (16, dict(match=300, mismatch=-32768, open=-32000, extend=-768)),   # past it: 32-bit lanes
    (8, dict(match=1, mismatch=-128, open=-100, extend=-28)),
])
def test_gpu_weights_at_the_element_limits(bits, P):
    """Weights at the limits of the element type, lengths up to what the score
    bound allows, ragged neighbours: scores equal the oracle's."""
    rng = np.random.default_rng(bits)
    hi = {8: 100, 16: 100}[bits]
    b = swdata.generate(2001, 0, hi, bits=bits, seed=5)
    b.pairs["len1"] = rng.integers(0, hi + 1, b.n)
    b.pairs["len2"] = rng.integers(0, hi + 1, b.n)
    exp = oracle.sw(b.pairs, b.seqbuf, b.stride, P, nthreads=8)
    got = b.pairs.copy()
    with _sw(P, bits) as sw:
        sw.getScores(got, b.seqbuf, b.n, 1)
    assert (got["score"] == exp["score"]).all()
