"""The anchor chaining DP (dp_chain::mm_dp_vectorized drop-in) on the GPU
against the reference's golden outputs and the oracle; refusals."""
import glob
import os

import numpy as np
import pytest

import oracle
from tal_bsw import chaindata
from tal_bsw.api import TAL_EDOMAIN, TAL_EINVAL, TalBswError
from tal_bsw.chain import dp_chain

pytestmark = pytest.mark.gpu
GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "chain", "*.npz")))


def _params(d):
    return tuple(int(x) if k != 5 else float(x) for k, x in enumerate(d["params"]))


@pytest.mark.parametrize("f", GOLDEN, ids=os.path.basename)
def test_gpu_matches_golden(f):
    d = np.load(f)
    with dp_chain(*_params(d), device=0) as ch:
        gf, gp, gv = ch.mm_dp_batch(d["anchors"], d["offsets"], int(d["dr"]), int(d["dq"]))
    for name, g, e in (("f", gf, d["f"]), ("p", gp, d["p"]), ("v", gv, d["v"])):
        bad = np.nonzero(g != e)[0]
        assert bad.size == 0, f"{name}: {bad.size} differ, first #{bad[0]}: gpu {g[bad[0]]} ref {e[bad[0]]}"


@pytest.mark.parametrize("seed,jitter,spacing", [(1, 0, 11), (2, 60, 4), (3, 5, 25)])
def test_gpu_matches_oracle(seed, jitter, spacing):
    b = chaindata.generate(400, 200, 8000, seed=seed, l_jitter=jitter, spacing=spacing)
    P = chaindata.DRIVER_PARAMS
    ef, ep, ev = oracle.chain(b.anchors, b.offsets, P[2], P[4], 5000, 5000, nthreads=8)
    with dp_chain(*P, device=0) as ch:
        gf, gp, gv = ch.mm_dp_batch(b.anchors, b.offsets, 5000, 5000)
        assert ch.last_evals > 0
    assert (gf == ef).all() and (gp == ep).all() and (gv == ev).all()


def test_gpu_single_read_call_and_device_path():
    import torch
    b = chaindata.generate(50, 500, 3000, seed=9)
    P = chaindata.DRIVER_PARAMS
    ef, ep, ev = oracle.chain(b.anchors, b.offsets, P[2], P[4], 5000, 5000)
    with dp_chain(*P, device=0) as ch:
        # the reference's per-read call
        o0, o1 = int(b.offsets[3]), int(b.offsets[4])
        a = b.anchors[o0:o1].copy()
        f = np.zeros(a.shape[0], np.uint32)
        p = np.zeros(a.shape[0], np.int32)
        v = np.zeros(a.shape[0], np.int32)
        ch.mm_dp_vectorized(a.shape[0], a, f, p, v, 5000, 5000)
        ef1, ep1, ev1 = oracle.chain(a, np.array([0, a.shape[0]]), P[2], P[4], 5000, 5000)
        assert (f == ef1).all() and (p == ep1).all() and (v == ev1).all()
        # device-resident batch
        da = torch.from_numpy(b.anchors.view(np.uint8).copy()).cuda()
        do = torch.from_numpy(b.offsets.copy()).cuda()
        n = b.n
        df = torch.zeros(n, dtype=torch.int32, device="cuda")
        dp = torch.zeros(n, dtype=torch.int32, device="cuda")
        dv = torch.zeros(n, dtype=torch.int32, device="cuda")
        ch.mm_dp_device(da.data_ptr(), do.data_ptr(), b.n_reads, 5000, 5000, df.data_ptr(),
                        dp.data_ptr(), dv.data_ptr())
        assert (df.cpu().numpy().view(np.uint32) == ef).all()
        assert (dp.cpu().numpy() == ep).all() and (dv.cpu().numpy() == ev).all()


def test_gpu_refusals():
    P = chaindata.DRIVER_PARAMS
    b = chaindata.generate(5, 200, 500, seed=4)
    with dp_chain(*P, device=0) as ch:
        a = b.anchors.copy()
        a["l"][int(b.offsets[2]) + 1] = -3
        with pytest.raises(TalBswError) as ei:
            ch.mm_dp_batch(a, b.offsets, 5000, 5000)
        assert ei.value.status == TAL_EDOMAIN and ei.value.bad_pair == 2
        bad_offs = b.offsets.copy()
        bad_offs[3] = bad_offs[2] - 1
        with pytest.raises(TalBswError) as ei:
            ch.mm_dp_batch(b.anchors, bad_offs, 5000, 5000)
        assert ei.value.status == TAL_EINVAL
        # an empty batch and empty reads are fine
        f, p, v = ch.mm_dp_batch(b.anchors[:0], np.array([0, 0, 0], np.int64), 5000, 5000)
        assert f.shape == (0,)
