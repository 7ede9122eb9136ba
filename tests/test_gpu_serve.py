"""The serving loop (tal_bsw_server_*, tal_bsw_submit, tal_bsw_poll): each
request's outputs are the same alone and in a mix of concurrent requests and
equal the oracle; admission waits for pool memory; one request's bad pair
fails only that request."""
import numpy as np
import pytest

import oracle
import tal_bsw
from tal_bsw import synth
from tal_bsw.api import TAL_EDOMAIN, TAL_ENOMEM, TAL_OK, TalBswError
from tal_bsw.seqpair import outputs

pytestmark = pytest.mark.gpu


def _bsw(P):
    return tal_bsw.BandedPairWiseSW(P["o_del"], P["e_del"], P["o_ins"], P["e_ins"], P["zdrop"],
                                    P["end_bonus"], None, P["a"], P["b"], 1, device=0)


def _same(exp, got, what):
    e, g = outputs(exp), outputs(got)
    bad = np.nonzero((e != g).any(axis=1))[0]
    assert bad.size == 0, (f"{what}: {bad.size}/{len(e)} differ; first #{bad[0]}: "
                           f"gpu {g[bad[0]].tolist()} expected {e[bad[0]].tolist()}")


def _pinned(a):
    """A page-locked copy of numpy array a (torch allocates the pinned memory;
    keep the returned tensor alive as long as the view)."""
    import torch
    t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
    out = t.numpy().view(a.dtype).reshape(a.shape)
    out[...] = a
    return out, t


def _wait(srv, ticket):
    info = srv.poll(ticket, timeout_us=120_000_000)
    assert info is not None, "request not complete after 120 s"
    return info


def _requests(b, sizes):
    """Consecutive slices of batch b as requests (start, stop)."""
    out, lo = [], 0
    for s in sizes:
        hi = min(lo + int(s), b.n)
        out.append((lo, hi))
        lo = hi
    return out


@pytest.fixture(scope="module")
def c3():
    wl = synth.C3
    b = synth.generate(wl, 60000)
    P = wl.params()
    exp = oracle.routed(b.pairs, b.ref, b.qer, b.w, P, bits=0, nthreads=8)
    return wl, b, P, exp


def test_serving_alone_equals_mixed_equals_oracle(c3):
    wl, b, P, exp = c3
    rng = np.random.default_rng(5)
    sizes = np.exp(rng.uniform(np.log(50), np.log(6000), 40)).astype(int)
    spans = _requests(b, sizes)
    ref_p, ref_t = _pinned(b.ref)
    qer_p, qer_t = _pinned(b.qer)
    w_p, w_t = _pinned(b.w.astype(np.int32))
    with _bsw(P) as bsw:
        # autotune the bins on this mix first (the server takes the tuning)
        warm = b.pairs.copy()
        bsw.scores_batched(warm, b.ref, b.qer, b.n, 100, wpair=b.w, bits=tal_bsw.AUTO)
        _same(exp, warm, "batched warm-up")
        with tal_bsw.BswServer(bsw, pool_bytes=1 << 30) as srv:
            # alone: one request at a time
            alone = b.pairs.copy()
            for lo, hi in spans:
                t = srv.submit(alone[lo:hi], b.ref, b.qer, w=100, wpair=b.w[lo:hi], bits=tal_bsw.AUTO)
                info = _wait(srv, t)
                assert info.status == TAL_OK and info.tick_requests == 1
            # mixed: all at once; even requests from pinned buffers, odd from pageable
            mixed_pg = b.pairs.copy()
            mixed_pn, pn_t = _pinned(b.pairs)
            tickets = []
            for k, (lo, hi) in enumerate(spans):
                if k % 2 == 0:
                    t = srv.submit(mixed_pn[lo:hi], ref_p, qer_p, w=100, wpair=w_p[lo:hi], bits=0)
                else:
                    t = srv.submit(mixed_pg[lo:hi], b.ref, b.qer, w=100, wpair=b.w[lo:hi], bits=0)
                tickets.append(t)
            infos = [_wait(srv, t) for t in tickets]
            st = srv.stats()
    assert all(i.status == TAL_OK for i in infos)
    assert all(i.done_ns >= i.launch_ns >= i.admit_ns >= i.submit_ns for i in infos)
    assert st["max_tick_requests"] > 1, "requests submitted together never shared a tick"
    assert st["completed"] == st["submitted"] == 2 * len(spans)
    assert st["pool_used_bytes"] == 0
    n = spans[-1][1]
    mixed = mixed_pg.copy()
    for k, (lo, hi) in enumerate(spans):
        if k % 2 == 0:
            mixed[lo:hi] = mixed_pn[lo:hi]
    _same(exp[:n], alone[:n], "alone")
    _same(alone[:n], mixed[:n], "mixed vs alone")


def test_serving_admission_waits_for_pool_memory(c3):
    """A pool far smaller than the submitted work: requests wait for memory in
    arrival order and all complete; one larger than the pool is refused."""
    wl, b, P, exp = c3
    pool = 4 << 20
    with _bsw(P) as bsw, tal_bsw.BswServer(bsw, pool_bytes=pool, latency_pairs=-1) as srv:
        got = b.pairs.copy()
        spans = [(lo, lo + 4000) for lo in range(0, 48000, 4000)]   # ~1.5 MB each
        tickets = [srv.submit(got[lo:hi], b.ref, b.qer, w=100, wpair=b.w[lo:hi], bits=0)
                   for lo, hi in spans]
        infos = [_wait(srv, t) for t in tickets]
        st = srv.stats()
        with pytest.raises(TalBswError) as ei:
            srv.submit(got[:40000], b.ref, b.qer, w=100, wpair=b.w[:40000], bits=0)
        assert ei.value.status == TAL_ENOMEM
    assert all(i.status == TAL_OK for i in infos)
    assert 0 < st["pool_peak_bytes"] <= pool
    _same(exp[:48000], got[:48000], "pool-limited serving")


def test_serving_bad_pair_fails_only_its_request(c3):
    wl, b, P, exp = c3
    got = b.pairs.copy()
    qer = b.qer.copy()
    # request 1's pair 7 gets a query base code above 4: the kernel flags it
    bad_pair = 1000 + 7
    qer[got["idq"][bad_pair]] = 9
    spans = [(0, 1000), (1000, 2000), (2000, 3000)]
    with _bsw(P) as bsw, tal_bsw.BswServer(bsw, pool_bytes=256 << 20) as srv:
        tickets = [srv.submit(got[lo:hi], b.ref, qer, w=100, wpair=b.w[lo:hi], bits=0)
                   for lo, hi in spans]
        infos = [_wait(srv, t) for t in tickets]
        empty = _wait(srv, srv.submit(got[:0], b.ref, qer, numPairs=0))
        with pytest.raises(TalBswError):
            srv.poll(123456789)
    assert infos[0].status == TAL_OK and infos[2].status == TAL_OK
    assert infos[1].status == TAL_EDOMAIN and infos[1].bad_pair == 7
    assert empty.status == TAL_OK
    _same(exp[0:1000], got[0:1000], "request before the bad one")
    _same(exp[2000:3000], got[2000:3000], "request after the bad one")
    keep = np.r_[1000:bad_pair, bad_pair + 1:2000]
    _same(exp[keep], got[keep], "good pairs of the bad request")


def test_serving_one_large_tick_is_exact(c3):
    """A tick run like the batched form (one launch per non-empty segment, each
    on its own stream while they last, the shortest-query ones queued behind
    the shortest before them): every segment of the C3 mix in one request, and
    the outputs equal the reference's."""
    wl, b, P, exp = c3
    with _bsw(P) as bsw, tal_bsw.BswServer(bsw, pool_bytes=1 << 30, latency_pairs=-1) as srv:
        got = b.pairs.copy()
        t = srv.submit(got, b.ref, b.qer, w=100, wpair=b.w, bits=0)
        info = _wait(srv, t)
        assert info.status == TAL_OK and info.tick_requests == 1
    _same(exp, got, "one large tick")
