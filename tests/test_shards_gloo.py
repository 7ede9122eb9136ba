"""Multi-rank path of the benchmark on CPU (gloo, world size 2): each rank takes
its own shard of pairs (pairs [rank*n, (rank+1)*n) of the seeded workload), no
data-path collective, and the ranks combine only their timings and counts.
The shards together are exactly the single-process workload, and the outputs
per shard (scored here by the oracle, which stands in for the GPU on a CPU
host) equal the single-process ones."""
import os
import socket
import sys
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, out_dir, n):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    for p in (ROOT, os.path.join(ROOT, "trans-omics-acceleration-library_gb300"),
              os.path.join(ROOT, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import bench
    import oracle
    from tal_bsw import synth
    d = bench.Dist("gloo")
    assert (d.ws, d.rank) == (ws, rank)
    wl = synth.C2
    b = synth.generate(wl, n, first=rank * n)
    got = oracle.vector(b.pairs, b.ref, b.qer, wl.w, wl.params(), bits=16, lanes=1)
    cells = float(got["score"].sum())
    total = d.sum(cells)
    slowest = d.max(float(rank + 1))
    d.barrier()
    np.savez(os.path.join(out_dir, f"rank{rank}.npz"), pairs=got, total=total, slowest=slowest,
             cells=cells)
    d.close()


def test_two_gloo_ranks_shard_the_workload():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import oracle
    from tal_bsw import synth
    from tal_bsw.seqpair import outputs
    n = 48
    with tempfile.TemporaryDirectory() as tmp:
        mp.start_processes(_rank, args=(2, _free_port(), tmp, n), nprocs=2, join=True,
                           start_method="spawn")
        r = [np.load(os.path.join(tmp, f"rank{k}.npz")) for k in range(2)]
    whole = synth.generate(synth.C2, 2 * n)
    exp = oracle.vector(whole.pairs, whole.ref, whole.qer, synth.C2.w, synth.C2.params(), bits=16,
                        lanes=1)
    got = np.concatenate([r[0]["pairs"], r[1]["pairs"]])
    # same pairs (lengths, h0) and the same outputs as one process over 2n pairs
    for f in ("len1", "len2", "h0"):
        assert (got[f] == whole.pairs[f]).all()
    assert (outputs(got) == outputs(exp)).all()
    assert float(r[0]["total"]) == float(r[1]["total"]) == float(r[0]["cells"] + r[1]["cells"])
    assert float(r[0]["slowest"]) == float(r[1]["slowest"]) == 2.0
