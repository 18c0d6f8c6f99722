"""The multi-GPU path is replicas only (frames and codewords are independent; no exchange step): bench.py's rank
plumbing (barrier, max over ranks of the step time, the whole-job aggregate) run as two gloo ranks on the CPU, and a
batch split across ranks decoding to the same results as the whole batch."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def worker(rank, ws, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(ws), "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import torch.distributed as dist
    import bench
    import oracle
    from lizard_gb300_testing import synth
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    # each replica decodes its own shard of one batch with the CPU decoder (the oracle stands in for a GPU here)
    b = synth.ldpc_batch(64, seed=9)
    lo, hi = rank * 32, (rank + 1) * 32
    n_end = int(b["offsets"][hi]) if hi < 64 else b["llr"].size
    bits, its, ok = oracle.ldpc_batch(oracle.port(), b["llr"][int(b["offsets"][lo]):n_end], b["offsets"][lo:hi] - b["offsets"][lo],
                                      b["rates"][lo:hi], 20, 9, 0.95)
    bench.barrier(ws)
    t = bench.max_over_ranks(float(rank + 1), ws)
    out[rank] = (t, its.tolist(), ok.tolist())
    dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_replicas_over_gloo():
    import oracle
    from lizard_gb300_testing import synth
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(240)
        assert p.exitcode == 0
    # the max over ranks is the slowest rank's time on every rank
    assert out[0][0] == 2.0 and out[1][0] == 2.0
    b = synth.ldpc_batch(64, seed=9)
    _, its, ok = oracle.ldpc_batch(oracle.port(), b["llr"], b["offsets"], b["rates"], 20, 9, 0.95)
    assert np.array_equal(np.array(out[0][1] + out[1][1]), its)
    assert np.array_equal(np.array(out[0][2] + out[1][2]), ok)
