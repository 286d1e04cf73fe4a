"""The multi-rank path of the benchmark (replicas: one process per GPU, no
data-path exchange) with world size 2 on the gloo backend, on CPU: the timing
reductions every rank sees and the whole-job throughput built from them."""
import os
import socket

import torch
import torch.multiprocessing as mp

from vcfpop_gb300 import replicas


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    r, w, local = replicas.init("gloo")
    replicas.barrier()
    ms = 10.0 + 5.0 * r                       # the ranks' own timed regions
    slowest = replicas.max_over_ranks(ms)
    units = replicas.sum_over_ranks(1000.0)   # each rank processed the same work
    replicas.barrier()
    replicas.finish()
    out.put((r, w, local, slowest, units, units / (slowest / 1e3)))


def test_two_gloo_ranks_agree_on_the_job_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [x[0] for x in res] == [0, 1] and all(x[1] == 2 for x in res)
    for r, w, local, slowest, units, rate in res:
        assert local == r
        assert slowest == 15.0                 # the max over ranks, on every rank
        assert units == 2000.0
        assert abs(rate - 2000.0 / 0.015) < 1e-6


def test_single_process_needs_no_group():
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    assert replicas.init("gloo") == (0, 1, 0)
    assert not torch.distributed.is_initialized()
    assert replicas.max_over_ranks(3.0) == 3.0 and replicas.sum_over_ranks(2.0) == 2.0
