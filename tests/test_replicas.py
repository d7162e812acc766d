"""Host-side logic of bench.py's multi-GPU mode on CPU: two ranks over gloo.

The engine does not shard: `bench.py --gpus N` runs N independent replicas of
the workload (one per GPU), which meet only at barriers and in the max-over-ranks
step time.  These ranks exercise that logic without a GPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(WORLD_SIZE=str(ws), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    import torch.distributed as dist
    got_ws, got_rank, _ = bench.dist_setup()
    assert dist.get_backend() == "gloo"
    bench.barrier(got_ws)
    t = 0.5 + 0.25 * got_rank  # the replicas' step times differ
    tmax = bench.allmax(got_ws, t)
    out[got_rank] = (got_ws, tmax, bench.replica_value(got_ws, 86016, tmax))
    bench.barrier(got_ws)
    dist.destroy_process_group()


def test_two_replicas_over_gloo():
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, ws, port, out)) for r in range(ws)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        res = dict(out)
    assert sorted(res) == [0, 1]
    for r in range(ws):
        got_ws, tmax, value = res[r]
        assert got_ws == 2
        assert tmax == pytest.approx(0.75)  # the slowest rank's time on every rank
        assert value == pytest.approx(2 * 86016 / 0.75)

