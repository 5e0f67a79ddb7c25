"""The multi-GPU form is independent replicas (bench.py --gpus N under torchrun): the ranks share
only a barrier and the maximum of their times.  Checked here with two gloo ranks on the host:
the slowest rank's time reaches every rank, the whole job's rate counts every rank's units over
that time, and a rank that never joins makes the others fail at the barrier instead of hanging."""
import datetime
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    import torch.distributed as dist
    from fdfk2d_gb300 import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=30))
    try:
        replicas.barrier()
        t = replicas.max_over_ranks(times[rank])
        rate = replicas.whole_job_rate(1000.0, t)
        replicas.barrier()
        out.put((rank, replicas.world_size(), t, rate))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    times = [0.25, 0.5]
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1]
    for rank, world, t, rate in got:
        assert world == 2
        assert t == 0.5                      # every rank sees the slowest rank's time
        assert rate == pytest.approx(4000.0)  # 2 ranks x 1000 units / 0.5 s


def _lonely_rank(port, out):
    import torch.distributed as dist
    from fdfk2d_gb300 import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    try:
        dist.init_process_group("gloo", rank=0, world_size=2, timeout=datetime.timedelta(seconds=3))
        replicas.barrier()
        out.put("joined")
    except Exception as e:   # the second rank never joins: rendezvous or barrier times out
        out.put(type(e).__name__)


def test_missing_replica_fails_instead_of_hanging():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    p = ctx.Process(target=_lonely_rank, args=(_free_port(), out))
    p.start()
    msg = out.get(timeout=120)
    p.join(timeout=60)
    assert msg != "joined"


def test_single_process_needs_no_group():
    from fdfk2d_gb300 import replicas
    assert replicas.world_size() == 1
    assert replicas.max_over_ranks(0.125) == 0.125
    assert replicas.whole_job_rate(10.0, 2.0) == 5.0
    with pytest.raises(ValueError):
        replicas.whole_job_rate(10.0, 0.0)
