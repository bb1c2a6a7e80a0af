"""Multi-process (world size 2, gloo, CPU) checks of the replica path: the
footprint-balanced assignment of independent systems to ranks, the
max-over-ranks timing reduction bench.py uses, and a rank that fails
between steps being detected by the others instead of hanging them."""
import datetime
import os
import socket

import torch.multiprocessing as mp

from gbfv import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _init(rank, world, port, timeout_s=20):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=timeout_s))
    return dist


def _sizes():
    return [10000 + 7919 * i % 190000 for i in range(37)]


def _worker_assign(rank, world, port, q):
    dist = _init(rank, world, port)
    sizes = _sizes()
    mine = replicas.assign(sizes, world)[rank]
    work = sum(sizes[i] for i in mine)
    ms, tot = replicas.reduce_timing(10.0 + rank, work)
    got = [None] * world
    dist.all_gather_object(got, mine)
    q.put((rank, ms, tot, got))
    dist.destroy_process_group()


def test_assignment_and_timing_reduction_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker_assign, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    sizes = _sizes()
    for rank, ms, tot, got in res:
        assert ms == 11.0                      # max over ranks
        assert tot == sum(sizes)               # every system counted once
        flat = sorted(i for part in got for i in part)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[i] for i in part) for part in got]
        assert max(loads) - min(loads) <= max(sizes)


def test_assign_balances_and_is_deterministic():
    sizes = [5, 9, 3, 3, 8, 1, 7]
    a = replicas.assign(sizes, 3)
    assert a == replicas.assign(sizes, 3)
    assert sorted(i for p in a for i in p) == list(range(7))
    loads = [sum(sizes[i] for i in p) for p in a]
    assert max(loads) <= 13
    assert replicas.assign(sizes, 1) == [list(range(7))]


def _worker_fail(rank, world, port, q):
    _init(rank, world, port, timeout_s=10)
    replicas.reduce_timing(1.0, 1.0)           # one healthy step on both ranks
    if rank == 1:
        q.put((rank, "left"))
        q.close()
        q.join_thread()                        # the message is out before the process goes
        os._exit(3)                            # leaves between steps, nothing in flight
    try:
        replicas.reduce_timing(2.0, 1.0)
        q.put((rank, "no error"))
    except Exception as e:                     # the peer is gone: the collective fails
        q.put((rank, "error: " + type(e).__name__))


def test_rank_leaving_is_detected_not_hung():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker_fail, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode is not None          # neither process hangs
    assert res[1] == "left"
    assert res[0].startswith("error"), res[0]
