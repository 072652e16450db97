"""Multi-GPU host logic on CPU: two gloo ranks run the measurement protocol
of bench.py --gpus N (replicas on their own frames, barrier, the slowest
rank's time, whole-job throughput), as torchrun would start them."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    from sa_gb300 import replicas, synth
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    r, w, lr = replicas.rank_env()
    assert (r, w, lr) == (rank, world, rank)
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    seed = replicas.replica_seed(1, rank)
    wl = synth.make_workload(0, frames=1, seed=seed)
    units = len(wl["guesses"][0]["x"])
    dist.barrier()
    ms = 10.0 + 5.0 * rank            # the ranks' own step times
    slowest = replicas.max_over_ranks(ms, dist)
    value = replicas.job_throughput(units, world, slowest)
    gathered = [None] * world
    dist.all_gather_object(gathered, (seed, units, slowest, value))
    if rank == 0:
        out.put(gathered)
    dist.destroy_process_group()


def test_two_gloo_replicas():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (s0, u0, t0, v0), (s1, u1, t1, v1) = res
    assert s0 != s1                                   # each replica its own frames
    assert t0 == t1 == 15.0                           # both see the slowest rank
    assert v0 == v1 == pytest.approx(u0 * 2 / 0.015)  # whole-job units per second


def test_single_process_defaults(monkeypatch):
    from sa_gb300 import replicas
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert replicas.rank_env() == (0, 1, 0)
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.job_throughput(1000, 1, 500.0) == pytest.approx(2000.0)
