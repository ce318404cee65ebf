"""The replica path of bench.py on the CPU: under torchrun every GPU runs its
own replica, the ranks reduce their timed region to the slowest one, and the
whole-job rate counts the work of all ranks; the reference arm runs on rank 0
only.  Two gloo ranks (spawned processes, rendezvous on 127.0.0.1) stand in for
two GPUs."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        r, w, _ = bench.dist_env()
        # replica r took 10 + r ms for 1000 units of work
        ms = bench.max_over_ranks(10.0 + rank, w, device="cpu")
        rate = bench.job_rate(w, 1000, ms / 1e3)
        dist.barrier()
        q.put((rank, r, w, ms, rate))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_time_and_the_whole_job_rate():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    for rank, r, w, ms, rate in res:
        assert (r, w) == (rank, 2)
        assert ms == 11.0  # the slower replica's time, on every rank
        assert rate == pytest.approx(2 * 1000 / 0.011)


def test_single_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.job_rate(1, 100, 0.5) == 200.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    # rank 1 returns before it looks at its arguments or does any work
    assert bench.run_reference(None) == 0
