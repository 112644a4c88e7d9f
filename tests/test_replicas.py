"""Multi-GPU is replicas only: each rank runs the whole workload, the job's
time is the slowest rank's and its throughput counts every rank's work.  The
reduction runs here on two gloo ranks (CPU)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 100.0 + 50.0 * rank          # rank 1 is slower
        slowest = bench.max_over_ranks(local_ms)
        q.put((rank, slowest, bench.replica_throughput(world, 10, 1_000_000, slowest)))
    finally:
        dist.destroy_process_group()


def test_replicas_report_the_slowest_rank():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [150.0, 150.0]
    assert all(o[2] == pytest.approx(2 * 10 * 1_000_000 / 0.150) for o in out)


def test_single_process_is_unchanged():
    import bench
    assert bench.max_over_ranks(42.0) == 42.0
    assert bench.replica_throughput(1, 4, 1000, 2000.0) == 2000.0


def test_reference_arm_only_rank0_prints(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        warmup, steps, gpus = 3, 1, 2
    assert bench.run_reference_arm(Args()) is None
    assert capsys.readouterr().out == ""


def test_term_bytes_and_ops_follow_the_unit_of_work():
    """One neighbour term: the 4-byte corpus word, a 16-bit table read per
    colour channel, the map byte and a 32-bit table read per map channel."""
    import bench
    assert bench.term_bytes(3, 0) == 10 and bench.term_ops(3, 0) == 13
    assert bench.term_bytes(3, 1) == 15 and bench.term_ops(3, 1) == 16
    assert bench.term_bytes(1, 0) == 6
    assert set(bench.WAVE_DRAM_BYTES) <= {"render1024", "heal4096", "mapstyle2048", "heal256"}
