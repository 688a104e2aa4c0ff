"""The N>1 path of bench.py as world_size-2 gloo ranks on CPU: a replica
run (one process per GPU, each rendering its own frames) reduces its
timings once, after the timed region -- each time the maximum over the
ranks, each unit count the sum -- and the CPU reference arm runs on rank 0
alone."""
import multiprocessing as mp
import os
import socket


ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    times, units = bench.job_totals([1.0 + rank, 5.0 - rank], [100 * (rank + 1), 7], dist, "cpu")
    q.put((rank, times, units))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timings_reduce_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict()
    for _ in range(2):
        r, times, units = q.get(timeout=120)
        got[r] = (times, units)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        assert got[r] == ([2.0, 5.0], [300, 14]), got


def test_single_process_totals_are_its_own():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_totals([1.5, 2.5], [10, 20]) == ([1.5, 2.5], [10, 20])


def test_reference_arm_runs_on_rank_zero_only(capsys):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    old = sys.argv
    sys.argv = ["bench.py", "--impl", "reference"]
    try:
        args = bench.parse()
    finally:
        sys.argv = old
    bench.run_reference(args, 1, 2)     # rank 1 of 2: no work, no line
    assert capsys.readouterr().out == ""
