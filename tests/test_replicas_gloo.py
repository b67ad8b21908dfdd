"""The N > 1 reporting path of bench.py on CPU: two gloo ranks, each timing
its own replica, report the slowest rank's duration and the units of all
ranks (the multi-GPU run is replicas only: no data-path collective)."""
import os
import socket


ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        ms, units = bench.aggregate_over_ranks(10.0 + 5.0 * rank, 1000 * (rank + 1), "cpu")
        out_q.put((rank, ms, units))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_max_time_and_summed_units():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(results) == [(0, 15.0, 3000), (1, 15.0, 3000)]


def test_single_process_is_identity():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_over_ranks(12.5, 7, "cpu") == (12.5, 7)
