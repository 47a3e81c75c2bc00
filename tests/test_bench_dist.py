"""bench.py's multi-rank path on CPU: world size 2 over gloo (127.0.0.1).
Replicas run independently; the slowest rank's time and the whole-job rate
are agreed on by all ranks, and the reference arm runs on rank 0 only."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    bench.barrier(ws)
    ms = 100.0 + 50.0 * rank  # per-rank time of 10 steps
    slowest = bench.max_over_ranks(ws, ms, device="cpu")
    q.put((rank, slowest, bench.throughput(ws, 10, slowest)))
    dist.destroy_process_group()


def test_two_ranks_agree_on_slowest_time_and_rate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [150.0, 150.0]
    assert all(abs(r[2] - 2 * 10 / 0.150) < 1e-9 for r in res)


def test_reference_arm_is_rank0_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        warmup, steps, n, log2_c, gpus = 1, 1, 4, 1, 2

    bench.run_reference(A, 2, 1)  # rank 1: no work, no output
    assert capsys.readouterr().out == ""
