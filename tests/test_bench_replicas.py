"""The benchmark's multi-process form (one independent replica per GPU, no data exchange):
two gloo ranks on the CPU take the barriers around the timed region and agree on the max
over ranks of their times, which the whole-job throughput divides by."""
import importlib.util
import multiprocessing as mp
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    r, w, loc = bench.dist_info()
    reps = bench.Replicas(w)
    reps.barrier()
    t = reps.max(10.0 + 5.0 * r)  # rank 1 is the slower replica
    reps.barrier()
    q.put((r, w, loc, t))
    reps.dist.destroy_process_group()


def test_replicas_barrier_and_max_over_ranks():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 0, 15.0), (1, 2, 1, 15.0)]


def test_single_process_needs_no_group():
    spec = importlib.util.spec_from_file_location("bench_mod1", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    reps = bench.Replicas(1)
    reps.barrier()
    assert reps.dist is None and reps.max(3.5) == 3.5
