"""The multi-GPU bench path is N independent replicas: each rank proves its own
seeded files and the ranks only meet at a barrier and a max of elapsed times.
This runs that coordination as two gloo ranks on the CPU."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    r, w, _ = bench.dist_env()
    ranks = bench.Ranks(w, "gloo")
    files = bench.workload_files(bench.WORKLOADS["batched"], r)
    ranks.barrier()
    slowest = ranks.max(float(10 + r))
    out.put((r, slowest, [len(d) for d, _, _ in files[:8]], files[0][1]))
    ranks.close()


def test_two_gloo_replicas_share_only_a_barrier_and_a_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, m0, sizes0, seed0), (r1, m1, sizes1, seed1) = res
    assert (r0, r1) == (0, 1)
    assert m0 == m1 == 11.0  # the slowest rank's time is the job's time
    # each replica works on its own files: different sizes and per-file seeds
    assert sizes0 != sizes1 and seed0 != seed1
