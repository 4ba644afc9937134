"""The multi-GPU form of bench.py (replicas only: every rank anneals its own
populations, no data-path collective) on two gloo ranks on the CPU: rank
setup, distinct per-rank seeds, the whole-job reduction (slowest rank's time,
all ranks' attempts), and the reference arm's rank-0-only rule."""
import os
import socket
import sys

import pytest

from conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, _, ws, dist = bench.dist_init()
    # rank r: (10 + 2r) ms for 100 (r + 1) attempts
    got = bench.reduce_over_ranks(dist, "cpu", 10.0 + 2 * r, 100.0 * (r + 1))
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, ws, got, bench.rank_seed(r)))


def test_two_ranks_reduce_to_whole_job_figures():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get() for _ in range(2))
    assert [x[0] for x in res] == [0, 1] and all(x[1] == 2 for x in res)
    assert res[0][2] == res[1][2] == (12.0, 300.0)  # max time, summed attempts
    assert res[0][3] != res[1][3]                   # independent replicas per rank


def test_single_rank_reduction_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(None, "cpu", 3.5, 7.0) == (3.5, 7.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    assert bench.run_reference(bench.parse_args(["--impl", "reference"])) is None
