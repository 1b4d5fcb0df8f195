"""bench.py's host logic on CPU: the replica mode on two gloo ranks, and
the whole-step byte count of its step_hbm figure.

Under torchrun every rank solves its own copy of the workload and nothing is
exchanged on the data path; the host only takes the maximum time and the sum
of the work over ranks.  These tests run that host logic (bench.Dist and
bench.whole_job_rate) in two processes on the gloo backend.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "WORLD_SIZE": str(world), "RANK": str(rank),
                       "LOCAL_RANK": str(rank), "TEA_DIST_BACKEND": "gloo"})
    import bench
    dist = bench.Dist()
    try:
        dist.barrier()
        # rank r did (r + 1) * 1000 cell-iterations in (r + 1) * 0.5 s
        work, secs = (rank + 1) * 1000.0, (rank + 1) * 0.5
        out[rank] = (dist.world, dist.max(secs), dist.sum(work),
                     bench.whole_job_rate(dist, work, secs))
        dist.barrier()
    finally:
        dist.close()


def test_two_gloo_ranks_aggregate_the_whole_job():
    world, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert sorted(res) == [0, 1]
    for r in (0, 1):
        n, tmax, total, rate = res[r]
        assert n == 2
        assert tmax == 1.0               # the slower rank's time
        assert total == 3000.0           # both ranks' work
        assert rate == 3000.0 / 1.0      # the same number on every rank


def test_single_process_needs_no_process_group():
    import bench

    class Solo(bench.Dist):
        def __init__(self):
            self.world, self.rank, self.local, self.pg = 1, 0, 0, None

    d = Solo()
    assert d.max(2.5) == 2.5 and d.sum(7.0) == 7.0
    assert bench.whole_job_rate(d, 100.0, 4.0) == 25.0


def test_step_bytes_follow_the_reference_kernels():
    """step_hbm's bytes per cell-iteration: the reference kernels' fields of
    one solver iteration, each once (PPCG: calc_w 32, calc_ur 88, init_sd
    48, ten inner steps of update_r 56 and calc_sd 56, r.z 16, calc_p 24,
    over 11 cell-iterations)."""
    import bench
    assert bench.step_bytes_per_cell_iteration("ppcg4096") == (32 + 88 + 48 + 16 + 24 +
                                                              10 * (56 + 56)) / 11
    assert bench.step_bytes_per_cell_iteration("cg4096") == 32 + 88 + 24
    assert bench.step_bytes_per_cell_iteration("cg512") == 32 + 64 + 24
    assert bench.step_bytes_per_cell_iteration("cheby4096") == 96 + 24
    # the one-pass inner step counts both reference kernels' fields
    kb = bench.KERNEL_BYTES
    assert kb["tea_leaf_ppcg_solve_inner_step"]["jac_block"] == \
        kb["tea_leaf_ppcg_solve_update_r"] + kb["tea_leaf_ppcg_solve_calc_sd"]["jac_block"]
