"""The multi-rank path on the CPU: two `gloo` ranks on 127.0.0.1.

One all-vs-all splits into row ranges of nearly equal pair counts
(bs_partition_rows, host only), one range per GPU, with no exchange between
ranks.  Here each rank computes its range with the FP64 oracle (the GPU's
part on a GPU machine) into its slice of the packed triangle; the slices gathered
on rank 0 must be the full matrix, each pair exactly once.  The bench's
whole-job rate takes the slowest rank's time (all_reduce MAX), which a rank
with a planted slow time must set.
"""
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, n, L, result_dir):
    import sys

    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from bench import whole_job_rate
        from bioshell_gb300 import synth
        from bioshell_gb300.crmsd import partition_rows
        from oracle import oracle

        rng = np.random.default_rng(3)
        x = synth.decoys(synth.base_chain(L, rng), n, rng, near_dup_frac=0.1)
        b = partition_rows(n, world)
        lo, hi = int(b[rank]), int(b[rank + 1])
        # this rank's rows: pairs (i, j), lo <= i < hi, j > i, in packed order
        ii = np.concatenate([np.full(n - 1 - i, i, dtype=np.int64) for i in range(lo, hi)] or [np.zeros(0, np.int64)])
        jj = np.concatenate([np.arange(i + 1, n, dtype=np.int64) for i in range(lo, hi)] or [np.zeros(0, np.int64)])
        part = oracle.crmsd_pairs(x, ii, jj, nthreads=1)
        counts = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(counts, torch.tensor([part.size], dtype=torch.int64))
        width = int(max(c.item() for c in counts))
        buf = torch.zeros(width, dtype=torch.float64)
        buf[: part.size] = torch.from_numpy(part)
        slices = [torch.zeros(width, dtype=torch.float64) for _ in range(world)]
        dist.all_gather(slices, buf)
        # the slowest rank sets the job's time: rank 1 plants 3x the time
        ms, rate = whole_job_rate(10.0 * (3 if rank == 1 else 1), n * (n - 1) / 2 / world, 2, world, dist,
                                  device="cpu")
        if rank == 0:
            full = np.concatenate([s[: int(c.item())].numpy() for s, c in zip(slices, counts)])
            np.savez(os.path.join(result_dir, "r0.npz"), full=full, ref=oracle.crmsd_all_vs_all(x, nthreads=1),
                     counts=np.array([int(c.item()) for c in counts]), bounds=b, ms=ms, rate=rate)
    finally:
        dist.destroy_process_group()


def test_row_ranges_over_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    from oracle import oracle

    oracle.build()
    n, L, world = 203, 24, 2
    mp.start_processes(_rank_main, args=(world, _free_port(), n, L, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    r = np.load(tmp_path / "r0.npz")
    # the ranges tile the rows, and their pairs make the full triangle in order
    b = r["bounds"]
    assert b[0] == 0 and b[-1] == n and np.all(np.diff(b) >= 0)
    assert all(v % 40 == 0 or v == n for v in b[1:-1])
    assert r["counts"].sum() == n * (n - 1) // 2
    np.testing.assert_array_equal(r["full"], r["ref"])
    # balanced to within one 40-row block of pairs
    assert abs(int(r["counts"][0]) - int(r["counts"][1])) <= 40 * n
    # the whole job's time is the slowest rank's
    assert float(r["ms"]) == 30.0
    assert float(r["rate"]) == pytest.approx(n * (n - 1) / 2 * 2 / 30e-3)
