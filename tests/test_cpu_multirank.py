"""World-size-2 tests of the multi-process path, on CPU with the gloo backend.

Under torchrun every rank runs an independent replica of the workload on its
own GPU: the only collectives are the barrier around the timed region and the
max over ranks of its duration. These tests run that host logic as two gloo
ranks, check that the non-zero ranks of the reference arm exit without work,
and check with the oracle the two facts that make replicas valid shards:
MX rounding split at block boundaries and the emulated GEMM split by output
rows need no exchange between ranks (each shard equals the same rows of the
whole result, bit for bit).
"""
import contextlib
import io
import os
import socket
import sys
import types

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
WORLD = 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _init(rank, port):
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=WORLD)


def _timing_rank(rank, port):
    import bench
    _init(rank, port)
    try:
        # rank 0 is the slower one for the first figure, rank 1 for the second
        mine = [2.0 - rank, 3.0 + 4.0 * rank]
        dist.barrier()
        got = bench.max_over_ranks(dist, mine, "cpu")
        assert got == [2.0, 7.0], got
        # value: both replicas' bytes over the slowest rank's time
        assert bench.whole_job_gbs(WORLD, 5, 8e9, got[0]) == pytest.approx(40.0)
    finally:
        dist.destroy_process_group()


def _shard_rank(rank, port):
    from oracle import oracle as O
    _init(rank, port)
    try:
        rng = np.random.default_rng(11)
        rows, cols, block = 64, 256, 32
        x = rng.standard_normal((rows, cols)).astype(np.float32)
        x[rng.random(x.shape) < 0.02] *= 4096.0
        ef, sf = O.fmt(8, 3, 7), O.fmt(8, 0, 127, saturating=False, signed=False)
        lo, hi = rank * rows // WORLD, (rank + 1) * rows // WORLD
        part = O.mx_round(x[lo:hi], block, ef, sf)
        parts = [torch.empty((rows // WORLD, cols), dtype=torch.float32) for _ in range(WORLD)]
        dist.all_gather(parts, torch.from_numpy(part))
        whole = O.mx_round(x, block, ef, sf)
        assert np.array_equal(torch.cat(parts).numpy().view(np.uint32), whole.view(np.uint32))

        M, N, K = 48, 40, 96
        A = rng.standard_normal((M, K)).astype(np.float32)
        B = rng.standard_normal((K, N)).astype(np.float32)
        r0, nr = rank * M // WORLD, M // WORLD
        d = O.gemm_rows(A, B, 10, r0, nr)
        ds = [torch.empty((nr, N), dtype=torch.float32) for _ in range(WORLD)]
        dist.all_gather(ds, torch.from_numpy(np.ascontiguousarray(d)))
        full = O.gemm(A, B, 10)
        assert np.array_equal(torch.cat(ds).numpy().view(np.uint32), full.view(np.uint32))
    finally:
        dist.destroy_process_group()


def _spawn(fn):
    mp.spawn(fn, args=(_free_port(),), nprocs=WORLD, join=True)


def test_max_over_ranks_and_whole_job_value():
    _spawn(_timing_rank)


def test_row_shards_equal_whole_result():
    pytest.importorskip("oracle.oracle")
    _spawn(_shard_rank)


def test_reference_arm_runs_on_rank_zero_only():
    import bench
    args = types.SimpleNamespace(steps=1, warmup=0, gpus=WORLD)
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        bench.run_reference(args, WORLD, 1)
    assert out.getvalue() == ""
