"""Grouped tensor-core GEMM: every task equals the single-GEMM tensor-core
path bit for bit (the same products summed per output, whether a tile is
128 or 64 columns wide), under every tile shape and schedule, from a
captured CUDA graph, and with ragged shapes; the autotuner picks and caches
a (tile shape, schedule) pair."""
import json

import pytest
import torch

import lofloat_gb300 as lg
from lofloat_gb300 import autotune

pytestmark = pytest.mark.gpu


def _tasks(count, seed, dims=(128, 640), ragged=False):
    g = torch.Generator().manual_seed(seed)
    out = []
    for i in range(count):
        M, N, K = (int(torch.randint(dims[0], dims[1], (1,), generator=g)) for _ in range(3))
        if not ragged:
            M, N, K = (x // 64 * 64 for x in (M, N, K))
        ta, tb = i % 2, (i // 2) % 2
        A = torch.randn((K, M) if ta else (M, K), generator=g).cuda()
        B = torch.randn((N, K) if tb else (K, N), generator=g).cuda()
        out.append(dict(A=A, B=B, D=torch.empty(M, N, device="cuda"), trans_a=ta, trans_b=tb,
                        accum_mant_bits=int(7 + i % 6), alpha=float(0.5 + i % 3),
                        chunk=[16, 32, 64, 48][i % 4]))
    return out


def _reference(t):
    return lg.gemm(t["A"], t["B"], t["accum_mant_bits"], trans_a=bool(t["trans_a"]),
                   trans_b=bool(t["trans_b"]), alpha=t["alpha"], variant="tc", chunk=t["chunk"])


@pytest.mark.parametrize("schedule", ["task", "lpt", "lpt_snake", "128x64/task", "128x64/lpt",
                                      "128x64/lpt_snake", "128x256/task", "128x256/lpt",
                                      "128x256/lpt_snake"])
def test_grouped_matches_single(schedule):
    tasks = _tasks(10, 1)
    gg = lg.GroupedGemm(tasks, schedule=schedule)
    gg.ws.fill_(0xFF)  # the launch must clear the status word itself
    gg()
    torch.cuda.synchronize()
    assert gg.status() == 0
    for i, t in enumerate(tasks):
        assert torch.equal(t["D"], _reference(t)), i


@pytest.mark.parametrize("schedule", ["lpt_snake", "128x64/lpt_snake", "128x256/lpt_snake"])
def test_grouped_ragged_and_graph(schedule):
    tasks = _tasks(7, 2, dims=(1, 300), ragged=True)
    gg = lg.GroupedGemm(tasks, schedule=schedule, grid=37)
    gg.capture()
    for t in tasks:
        t["D"].zero_()
    gg.replay()
    torch.cuda.synchronize()
    assert gg.status() == 0
    for i, t in enumerate(tasks):
        assert torch.equal(t["D"], _reference(t)), i


def test_autotuner_caches(tmp_path, monkeypatch):
    monkeypatch.setattr(autotune, "CACHE_PATH", str(tmp_path / "tune.json"))
    tasks = _tasks(6, 3)
    gg = lg.GroupedGemm(tasks, schedule="auto", tune_reps=2)
    assert gg.schedule in autotune.CHOICES
    cache = json.loads((tmp_path / "tune.json").read_text())
    assert gg.signature in cache and set(cache[gg.signature]["ms"]) == set(autotune.CHOICES)
    again = lg.GroupedGemm(tasks, schedule="auto")
    assert again.schedule == gg.schedule
    again()
    torch.cuda.synchronize()
    for i, t in enumerate(tasks):
        assert torch.equal(t["D"], _reference(t)), i


@pytest.mark.parametrize("schedule", ["lpt_snake", "128x64/lpt_snake", "128x256/lpt_snake"])
def test_generic_launch_matches_width_launch(schedule):
    """lofgb_gemm_grouped_launch (tile width read from the table on the
    device) gives the bits of lofgb_gemm_grouped_launch_w (the kernel built
    for the width); a width other than the table's is refused on the device."""
    tasks = _tasks(5, 4)
    gg = lg.GroupedGemm(tasks, schedule=schedule)
    gg()
    torch.cuda.synchronize()
    want = [t["D"].clone() for t in tasks]
    for t in tasks:
        t["D"].zero_()
    L = lg._native.lib()
    stream = torch.cuda.current_stream().cuda_stream
    assert L.lofgb_gemm_grouped_launch(gg.table.data_ptr(), gg.num_tiles, gg.split_items, gg.grid,
                                       stream) == 0
    torch.cuda.synchronize()
    assert gg.status() == 0
    for t, w in zip(tasks, want):
        assert torch.equal(t["D"], w)
    other = 128 if gg.tile_n != 128 else 256
    assert L.lofgb_gemm_grouped_launch_w(gg.table.data_ptr(), gg.num_tiles, gg.split_items, gg.grid,
                                         other, stream) == 0
    torch.cuda.synchronize()
    assert gg.status() == -7   # LOFGB_ERR_UNSUPPORTED
    assert L.lofgb_gemm_grouped_launch_w(gg.table.data_ptr(), gg.num_tiles, gg.split_items, gg.grid,
                                         96, stream) == -7
