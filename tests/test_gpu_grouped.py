"""Grouped rounding: one launch over many tensors with per-tensor formats;
every task bit-identical to the oracle (and so to the single-tensor path)."""
import numpy as np
import pytest
import torch

import lofloat_gb300 as lg
from golden_io import same_bits
from gpu_util import ofmt
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _random_tasks(count, seed, max_log2=18):
    rng = np.random.default_rng(seed)
    xs, fmts, modes, lens, seeds = [], [], [], [], []
    for i in range(count):
        n = int(2 ** rng.uniform(0, max_log2))
        x = (rng.standard_normal(n) * 2.0 ** rng.uniform(-10, 10)).astype(np.float32)
        e = int(rng.integers(2, 9))
        m = int(rng.integers(1, 11))
        sat = bool(rng.integers(0, 2))
        fmts.append(lg.make_format(e, m, saturating=sat))
        modes.append(int(rng.choice([0, 1, 12, 3, 5, 8, 10])))
        lens.append(int(rng.integers(1, 9)) if modes[-1] in (3, 8) else 0)
        seeds.append(int(rng.integers(0, 2**63)))
        xs.append(x)
    return xs, fmts, modes, lens, seeds


def test_grouped_matches_oracle():
    xs, fmts, modes, lens, seeds = _random_tasks(96, 0)
    ins = [torch.from_numpy(x).cuda() for x in xs]
    outs = [torch.empty_like(t) for t in ins]
    offsets = [i * 7 for i in range(len(xs))]
    g = lg.GroupedRound(ins, outs, fmts, modes, stoch_lens=lens, seeds=seeds, offsets=offsets)
    g()
    torch.cuda.synchronize()
    for i, x in enumerate(xs):
        want = O.round(x, ofmt(fmts[i]), modes[i], lens[i], seed=seeds[i], offset=offsets[i])
        assert same_bits(outs[i].cpu().numpy(), want), i


def test_grouped_graph_replay_and_misaligned():
    xs, fmts, modes, lens, seeds = _random_tasks(40, 1, max_log2=16)
    base = torch.from_numpy(np.concatenate(xs + [np.zeros(1, np.float32)])).cuda()
    # slices of one buffer: most start off a 16-byte boundary
    ins, pos = [], 1
    flat = torch.cat([torch.zeros(1, device="cuda"), base])
    for x in xs:
        ins.append(flat[pos:pos + x.size])
        pos += x.size
    outs = [torch.empty(x.size, device="cuda")[:] for x in xs]
    g = lg.GroupedRound(ins, outs, fmts, modes, stoch_lens=lens, seeds=seeds)
    g.capture()
    for o in outs:
        o.zero_()
    g.replay()
    torch.cuda.synchronize()
    for i, x in enumerate(xs):
        want = O.round(x, ofmt(fmts[i]), modes[i], lens[i], seed=seeds[i], offset=0)
        assert same_bits(outs[i].cpu().numpy(), want), i


def test_grouped_single_task_equals_virtual_round():
    x = torch.randn(1_000_003, device="cuda") * 100
    f = lg.create_p3109_params(8, 4)
    y = torch.empty_like(x)
    lg.GroupedRound([x], [y], [f], [3], stoch_lens=[8], seeds=[5])()
    ref = lg.virtual_round(x, f, round_mode=3, stoch_len=8, seed=5, offset=0)
    assert torch.equal(y, ref)


@pytest.mark.parametrize("item", [1 << 10, 1 << 14, 1 << 17, "auto"])
def test_grouped_item_sizes(item, tmp_path, monkeypatch):
    """Any work-item size (and the timed choice) gives the oracle's bits."""
    monkeypatch.setattr(lg.autotune, "CACHE_PATH", str(tmp_path / "tune.json"))
    xs, fmts, modes, lens, seeds = _random_tasks(48, 3)
    ins = [torch.from_numpy(x).cuda() for x in xs]
    outs = [torch.empty_like(t) for t in ins]
    g = lg.GroupedRound(ins, outs, fmts, modes, stoch_lens=lens, seeds=seeds, item=item)
    if item == "auto":
        assert g.item in lg.grouped.ITEM_CANDIDATES and len(g.tuning_ms) == 4
        again = lg.GroupedRound(ins, outs, fmts, modes, stoch_lens=lens, seeds=seeds, item="auto")
        assert again.item == g.item and again.tuning_ms == {}   # from the cache
    for o in outs:
        o.zero_()
    g()
    torch.cuda.synchronize()
    for i, x in enumerate(xs):
        want = O.round(x, ofmt(fmts[i]), modes[i], lens[i], seed=seeds[i], offset=0)
        assert same_bits(outs[i].cpu().numpy(), want), i
