"""Grouped rounding: hundreds of FP32 tensors, each with its own format, mode,
scale and RNG stream, rounded by one persistent kernel launch
(lofgb_round_grouped_f32), optionally replayed from a captured CUDA graph.

    g = GroupedRound(ins, outs, formats, modes, stoch_lens=..., seeds=...)
    g()                 # one launch on the current stream
    g.capture()         # capture that launch in a CUDA graph
    g.replay()          # replay it

Each task gives the same bits as ``virtual_round(in, fmt, mode, stoch_len,
scale, seed=..., offset=...)`` on that tensor alone.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native
from ._native import LofgbRoundTask, check
from .autotune import _load_cache, _store_cache, round_signature
from .binding import FloatFormatDescriptor, _stream


ITEM_CANDIDATES = (1 << 14, 1 << 15, 1 << 16, 1 << 17)


class GroupedRound:
    """`item`: elements per work item, a power of two in [2^10, 2^24], or
    "auto" to time ITEM_CANDIDATES on these tensors and keep the fastest
    (cached per problem signature, like GroupedGemm's schedule)."""

    def __init__(self, ins, outs, formats, modes, stoch_lens=None, scales=None, seeds=None,
                 offsets=None, item=1 << 16, tune_reps: int = 3):
        n = len(ins)
        if not (len(outs) == len(formats) == len(modes) == n):
            raise ValueError("ins, outs, formats and modes must have the same length")
        stoch_lens = stoch_lens or [0] * n
        scales = scales or [1.0] * n
        seeds = seeds or [0] * n
        offsets = offsets or [0] * n
        dev = None
        for x, y in zip(ins, outs):
            if x.dtype != torch.float32 or y.dtype != torch.float32:
                raise RuntimeError("grouped rounding: float32 tensors only")
            if not (x.is_cuda and y.is_cuda and x.is_contiguous() and y.is_contiguous()):
                raise RuntimeError("grouped rounding: contiguous CUDA tensors only")
            if x.numel() != y.numel():
                raise RuntimeError("grouped rounding: input and output sizes differ")
            dev = dev or x.device
        self.device = dev
        self.ins, self.outs = list(ins), list(outs)  # keep the buffers alive
        tasks = (LofgbRoundTask * n)()
        for i in range(n):
            f = formats[i]
            if not isinstance(f, FloatFormatDescriptor):
                raise TypeError("formats must be FloatFormatDescriptor objects")
            tasks[i] = LofgbRoundTask(ins[i].data_ptr(), outs[i].data_ptr(), ins[i].numel(),
                                      f.c_format, int(modes[i]), int(stoch_lens[i]),
                                      float(scales[i]), 0, int(seeds[i]) & ((1 << 64) - 1),
                                      int(offsets[i]))
        self._tasks = tasks
        self.ntasks = n
        self.bytes = sum(8 * x.numel() for x in ins)
        self.graph = None
        self.tuning_ms = {}
        if item == "auto":
            sig = round_signature([(int(x.numel()), int(m)) for x, m in zip(ins, modes)])
            cached = _load_cache().get(sig)
            if cached and cached.get("item") in ITEM_CANDIDATES:
                item = int(cached["item"])
            else:
                for cand in ITEM_CANDIDATES:
                    self._prepare(cand)
                    self.tuning_ms[cand] = self._time(tune_reps)
                item = min(self.tuning_ms, key=self.tuning_ms.get)
                _store_cache(sig, {"item": item, "ms": self.tuning_ms})
        self._prepare(int(item))

    def _prepare(self, item: int) -> None:
        L = _native.lib()
        n = self.ntasks
        nbytes = int(L.lofgb_round_grouped_table_size(n))
        host = np.zeros(max(nbytes, 1), np.uint8)
        items = C.c_int64(0)
        check(L.lofgb_round_grouped_prepare_items(self._tasks, n, host.ctypes.data_as(C.c_void_p),
                                                  nbytes, int(item), C.byref(items)),
              "grouped_round_prepare")
        self.item = int(item)
        self.num_items = int(items.value)
        self.table = torch.from_numpy(host).to(self.device)  # caching allocator: 512-byte aligned
        self.graph = None

    def _time(self, reps: int) -> float:
        self()
        torch.cuda.synchronize(self.device)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(reps):
            self()
        e.record()
        torch.cuda.synchronize(self.device)
        return s.elapsed_time(e) / reps

    def __call__(self):
        with torch.cuda.device(self.device):
            check(_native.lib().lofgb_round_grouped_f32(self.table.data_ptr(), self.ntasks,
                                                        self.num_items, _stream(self.table)),
                  "grouped_round")

    def capture(self):
        """Capture one launch in a CUDA graph (warm-up launch first)."""
        self()
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self()
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()
