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
from .binding import FloatFormatDescriptor, _stream


class GroupedRound:
    def __init__(self, ins, outs, formats, modes, stoch_lens=None, scales=None, seeds=None,
                 offsets=None):
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
        L = _native.lib()
        nbytes = int(L.lofgb_round_grouped_table_size(n))
        host = np.zeros(max(nbytes, 1), np.uint8)
        items = C.c_int64(0)
        check(L.lofgb_round_grouped_prepare(tasks, n, host.ctypes.data_as(C.c_void_p), nbytes,
                                            C.byref(items)), "grouped_round_prepare")
        self.ntasks = n
        self.num_items = int(items.value)
        self.table = torch.from_numpy(host).to(dev)  # caching allocator: 512-byte aligned
        self.bytes = sum(8 * x.numel() for x in ins)
        self.graph = None

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
