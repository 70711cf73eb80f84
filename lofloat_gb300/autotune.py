"""Grouped tensor-core GEMMs and the schedule autotuner.

``GroupedGemm`` runs many emulated-accumulation GEMMs of different shapes,
each with its own accumulator width, chunk and alpha, as one operand-split
launch plus one persistent tcgen05 launch (lofgb_gemm_grouped_launch_w, the
kernel built for the table's tile width), and can capture both in a CUDA
graph.

The tile shape (128 x 128; 128 x 64: twice the tiles, finer load balance
over uneven GEMMs, more operand traffic per product; 128 x 256: half the
tiles, one MMA per 256 columns) and the tile schedule —
the order in which the persistent CTAs take the output tiles of all GEMMs —
decide load balance when the GEMMs differ in size. ``GroupedGemm(...,
schedule="auto")`` times every (shape, schedule) pair the library offers
(shapes 128x128, 128x64 and 128x256; task order, longest-K first dealt round-robin,
longest-K first dealt boustrophedon) on the actual problem, keeps the
fastest, and caches the choice in a JSON table keyed by the problem's shape
signature (bucketed to powers of two), so later problems of the same shape
reuse it without timing. A choice is named "<shape>/<schedule>", e.g.
"128x64/lpt_snake"; a bare schedule name means the 128 x 128 tile.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import threading

import numpy as np
import torch

from . import _native
from ._native import LofgbGemmTask, check
from .binding import _stream

SCHEDULES = {"task": 0, "lpt": 1, "lpt_snake": 2}
TILES = {"128x128": 0, "128x64": 16, "128x256": 32}   # LOFGB_GROUPED_TILE_N64 / _N256
TILE_N = {"128x128": 128, "128x64": 64, "128x256": 256}
CHOICES = [f"{t}/{s}" for t in TILES for s in SCHEDULES]


def _code(choice: str) -> int:
    """Library schedule code of "<shape>/<schedule>" (or a bare schedule)."""
    tile, _, sched = choice.rpartition("/")
    return TILES[tile or "128x128"] | SCHEDULES[sched]
CACHE_PATH = os.environ.get(
    "LOFGB_AUTOTUNE_CACHE",
    os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json"))
_cache_lock = threading.Lock()


def _bucket(v: int) -> int:
    return 1 << max(0, int(v - 1).bit_length())


def signature(shapes) -> str:
    """Shape signature of a grouped problem: sorted (M, N, K, chunk) buckets."""
    b = sorted((_bucket(m), _bucket(n), _bucket(k), c) for m, n, k, c in shapes)
    return json.dumps(b)


def round_signature(sizes_modes) -> str:
    """Signature of a grouped rounding problem: sorted (size bucket, mode)."""
    return "round:" + json.dumps(sorted((_bucket(n), int(m)) for n, m in sizes_modes))


def _load_cache() -> dict:
    try:
        with open(CACHE_PATH) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store_cache(sig: str, entry: dict) -> None:
    with _cache_lock:
        cache = _load_cache()
        cache[sig] = entry
        os.makedirs(os.path.dirname(CACHE_PATH), exist_ok=True)
        tmp = CACHE_PATH + f".tmp{os.getpid()}"
        with open(tmp, "w") as fh:
            json.dump(cache, fh, indent=1, sort_keys=True)
        os.replace(tmp, CACHE_PATH)


class GroupedGemm:
    """tasks: list of dicts with keys A, B, D (CUDA float32 tensors), and
    optionally trans_a, trans_b, accum_mant_bits (10), alpha (1.0), chunk (32)."""

    def __init__(self, tasks, schedule="auto", grid: int = 0, tune_reps: int = 3):
        if not tasks:
            raise ValueError("no tasks")
        self.device = tasks[0]["A"].device
        self.tasks = tasks
        n = len(tasks)
        arr = (LofgbGemmTask * n)()
        shapes = []
        for i, t in enumerate(tasks):
            A, B, D = t["A"], t["B"], t["D"]
            for x in (A, B, D):
                if x.dtype != torch.float32 or not x.is_cuda or not x.is_contiguous() or x.dim() != 2:
                    raise RuntimeError("grouped GEMM: contiguous 2-D float32 CUDA tensors only")
            ta, tb = int(t.get("trans_a", 0)), int(t.get("trans_b", 0))
            M, K = (A.shape[1], A.shape[0]) if ta else (A.shape[0], A.shape[1])
            Kb, N = (B.shape[1], B.shape[0]) if tb else (B.shape[0], B.shape[1])
            if K != Kb or tuple(D.shape) != (M, N):
                raise RuntimeError(f"grouped GEMM task {i}: shapes do not match")
            chunk = int(t.get("chunk", 32))
            arr[i] = LofgbGemmTask(A.data_ptr(), A.shape[1], B.data_ptr(), B.shape[1], D.data_ptr(), N,
                                   ta, tb, M, N, K, int(t.get("accum_mant_bits", 10)),
                                   float(t.get("alpha", 1.0)), chunk)
            shapes.append((M, N, K, chunk))
        self._arr = arr
        self.flops = sum(2.0 * m * n * k for m, n, k, _ in shapes)
        L = _native.lib()
        self.ws = torch.empty(max(1024, int(L.lofgb_gemm_grouped_workspace_size(arr, n))),
                              dtype=torch.uint8, device=self.device)
        self.table_bytes = int(L.lofgb_gemm_grouped_table_size(arr, n))
        self.grid = int(grid)
        self.signature = signature(shapes)
        self.graph = None
        if schedule == "auto":
            cached = _load_cache().get(self.signature)
            if cached is not None and cached.get("schedule") not in CHOICES:
                cached = None   # an entry from before tile shapes were tuned
            if cached is not None:
                self.schedule = cached["schedule"]
                self.tuning = cached
            else:
                self.schedule, self.tuning = self._tune(tune_reps)
        else:
            self.schedule = schedule
            self.tuning = None
        self._prepare(self.schedule)

    def _prepare(self, schedule: str) -> None:
        L = _native.lib()
        host = np.zeros(self.table_bytes, np.uint8)
        nt, si = C.c_int64(0), C.c_int64(0)
        with torch.cuda.device(self.device):
            check(L.lofgb_gemm_grouped_prepare(self._arr, len(self.tasks), self.ws.data_ptr(),
                                               self.ws.numel(), _code(schedule), self.grid,
                                               host.ctypes.data_as(C.c_void_p), self.table_bytes,
                                               C.byref(nt), C.byref(si)), "gemm_grouped_prepare")
        self.table = torch.from_numpy(host).to(self.device)
        self.num_tiles, self.split_items = int(nt.value), int(si.value)
        self.tile_n = TILE_N[schedule.rpartition("/")[0] or "128x128"]
        self.graph = None

    def _tune(self, reps: int):
        times = {}
        for name in CHOICES:
            self._prepare(name)
            self()  # warm up
            torch.cuda.synchronize(self.device)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            for _ in range(reps):
                self()
            e.record()
            torch.cuda.synchronize(self.device)
            times[name] = s.elapsed_time(e) / reps
        best = min(times, key=times.get)
        entry = {"schedule": best, "ms": times}
        _store_cache(self.signature, entry)
        return best, entry

    def __call__(self):
        with torch.cuda.device(self.device):
            check(_native.lib().lofgb_gemm_grouped_launch_w(self.table.data_ptr(), self.num_tiles,
                                                            self.split_items, self.grid, self.tile_n,
                                                            _stream(self.table)), "gemm_grouped_launch")

    def status(self) -> int:
        """Device status word (0, or LOFGB_ERR_TIMEOUT); synchronises."""
        return int(self.ws[:4].view(torch.int32).item())

    def capture(self):
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
