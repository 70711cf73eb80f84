"""Helpers shared by the GPU parity tests."""
import numpy as np
import torch

from oracle import oracle as O


def dev():
    return torch.device("cuda:0")


def to_gpu(a: np.ndarray) -> torch.Tensor:
    if a.dtype == np.uint16:
        return torch.from_numpy(a.view(np.int16).copy()).to(dev()).view(torch.float16)
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev())


def from_gpu(t: torch.Tensor) -> np.ndarray:
    t = t.detach().cpu()
    if t.dtype == torch.float16:
        return t.view(torch.int16).numpy().view(np.uint16)
    return t.numpy()


def ofmt(d):
    """oracle Format from a FloatFormatDescriptor."""
    return O.Format(d.total_bits, d.mantissa_bits, d.bias, int(d.inf_behavior), int(d.nan_behavior),
                    int(d.signedness), 0)


def round_data_2p24(n=1 << 24, seed=0):
    """N(0,1)·2^u, u ~ U{-20..20}, float32 (the plain-rounding workload)."""
    g = torch.Generator().manual_seed(seed)
    x = torch.randn(n, generator=g, dtype=torch.float32)
    u = torch.randint(-20, 21, (n,), generator=g, dtype=torch.int32)
    return (x * torch.exp2(u.float())).numpy()


def mx_matrix_data(rows=8192, cols=8192, seed=2):
    """N(0,1) with 1% of elements scaled by 2^12, float32 (the MX workload)."""
    g = torch.Generator().manual_seed(seed)
    x = torch.randn(rows * cols, generator=g, dtype=torch.float32)
    mask = torch.rand(rows * cols, generator=g) < 0.01
    x[mask] *= 4096.0
    return x.numpy().reshape(rows, cols)


def mismatch_report(x, got, want, limit=5):
    u = {2: np.uint16, 4: np.uint32, 8: np.uint64}[got.dtype.itemsize]
    g, w = got.view(u).ravel(), want.view(u).ravel()
    idx = np.nonzero(g != w)[0]
    xs = x.ravel()
    return f"{idx.size} mismatches; first: " + ", ".join(
        f"[{i}] x={xs[i]!r} got={got.ravel()[i]!r} want={want.ravel()[i]!r}" for i in idx[:limit])
