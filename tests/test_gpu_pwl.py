"""GPU parity of the piecewise-linear SiLU (pwl_silu) against the oracle:
bit-exact for float32, and for float64 / float16 inputs widened to float32 and
the result narrowed back, as the reference's kernel does."""
import numpy as np
import pytest
import torch

import lofloat_gb300 as lg
from golden_io import same_bits
from gpu_util import from_gpu, mismatch_report, to_gpu
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _inputs(n, R, seed):
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal(n) * R * 0.7).astype(np.float32)
    edges = np.array([0.0, -0.0, R, -R, np.nextafter(np.float32(R), np.float32(np.inf)),
                      np.nextafter(np.float32(-R), np.float32(-np.inf)), np.inf, -np.inf, np.nan,
                      1e-45, -1e-45, 3e38, -3e38], np.float32)
    k = min(n, edges.size)
    x[:k] = edges[:k]
    return x


@pytest.mark.parametrize("bits", [1, 4, 8, 12])
@pytest.mark.parametrize("method", ["uniform", "midpoint", "minimax"])
def test_f32_vs_oracle(bits, method):
    m = lg.PWLSiLU(R=6.0, lut_bits=bits, lut_method=method)
    lut = m.lut.numpy()
    x = _inputs(100_003, 6.0, bits)
    got = from_gpu(lg.pwl_silu(to_gpu(x), torch.from_numpy(lut), 6.0))
    want = O.pwl_silu(x, lut, 6.0)
    assert same_bits(got, want), mismatch_report(x, got, want)


@pytest.mark.parametrize("dtype", [np.float64, np.float16])
def test_other_dtypes(dtype):
    m = lg.PWLSiLU(R=8.0, lut_bits=5)
    lut = m.lut.numpy()
    with np.errstate(over="ignore"):
        x = _inputs(50_001, 8.0, 3).astype(dtype)
    got = lg.pwl_silu(torch.from_numpy(x).cuda(), m.lut, 8.0).cpu().numpy()
    want = O.pwl_silu(x.astype(np.float32), lut, 8.0).astype(dtype)
    assert got.dtype == dtype
    u = np.uint64 if dtype == np.float64 else np.uint16
    nan = np.isnan(got) & np.isnan(want)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    assert np.array_equal(got.view(u)[~nan], want.view(u)[~nan])


@pytest.mark.parametrize("n", [0, 1, 3, 5, 17, 1029])
def test_sizes_and_misaligned(n):
    m = lg.PWLSiLU(R=4.0, lut_bits=4)
    x = _inputs(n + 1, 4.0, n)
    xg = to_gpu(x)[1:]  # 4-byte offset: not 16-byte aligned
    got = from_gpu(lg.pwl_silu(xg, m.lut, 4.0))
    assert same_bits(got, O.pwl_silu(x[1:], m.lut.numpy(), 4.0))


def test_module_matches_oracle_and_grad():
    m = lg.PWLSiLU(R=8.0, lut_bits=6).cuda()
    x = torch.randn(4096, device="cuda", requires_grad=True) * 3
    x.retain_grad()
    y = m(x)
    xs = from_gpu(x.detach())
    assert same_bits(from_gpu(y.detach()), O.pwl_silu(xs, m.lut.cpu().numpy(), 8.0))
    assert (y - torch.nn.functional.silu(x)).abs().max() < 0.05
    y.sum().backward()
    s = torch.sigmoid(x.detach())
    assert torch.allclose(x.grad, s * (1 + x.detach() * (1 - s)))


def test_errors():
    x = torch.zeros(8, device="cuda")
    with pytest.raises(RuntimeError):
        lg.pwl_silu(x, torch.zeros(6), 1.0)  # 5 segments: not a power of 2
    with pytest.raises(RuntimeError):
        lg.pwl_silu(x, torch.zeros(5), 0.0)
    with pytest.raises(RuntimeError):
        lg.pwl_silu(x, torch.zeros(1), 1.0)
