"""BatchNorm approximations (LoFloat/layers.py:805-1047), host side.

The modules run on two CUDA kernels (tests/test_gpu_norms.py checks them);
their backward differentiates the reference's own FP32 formulation, restated
in lofloat_gb300.norms._chain. Here, on the CPU: that restatement against
outputs and gradients recorded from the reference's modules
(tests/golden/golden_layers.npz, tests/golden/make_layers_golden.py), the
buffers and arguments of the modules, and the CUDA-only forward."""
import math

import numpy as np
import pytest
import torch

import lofloat_gb300 as lg
from golden_io import load, same_bits
from lofloat_gb300 import norms

SHAPES = ("nchw", "nc", "ncl")
VARIANTS = {
    "l1": ("l1", lambda c: lg.L1BatchNorm(c)),
    "l1_tensor_scale": ("l1", lambda c: lg.L1BatchNorm(c, scale=torch.linspace(0.5, 1.5, c))),
    "linf": ("linf", lambda c: lg.LinfBatchNorm(c)),
    "linf_scale": ("linf", lambda c: lg.LinfBatchNorm(c, scale=0.75, momentum=0.3)),
    "fisr": ("fisr", lambda c: lg.FISRBatchNorm(c)),
    "pwl_minimax": ("pwl", lambda c: lg.PWLBatchNorm(c)),
    "pwl_uniform6": ("pwl", lambda c: lg.PWLBatchNorm(c, lut_bits=6, lut_method="uniform")),
    "l1_noaffine": ("l1", lambda c: lg.L1BatchNorm(c, affine=False)),
    "fisr_noaffine_eps": ("fisr", lambda c: lg.FISRBatchNorm(c, affine=False, eps=1e-3)),
}


@pytest.fixture(scope="module")
def golden():
    return load("golden_layers.npz")


def _chain_of(mod, kind, x, stats=None, w=None, b=None):
    return norms._chain(kind, x, w, b, getattr(mod, "scale", None), mod.eps,
                        getattr(mod, "lut", None), stats)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("vname", list(VARIANTS))
def test_restated_chain_matches_reference(golden, shape, vname):
    """Training outputs and gradients, and eval outputs from the recorded
    running statistics, bit for bit."""
    kind, make = VARIANTS[vname]
    key = f"bn_{shape}_{vname}"
    x = torch.from_numpy(golden[f"bn_{shape}_x"]).requires_grad_(True)
    c = x.shape[1]
    mod = make(c)
    w = b = None
    if mod.affine:
        w = torch.from_numpy(golden[f"bn_{shape}_w"]).requires_grad_(True)
        b = torch.from_numpy(golden[f"bn_{shape}_b"]).requires_grad_(True)
    y = _chain_of(mod, kind, x, None, w, b)
    assert same_bits(y.detach().numpy(), golden[key + "_y_train"])
    y.backward(torch.from_numpy(golden[key + "_gy"]))
    assert same_bits(x.grad.numpy(), golden[key + "_dx"])
    if w is not None:
        assert same_bits(w.grad.numpy(), golden[key + "_dw"])
        assert same_bits(b.grad.numpy(), golden[key + "_db"])
    dev_name = {"l1": "running_mad", "linf": "running_maxdev"}.get(kind, "running_var")
    stats = (torch.from_numpy(golden[key + "_running_mean"]), torch.from_numpy(golden[key + "_" + dev_name]))
    x2 = torch.from_numpy(golden[f"bn_{shape}_x2"])
    y2 = _chain_of(mod, kind, x2, stats, w.detach() if w is not None else None,
                   b.detach() if b is not None else None)
    assert same_bits(y2.numpy(), golden[key + "_y_eval"])


def test_module_buffers_and_arguments():
    l1 = lg.L1BatchNorm(3)
    assert abs(l1.scale[0].item() - math.sqrt(2 / math.pi)) < 1e-7
    assert [n for n, _ in l1.named_buffers()] == ["running_mean", "running_mad", "num_batches_tracked", "scale"]
    assert [n for n, _ in lg.LinfBatchNorm(3).named_buffers()] == ["running_mean", "running_maxdev", "scale"]
    assert [n for n, _ in lg.FISRBatchNorm(3).named_buffers()] == ["running_mean", "running_var",
                                                                   "num_batches_tracked"]
    assert [n for n, _ in lg.PWLBatchNorm(3).named_buffers()] == ["running_mean", "running_var",
                                                                  "num_batches_tracked", "lut"]
    assert lg.L1BatchNorm(4, affine=False).weight is None
    assert torch.equal(lg.L1BatchNorm(3, scale=torch.tensor([2.0])).scale, torch.full((3,), 2.0))
    with pytest.raises(ValueError):
        lg.L1BatchNorm(3, scale=torch.ones(2))


def test_rsqrt_approximations():
    v = torch.logspace(-6, 6, 2001)
    assert ((lg.FISRBatchNorm._fast_rsqrt(v) * v.sqrt() - 1).abs().max() < 1e-5)
    for method, tol in (("uniform", 1e-3), ("midpoint", 2e-2), ("minimax", 1e-3)):
        p = lg.PWLBatchNorm(4, lut_bits=4, lut_method=method)
        assert ((p._rsqrt_pwl(v) * v.sqrt() - 1).abs().max() < tol)


def test_forward_needs_cuda():
    with pytest.raises(RuntimeError):
        lg.L1BatchNorm(3)(torch.zeros(2, 3, 4))


def test_golden_fixture_is_consistent(golden):
    assert golden["bn_nchw_x"].shape == (8, 6, 5, 7)
    assert np.isfinite(golden["bn_nchw_fisr_y_train"]).all()


def _max_centred(x, m):
    """max |x - m| over FP32 differences, NaN if any difference is NaN."""
    d = np.abs(x - m)
    return np.float32(np.nan) if np.isnan(d).any() else d.max()


def _max_from_range(x, m):
    """max(max x - m, m - min x) in FP32 with the sign cleared (the larger
    difference is never below zero, but is -0 for x all -0 about m = +0), NaN
    if either difference is; NaN inputs are skipped by the range, as fmaxf /
    fminf do."""
    hi, lo = np.nanmax(x), np.nanmin(x)
    d1, d2 = np.float32(hi - m), np.float32(m - lo)
    return np.float32(np.nan) if np.isnan(d1) or np.isnan(d2) else np.abs(max(d1, d2))


def test_max_deviation_identity_in_fp32():
    """LinfBatchNorm's max |x - mean| from one pass: with FP32 subtraction
    rounded monotonically, the largest rounded |x - m| comes from max x or
    min x, for any FP32 m (the mean the kernel computes, or one placed
    anywhere, ties and signed zeros included); a NaN x makes the mean NaN."""
    rng = np.random.default_rng(17)
    with np.errstate(invalid="ignore", over="ignore"):
        for trial in range(3000):
            n = int(rng.integers(1, 200))
            scale = np.float32(10.0 ** rng.integers(-40, 38))
            x = (rng.standard_normal(n) * scale).astype(np.float32)
            if trial % 7 == 0:
                x[rng.integers(0, n)] = np.float32(rng.choice([np.inf, -np.inf, 0.0, -0.0]))
            if trial % 11 == 0:
                x[:] = x[0]
            if trial % 17 == 0:
                x[:] = np.float32(-0.0)
            m = np.float32(x.astype(np.float64).mean())
            if trial % 2 == 0:      # the kernel's sums start at +0
                m = np.float32(m + np.float32(0.0))
            if trial % 5 == 0:      # a centre off the mean, inside or outside the range
                m = np.float32(m + rng.standard_normal() * scale)
            if trial % 13 == 0:
                x[rng.integers(0, n)] = np.float32(np.nan)
                m = np.float32(np.nan)
            want, got = _max_centred(x, m), _max_from_range(x, m)
            assert (np.isnan(want) and np.isnan(got)) or \
                (want == got and np.signbit(want) == np.signbit(got)), (trial, x, m, want, got)
