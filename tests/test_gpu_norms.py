"""BatchNorm approximations on the GPU (csrc/norms.cu: per-channel statistics,
fused normalise + affine), through the modules and through bn_stats /
bn_apply.

  * eval mode from the reference's recorded running statistics: bit for bit
    against the outputs the reference's own modules produced
    (tests/golden/golden_layers.npz);
  * training mode: statistics are reductions, summed here in another order
    (FP32 per thread, double across threads) than torch's, so outputs,
    running statistics and gradients agree within stated tolerances;
  * statistics against an FP64 restatement (mean, mean |x - mean|,
    max |x - mean|, biased variance) and outputs against the FP64 formula
    from the kernel's own statistics, at the bench's NCHW 32x256x56x56 too;
  * flat (short-row), unaligned and in-place buffers, and argument errors.
"""
import numpy as np
import pytest
import torch

import lofloat_gb300 as lg
from golden_io import load, same_bits
from lofloat_gb300 import binding as lof
from lofloat_gb300 import norms
from test_cpu_norms import SHAPES, VARIANTS

pytestmark = pytest.mark.gpu

DEV_BUF = {"l1": "running_mad", "linf": "running_maxdev", "fisr": "running_var", "pwl": "running_var"}
# training-mode tolerances: FP32 outputs of O(1) whose statistics differ from
# torch's in the last bits
OUT_RTOL, OUT_ATOL = 2e-5, 2e-5
GRAD_RTOL, GRAD_ATOL = 1e-4, 1e-5


@pytest.fixture(scope="module")
def golden():
    return load("golden_layers.npz")


def _module(golden, shape, vname):
    kind, make = VARIANTS[vname]
    c = golden[f"bn_{shape}_x"].shape[1]
    mod = make(c).cuda()
    if mod.affine:
        with torch.no_grad():
            mod.weight.copy_(torch.from_numpy(golden[f"bn_{shape}_w"]))
            mod.bias.copy_(torch.from_numpy(golden[f"bn_{shape}_b"]))
    return kind, mod


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("vname", list(VARIANTS))
def test_eval_bitexact_against_reference(golden, shape, vname):
    kind, mod = _module(golden, shape, vname)
    key = f"bn_{shape}_{vname}"
    with torch.no_grad():
        mod.running_mean.copy_(torch.from_numpy(golden[key + "_running_mean"]))
        getattr(mod, DEV_BUF[kind]).copy_(torch.from_numpy(golden[key + "_" + DEV_BUF[kind]]))
    mod.eval()
    y = mod(torch.from_numpy(golden[f"bn_{shape}_x2"]).cuda())
    assert same_bits(y.detach().cpu().numpy(), golden[key + "_y_eval"])


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("vname", list(VARIANTS))
def test_training_step_against_reference(golden, shape, vname):
    kind, mod = _module(golden, shape, vname)
    key = f"bn_{shape}_{vname}"
    x = torch.from_numpy(golden[f"bn_{shape}_x"]).cuda().requires_grad_(True)
    y = mod(x)
    np.testing.assert_allclose(y.detach().cpu().numpy(), golden[key + "_y_train"], OUT_RTOL, OUT_ATOL)
    np.testing.assert_allclose(mod.running_mean.cpu().numpy(), golden[key + "_running_mean"], 1e-6, 1e-7)
    np.testing.assert_allclose(getattr(mod, DEV_BUF[kind]).cpu().numpy(),
                               golden[key + "_" + DEV_BUF[kind]], 1e-5, 1e-7)
    if hasattr(mod, "num_batches_tracked"):
        assert int(mod.num_batches_tracked) == 1
    y.backward(torch.from_numpy(golden[key + "_gy"]).cuda())
    np.testing.assert_allclose(x.grad.cpu().numpy(), golden[key + "_dx"], GRAD_RTOL, GRAD_ATOL)
    if mod.affine:
        np.testing.assert_allclose(mod.weight.grad.cpu().numpy(), golden[key + "_dw"], GRAD_RTOL, 1e-4)
        np.testing.assert_allclose(mod.bias.grad.cpu().numpy(), golden[key + "_db"], GRAD_RTOL, 1e-4)


def _fp64_stats(x, stat):
    xd = x.double()
    dims = [0] + list(range(2, x.dim()))
    mean = xd.mean(dim=dims)
    if stat == lof.BnStat.VARIANCE:
        return mean, xd.var(dim=dims, unbiased=False)
    # the deviation is taken about the FP32 mean, in FP32, as the reference does
    shape = [1, -1] + [1] * (x.dim() - 2)
    xc = (x - mean.float().view(shape)).abs().double()
    return mean, (xc.mean(dim=dims) if stat == lof.BnStat.MEAN_ABS_DEV else xc.amax(dim=dims))


@pytest.mark.parametrize("shape", [(32, 256, 56, 56), (16, 64, 9, 13), (4096, 24), (7, 5, 3),
                                   (2, 3, 1000)])
@pytest.mark.parametrize("stat", list(lof.BnStat))
def test_stats_against_fp64(shape, stat):
    g = torch.Generator(device="cuda").manual_seed(sum(shape) + int(stat))
    x = torch.randn(*shape, device="cuda", generator=g) * 2 + 0.5
    mean, dev = lof.bn_stats(x, stat)
    m64, d64 = _fp64_stats(x, stat)
    torch.testing.assert_close(mean.double(), m64, rtol=0, atol=2e-6)
    torch.testing.assert_close(dev.double(), d64, rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("norm", list(lof.BnNorm))
def test_apply_against_fp64_formula(norm):
    """Outputs at the bench's size against the formula in FP64 from the same
    statistics (the approximate 1/sqrt taken from the FP32 restatement)."""
    g = torch.Generator(device="cuda").manual_seed(11 + int(norm))
    x = torch.randn(32, 256, 56, 56, device="cuda", generator=g) * 3 - 1
    c = x.shape[1]
    w = torch.rand(c, device="cuda", generator=g) + 0.5
    b = torch.randn(c, device="cuda", generator=g)
    sc = torch.rand(c, device="cuda", generator=g) + 0.5
    stat = lof.BnStat.VARIANCE if norm != lof.BnNorm.DIVIDE else lof.BnStat.MEAN_ABS_DEV
    mean, dev = lof.bn_stats(x, stat)
    lut = lg.PWLBatchNorm(c).lut.cuda()
    y = lof.bn_apply(x, mean, dev, 1e-5, norm, scale=sc if norm == lof.BnNorm.DIVIDE else None,
                     weight=w, bias=b, lut=lut)
    v = dev + 1e-5
    if norm == lof.BnNorm.DIVIDE:
        f = sc.double() / v.double()
    elif norm == lof.BnNorm.FISR:
        f = norms._fisr_chain(v).double()
    else:
        f = norms._pwl_chain(v, lut).double()
    v4 = [1, -1, 1, 1]
    want = (x.double() - mean.double().view(v4)) * f.view(v4) * w.double().view(v4) + b.double().view(v4)
    torch.testing.assert_close(y.double(), want, rtol=4e-6, atol=4e-6)


def test_unaligned_in_place_and_flat_paths():
    g = torch.Generator(device="cuda").manual_seed(5)
    base = torch.randn(1 + 3 * 4 * 80, device="cuda", generator=g)
    x = base[1:].view(3, 4, 80)            # 4-byte offset: no 16-byte vectors
    mean, dev = lof.bn_stats(x, lof.BnStat.VARIANCE)
    m64, d64 = _fp64_stats(x, lof.BnStat.VARIANCE)
    torch.testing.assert_close(dev.double(), d64, rtol=1e-5, atol=1e-7)
    want = lof.bn_apply(x.clone(), mean, dev, 1e-5, lof.BnNorm.FISR)
    got = lof.bn_apply(x, mean, dev, 1e-5, lof.BnNorm.FISR, out=x)   # in place
    assert torch.equal(got, want)
    x2 = torch.randn(5000, 3, device="cuda", generator=g)              # (N, C): inner = 1
    mean, dev = lof.bn_stats(x2, lof.BnStat.MAX_ABS_DEV)
    assert torch.equal(dev, (x2 - mean).abs().amax(dim=0))


@pytest.mark.parametrize("shape", [(32, 256, 56, 56), (16, 64, 9, 13), (5000, 3), (2, 3, 1000)])
def test_max_deviation_equals_centred_amax(shape):
    """The single pass's max(max x - mean, mean - min x) has the bits of the
    maximum over every centred value, taken about the same FP32 mean."""
    g = torch.Generator(device="cuda").manual_seed(31 + sum(shape))
    x = torch.randn(*shape, device="cuda", generator=g) * 3 + 1
    mean, dev = lof.bn_stats(x, lof.BnStat.MAX_ABS_DEV)
    view = [1, -1] + [1] * (x.dim() - 2)
    dims = [0] + list(range(2, x.dim()))
    assert torch.equal(dev, (x - mean.view(view)).abs().amax(dim=dims))


def test_max_deviation_with_infinities_and_nan():
    x = torch.randn(6, 7, 50, device="cuda")
    x[1, 0, 3] = float("inf")                                   # mean inf: inf - inf
    x[2, 1, 4] = float("-inf")                                  # mean -inf
    x[0, 2, 5], x[3, 2, 6] = float("inf"), float("-inf")        # mean NaN
    x[4, 3, 7] = float("nan")
    x[:, 4] = 2.5                                               # constant: deviation +0
    x[:, 5] = 1.0e30                                            # large, equal values
    x[:, 6] = -0.0                                              # mean +0, deviation +0
    mean, dev = lof.bn_stats(x, lof.BnStat.MAX_ABS_DEV)
    want = (x - mean.view(1, -1, 1)).abs().amax(dim=(0, 2))
    torch.testing.assert_close(dev, want, rtol=0, atol=0, equal_nan=True)
    assert torch.isnan(dev[:4]).all() and not torch.isnan(dev[4:]).any()
    assert dev[4].item() == 0.0 and not torch.signbit(dev[4])
    assert dev[6].item() == 0.0 and not torch.signbit(dev[6])


def test_nan_propagates_to_max_deviation():
    x = torch.randn(4, 3, 100, device="cuda")
    x[2, 1, 7] = float("nan")
    _, dev = lof.bn_stats(x, lof.BnStat.MAX_ABS_DEV)
    assert torch.isnan(dev[1]) and not torch.isnan(dev[0]) and not torch.isnan(dev[2])


def test_errors():
    x = torch.randn(2, 3, 4, device="cuda")
    m = torch.zeros(3, device="cuda")
    with pytest.raises(RuntimeError):
        lof.bn_apply(x, m, m, 1e-5, lof.BnNorm.PWL)                     # no table
    with pytest.raises(RuntimeError):
        lof.bn_apply(x, m, torch.zeros(2, device="cuda"), 1e-5, lof.BnNorm.DIVIDE)
    with pytest.raises(RuntimeError):
        lof.bn_stats(x.double(), lof.BnStat.VARIANCE)
    L = lg._native.lib()
    assert L.lofgb_bn_stats_f32(x.data_ptr(), 2, 3, 4, 7, m.data_ptr(), m.data_ptr(), None, None,
                                0.1, None, 0, None) == -7
