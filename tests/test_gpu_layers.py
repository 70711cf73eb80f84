"""torch.ops.lofloat.* registrations, STE functions, LoF_Linear, and the
hand-written backward of the emulated linear layer."""
import numpy as np
import pytest
import torch

import lofloat_gb300 as lg
from golden_io import same_bits
from gpu_util import from_gpu, ofmt, to_gpu
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_custom_ops_match_binding():
    e4m3 = lg.create_p3109_params(8, 4)
    fid = lg.register_format(e4m3)
    assert lg.register_format(e4m3) == fid
    x = torch.randn(1000, device="cuda") * 10
    y1 = torch.ops.lofloat.virtual_round(x, fid, 0, 0, 2.0)
    y2 = lg.virtual_round(x, e4m3, scale=2.0)
    assert torch.equal(y1, y2)
    e8 = lg.register_format(lg.create_e8m0_params())
    z1 = torch.ops.lofloat.virtual_mx_round(x, 32, fid, e8, 0, 0, 0)
    z2 = lg.virtual_mx_round(x, 32, e4m3, lg.create_e8m0_params())
    assert torch.equal(z1, z2)


def test_fake_kernels_trace():
    fid = lg.register_format(lg.create_p3109_params(8, 4))
    from torch._subclasses.fake_tensor import FakeTensorMode
    with FakeTensorMode():
        x = torch.empty(4, 8, device="cuda")
        assert torch.ops.lofloat.virtual_round(x, fid, 0, 0, 1.0).shape == (4, 8)
        assert torch.ops.lofloat.lof_gemm(x, torch.empty(8, 3, device="cuda"), 10, 0, 0, 1.0, 1.0).shape == (4, 3)


def test_ste_gradients():
    e4m3 = lg.create_p3109_params(8, 4)
    x = (torch.rand(4, 256, device="cuda") - 0.5).mul(10).requires_grad_(True)
    q = lg.LoF_Quantize(e4m3, scaling="mx", mx_block_size=32)
    q(x).sum().backward()
    assert torch.equal(x.grad, torch.ones_like(x))
    x.grad = None
    lg.STERound.apply(x, lg.register_format(e4m3), 0, 3.0).sum().backward()
    assert torch.allclose(x.grad, torch.full_like(x, 3.0))
    with pytest.raises(ValueError):
        lg.LoF_Quantize(e4m3, scaling="mx", mx_block_size=32)(torch.rand(3, 30, device="cuda"))


def test_lof_linear_forward_matches_reference_path():
    torch.manual_seed(0)
    lin = lg.LoF_Linear(256, 64, act_exp=4, act_mant=3, weight_exp=4, weight_mant=3, bias=False,
                        scaling="mx", mx_block_size=32, accum_mant_bits=10).cuda()
    x = torch.randn(4, 256, device="cuda")
    y = lin(x)
    # reference path: MX both operands, then lof_gemm on x_q and the transposed weight
    xq = lg.virtual_mx_round(x, 32, lin.act_params, lin.scale_format)
    wq = lg.virtual_mx_round(lin.weight.detach(), 32, lin.weight_params, lin.scale_format)
    ref = lg.lof_gemm(xq, wq.t().contiguous(), 10)
    assert torch.equal(y.detach(), ref)
    assert y.requires_grad


def test_lof_linear_per_tensor_scales():
    torch.manual_seed(1)
    lin = lg.LoF_Linear(64, 32, act_exp=4, act_mant=3, weight_exp=4, weight_mant=3, bias_exp=5,
                        bias_mant=2, act_scale_factor=2.0, w_scale_factor=0.5, accum_mant_bits=12,
                        differentiable=False).cuda()
    x = torch.randn(8, 64, device="cuda")
    y = lin(x)
    xq = lg.virtual_round(x, lin.act_params, scale=2.0)
    wq = lg.virtual_round(lin.weight.detach(), lin.weight_params, scale=0.5)
    ref = lg.lof_gemm(xq, wq.t().contiguous(), 12, scale_a=2.0, scale_b=0.5)
    ref = ref + lg.virtual_round(lin.bias.detach(), lin.bias_params)
    assert torch.equal(y, ref)


def _fd_check(M=6, K=64, N=5):
    """Central finite differences of loss = sum(Y^2) in FP64 with rounding
    disabled vs the hand-written backward with a 23-bit accumulator."""
    torch.manual_seed(2)
    x = torch.randn(M, K, dtype=torch.float64)
    w = torch.randn(N, K, dtype=torch.float64) * 0.1
    cfg = lg.LinearConfig(accum_mant_bits=23)
    xg = x.float().cuda().requires_grad_(True)
    wg = w.float().cuda().requires_grad_(True)
    (lg.lof_linear(xg, wg, cfg) ** 2).sum().backward()

    def loss(xx, ww):
        return float(((xx @ ww.T) ** 2).sum())

    h = 1e-6
    gx = torch.zeros_like(x)
    for i in range(M):
        for k in range(K):
            e = torch.zeros_like(x)
            e[i, k] = h
            gx[i, k] = (loss(x + e, w) - loss(x - e, w)) / (2 * h)
    gw = torch.zeros_like(w)
    for j in range(N):
        for k in range(K):
            e = torch.zeros_like(w)
            e[j, k] = h
            gw[j, k] = (loss(x, w + e) - loss(x, w - e)) / (2 * h)
    return xg.grad.double().cpu(), wg.grad.double().cpu(), gx, gw


def test_backward_vs_finite_differences():
    dx, dw, gx, gw = _fd_check()
    assert torch.allclose(dx, gx, rtol=1e-4, atol=1e-4)
    assert torch.allclose(dw, gw, rtol=1e-4, atol=1e-4)


def test_backward_vs_surrogate_autograd():
    """Against autograd through STE MX rounding and an FP64 matmul of the
    rounded operands (the reference's gradient definition for the rounding,
    with the GEMM exact)."""
    torch.manual_seed(3)
    M, K, N = 128, 256, 96
    e4m3 = lg.create_p3109_params(8, 4)
    e8 = lg.create_e8m0_params()
    e5m2 = lg.make_format(5, 2)
    x = torch.randn(M, K, device="cuda").bfloat16().requires_grad_(True)
    w = (torch.randn(N, K, device="cuda") * 0.02).bfloat16().requires_grad_(True)
    cfg = lg.LinearConfig(act_format=e4m3, weight_format=e4m3, scale_format=e8, accum_mant_bits=10,
                          grad_format=e5m2)
    y = lg.lof_linear(x, w, cfg)
    (y.float() ** 2).sum().backward()
    xq = lg.virtual_mx_round(x.detach().float(), 32, e4m3, e8).double()
    wq = lg.virtual_mx_round(w.detach().float(), 32, e4m3, e8).double()
    xr = xq.clone().requires_grad_(True)
    wr = wq.clone().requires_grad_(True)
    ((xr @ wr.T) ** 2).sum().backward()
    # dY stochastic-rounded to E5M2 (2 mantissa bits) carries ~2^-3 relative
    # noise per element; the GEMMs add 10-bit accumulation error
    for got, ref in ((x.grad, xr.grad), (w.grad, wr.grad)):
        rel = ((got.double() - ref).norm() / ref.norm()).item()
        assert rel < 0.15, rel
    assert x.grad.dtype == torch.bfloat16 and w.grad.dtype == torch.bfloat16
    # without gradient rounding only the 10-bit accumulation remains
    x.grad = w.grad = None
    cfg.grad_format = None
    (lg.lof_linear(x, w, cfg).float() ** 2).sum().backward()
    for got, ref in ((x.grad, xr.grad), (w.grad, wr.grad)):
        rel = ((got.double() - ref).norm() / ref.norm()).item()
        assert rel < 2e-2, rel


def test_stochastic_gradient_is_unbiased():
    """Averaged over seeds, the SR-rounded gradient approaches the unrounded one."""
    torch.manual_seed(5)
    x = torch.randn(64, 128, device="cuda").requires_grad_(True)
    w = (torch.randn(32, 128, device="cuda") * 0.05).requires_grad_(True)
    cfg = lg.LinearConfig(accum_mant_bits=23, grad_format=lg.make_format(5, 2), grad_stoch_len=16)
    dy = torch.randn(64, 32, device="cuda")
    acc = torch.zeros_like(x)
    for s in range(64):
        lg.set_seed(1000 + s)
        x.grad = None
        lg.lof_linear(x, w, cfg).backward(dy)
        acc += x.grad
    exact = dy @ w.detach()
    rel = ((acc / 64 - exact).norm() / exact.norm()).item()
    assert rel < 0.03, rel
