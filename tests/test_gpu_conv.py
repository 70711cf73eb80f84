"""GPU parity of the emulated-accumulation conv2d.

The CUDA-core form is bit-exact against the oracle in both reduction orders:
"crs" (the reference's default LoF_Conv2d path, im2col + lof_gemm per image)
and "tiled8" (lof_conv2d's implicit GEMM with 8-channel k-tiles). The "crs"
order is additionally pinned against unfold + the GEMM on the GPU. The
tensor-core form is checked against the FP64 conv2d with the tolerance the
chunked accumulator allows."""
import numpy as np
import pytest
import torch
import torch.nn.functional as F

import lofloat_gb300 as lg
from golden_io import same_bits, same_bits_nan_class
from gpu_util import from_gpu, mismatch_report, to_gpu
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# (N, C, H, W, K, R, S, stride, padding, dilation)
SHAPES = [
    (1, 1, 1, 1, 1, 1, 1, (1, 1), (0, 0), (1, 1)),
    (2, 3, 9, 7, 5, 3, 3, (1, 1), (1, 1), (1, 1)),
    (1, 8, 12, 12, 16, 3, 3, (2, 2), (1, 1), (1, 1)),
    (3, 13, 10, 11, 7, 3, 2, (1, 2), (2, 0), (2, 1)),
    (2, 16, 6, 6, 130, 1, 1, (1, 1), (0, 0), (1, 1)),
    (1, 5, 20, 18, 9, 5, 5, (3, 2), (2, 2), (1, 1)),
    (2, 32, 8, 8, 24, 3, 3, (1, 1), (1, 1), (1, 1)),
    (1, 4, 40, 40, 3, 7, 7, (2, 2), (3, 3), (1, 1)),
]


def _data(shape, seed):
    n, c, h, w, k, r, s = shape[:7]
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, c, h, w)).astype(np.float32)
    wt = (rng.standard_normal((k, c, r, s)) * 0.3).astype(np.float32)
    return x, wt


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s[:7])))
@pytest.mark.parametrize("order", ["crs", "tiled8"])
@pytest.mark.parametrize("mbits", [10, 23])
def test_plain_vs_oracle(shape, order, mbits):
    x, wt = _data(shape, hash((shape, order, mbits)) & 0xFFFF)
    st, pd, dl = shape[7:]
    got = from_gpu(lg.conv2d(to_gpu(x), to_gpu(wt), mbits, stride=st, padding=pd, dilation=dl,
                             order=order))
    want = O.conv2d(x, wt, mbits, stride=st, padding=pd, dilation=dl, order=order)
    assert got.shape == want.shape
    assert same_bits(got, want), mismatch_report(got, got, want)


@pytest.mark.parametrize("mbits", [4, 7, 12])
def test_narrow_accumulators(mbits):
    shape = (2, 11, 9, 9, 20, 3, 3, (1, 1), (1, 1), (1, 1))
    x, wt = _data(shape, mbits)
    for order in ("crs", "tiled8"):
        got = from_gpu(lg.conv2d(to_gpu(x), to_gpu(wt), mbits, padding=1, order=order, alpha=0.75))
        want = O.conv2d(x, wt, mbits, padding=(1, 1), order=order, alpha=0.75)
        assert same_bits(got, want), (order, mismatch_report(got, got, want))


def test_crs_equals_unfold_gemm():
    """The reference's default path: F.unfold then lof_gemm per image."""
    rng = np.random.default_rng(5)
    x = rng.standard_normal((3, 6, 11, 10)).astype(np.float32)
    wt = rng.standard_normal((9, 6, 3, 2)).astype(np.float32)
    xg, wg = to_gpu(x), to_gpu(wt)
    kw = dict(kernel_size=(3, 2), dilation=(1, 2), padding=(1, 0), stride=(2, 1))
    cols = F.unfold(xg, **kw)
    ref = torch.stack([lg.lof_gemm(wg.reshape(9, -1), cols[b].contiguous(), 10, scale_a=0.5,
                                   scale_b=2.0) for b in range(3)])
    got = lg.conv2d(xg, wg, 10, stride=(2, 1), padding=(1, 0), dilation=(1, 2),
                    alpha=lg.gemm_alpha(0.5, 2.0), order="crs")
    assert same_bits(from_gpu(got).reshape(3, 9, -1), from_gpu(ref))


def test_dropin_lof_conv2d():
    rng = np.random.default_rng(6)
    x = rng.standard_normal((2, 12, 10, 10)).astype(np.float32)
    wt = rng.standard_normal((7, 12, 3, 3)).astype(np.float32)
    got = from_gpu(lg.lof_conv2d(to_gpu(x), to_gpu(wt), 1, 1, 1, 1, 1, 1, 10,
                                 lg.RoundingMode.RoundTowardsZero, 3, 0.3, 7.0))
    alpha = float(np.float32(1.0 / (0.3 * 7.0)))
    assert lg.conv2d_alpha(0.3, 7.0) == alpha
    want = O.conv2d(x, wt, 10, padding=(1, 1), alpha=alpha, order="tiled8")
    assert same_bits(got, want), mismatch_report(got, got, want)
    zero = from_gpu(lg.lof_conv2d(to_gpu(x), to_gpu(wt), 1, 1, 1, 1, 1, 1, 10, weight_scale=0.0))
    assert same_bits(zero, O.conv2d(x, wt, 10, padding=(1, 1), order="tiled8"))


def test_special_values_and_signed_zero():
    rng = np.random.default_rng(7)
    x = rng.standard_normal((1, 9, 6, 6)).astype(np.float32)
    wt = rng.standard_normal((4, 9, 3, 3)).astype(np.float32)
    x[0, 2, 3, 3] = np.nan
    x[0, 4, 0, 0] = np.inf
    wt[1] = -np.abs(wt[1])
    x[0, :, 4:, 4:] = 0.0   # all-zero windows with negative weights: signed zeros
    wt[2, 3, 1, 1] = 3e38
    for order in ("crs", "tiled8"):
        got = from_gpu(lg.conv2d(to_gpu(x), to_gpu(wt), 10, padding=1, order=order))
        want = O.conv2d(x, wt, 10, padding=(1, 1), order=order)
        ok, _ = same_bits_nan_class(got, want)
        assert ok, (order, mismatch_report(got, got, want))


def test_empty_batch_and_errors():
    xg = torch.zeros((0, 3, 5, 5), device="cuda")
    wg = torch.zeros((4, 3, 3, 3), device="cuda")
    assert lg.conv2d(xg, wg, 10).shape == (0, 4, 3, 3)
    with pytest.raises(RuntimeError):
        lg.conv2d(torch.zeros((1, 3, 2, 2), device="cuda"), wg, 10)  # no output pixels
    with pytest.raises(RuntimeError):
        lg.conv2d(torch.zeros((1, 2, 5, 5), device="cuda"), wg, 10)  # C mismatch
    with pytest.raises(RuntimeError):
        lg.conv2d(torch.zeros((1, 3, 5, 5)), wg.cpu(), 10)  # CPU tensors


def _fp64_conv(x, wt, **kw):
    return F.conv2d(torch.from_numpy(x).double().cuda(), torch.from_numpy(wt).double().cuda(),
                    **kw).cpu().numpy()


@pytest.mark.parametrize("order", ["crs", "tiled8"])
@pytest.mark.parametrize("chunk", [16, 64])
def test_tc_error_vs_fp64(order, chunk):
    rng = np.random.default_rng(8)
    x = rng.standard_normal((4, 64, 14, 14)).astype(np.float32)
    wt = (rng.standard_normal((96, 64, 3, 3)) * 0.05).astype(np.float32)
    got = from_gpu(lg.conv2d(to_gpu(x), to_gpu(wt), 10, padding=1, order=order, variant="tc",
                             chunk=chunk))
    ref = _fp64_conv(x, wt, padding=1)
    plain = from_gpu(lg.conv2d(to_gpu(x), to_gpu(wt), 10, padding=1, order=order))
    # the chunked accumulator rounds K/chunk times instead of K times: its error
    # is bounded by the per-MAC form's bound
    scale = np.abs(ref).mean()
    err_tc = np.abs(got - ref).max() / scale
    err_plain = np.abs(plain - ref).max() / scale
    assert err_tc <= 1.5 * err_plain + 1e-3, (err_tc, err_plain)
    assert np.abs(got - ref).mean() / scale < 2e-3


def test_tc_exact_inputs_are_exact():
    """Small integers: every chunk sum and accumulator value is exact, so the
    tensor-core form equals the plain form bit for bit."""
    rng = np.random.default_rng(9)
    x = rng.integers(-4, 5, (2, 24, 9, 9)).astype(np.float32)
    wt = rng.integers(-3, 4, (40, 24, 3, 3)).astype(np.float32)
    for order in ("crs", "tiled8"):
        tc = from_gpu(lg.conv2d(to_gpu(x), to_gpu(wt), 23, padding=1, order=order, variant="tc"))
        plain = from_gpu(lg.conv2d(to_gpu(x), to_gpu(wt), 23, padding=1, order=order))
        assert np.array_equal(tc, plain)
        assert np.array_equal(tc.astype(np.float64), _fp64_conv(x, wt, padding=1))
    assert lg.binding.tc_device_status() == 0


def _p3109(bits, mant_with_implicit):
    return lg.create_p3109_params(bits, mant_with_implicit)


def test_layer_im2col_matches_reference_path():
    """LoF_Conv2d(backend="im2col") = STERound of x and W, unfold, lof_gemm per
    image, quantised bias (LoFloat/layers.py:679-713)."""
    torch.manual_seed(0)
    layer = lg.LoF_Conv2d(6, 10, 3, stride=1, padding=1, act_params=_p3109(8, 4),
                          weight_params=_p3109(8, 4), bias_params=_p3109(16, 11),
                          accum_mant_bits=10, act_scale_factor=2.0, w_scale_factor=0.5,
                          b_scale_factor=4.0).cuda()
    with torch.no_grad():
        layer.bias.uniform_(-1, 1)
    x = torch.randn(2, 6, 8, 8, device="cuda")
    with torch.no_grad():
        got = layer(x)
        xq = lg.virtual_round(x, layer.act_params, scale=2.0)
        wq = lg.virtual_round(layer.weight, layer.weight_params, scale=0.5)
        cols = F.unfold(xq, kernel_size=3, padding=1)
        ref = torch.stack([lg.lof_gemm(wq.reshape(10, -1), cols[b].contiguous(), 10,
                                       scale_a=0.5, scale_b=2.0) for b in range(2)])
        bq = lg.virtual_round(layer.bias, layer.bias_params, scale=4.0) / 4.0
        ref = ref.view(2, 10, 8, 8) + bq.view(1, -1, 1, 1)
    assert same_bits(from_gpu(got), from_gpu(ref))


def test_layer_groups_and_cutlass_backend():
    torch.manual_seed(1)
    g = lg.LoF_Conv2d(8, 12, 3, padding=1, groups=4, act_params=_p3109(8, 4),
                      weight_params=_p3109(8, 4), bias=False, accum_mant_bits=12).cuda()
    x = torch.randn(2, 8, 7, 7, device="cuda")
    with torch.no_grad():
        got = g(x)
        xq = lg.virtual_round(x, g.act_params)
        wq = lg.virtual_round(g.weight, g.weight_params)
        cols = F.unfold(xq, kernel_size=3, padding=1).view(2, 4, 2 * 9, 49)
        wcol = wq.view(4, 3, -1)
        ref = torch.stack([torch.cat([lg.lof_gemm(wcol[k], cols[b, k].contiguous(), 12)
                                      for k in range(4)]) for b in range(2)]).view(2, 12, 7, 7)
    assert same_bits(from_gpu(got), from_gpu(ref))

    c = lg.LoF_Conv2d(5, 6, 3, padding=1, act_params=_p3109(8, 4), weight_params=_p3109(8, 4),
                      bias=False, accum_mant_bits=10, backend="cutlass").cuda()
    x = torch.randn(1, 5, 6, 6, device="cuda")
    with torch.no_grad():
        got = c(x)
        xq = lg.virtual_round(x, c.act_params)
        wq = lg.virtual_round(c.weight, c.weight_params)
    want = O.conv2d(from_gpu(xq), from_gpu(wq), 10, padding=(1, 1), order="tiled8")
    assert same_bits(from_gpu(got), want)


def test_layer_mx_scaling():
    torch.manual_seed(2)
    layer = lg.LoF_Conv2d(32, 16, 3, padding=1, act_params=_p3109(8, 4),
                          weight_params=_p3109(8, 4), bias=False, accum_mant_bits=10,
                          scaling="mx", mx_block_size=32).cuda()
    x = torch.randn(2, 32, 8, 8, device="cuda")
    with torch.no_grad():
        got = layer(x)
        e8 = lg.create_e8m0_params()
        cols = F.unfold(x, kernel_size=3, padding=1)
        xq = lg.virtual_mx_round(cols.transpose(1, 2).contiguous(), 32, layer.act_params, e8)
        xq = xq.transpose(1, 2).contiguous()
        wq = lg.virtual_mx_round(layer.weight.reshape(16, -1), 32, layer.weight_params, e8)
        ref = torch.stack([lg.lof_gemm(wq, xq[b].contiguous(), 10) for b in range(2)])
    assert got.shape == (2, 16, 8, 8)
    assert same_bits(from_gpu(got).reshape(2, 16, -1), from_gpu(ref))


def test_layer_cutlass_backend_with_groups():
    """backend="cutlass" with groups: each group an independent implicit-GEMM
    convolution over its channels, in the kernel's tiled reduction order."""
    torch.manual_seed(3)
    layer = lg.LoF_Conv2d(12, 6, 3, padding=1, groups=3, act_params=_p3109(8, 4),
                          weight_params=_p3109(8, 4), bias=False, accum_mant_bits=10,
                          backend="cutlass").cuda()
    x = torch.randn(2, 12, 7, 6, device="cuda")
    with torch.no_grad():
        got = from_gpu(layer(x))
        xq = from_gpu(lg.virtual_round(x, layer.act_params))
        wq = from_gpu(lg.virtual_round(layer.weight, layer.weight_params))
    want = np.concatenate([O.conv2d(np.ascontiguousarray(xq[:, 4 * g:4 * g + 4]),
                                    np.ascontiguousarray(wq[2 * g:2 * g + 2]), 10, padding=(1, 1),
                                    order="tiled8") for g in range(3)], axis=1)
    assert same_bits(got, want)


def _mx_cols(x, layer, g, cin, cout):
    e8 = lg.create_e8m0_params()
    cols = F.unfold(x[:, g * cin:(g + 1) * cin], kernel_size=3, padding=1)
    xq = lg.virtual_mx_round(cols.transpose(1, 2).contiguous(), 32, layer.act_params, e8)
    wq = lg.virtual_mx_round(layer.weight[g * cout:(g + 1) * cout].reshape(cout, -1), 32,
                             layer.weight_params, e8)
    return from_gpu(xq), from_gpu(wq)          # (N, L, K), (cout, K)


@pytest.mark.parametrize("backend", ["im2col", "cutlass"])
def test_layer_mx_scaling_with_groups(backend):
    """scaling="mx" with groups: MX blocks along each group's im2col reduction;
    im2col sums it in order, cutlass in the implicit-GEMM kernel's tiled order
    (the same rounded values, the reduction axis permuted)."""
    from lofloat_gb300.layers import _tiled8_order
    torch.manual_seed(4)
    G, cin, cout = 2, 32, 3
    layer = lg.LoF_Conv2d(G * cin, G * cout, 3, padding=1, groups=G, act_params=_p3109(8, 4),
                          weight_params=_p3109(8, 4), bias=False, accum_mant_bits=10,
                          scaling="mx", mx_block_size=32, backend=backend).cuda()
    x = torch.randn(2, G * cin, 5, 6, device="cuda")
    with torch.no_grad():
        got = from_gpu(layer(x)).reshape(2, G * cout, -1)
        parts = []
        for g in range(G):
            xq, wq = _mx_cols(x, layer, g, cin, cout)
            if backend == "cutlass":
                perm = _tiled8_order(cin, 9, "cpu").numpy()
                xq, wq = xq[..., perm], wq[:, perm]
            parts.append(np.stack([O.gemm(np.ascontiguousarray(wq), np.ascontiguousarray(xq[n].T), 10)
                                   for n in range(2)]))
    assert same_bits(got, np.concatenate(parts, axis=1))
