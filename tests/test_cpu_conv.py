"""CPU checks of the conv2d and PWL-SiLU oracles and of the host-side layer
logic (no GPU).

The conv2d oracle is pinned to the GEMM oracle (itself pinned to the
reference's compiled leaf through the golden vectors): in "crs" order it must
equal F.unfold followed by the sequential-k GEMM per image — the reference's
default LoF_Conv2d path — and in "tiled8" order it must equal the GEMM over an
explicitly permuted im2col matrix whose rows follow CUTLASS's analytic
iterator order (8-channel tile, r, s, channel in tile) with zero rows for
channels past C."""
import numpy as np
import pytest
import torch
import torch.nn.functional as F

from golden_io import same_bits
from oracle import oracle as O


def _tiled8_rows(c, r, s):
    rows = []
    for ct in range((c + 7) // 8):
        for rr in range(r):
            for ss in range(s):
                for ci in range(8):
                    ch = ct * 8 + ci
                    rows.append(ch * r * s + rr * s + ss if ch < c else -1)
    return rows


@pytest.mark.parametrize("shape", [(2, 6, 9, 8, 5, 3, 2, (2, 1), (1, 0), (1, 2)),
                                   (1, 3, 7, 7, 4, 3, 3, (1, 1), (1, 1), (1, 1)),
                                   (3, 17, 5, 6, 6, 1, 3, (1, 1), (0, 2), (1, 1))])
def test_conv_oracle_pinned_to_gemm_oracle(shape):
    n, c, h, w, k, r, s, st, pd, dl = shape
    rng = np.random.default_rng(c * 31 + k)
    x = rng.standard_normal((n, c, h, w)).astype(np.float32)
    wt = rng.standard_normal((k, c, r, s)).astype(np.float32)
    cols = F.unfold(torch.from_numpy(x), kernel_size=(r, s), dilation=dl, padding=pd,
                    stride=st).numpy()                       # (n, c*r*s, L), rows (c, r, s)
    p, q = O.conv_out_size(h, w, r, s, st, pd, dl)
    crs = O.conv2d(x, wt, 10, stride=st, padding=pd, dilation=dl, alpha=0.5, order="crs")
    want = np.stack([O.gemm(wt.reshape(k, -1), cols[b], 10, alpha=0.5) for b in range(n)])
    assert same_bits(crs, want.reshape(n, k, p, q))

    rows = _tiled8_rows(c, r, s)
    idx = np.array([max(v, 0) for v in rows])
    live = np.array([v >= 0 for v in rows])
    wt8 = wt.reshape(k, -1)[:, idx] * live
    t8 = O.conv2d(x, wt, 10, stride=st, padding=pd, dilation=dl, alpha=0.5, order="tiled8")
    want8 = np.stack([O.gemm(wt8.astype(np.float32), (cols[b][idx] * live[:, None]).astype(np.float32),
                             10, alpha=0.5) for b in range(n)])
    assert same_bits(t8, want8.reshape(n, k, p, q))


def test_conv_oracle_exact_inputs_match_fp64():
    rng = np.random.default_rng(1)
    x = rng.integers(-3, 4, (2, 5, 7, 6)).astype(np.float32)
    wt = rng.integers(-2, 3, (4, 5, 3, 3)).astype(np.float32)
    ref = F.conv2d(torch.from_numpy(x).double(), torch.from_numpy(wt).double(), stride=(1, 2),
                   padding=1).numpy()
    for order in ("crs", "tiled8"):
        y = O.conv2d(x, wt, 23, stride=(1, 2), padding=(1, 1), order=order)
        assert np.array_equal(y.astype(np.float64), ref)


def test_conv_oracle_column_sample():
    rng = np.random.default_rng(2)
    x = rng.standard_normal((2, 4, 6, 6)).astype(np.float32)
    wt = rng.standard_normal((3, 4, 3, 3)).astype(np.float32)
    full = O.conv2d(x, wt, 10, padding=(1, 1))
    part = O.conv2d(x, wt, 10, padding=(1, 1), col0=40, ncols=20)
    flat_full = full.transpose(0, 2, 3, 1).reshape(-1, 3)
    flat_part = part.transpose(0, 2, 3, 1).reshape(-1, 3)
    assert same_bits(flat_part[40:60], flat_full[40:60])
    assert not flat_part[:40].any() and not flat_part[60:].any()


def test_pwl_oracle_against_interpolation_formula():
    """The oracle against the table interpolation written out in float64:
    u = (clamp(x) + R) n / 2R, i = min(floor(u), n - 1),
    y = T_i + (u - i)(T_(i+1) - T_i), relu outside [-R, R]."""
    import lofloat_gb300 as lg
    m = lg.PWLSiLU(R=8.0, lut_bits=6)
    x = (np.random.default_rng(3).standard_normal(20000) * 5).astype(np.float32)
    got = O.pwl_silu(x, m.lut.numpy(), 8.0)
    t = m.lut.numpy().astype(np.float64)
    u = (np.clip(x.astype(np.float64), -8, 8) + 8) * (64 / 16)
    i = np.minimum(np.floor(u).astype(np.int64), 63)
    ref = t[i] + (u - i) * (t[i + 1] - t[i])
    ref = np.where(np.abs(x) > 8, np.maximum(x, 0), ref)
    assert np.allclose(got, ref, atol=2e-6, rtol=1e-6)
    knots = np.linspace(-8.0, 8.0, 65, dtype=np.float32)[:-1]
    assert same_bits(O.pwl_silu(knots, m.lut.numpy(), 8.0), m.lut.numpy()[:-1])
    outside = np.array([-9.0, 9.0, np.inf, -np.inf], np.float32)
    assert same_bits(O.pwl_silu(outside, m.lut.numpy(), 8.0),
                     np.array([0.0, 9.0, np.inf, 0.0], np.float32))


def test_layer_constructor_validation():
    import lofloat_gb300 as lg
    e4m3 = lg.create_p3109_params(8, 4)
    with pytest.raises(ValueError):
        lg.LoF_Conv2d(3, 4, 3, act_params=e4m3, weight_params=e4m3, scaling="mx", mx_block_size=32)
    # every backend takes groups and MX scaling
    lg.LoF_Conv2d(32, 4, 1, act_params=e4m3, weight_params=e4m3, scaling="mx", backend="cutlass")
    lg.LoF_Conv2d(4, 4, 3, groups=2, act_params=e4m3, weight_params=e4m3, backend="cutlass")
    lg.LoF_Conv2d(64, 4, 1, groups=2, act_params=e4m3, weight_params=e4m3, scaling="mx")
    with pytest.raises(ValueError):   # the group's reduction 16 * 1 * 1 is not a whole MX block
        lg.LoF_Conv2d(32, 4, 1, groups=2, act_params=e4m3, weight_params=e4m3, scaling="mx")
    with pytest.raises(ValueError):
        lg.LoF_Conv2d(6, 4, 3, act_params=e4m3, weight_params=e4m3, hadamard_transform=True)
    with pytest.raises(ValueError):
        lg.LoF_Conv2d(6, 4, 3, act_params=e4m3, weight_params=e4m3, backend="cudnn")
    layer = lg.LoF_Conv2d(8, 4, 3, act_exp=4, act_mant=3, weight_exp=4, weight_mant=3,
                          bias_exp=5, bias_mant=10, accum_mant_bits=12)
    assert layer.weight.shape == (4, 8, 3, 3)
    import copy
    twin = copy.deepcopy(layer)
    assert torch.equal(twin.weight, layer.weight) and twin.accum_mant_bits == 12
    conv = torch.nn.Conv2d(8, 4, 3, padding=1, bias=True)
    lifted = lg.LoF_Conv2d.from_conv2d(conv, e4m3, e4m3, bias_params=e4m3)
    assert torch.equal(lifted.weight, conv.weight) and lifted.padding == (1, 1)


def test_format_accumulator_oracle_reduces_to_mantissa_rounding():
    """With FP32's exponent range (8 exponent bits, bias 127) and no
    overflow or subnormal sums, rounding the accumulator into the format is
    the mantissa-only rounding of the reference leaf."""
    rng = np.random.default_rng(3)
    A = rng.standard_normal((20, 300)).astype(np.float32)
    B = rng.standard_normal((300, 16)).astype(np.float32)
    for m in (7, 10, 12):
        fmt = O.fmt(9 + m, m, 127, saturating=False)
        assert same_bits(O.gemm_accfmt(A, B, fmt, alpha=0.25), O.gemm(A, B, m, alpha=0.25))


@pytest.mark.parametrize("c", [3, 8, 10, 17])
def test_tiled8_order_is_the_conv_kernels_reduction_order(c):
    """The implicit-GEMM conv's 8-channel-tile reduction order, as the layer's
    permutation of the im2col reduction axis: a sequential emulated GEMM over
    the permuted columns gives the conv oracle's tiled-order bits."""
    from lofloat_gb300.layers import _tiled8_order
    rng = np.random.default_rng(c)
    x = rng.standard_normal((2, c, 6, 5)).astype(np.float32)
    w = rng.standard_normal((4, c, 3, 3)).astype(np.float32)
    want = O.conv2d(x, w, 9, padding=(1, 1), order="tiled8")
    perm = _tiled8_order(c, 9, "cpu").numpy()
    cols = F.unfold(torch.from_numpy(x), kernel_size=3, padding=1).numpy()     # (N, C*9, L)
    wc = np.ascontiguousarray(w.reshape(4, -1)[:, perm])
    for n in range(2):
        got = O.gemm(wc, np.ascontiguousarray(cols[n][perm]), 9)
        assert same_bits(got, want[n].reshape(4, -1)), n
