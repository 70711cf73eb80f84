"""GPU parity of the strided-batched emulated GEMM and of the attention layer
built on it: every product of a batch is bit-identical to the single GEMM
(plain: to the oracle; tensor cores: to the single tensor-core launch), and
LoF_MultiHeadAttention reproduces the reference's per-(batch, head) loop of
lof_gemm calls (LoFloat/layers.py:1152-1410) bit for bit."""
import numpy as np
import pytest
import torch

import lofloat_gb300 as lg
from golden_io import same_bits
from gpu_util import from_gpu, mismatch_report, to_gpu
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("batch", [1, 3, 17])
@pytest.mark.parametrize("ta,tb", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_plain_batched_vs_oracle(batch, ta, tb):
    rng = np.random.default_rng(batch * 4 + ta * 2 + tb)
    M, N, K = 70, 130, 90
    A = rng.standard_normal((batch, K, M) if ta else (batch, M, K)).astype(np.float32)
    B = rng.standard_normal((batch, N, K) if tb else (batch, K, N)).astype(np.float32)
    got = from_gpu(lg.gemm(to_gpu(A), to_gpu(B), 10, trans_a=bool(ta), trans_b=bool(tb), alpha=0.5))
    assert got.shape == (batch, M, N)
    for b in range(batch):
        want = O.gemm(A[b], B[b], 10, alpha=0.5, trans_a=ta, trans_b=tb)
        assert same_bits(got[b], want), (b, mismatch_report(got[b], got[b], want))


def test_plain_batched_broadcast_operand():
    rng = np.random.default_rng(11)
    A = rng.standard_normal((40, 64)).astype(np.float32)
    B = rng.standard_normal((5, 64, 24)).astype(np.float32)
    got = from_gpu(lg.gemm(to_gpu(A), to_gpu(B), 12))
    for b in range(5):
        assert same_bits(got[b], O.gemm(A, B[b], 12))


@pytest.mark.parametrize("batch", [2, 5])
def test_tc_batched_equals_single(batch):
    rng = np.random.default_rng(batch)
    M, N, K = 200, 136, 320
    A = rng.standard_normal((batch, M, K)).astype(np.float32)
    Bt = rng.standard_normal((batch, N, K)).astype(np.float32)
    Ag, Bg = to_gpu(A), to_gpu(Bt)
    got = from_gpu(lg.gemm(Ag, Bg, 10, trans_b=True, variant="tc", chunk=32))
    for b in range(batch):
        single = from_gpu(lg.gemm(Ag[b], Bg[b], 10, trans_b=True, variant="tc", chunk=32))
        assert same_bits(got[b], single), b
    assert lg.binding.tc_device_status() == 0


def test_lof_gemm_2d_batch_matches_loop():
    """_lof_gemm_2d on 4-D operands = the reference's loop of lof_gemm calls."""
    rng = np.random.default_rng(3)
    q = to_gpu(rng.standard_normal((2, 3, 17, 16)).astype(np.float32))
    k = to_gpu(rng.standard_normal((2, 3, 23, 16)).astype(np.float32))
    got = lg._lof_gemm_2d(q, k.transpose(-2, -1), 10, 0, 0)     # K^T read in place
    loop = torch.stack([lg.lof_gemm(q.reshape(-1, 17, 16)[i].contiguous(),
                                    k.transpose(-2, -1).reshape(-1, 16, 23)[i].contiguous(), 10)
                        for i in range(6)]).reshape(2, 3, 17, 23)
    assert same_bits(from_gpu(got), from_gpu(loop))
    v = to_gpu(rng.standard_normal((2, 3, 23, 16)).astype(np.float32))
    got2 = lg._lof_gemm_2d(got, v, 10, 0, 0, scale_a=2.0, scale_b=0.5)
    loop2 = torch.stack([lg.lof_gemm(got.reshape(-1, 17, 23)[i].contiguous(),
                                     v.reshape(-1, 23, 16)[i].contiguous(), 10, scale_a=2.0,
                                     scale_b=0.5) for i in range(6)]).reshape(2, 3, 17, 16)
    assert same_bits(from_gpu(got2), from_gpu(loop2))


def _reference_mha(layer, query, key, value, attn_mask=None, key_padding_mask=None):
    """The reference's forward (LoFloat/layers.py:1306-1350) written with
    one lof_gemm call per product, as its _lof_linear / _lof_gemm_2d do."""
    def lin(x, w, b):
        k = x.shape[-1]
        out = lg.lof_gemm(x.reshape(-1, k).contiguous(), w.t().contiguous(), layer.accum_mant_bits)
        out = out.reshape(*x.shape[:-1], w.shape[0])
        return out + b if b is not None else out

    def bmm(a, b):
        m, kk, n = a.shape[-2], a.shape[-1], b.shape[-1]
        af, bf = a.reshape(-1, m, kk).contiguous(), b.reshape(-1, kk, n).contiguous()
        return torch.stack([lg.lof_gemm(af[i], bf[i], layer.accum_mant_bits)
                            for i in range(af.shape[0])]).reshape(*a.shape[:-2], m, n)

    B, T, E = query.shape
    S = key.shape[1]
    qz = lambda t, p: layer._quantize(t, p)  # noqa: E731
    query, key, value = qz(query, layer.act_params), qz(key, layer.act_params), qz(value, layer.act_params)
    wq, wk, wv, wo = (qz(w, layer.weight_params) for w in
                      (layer.q_weight, layer.k_weight, layer.v_weight, layer.out_weight))
    bq, bk, bv, bo = (qz(b, layer.bias_params) if b is not None else None for b in
                      (layer.q_bias, layer.k_bias, layer.v_bias, layer.out_bias))
    h, d = layer.num_heads, layer.head_dim
    q = lin(query, wq, bq).view(B, T, h, d).transpose(1, 2)
    k = lin(key, wk, bk).view(B, S, h, d).transpose(1, 2)
    v = lin(value, wv, bv).view(B, S, h, d).transpose(1, 2)
    attn = bmm(q, k.transpose(-2, -1)) * layer.scale
    if attn_mask is not None:
        attn = attn + attn_mask
    if key_padding_mask is not None:
        attn = attn.masked_fill(key_padding_mask.unsqueeze(1).unsqueeze(2), float("-inf"))
    attn = torch.softmax(attn, dim=-1)
    out = bmm(attn, v).transpose(1, 2).contiguous().view(B, T, E)
    return lin(out, wo, bo)


@pytest.mark.parametrize("scaling", ["per_tensor", "mx"])
def test_mha_matches_reference_forward(scaling):
    torch.manual_seed(0)
    e4m3 = lg.create_p3109_params(8, 4)
    layer = lg.LoF_MultiHeadAttention(64, 4, act_params=e4m3, weight_params=e4m3,
                                      bias_params=lg.create_p3109_params(16, 11),
                                      accum_mant_bits=10, scaling=scaling).cuda().eval()
    with torch.no_grad():
        for b in (layer.q_bias, layer.k_bias, layer.v_bias, layer.out_bias):
            b.uniform_(-0.1, 0.1)
        x = torch.randn(3, 20, 64, device="cuda")
        kv = torch.randn(3, 12, 64, device="cuda")
        mask = torch.zeros(20, 12, device="cuda")
        mask[:, -2:] = -1e4
        kpm = torch.zeros(3, 12, dtype=torch.bool, device="cuda")
        kpm[1, :3] = True
        got, w = layer(x, kv, kv, attn_mask=mask, key_padding_mask=kpm, need_weights=True)
        want = _reference_mha(layer, x, kv, kv, attn_mask=mask, key_padding_mask=kpm)
    assert w.shape == (3, 4, 20, 12)
    assert same_bits(from_gpu(got), from_gpu(want))


def test_mha_from_torch_module_and_tc():
    torch.manual_seed(1)
    mha = torch.nn.MultiheadAttention(32, 2, batch_first=True).cuda()
    e5m2 = lg.create_p3109_params(8, 3)
    layer = lg.LoF_MultiHeadAttention.from_mha(mha, e5m2, e5m2, accum_mant_bits=23).eval()
    x = torch.randn(2, 9, 32, device="cuda")
    with torch.no_grad():
        got, _ = layer(x, x, x)
        ref, _ = mha(x, x, x)
    # E5M2 weights and activations: close to the FP32 module, not equal
    assert (got - ref).abs().max() < 0.25 * ref.abs().max()
    layer.gemm_variant = "tc"
    with torch.no_grad():
        tc, _ = layer(x, x, x)
    assert (tc - got).abs().max() < 1e-3 * got.abs().max() + 1e-6
