"""The no-allocation tensor-core GEMM entry point (lofgb_gemm_tc_noalloc_f32).

It exists for callers that may not allocate device memory when they run a
GEMM, for example a plugin whose host framework owns all device memory. It
uses a fixed 64 MiB scratch array inside liblofgb.so instead of a workspace
from the caller. This file runs it through the C ABI and checks it against
the workspace-taking entry point (lofgb_gemm_f32, LOFGB_GEMM_TC) on two calls
in a row. Both run the same kernels, so the outputs must agree bit for bit,
which is stricter than the tolerance the tensor-core tests use against the
CPU model. It also checks that warmed-up calls allocate no device memory,
the size limit, and that argument errors come before the size check. The
file is named so pytest collects it last.
"""
import ctypes as C

import pytest
import torch

import lofloat_gb300 as lg
from lofloat_gb300 import _native

pytestmark = pytest.mark.gpu


def _noalloc(A, B, mbits, alpha=1.0, chunk=32, trans_a=False, trans_b=False):
    M, K = (A.shape[1], A.shape[0]) if trans_a else A.shape
    N = B.shape[0] if trans_b else B.shape[1]
    D = torch.empty(M, N, device=A.device)
    st = _native.lib().lofgb_gemm_tc_noalloc_f32(
        A.data_ptr(), A.shape[1], int(trans_a), B.data_ptr(), B.shape[1], int(trans_b),
        D.data_ptr(), N, M, N, K, mbits, alpha, chunk,
        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, _native.lib().lofgb_last_error_detail().decode()
    return D


def test_noalloc_matches_workspace_entry_point_twice():
    torch.manual_seed(0)
    cases = [  # two calls in a row with different shapes, layouts and widths
        dict(M=300, N=200, K=520, mbits=10, chunk=32, trans_a=False, trans_b=True, alpha=1.0),
        dict(M=128, N=384, K=256, mbits=7, chunk=64, trans_a=True, trans_b=False, alpha=0.25),
    ]
    for c in cases:
        A = torch.randn(c["K"], c["M"], device="cuda") if c["trans_a"] else torch.randn(c["M"], c["K"], device="cuda")
        B = torch.randn(c["N"], c["K"], device="cuda") if c["trans_b"] else torch.randn(c["K"], c["N"], device="cuda")
        got = _noalloc(A, B, c["mbits"], c["alpha"], c["chunk"], c["trans_a"], c["trans_b"])
        want = lg.gemm(A, B, c["mbits"], trans_a=c["trans_a"], trans_b=c["trans_b"], alpha=c["alpha"],
                       variant="tc", chunk=c["chunk"])
        torch.cuda.synchronize()
        assert torch.equal(got, want)


def test_noalloc_call_allocates_no_device_memory():
    """After the first call on the device (set-up: it resolves the scratch
    array's address and may load the module), further calls must leave the
    device's free memory and torch's allocator untouched."""
    torch.manual_seed(1)
    A = torch.randn(256, 320, device="cuda")
    B = torch.randn(320, 192, device="cuda")
    D = torch.empty(256, 192, device="cuda")
    L = _native.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def call():
        st = L.lofgb_gemm_tc_noalloc_f32(A.data_ptr(), 320, 0, B.data_ptr(), 192, 0, D.data_ptr(),
                                         192, 256, 192, 320, 10, 1.0, 32, stream)
        assert st == 0, L.lofgb_last_error_detail().decode()

    call()  # first call on this device: set-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    reserved0 = torch.cuda.memory_reserved()
    call()
    call()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_allocated() == alloc0
    assert torch.cuda.memory_reserved() == reserved0


def test_noalloc_rejects_sizes_beyond_its_scratch():
    L = _native.lib()
    need = L.lofgb_gemm_tc_workspace_size(4096, 4096, 4096)
    assert need > 64 * 2**20
    # valid operands of the oversize shape: only the scratch limit is at fault
    A = torch.empty(4096, 4096, device="cuda")
    B = torch.empty(4096, 4096, device="cuda")
    D = torch.empty(4096, 4096, device="cuda")
    st = L.lofgb_gemm_tc_noalloc_f32(A.data_ptr(), 4096, 0, B.data_ptr(), 4096, 0, D.data_ptr(),
                                     4096, 4096, 4096, 4096, 10, 1.0, 32, None)
    assert st == -9
    assert "scratch" in L.lofgb_last_error_detail().decode()
    # invalid arguments give the codes lofgb_gemm_f32 gives, whatever the size
    st = L.lofgb_gemm_tc_noalloc_f32(A.data_ptr(), 4095, 0, B.data_ptr(), 4096, 0, D.data_ptr(),
                                     4096, 4096, 4096, 4096, 10, 1.0, 32, None)
    assert st == -2
    st = L.lofgb_gemm_tc_noalloc_f32(None, 4096, 0, B.data_ptr(), 4096, 0, D.data_ptr(),
                                     4096, 4096, 4096, 4096, 10, 1.0, 32, None)
    assert st == -1
