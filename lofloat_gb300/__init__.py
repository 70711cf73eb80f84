"""lofloat_gb300 — GB300 (sm_103a) kernels for LoFloat's emulation hot path.

Drop-in surface of the reference package ``LoFloat`` for that path:

* ``virtual_round`` / ``virtual_mx_round`` / ``lof_gemm`` and the enums and
  ``FloatFormatDescriptor`` of the compiled module (src/LoPy_bind.cpp);
* ``torch.ops.lofloat.virtual_round / virtual_mx_round / lof_gemm`` with the
  reference's schemas (LoFloat/_custom_ops.py);
* the format factories (LoFloat/formats.py);
* ``lof_conv2d`` and ``pwl_silu`` of the compiled module;
* ``STERound``, ``STEMXRound``, ``LoF_Quantize``, ``LoF_Linear``, ``LoF_Conv2d``,
  ``PWLSiLU`` (LoFloat/layers.py), plus a differentiable emulated linear
  (``lof_linear``).

All compute runs in liblofgb.so (include/lofgb.h) on CUDA tensors.
"""
from . import _custom_ops  # noqa: F401  (registers torch.ops.lofloat.*)
from .binding import (FloatFormatDescriptor, InfBehavior, NaNBehavior, RoundingMode, Signedness,
                      SaturationMode, codec_format, conv2d, conv2d_alpha, gemm, gemm_alpha,
                      gemm_f64_reference, get_rng_state, lof_conv2d, lof_decode, lof_encode, lof_gemm,
                      mx_decode, mx_encode, packed_size, pwl_silu, set_rng_state, set_seed,
                      virtual_mx_round, virtual_round)
from .formats import (create_e8m0_params, create_half_params, create_p3109_params,
                      create_single_params, make_format)
from .layers import (LinearConfig, LoF_Conv2d, LoF_Linear, LoF_MultiHeadAttention, LoF_Quantize,
                     LoFLinearFunction, PWLSiLU, STEMXRound, STERound, _fwht, _lof_gemm_2d,
                     _lof_linear, _quantize, exp_mant_quantize, lof_linear, mantissa_quantize)
from ._custom_ops import get_format, register_format
from .grouped import GroupedRound
from .norms import FISRBatchNorm, L1BatchNorm, LinfBatchNorm, PWLBatchNorm
from .autotune import GroupedGemm

__all__ = [
    "FloatFormatDescriptor", "InfBehavior", "NaNBehavior", "RoundingMode", "Signedness",
    "virtual_round", "virtual_mx_round", "lof_gemm", "gemm", "gemm_alpha", "gemm_f64_reference",
    "set_seed", "get_rng_state", "set_rng_state", "create_p3109_params", "create_e8m0_params",
    "create_half_params", "create_single_params", "make_format", "STERound", "STEMXRound",
    "LoF_Quantize", "LoF_Linear", "LoFLinearFunction", "LinearConfig", "lof_linear",
    "mantissa_quantize", "exp_mant_quantize",
    "register_format", "get_format", "GroupedRound", "GroupedGemm", "lof_conv2d", "conv2d",
    "conv2d_alpha", "pwl_silu", "LoF_Conv2d", "PWLSiLU", "LoF_MultiHeadAttention",
    "SaturationMode", "codec_format", "packed_size", "lof_encode", "lof_decode", "mx_encode",
    "mx_decode",
    "L1BatchNorm", "LinfBatchNorm", "FISRBatchNorm", "PWLBatchNorm",
]
