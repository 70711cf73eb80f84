"""Golden fixtures for the PWL tables and the BatchNorm approximations, made
by importing the reference's own Python layers (LoFloat/layers.py) here.

    python tests/golden/make_layers_golden.py

The reference package imports its compiled extension at import time; these
layers never call it, so a stand-in module takes its place (every attribute
a harmless placeholder). The script records, with torch on the CPU:
  * PWLSiLU tables (R, lut_bits, method) and PWLBatchNorm tables (lut_bits,
    method), as float32;
  * the four BatchNorm variants on seeded inputs: training-mode outputs, the
    gradients for a seeded upstream gradient and the updated running
    statistics, then eval-mode outputs on a second input.
It writes tests/golden/golden_layers.npz and its entry in MANIFEST.json. The
tests read only the fixture, never the reference.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("LOFGB_REFERENCE", "/root/reference")


class _Anything:
    """Placeholder for every name of the reference's compiled extension."""

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Anything()

    def __call__(self, *a, **k):
        return _Anything()


class _StandIn(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Anything()


def import_reference_layers():
    sys.modules["LoFloat.LoFloat"] = _StandIn("LoFloat.LoFloat")
    sys.path.insert(0, REF)
    import LoFloat.layers as L  # noqa: E402
    return L


BN_SHAPES = {"nchw": (8, 6, 5, 7), "nc": (64, 10), "ncl": (4, 3, 17)}
PWL_SILU = [(8.0, b, m) for b in (1, 2, 3, 4, 5, 6, 8, 10, 12) for m in ("uniform", "midpoint", "minimax")]
PWL_SILU += [(r, 4, "minimax") for r in (1.0, 3.3, 6.0, 16.0)]
PWL_BN = [(b, m) for b in (1, 2, 3, 4, 6, 8) for m in ("uniform", "midpoint", "minimax")]


def main():
    L = import_reference_layers()
    out = {}
    for r, bits, m in PWL_SILU:
        mod = L.PWLSiLU(R=r, lut_bits=bits, lut_method=m, use_ext=False)
        out[f"silu_lut_R{r}_b{bits}_{m}"] = mod.lut.numpy().copy()
    for bits, m in PWL_BN:
        mod = L.PWLBatchNorm(3, lut_bits=bits, lut_method=m)
        out[f"bn_lut_b{bits}_{m}"] = mod.lut.numpy().copy()
    variants = {
        "l1": lambda c: L.L1BatchNorm(c),
        "l1_tensor_scale": lambda c: L.L1BatchNorm(c, scale=torch.linspace(0.5, 1.5, c)),
        "linf": lambda c: L.LinfBatchNorm(c),
        "linf_scale": lambda c: L.LinfBatchNorm(c, scale=0.75, momentum=0.3),
        "fisr": lambda c: L.FISRBatchNorm(c),
        "pwl_minimax": lambda c: L.PWLBatchNorm(c),
        "pwl_uniform6": lambda c: L.PWLBatchNorm(c, lut_bits=6, lut_method="uniform"),
        "l1_noaffine": lambda c: L.L1BatchNorm(c, affine=False),
        "fisr_noaffine_eps": lambda c: L.FISRBatchNorm(c, affine=False, eps=1e-3),
    }
    for sname, shape in BN_SHAPES.items():
        g = torch.Generator().manual_seed(len(shape) * 100 + shape[1])
        x = torch.randn(*shape, generator=g) * 3 + 1
        x2 = torch.randn(*shape, generator=g) * 2 - 0.5
        c = shape[1]
        w = torch.randn(c, generator=g) * 0.5 + 1
        b = torch.randn(c, generator=g) * 0.1
        out[f"bn_{sname}_x"] = x.numpy()
        out[f"bn_{sname}_x2"] = x2.numpy()
        out[f"bn_{sname}_w"] = w.numpy()
        out[f"bn_{sname}_b"] = b.numpy()
        for vname, make in variants.items():
            mod = make(c)
            if mod.affine:
                with torch.no_grad():
                    mod.weight.copy_(w)
                    mod.bias.copy_(b)
            mod.train()
            xg = x.clone().requires_grad_(True)
            y = mod(xg)
            gy = torch.randn(*shape, generator=g)
            y.backward(gy)
            key = f"bn_{sname}_{vname}"
            out[key + "_y_train"] = y.detach().numpy()
            out[key + "_gy"] = gy.numpy()
            out[key + "_dx"] = xg.grad.numpy()
            if mod.affine:
                out[key + "_dw"] = mod.weight.grad.numpy().copy()
                out[key + "_db"] = mod.bias.grad.numpy().copy()
            for buf in ("running_mean", "running_mad", "running_maxdev", "running_var"):
                if hasattr(mod, buf):
                    out[key + "_" + buf] = getattr(mod, buf).numpy().copy()
            mod.eval()
            with torch.no_grad():
                out[key + "_y_eval"] = mod(x2).numpy()
    path = os.path.join(HERE, "golden_layers.npz")
    np.savez_compressed(path, **out)
    with open(path, "rb") as fh:
        sha = hashlib.sha256(fh.read()).hexdigest()
    mpath = os.path.join(HERE, "MANIFEST.json")
    with open(mpath) as fh:
        man = json.load(fh)
    man["files"]["golden_layers.npz"] = {"cases": sorted(out), "sha256": sha,
                                        "generator": "python tests/golden/make_layers_golden.py",
                                        "reference": "LoFloat/layers.py (PWLSiLU, BatchNorm variants)"}
    with open(mpath, "w") as fh:
        json.dump(man, fh, indent=1, sort_keys=True)
        fh.write("\n")
    print(f"wrote {path} ({len(out)} arrays)")


if __name__ == "__main__":
    main()
