"""PWL knot tables (lofloat_gb300.pwl.pwl_table) against the tables of the
reference's own layers, recorded in tests/golden/golden_layers.npz by
tests/golden/make_layers_golden.py: PWLSiLU over several ranges, widths and
all three constructions, and PWLBatchNorm's 1/sqrt table. Bit for bit."""
import numpy as np
import pytest

import lofloat_gb300 as lg
from golden_io import load, same_bits


@pytest.fixture(scope="module")
def golden():
    return load("golden_layers.npz")


def test_silu_tables_match_reference(golden):
    keys = [k for k in golden.files if k.startswith("silu_lut_")]
    assert len(keys) >= 30
    for k in keys:
        _, _, r, b, method = k.split("_")
        m = lg.PWLSiLU(R=float(r[1:]), lut_bits=int(b[1:]), lut_method=method)
        assert same_bits(m.lut.numpy(), golden[k]), k


def test_batchnorm_tables_match_reference(golden):
    keys = [k for k in golden.files if k.startswith("bn_lut_")]
    assert len(keys) >= 18
    for k in keys:
        _, _, b, method = k.split("_")
        m = lg.PWLBatchNorm(3, lut_bits=int(b[1:]), lut_method=method)
        assert same_bits(m.lut.numpy(), golden[k]), k


def test_table_errors():
    with pytest.raises(ValueError):
        lg.PWLSiLU(lut_method="cubic")
    with pytest.raises(ValueError):
        lg.PWLSiLU(lut_bits=13)        # beyond the kernel's 4096 segments
    t = lg.pwl.pwl_table(lg.pwl.silu, -4.0, 4.0, 8, "minimax")
    assert t.shape == (9,) and np.isfinite(t.numpy()).all()
