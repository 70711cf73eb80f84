"""The oracle's per-element random stream: lanes of one SplitMix64 output,
64 >> lg bits each, from the low end; lg = 0 is one output per element."""
import pytest

from oracle import oracle as O

SR_A, SR_B, SR_C, TRUE_SR, PROB, SR_D = 3, 8, 9, 10, 11, 14


@pytest.mark.parametrize("mode,ln,lgl", [
    (0, 0, 3), (1, 0, 3), (12, 0, 3), (SR_A, 0, 3), (SR_A, 8, 3), (SR_A, 9, 2), (SR_A, 16, 2),
    (SR_A, 17, 1), (SR_A, 32, 1), (SR_A, 33, 0), (SR_A, 62, 0), (SR_B, 8, 3), (SR_C, 16, 2),
    (SR_D, 7, 3), (SR_D, 8, 2), (SR_D, 15, 2), (SR_D, 16, 1), (SR_D, 31, 1), (SR_D, 32, 0),
    (PROB, 0, 3), (PROB, 40, 3), (TRUE_SR, 0, 0), (TRUE_SR, 8, 0)])
def test_lane_width_table(mode, ln, lgl):
    assert O.rng_lanes_log2(mode, ln) == lgl


def test_lanes_are_slices_of_one_output():
    for seed in (0, 1, 0xDEADBEEF12345678):
        for lgl in range(4):
            per, bits = 1 << lgl, 64 >> lgl
            for g in list(range(0, 40)) + [(1 << 40) + 5, (1 << 63) + 3]:
                w = O.rng(seed, g >> lgl)
                lane = g % per
                r = O.rng_elem(seed, g, lgl)
                assert r == w >> (lane * bits)
                assert r & ((1 << bits) - 1) == (w >> (lane * bits)) & ((1 << bits) - 1)
    assert all(O.rng_elem(7, g, 0) == O.rng(7, g) for g in range(100))
