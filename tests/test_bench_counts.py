"""The work counts bench.py reports beside its measurements (CPU): the
reference's algorithmic 16 M^3 per slice, and the split of the executed work
between the FP64 pipe and the FP16 tensor pipe for each block level of the
slice inverse (RG_SPLIT_INVERSE)."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_algorithmic_count_is_the_reference_sweep():
    # src/waveguide.f90:426-440: inverse 8 M^3 + product 8 M^3 per slice, the first slice inverse only
    assert bench.flops_per_realization(256, 2000) == 16.0 * 256 ** 3 * 1999 + 8.0 * 256 ** 3


@pytest.mark.parametrize("levels, M, fp64, fp16", [
    # two levels at 256 modes: four 64-mode Gauss-Jordan blocks; 26 digit pairs x 4 real
    # products x 2 k^3 per k x k product for the propagator, 4 products of 128, 8 of 64
    ("2", 256, 4 * 4 * 64 ** 3, 208 * 256 ** 3 + 4 * 208 * 128 ** 3 + 8 * 208 * 64 ** 3),
    ("1", 256, 2 * 4 * 128 ** 3, 208 * 256 ** 3 + 4 * 208 * 128 ** 3),
    ("0", 256, 4 * 256 ** 3, 208 * 256 ** 3),
    # a level needs an even size of at least 128: 200 -> 100 stops after one
    ("2", 200, 2 * 4 * 100 ** 3, 208 * 200 ** 3 + 4 * 208 * 100 ** 3),
    ("2", 512, 4 * 4 * 128 ** 3, 208 * 512 ** 3 + 4 * 208 * 256 ** 3 + 8 * 208 * 128 ** 3),
])
def test_executed_split_follows_the_block_levels(monkeypatch, levels, M, fp64, fp16):
    monkeypatch.setenv("RG_SPLIT_INVERSE", levels)
    monkeypatch.delenv("RG_TENSOR_R", raising=False)
    assert bench.executed_flops(M, 3, "blocked_symmetric") == (3.0 * fp64, 3.0 * fp16)


def test_executed_without_tensor_products(monkeypatch):
    monkeypatch.setenv("RG_TENSOR_R", "0")
    # the symmetric sweep carrying B Gs1: 12 M^3 + 4 M^2 per slice, all FP64
    assert bench.executed_flops(256, 1, "blocked_symmetric") == (12.0 * 256 ** 3 + 4.0 * 256 ** 2, 0.0)
