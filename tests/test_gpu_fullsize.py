"""Parity at the full size of the metric's workload (4M clustered positions,
1M shapes, 27 jackknife regions), through properties that hold at any size:
the mixed form's integer counts equal the plain FP64 form's, its w agree to
the stated tolerance, and halving every weight divides DD and w_g+ by exactly
4 and their covariance by exactly 16 (the reference's test_weights.py:5-40
relations, exact here because the fixed-point scales move by powers of two)."""

import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def workload():
    import torch
    sys.path.insert(0, ROOT)
    import bench
    from measure_ia_gb300.engine import PairCounter
    data = bench.make_catalog()
    common = dict(boxsize=bench.L_BOX, r_bins=bench.R_BINS, r_min=0.1, r_max=20.0, p_bins=bench.PI_BINS,
                  l_subboxes=3, cell_size=4.0, cell_refine=2, shapes_per_unit=128, cell_size_los=20.0,
                  cell_refine_los=10)
    pcm = PairCounter("w", precision="mixed", **common)
    dcat = pcm.to_device(data)
    mixed = pcm.measure(dcat)
    fp64 = PairCounter("w", precision="fp64", **common).measure(dcat)
    half = dict(dcat, weight=dcat["weight"] * 0.5, weight_shape_sample=dcat["weight_shape_sample"] * 0.5)
    mixed_half = pcm.measure(half)
    torch.cuda.synchronize()
    return mixed, fp64, mixed_half


def test_counts_bit_exact_at_full_size(workload):
    mixed, fp64, _ = workload
    np.testing.assert_array_equal(mixed.npairs, fp64.npairs)
    assert mixed.stats["binned_pairs"] == fp64.stats["binned_pairs"] > 2e10


def test_w_within_tolerance_at_full_size(workload):
    """w_g+ and w_gg of the mixed form within 1e-6 of the FP64 form, relative
    to the vector's scale and per bin (no bin of this workload is near zero)."""
    mixed, fp64, _ = workload
    for key in ("proj_gp", "proj_gg"):
        a, b = mixed[key], fp64[key]
        assert np.max(np.abs(a - b)) / np.max(np.abs(b)) < 1e-6, key
        assert np.max(np.abs(a - b) / np.abs(b)) < 1e-6, key


def test_weight_scaling_is_exact(workload):
    mixed, _, half = workload
    np.testing.assert_array_equal(half.npairs, mixed.npairs)
    np.testing.assert_array_equal(4.0 * half["DD_all"], mixed["DD_all"])
    np.testing.assert_array_equal(4.0 * half["Splus_all"], mixed["Splus_all"])
    np.testing.assert_array_equal(4.0 * half["proj_gp"], mixed["proj_gp"])
    np.testing.assert_array_equal(16.0 * half["cov_gp"], mixed["cov_gp"])
