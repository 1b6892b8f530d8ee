"""Cross-dataset jackknife covariance: the oracle restatement against the
reference's own outputs (tests/golden/crosscov_los3.npz, made by running
MeasureJackknife.measure_covariance_multiple_datasets and
create_full_cov_matrix_projections on three projections)."""

import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
import ia_oracle as O  # noqa: E402

FIX = os.path.join(HERE, "golden", "crosscov_los3.npz")
NAMES = ("LOS_x", "LOS_y", "LOS_z")


def realisations(z, ct, d, n=8):
    return np.array([z[f"out/{ct}/{d}_jk{n}/{d}_{b}"] for b in range(n)])


@pytest.mark.parametrize("ct", ["w_g_plus", "w_gg"])
def test_single_and_pair(ct):
    z = np.load(FIX)
    cov, std = O.jackknife_cross_cov(realisations(z, ct, "LOS_y"), realisations(z, ct, "LOS_y"))
    np.testing.assert_array_equal(cov, z[f"res/{ct}/single_cov"])
    np.testing.assert_array_equal(std, z[f"res/{ct}/single_std"])
    cov, std = O.jackknife_cross_cov(realisations(z, ct, "LOS_x"), realisations(z, ct, "LOS_z"))
    np.testing.assert_array_equal(cov, z[f"res/{ct}/pair_cov"])
    np.testing.assert_array_equal(std, z[f"res/{ct}/pair_std"])    # NaN where the cross sum is negative
    assert np.isnan(std).any() or (std >= 0).all()
    # the written datasets carry the same arrays under the reference's names
    np.testing.assert_array_equal(z[f"out/{ct}/LOS_x_LOS_z_jackknife_cov_8"], z[f"res/{ct}/pair_cov"])


@pytest.mark.parametrize("ct", ["w_g_plus", "w_gg"])
def test_full_projection_matrices(ct):
    z = np.load(FIX)
    r = {d: realisations(z, ct, d) for d in NAMES}
    own = [O.jackknife_cross_cov(r[d], r[d])[0] for d in NAMES]
    pairs = [O.jackknife_cross_cov(r[a], r[b])[0] for a, b in ((0, 1), (0, 2), (1, 2)) for a, b in
             [(NAMES[a], NAMES[b])]]
    full = O.full_projection_cov(*own, *pairs)
    for m, tag in zip(full, ("cov3", "cov2xy", "cov2xz", "cov2yz")):
        np.testing.assert_array_equal(m, z[f"res/{ct}/{tag}"])
    np.testing.assert_array_equal(full[0], z[f"out/{ct}/LOS_x_LOS_y_LOS_z_combined_jackknife_cov_8"])


@pytest.mark.parametrize("cls_name", ["MeasureIABox", "MeasureIALightcone"])
def test_covariance_methods_on_stored_realisations(cls_name, tmp_path, monkeypatch):
    """The two covariance methods of both drop-in classes on realisations
    already in an output file (the reference's own, from the fixture), with
    the device arithmetic replaced by the oracle: the file handling, names and
    block assembly, on the CPU."""
    import torch
    import measure_ia_gb300 as P
    from measure_ia_gb300 import engine, hdf5, open_output
    z = np.load(FIX)
    out = str(tmp_path / "stored.hdf5")
    # the reference's stored datasets: realisations and each projection's own covariance
    hdf5.write_file(out, {k[4:]: z[k] for k in z.files if k.startswith("out/") and "combined" not in k})

    def cpu_cross_cov(a, b=None, device=0):
        cov, std = O.jackknife_cross_cov(a, a if b is None else b)
        return torch.from_numpy(np.asarray(cov)), torch.from_numpy(np.asarray(std))

    monkeypatch.setattr(engine, "jackknife_cross_cov", cpu_cross_cov)
    if cls_name == "MeasureIABox":
        obj = P.MeasureIABox(None, out, None, None, boxsize=205.0)
    else:
        obj = P.MeasureIALightcone(None, None, out, pi_max=20.0)
    assert obj.snap_group == ""
    for ct in ("w_g_plus", "w_gg"):
        c, s = obj.measure_covariance_multiple_datasets(ct, ["LOS_x", "LOS_z"], num_box=8, return_output=True)
        np.testing.assert_array_equal(c, z[f"res/{ct}/pair_cov"])
        full = obj.create_full_cov_matrix_projections(ct, ["LOS_x", "LOS_y", "LOS_z"], num_box=8, return_output=True)
        for m, tag in zip(full, ("cov3", "cov2xy", "cov2xz", "cov2yz")):
            np.testing.assert_array_equal(m, z[f"res/{ct}/{tag}"])
        obj.create_full_cov_matrix_projections(ct, ["LOS_x", "LOS_y", "LOS_z"], num_box=8)
    st = open_output(out)
    assert "w_g_plus/LOS_x_LOS_y_LOS_z_combined_jackknife_cov_8" in set(st.keys())
