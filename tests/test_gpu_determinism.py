"""Bitwise reproducibility, as the reference's internal-consistency tests
assert it (tests/test_m_sim_internal_consistency.py:36-57,
tests/test_w_sim_internal_consistency.py, tests/test_weights.py:5-43):

* w_g+ of a 'g+' run equals that of a 'both' run, and w_gg of a 'gg' run
  that of a 'both' run, bit for bit;
* halving every weight gives exactly a quarter of w_g+ and of DD;
* the same measurement twice gives the same bits (the pairs reach the sums
  in a different order on every run).

Both forms keep their sums as integers (64-bit in the mixed form, 128-bit in
the FP64 form), so none of this depends on the order of the adds.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L = 205.0


def _catalogue(seed, n_pos=6000, n_shape=2500):
    rng = np.random.default_rng(seed)
    cen = rng.uniform(0.0, L, (60, 3))
    pos = np.mod(cen[rng.integers(0, 60, n_pos)] + rng.normal(0.0, 4.0, (n_pos, 3)), L)
    pos[pos >= L] = 0.0
    pick = np.sort(rng.choice(n_pos, n_shape, replace=False))
    ang = rng.uniform(0.0, np.pi, n_shape)
    return {"Position": pos, "Position_shape_sample": pos[pick].copy(),
            "Axis_Direction": np.c_[np.cos(ang), np.sin(ang)], "q": rng.uniform(0.2, 1.0, n_shape),
            "weight": np.exp(rng.normal(0.0, 0.3, n_pos)), "weight_shape_sample": np.exp(rng.normal(0.0, 0.3, n_shape)),
            "LOS": 2}


def _box(data, out, precision):
    from measure_ia_gb300 import MeasureIABox
    d = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in data.items()}
    return MeasureIABox(d, out, "TNG300", 99, [0.1, 20.0], 8, 4, None, boxsize=L, precision=precision)


def _read(out):
    from measure_ia_gb300 import open_output
    s = open_output(out)
    return {k: s.read(k) for k in s.keys()}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["w", "m"])
def test_gg_gp_both(kind, precision, tmp_path):
    data = _catalogue(1)
    out = str(tmp_path / "o.hdf5")
    grp = {"w": ("w_g_plus", "w_gg"), "m": ("multipoles_g_plus", "multipoles_gg")}[kind]
    for name, ct in (("All_both", "both"), ("All_gp", "g+"), ("All_gg", "gg")):
        box = _box(data, out, precision)
        fn = box.measure_xi_w if kind == "w" else box.measure_xi_multipoles
        fn(name, ct, 0, temp_file_path=str(tmp_path))
    r = _read(out)
    g = "Snapshot_99/"
    np.testing.assert_array_equal(r[f"{g}{grp[0]}/All_gp"], r[f"{g}{grp[0]}/All_both"])
    np.testing.assert_array_equal(r[f"{g}{grp[1]}/All_gg"], r[f"{g}{grp[1]}/All_both"])
    sep = "_rp" if kind == "w" else "_r"
    np.testing.assert_array_equal(r[f"{g}{grp[0]}/All_gp{sep}"], r[f"{g}{grp[0]}/All_both{sep}"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["w", "m"])
def test_weights(kind, precision, tmp_path):
    data = _catalogue(2)
    data["weight"] = np.ones(len(data["Position"]))
    data["weight_shape_sample"] = np.ones(len(data["Position_shape_sample"]))
    out = str(tmp_path / "o.hdf5")
    box = _box(data, out, precision)
    fn = box.measure_xi_w if kind == "w" else box.measure_xi_multipoles
    fn("All_both", "both", 8, temp_file_path=str(tmp_path))
    data["weight"] = np.full(len(data["Position"]), 0.5)
    data["weight_shape_sample"] = np.full(len(data["Position_shape_sample"]), 0.5)
    box = _box(data, out, precision)
    fn = box.measure_xi_w if kind == "w" else box.measure_xi_multipoles
    fn("All_both_weight", "both", 8, temp_file_path=str(tmp_path))
    r = _read(out)
    g = "Snapshot_99/"
    gp, gg, xi = (("w_g_plus", "w_gg", "w/xi_gg") if kind == "w"
                  else ("multipoles_g_plus", "multipoles_gg", "multipoles/xi_gg"))
    np.testing.assert_array_equal(r[f"{g}{gp}/All_both"], 4 * r[f"{g}{gp}/All_both_weight"])
    np.testing.assert_array_equal(r[f"{g}{xi}/All_both_DD"], 4 * r[f"{g}{xi}/All_both_weight_DD"])
    np.testing.assert_allclose(r[f"{g}{gp}/All_both_jackknife_cov_8"],
                               16 * r[f"{g}{gp}/All_both_weight_jackknife_cov_8"])
    np.testing.assert_allclose(r[f"{g}{gg}/All_both_jackknife_cov_8"],
                               16 * r[f"{g}{gg}/All_both_weight_jackknife_cov_8"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["w", "m"])
def test_repeat_runs_identical(kind, precision, tmp_path):
    """The whole output file, jackknife realisations and covariances
    included, is the same on a second run."""
    data = _catalogue(3, n_pos=20000, n_shape=8000)
    runs = []
    for k in range(2):
        out = str(tmp_path / f"o{k}.hdf5")
        box = _box(data, out, precision)
        fn = box.measure_xi_w if kind == "w" else box.measure_xi_multipoles
        fn("All", "both", 27, temp_file_path=str(tmp_path))
        runs.append(_read(out))
    assert set(runs[0]) == set(runs[1])
    for k in runs[0]:
        np.testing.assert_array_equal(runs[0][k], runs[1][k], err_msg=k)
