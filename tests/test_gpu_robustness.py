"""Failure paths that must end in a clean error or a correct result, never a
wrong one: the mixed form's FP64 edge re-test queue overflowing, and the
autotuner meeting launch configurations that fail."""

import math
import warnings

import numpy as np
import pytest

from golden_io import assert_close

pytestmark = pytest.mark.gpu

R_BINS = np.logspace(-1, np.log10(20.0), 11)
PI_BINS = np.linspace(-20.0, 20.0, 9)


def _edge_catalogue():
    from measure_ia_gb300.catalogs import add_edge_pairs, neyman_scott_catalog
    data = neyman_scott_catalog(300, 205.0, 6000, 11, mean_children=40, sigma=1.0)
    return add_edge_pairs(data, 205.0, 5, R_BINS, PI_BINS, 400)


def _counter(precision, **knobs):
    from measure_ia_gb300.engine import PairCounter
    return PairCounter("w", boxsize=205.0, r_bins=R_BINS, r_min=0.1, r_max=20.0, p_bins=PI_BINS, l_subboxes=3,
                       precision=precision, **knobs)


def test_edge_queue_overflow_is_an_error(monkeypatch):
    """A queue of 16 entries cannot hold the re-tests of 400 planted edge
    pairs: the run reports MIA_ERR_OVERFLOW instead of binning them in FP32."""
    from measure_ia_gb300._lib import MIA_ERR_OVERFLOW, MiaError
    data = _edge_catalogue()
    monkeypatch.setenv("MIA_EDGE_CAPACITY", "16")
    pc = _counter("mixed")
    with pytest.raises(MiaError) as err:
        pc.measure(data)
    assert err.value.code == MIA_ERR_OVERFLOW
    # the device and the library stay usable: the default capacity succeeds
    monkeypatch.delenv("MIA_EDGE_CAPACITY")
    ok = _counter("mixed").measure(data)
    ref = _counter("fp64").measure(data)
    np.testing.assert_array_equal(ok.npairs, ref.npairs)


def test_box_falls_back_to_fp64_form_on_overflow(monkeypatch, tmp_path):
    """MeasureIABox(precision='mixed') re-measures in the FP64 form when the
    queue overflows, with a RuntimeWarning, and its products equal an FP64 run."""
    from measure_ia_gb300 import MeasureIABox, open_output
    data = _edge_catalogue()
    kw = dict(separation_limits=[0.1, 20.0], num_bins_r=10, num_bins_pi=8, pi_max=20.0, boxsize=205.0)
    ref = MeasureIABox(data, str(tmp_path / "fp64.hdf5"), **kw, precision="fp64")
    ref.measure_xi_w("d", "both", 27, temp_file_path=str(tmp_path))
    monkeypatch.setenv("MIA_EDGE_CAPACITY", "16")
    box = MeasureIABox(data, str(tmp_path / "mixed.hdf5"), **kw, precision="mixed")
    with warnings.catch_warnings(record=True) as caught:
        warnings.simplefilter("always")
        box.measure_xi_w("d", "both", 27, temp_file_path=str(tmp_path))
    assert any("overflow" in str(w.message) for w in caught)
    np.testing.assert_array_equal(box.last_measurement.npairs, ref.last_measurement.npairs)
    a, b = open_output(str(tmp_path / "fp64.hdf5")), open_output(str(tmp_path / "mixed.hdf5"))
    for path in a.keys():
        assert_close(b.read(path), a.read(path), 1e-12, path)


def test_autotune_skips_failing_candidates(tmp_path):
    """Candidates that raise are timed as infinite; the choice is one that ran."""
    from measure_ia_gb300 import autotune
    from measure_ia_gb300._lib import MIA_ERR_WORKSPACE, MiaError
    data = _edge_catalogue()
    pc = _counter("mixed")
    dcat = pc.to_device(data)
    rp, _ = pc.search_ranges()

    def make(**knobs):
        if knobs["cell_refine"] != 2 or knobs["shapes_per_unit"] == 256:
            raise MiaError(MIA_ERR_WORKSPACE, "candidate refused")
        return pc.with_knobs(**knobs)

    best = autotune.tune(make, dcat, rp)
    assert best["cell_refine"] == 2 and best["shapes_per_unit"] != 256 and math.isfinite(best["ms"])

    def refuse(**knobs):
        raise MiaError(MIA_ERR_WORKSPACE, "candidate refused")

    with pytest.raises(MiaError):
        autotune.tune(refuse, dcat, rp, key="k", path=str(tmp_path / "t.json"))
    assert autotune.load_cache(str(tmp_path / "t.json")) == {}


def test_mixed_form_is_bitwise_reproducible():
    """Every product of the mixed form comes from integer sums (the block
    partials and the dataset's 64-bit totals), so two runs agree exactly
    whatever order the work units and atomics took."""
    from measure_ia_gb300.catalogs import neyman_scott_catalog
    data = neyman_scott_catalog(600, 205.0, 12000, 21, mean_children=40, sigma=1.0)
    pc = _counter("mixed")
    dcat = pc.to_device(data)
    a, b = pc.measure(dcat), pc.measure(dcat)
    np.testing.assert_array_equal(a.npairs, b.npairs)
    for k in a.arrays:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("where,value", [("Position", 205.0), ("Position", -1e-9), ("Position", float("nan")),
                                         ("Position_shape_sample", float("nan")),
                                         ("Position_shape_sample", 205.0 + 1e-12)])
def test_coordinates_outside_the_box_raise(where, value, precision, tmp_path):
    """A coordinate at exactly L, a negative one or a NaN (positions or shape
    positions) is refused on the device: the preparation kernels flag it,
    the pair kernel skips the catalogue, and MeasureIABox raises ValueError
    with the first offending index (the reference's periodic KD-tree,
    ``KDTree(..., boxsize=L)`` at measure_w_box_jk.py:764, raises ValueError
    for such data).  The library stays usable: the next measurement of a valid
    catalogue equals one made before the error."""
    from measure_ia_gb300 import MeasureIABox
    from measure_ia_gb300.catalogs import neyman_scott_catalog
    data = neyman_scott_catalog(200, 205.0, 3000, 21, mean_children=30, sigma=1.0)
    kw = dict(separation_limits=[0.1, 20.0], num_bins_r=10, num_bins_pi=8, pi_max=20.0, boxsize=205.0,
              precision=precision)
    good = MeasureIABox({k: np.array(v) if k != "LOS" else v for k, v in data.items()}, None, **kw)
    good.measure_xi_w("ok", "both", 27, temp_file_path=str(tmp_path))
    before = good.last_measurement
    bad = {k: np.array(v) if k != "LOS" else v for k, v in data.items()}
    idx = 137
    bad[where][idx, 1] = value
    box = MeasureIABox(bad, None, **kw)
    with pytest.raises(ValueError, match=rf"outside \[0, boxsize\) or not finite.*first offending index {idx}"):
        box.measure_xi_w("bad", "both", 27, temp_file_path=str(tmp_path))
    again = MeasureIABox({k: np.array(v) if k != "LOS" else v for k, v in data.items()}, None, **kw)
    again.measure_xi_w("ok", "both", 27, temp_file_path=str(tmp_path))
    after = again.last_measurement
    np.testing.assert_array_equal(after.npairs, before.npairs)
    for key in ("proj_gp", "proj_gg", "cov_gp", "DD_all", "Splus_all"):
        np.testing.assert_array_equal(after[key], before[key])


def test_batch_reports_the_catalogue_with_bad_coordinates():
    """In a batch, the catalogue whose positions leave the box is named in the
    error, and the other catalogues' products are those of single runs."""
    from measure_ia_gb300.catalogs import neyman_scott_catalog
    from measure_ia_gb300.engine import BatchCounter
    pc = _counter("mixed")
    cats = [neyman_scott_catalog(150, 205.0, 2000, 30 + i, mean_children=30, sigma=1.0) for i in range(3)]
    cats[1]["Position"][5, 0] = float("nan")
    dcats = [pc.to_device(c) for c in cats]
    batch = BatchCounter(pc, dcats)
    batch.prepare()
    with pytest.raises(ValueError, match=r"catalogue 1, first offending index 5"):
        batch.run()
    for i in (0, 2):
        np.testing.assert_array_equal(batch.fetch(i).npairs, pc.measure(cats[i]).npairs)
