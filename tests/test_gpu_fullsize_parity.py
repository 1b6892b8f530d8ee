"""Parity at the headline catalogue sizes: the GPU path (plain FP64 and
mixed forms, through MeasureIABox and the C ABI) against the oracle on the
same inputs, with every position of the catalogue and a seeded subset of
the shapes, so that the oracle finishes in a minute on the host cores.

* clustered 4M positions / 1M shapes (80,000 Neyman-Scott parents, 2,000
  injected pairs on bin edges), w_gg + w_g+ with 27 jackknife regions, at
  the default launch geometry and at the autotuned one of the full
  measurement (4 x 4 x 20 Mpc/h shape cells, 2 x 2 x 10 position cells per
  shape cell, 64 shapes per work unit): 1,500 random shapes plus 500 of the
  edge-pair shapes;
* clustered 1M positions / 200k shapes (20,000 parents), w and multipoles
  (20 mu_r bins), 27 jackknife regions: 3,000 random shapes.

Reference code per pair: measure_w_box_jk.py:543-646 and
measure_m_box_jk.py:570-682.  Bar: pair counts per (bin, jackknife region)
bit-exact in both forms; every dataset within 1e-10 relative (FP64 form);
the mixed form within 2e-5 per dataset entry (with the array's max as the
floor) and its w_gg / w_g+ within 5e-6 of the vector's scale.  (The mixed
form's FP32 term errors are unbiased, ~7e-8 of a term, so a bin's error
shrinks as 1/sqrt(pairs): the full measurement, ~500 times the pairs of these
subsets, holds w_g+ to ~2e-8 of its scale.)
"""

import os

import numpy as np
import pytest

from golden_io import assert_close
from oracle import ia_oracle as O

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
MIXED_RTOL = 2e-5
MIXED_W_RTOL = 5e-6
PROCS = max(1, min(16, os.cpu_count() or 1))
R_BINS_KW = dict(r_min=0.1, r_max=20.0, num_bins_r=10)
TUNED = dict(cell_size=4.0, cell_refine=2, shapes_per_unit=64, cell_size_los=20.0, cell_refine_los=10)

_CACHE = {}


def _subset(data, idx):
    out = {k: data[k] for k in ("Position", "weight", "LOS")}
    for k in ("Position_shape_sample", "Axis_Direction", "q", "weight_shape_sample"):
        out[k] = np.ascontiguousarray(data[k][idx])
    return out


def _config2():
    if "c2" not in _CACHE:
        import bench
        data = bench.make_catalog()
        n_s = len(data["Position_shape_sample"])
        rng = np.random.default_rng(2)
        idx = np.concatenate([np.sort(rng.choice(n_s - 2000, 1500, replace=False)), np.arange(n_s - 500, n_s)])
        _CACHE["c2"] = _subset(data, idx)
    return _CACHE["c2"]


def _config1():
    if "c1" not in _CACHE:
        from measure_ia_gb300.catalogs import neyman_scott_catalog
        data = neyman_scott_catalog(20000, 205.0, 200_000, 11, mean_children=50, sigma=1.0, kappa=2.0)
        rng = np.random.default_rng(1)
        _CACHE["c1"] = _subset(data, np.sort(rng.choice(len(data["Position_shape_sample"]), 3000, replace=False)))
    return _CACHE["c1"]


def _oracle(key, kind, cat, n_p):
    k = (key, kind)
    if k not in _CACHE:
        b = O.Binning(boxsize=205.0, **R_BINS_KW, num_bins_pi=n_p, pi_max=20.0)
        data = {kk: (np.array(v) if kk != "LOS" else v) for kk, v in cat.items()}
        _CACHE[k] = O.measure(kind, b, data, "full", "both", 27, None, "distortion", "multiprocessing",
                              chunk=50, processes=PROCS)
    return _CACHE[k]


def _check(cat, ref, kind, n_p, precision, tmp_path, knobs=None):
    from measure_ia_gb300 import MeasureIABox, open_output
    ref = dict(ref)
    c = ref.pop("__counts__")
    out = str(tmp_path / f"full_{kind}_{precision}.hdf5")
    box = MeasureIABox({k: v for k, v in cat.items()}, out, None, None, [0.1, 20.0], 10, n_p, 20.0, boxsize=205.0,
                       num_nodes=2, precision=precision, launch_knobs=knobs)
    fn = box.measure_xi_w if kind == "w" else box.measure_xi_multipoles
    fn("full", "both", 27, temp_file_path=str(tmp_path))
    m = box.last_measurement
    assert c.npairs.sum() > 10_000_000
    np.testing.assert_array_equal(m.npairs[0], c.npairs)
    np.testing.assert_array_equal(m.npairs[1:], c.npairs_jk)
    assert m.stats["binned_pairs"] == int(c.npairs.sum())
    store = open_output(out)
    assert set(store.keys()) == set(ref), sorted(set(store.keys()) ^ set(ref))[:10]
    rtol = FP64_RTOL if precision == "fp64" else MIXED_RTOL
    for path, v in ref.items():
        assert_close(store.read(path), v, rtol, path)
    if precision == "mixed":
        top = "w" if kind == "w" else "multipoles"
        for name in ("gg", "g_plus"):
            want = ref[f"{top}_{name}/full"]
            got = store.read(f"{top}_{name}/full")
            assert np.max(np.abs(got - want)) <= MIXED_W_RTOL * np.max(np.abs(want)), name


@pytest.mark.parametrize("knobs", ["default", "tuned"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_config2_positions_w_jk27(precision, knobs, tmp_path):
    cat = _config2()
    assert len(cat["Position"]) > 3_990_000
    _check(cat, _oracle("c2", "w", cat, 8), "w", 8, precision, tmp_path, TUNED if knobs == "tuned" else None)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["w", "m"])
def test_config1_positions_jk27(kind, precision, tmp_path):
    cat = _config1()
    assert len(cat["Position"]) > 990_000
    n_p = 8 if kind == "w" else 20
    _check(cat, _oracle("c1", kind, cat, n_p), kind, n_p, precision, tmp_path)
