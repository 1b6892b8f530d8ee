"""Lightcone path on the GPU (MeasureIALightcone through mia_lc_count).

* Every dataset of the reference runs in ``tests/golden/lc_*.npz``:
  the same dataset names, values within 1e-10 relative (array scale as the
  floor), non-finite entries at the same places.
* Each counter alone against the oracle on randomised catalogues: integer
  pair counts per bin bit-exact for the full sample and for every patch
  realisation (the reference re-counts each patch; here one pass), sums
  within 1e-10.
* The reference's failures: IndexError past the last bin of an unclamped
  counter, KeyError for gg jackknife covariances.
"""

import numpy as np
import pytest

from golden_io import lc_case_names, lc_masks, load_lc_case
from oracle import lightcone_oracle as LO

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def _close(got, ref, what, rtol=RTOL):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    assert got.shape == ref.shape, (what, got.shape, ref.shape)
    fin = np.isfinite(ref)
    np.testing.assert_array_equal(np.isfinite(got), fin, err_msg=f"{what}: non-finite pattern")
    g, r = got[fin], ref[fin]
    if r.size:
        lim = rtol * np.abs(r) + rtol * np.max(np.abs(r))
        err = np.abs(g - r)
        assert np.all(err <= lim), f"{what}: max err {err.max():.3e} (scale {np.max(np.abs(r)):.3e})"


def _run_product(meta, data, rnd, jk, cosmo, out):
    from measure_ia_gb300 import MeasureIALightcone
    call = dict(meta["call"])
    call.pop("cosmology", None)
    call.pop("measure_cov", None)
    if call.pop("masks", False):
        call["masks"] = lc_masks(data)
    lc = MeasureIALightcone({k: np.array(v) for k, v in data.items()}, {k: np.array(v) for k, v in rnd.items()},
                            out, num_nodes=2, **meta["binning"])
    jkp = {k: np.array(v) for k, v in jk.items()} if meta["measure_cov"] else None
    if meta["kind"] == "w":
        lc.measure_xi_w(meta["estimator"], "lc", meta["corr_type"], jk_patches=jkp, measure_cov=meta["measure_cov"],
                        cosmology=cosmo, **call)
    else:
        lc.measure_xi_multipoles(meta["estimator"], "lc", meta["corr_type"], jk_patches=jkp,
                                 calc_errors=meta["measure_cov"], cosmology=cosmo, **call)
    return lc


@pytest.mark.parametrize("name", lc_case_names())
def test_matches_reference_runs(name, tmp_path):
    from measure_ia_gb300 import open_output, read_output
    meta, data, rnd, jk, outs, cosmo = load_lc_case(name)
    out = str(tmp_path / "lc.hdf5")
    _run_product(meta, data, rnd, jk, cosmo, out)
    store = open_output(out)
    assert set(store.keys()) == set(outs), sorted(set(store.keys()) ^ set(outs))[:10]
    for path, ref in outs.items():
        _close(store.read(path), ref, path)
    assert set(read_output(out)) == set(outs)


def test_gg_covariance_fails_like_the_reference(tmp_path):
    from measure_ia_gb300 import open_output
    meta, data, rnd, jk, outs, cosmo = load_lc_case("w_clusters_gg")
    meta = dict(meta, measure_cov=True)
    jk = {"position": np.arange(len(data["RA"])) % 3, "shape": np.arange(len(data["RA_shape_sample"])) % 3,
          "randoms": np.arange(len(rnd["RA"])) % 3}
    out = str(tmp_path / "gg.hdf5")
    with pytest.raises(KeyError):
        _run_product(meta, data, rnd, jk, cosmo, out)
    # the full-sample products and the realisation counts were written first
    keys = set(open_output(out).keys())
    assert "w/xi_gg/lc" in keys and "w/xi_gg/lc_jk3/lc_0_DD" in keys and "w/xi_gg/lc_jk3/lc_2_RR" in keys


# ---- single counters against the oracle --------------------------------------

def _catalogue(seed, n_p, n_s, ra, dec, z):
    rng = np.random.default_rng(seed)
    par = max(3, n_p // 25)
    cen = np.c_[rng.uniform(*ra, par), rng.uniform(*dec, par), rng.uniform(*z, par)]
    pick = rng.integers(0, par, n_p)
    spread = 0.02 * (ra[1] - ra[0])
    sel = {"RA": cen[pick, 0] + rng.normal(0, spread, n_p), "DEC": np.clip(cen[pick, 1] + rng.normal(0, spread, n_p),
                                                                            -89.99, 89.99),
           "Redshift": np.abs(cen[pick, 2] + rng.normal(0, 0.002, n_p)), "weight": np.exp(rng.normal(0, 0.3, n_p))}
    k = rng.choice(n_p, n_s, replace=False)
    sel.update({"RA_shape_sample": sel["RA"][k] + rng.normal(0, 1e-3, n_s), "DEC_shape_sample": sel["DEC"][k],
                "Redshift_shape_sample": sel["Redshift"][k] + rng.normal(0, 1e-3, n_s),
                "weight_shape_sample": np.exp(rng.normal(0, 0.3, n_s)),
                "e1": rng.uniform(-0.5, 0.5, n_s), "e2": rng.uniform(-0.5, 0.5, n_s)})
    return sel


SWEEP = [
    # kind, shapes, over_h, rp_cut, n_patch, RA range, DEC range, z range, r range, n_r, n_p, pi_max
    ("w", True, False, None, 4, (10, 40), (-10, 10), (0.1, 0.3), (0.3, 25.0), 6, 5, 30.0),
    ("w", False, True, None, 5, (350, 360), (60, 80), (0.05, 0.2), (0.2, 15.0), 5, 8, 20.0),
    ("w", True, True, None, 3, (0, 15), (-85, -70), (0.3, 0.5), (0.5, 40.0), 8, 6, 40.0),
    ("m", True, False, None, 4, (100, 130), (20, 40), (0.1, 0.25), (0.3, 25.0), 6, 10, 30.0),
    ("m", False, False, 1.5, 6, (200, 230), (-30, 0), (0.2, 0.4), (0.5, 30.0), 7, 8, 30.0),
    ("m", True, True, 0.5, 0, (40, 60), (0, 20), (0.05, 0.15), (0.2, 12.0), 4, 12, 12.0),
    ("w", False, False, None, 0, (0.5, 3.0), (88.0, 89.9), (0.1, 0.2), (0.1, 10.0), 5, 4, 10.0),
]


def _prep(sel, chi, with_shapes):
    dec = sel["DEC"]
    pos = {"ra": sel["RA"], "dec": dec, "chi": chi(sel["Redshift"]), "w": sel["weight"],
           "cos_dec": np.cos(dec / 180 * np.pi)}
    shp = {"ra": sel["RA_shape_sample"], "dec": sel["DEC_shape_sample"], "chi": chi(sel["Redshift_shape_sample"]),
           "w": sel["weight_shape_sample"]}
    if with_shapes:
        e1, e2 = sel["e1"], sel["e2"]
        theta = 1. / 2 * np.arctan2(e2, e1)
        semi = np.array([np.cos(theta), np.sin(theta)])
        axis = semi / np.sqrt(np.sum(semi ** 2, axis=0))
        phi = np.arctan2(axis[1], axis[0])
        shp.update(e=np.sqrt(e1 ** 2 + e2 ** 2), c2a=np.cos(2 * phi), s2a=np.sin(2 * phi))
    return pos, shp


def _subset(sel, mp, ms):
    pk = ("RA", "DEC", "Redshift", "weight")
    return {k: (v[mp] if k in pk else v[ms]) for k, v in sel.items()}


@pytest.mark.parametrize("case", range(len(SWEEP)))
def test_counter_against_oracle(case):
    from measure_ia_gb300.cosmology import FlatLCDM
    from measure_ia_gb300.lightcone import LightconeCounter
    kind, shapes, over_h, rp_cut, n_patch, ra, dec, z, rr, n_r, n_p, pi_max = SWEEP[case]
    sel = _catalogue(500 + case, 700, 500, ra, dec, z)
    cosmo = FlatLCDM()
    h = cosmo["h"]
    b = LO.LcBinning(rr[0], rr[1], n_r, n_p, pi_max)
    chi_raw = lambda a: cosmo.comoving_radial_distance(a)
    chi_h = lambda zz: chi_raw(1 / (1 + zz)) * (h if over_h else 1.0)
    rng = np.random.default_rng(900 + case)
    pp = rng.integers(0, max(1, n_patch), len(sel["RA"]))
    sp = rng.integers(0, max(1, n_patch), len(sel["RA_shape_sample"]))
    pos, shp = _prep(sel, chi_h, shapes)
    if n_patch:
        pos["patch"], shp["patch"] = pp, sp.astype(np.int32)
    counter = LightconeCounter(kind, shapes, b.r_bins, rr[0], rr[1], b.pi_bins if kind == "w" else b.mu_r_bins,
                               h_extra=h if over_h else 1.0, rp_cut=0.0 if rp_cut is None else rp_cut)
    sums, counts = counter.count(pos, shp, n_patch)
    unit = lambda s: dict(s, weight=np.ones(len(s["RA"])), weight_shape_sample=np.ones(len(s["RA_shape_sample"])))
    reals = [(np.ones(len(pp), bool), np.ones(len(sp), bool))] + [(pp != i, sp != i) for i in range(n_patch)]
    assert counts[0].sum() > 0
    for k, (mp, ms) in enumerate(reals):
        s = _subset(sel, mp, ms)
        _, _, cnt = LO.pair_counts(kind, False, b, unit(s), chi_raw, h, over_h, rp_cut)
        got = counts[k].astype(np.float64)
        got[got == 0] = 1
        np.testing.assert_array_equal(got, cnt, err_msg=f"counts of realisation {k}")
        SP, SX, DD = LO.pair_counts(kind, shapes, b, s, chi_raw, h, over_h, rp_cut)
        dd = sums[0, k].copy()
        dd[(dd == 0) | (counts[k] == 0)] = 1
        _close(dd, DD, f"DD {k}")
        if shapes:
            _close(sums[1, k], SP, f"S+D {k}")
            _close(sums[2, k], SX, f"SxD {k}")


def test_index_past_last_bin_raises():
    """mu = 1 exactly (a shape straight behind a position) indexes bin n in
    the multipole counter, which has no clamp: IndexError, as in the reference
    (reachable with rp_cut < 0, so that r_p = 0 passes the cut)."""
    from measure_ia_gb300.cosmology import FlatLCDM
    from measure_ia_gb300.lightcone import LightconeCounter
    sel = {"RA": np.array([20.0, 21.0]), "DEC": np.array([5.0, 5.5]), "Redshift": np.array([0.2, 0.2]),
           "weight": np.ones(2), "RA_shape_sample": np.array([20.0]), "DEC_shape_sample": np.array([5.0]),
           "Redshift_shape_sample": np.array([0.2005]), "weight_shape_sample": np.ones(1)}
    cosmo = FlatLCDM()
    b = LO.LcBinning(0.1, 20.0, 5, 4, 20.0)
    chi = lambda a: cosmo.comoving_radial_distance(a)
    with pytest.raises(IndexError):
        LO.pair_counts("m", False, b, sel, chi, 0.7, False, -1.0)
    pos, shp = _prep(sel, lambda zz: chi(1 / (1 + zz)), False)
    counter = LightconeCounter("m", False, b.r_bins, 0.1, 20.0, b.mu_r_bins, rp_cut=-1.0)
    with pytest.raises(IndexError):
        counter.count(pos, shp)
    # with rp_cut = 0 the pair is cut and both count the same
    counter = LightconeCounter("m", False, b.r_bins, 0.1, 20.0, b.mu_r_bins, rp_cut=0.0)
    _, counts = counter.count(pos, shp)
    _, _, dd = LO.pair_counts("m", False, b, sel, chi, 0.7, False, 0.0)
    got = counts[0].astype(np.float64)
    got[got == 0] = 1
    np.testing.assert_array_equal(got, dd)


def test_empty_samples():
    """No positions, no shapes, or no pair in range: zero counts, DD read as 1
    where empty (the reference's DD == 0 -> 1), no error."""
    from measure_ia_gb300.lightcone import LightconeCounter
    b = LO.LcBinning(0.5, 10.0, 4, 4, 10.0)
    one = {"ra": np.array([10.0]), "dec": np.array([0.0]), "chi": np.array([500.0]), "w": np.ones(1),
           "cos_dec": np.ones(1)}
    far = {"ra": np.array([50.0]), "dec": np.array([40.0]), "chi": np.array([900.0]), "w": np.ones(1),
           "e": np.full(1, 0.3), "c2a": np.ones(1), "s2a": np.zeros(1)}
    empty_p = {k: v[:0] for k, v in one.items()}
    empty_s = {k: v[:0] for k, v in far.items()}
    for shapes in (False, True):
        c = LightconeCounter("w", shapes, b.r_bins, 0.5, 10.0, b.pi_bins)
        for pos, shp in ((empty_p, far), (one, empty_s), (one, far), (empty_p, empty_s)):
            sums, counts = c.count(pos, shp, 0)
            assert counts.sum() == 0 and np.all(sums == 0.0)


@pytest.mark.parametrize("kind", ["w", "m"])
def test_counter_sums_are_order_free(kind):
    """The counter's sums are exact integers: a second run gives the same
    bits, and halving every weight gives exactly a quarter of DD, S+D, SxD
    in the total and in every realisation."""
    from measure_ia_gb300.cosmology import FlatLCDM
    from measure_ia_gb300.lightcone import LightconeCounter
    sel = _catalogue(77, 3000, 2000, (10, 40), (-10, 10), (0.1, 0.3))
    cosmo = FlatLCDM()
    b = LO.LcBinning(0.3, 25.0, 6, 5, 30.0)
    chi = lambda zz: cosmo.comoving_radial_distance(1 / (1 + zz))
    rng = np.random.default_rng(7)
    pos, shp = _prep(sel, chi, True)
    pos["patch"] = rng.integers(0, 5, len(sel["RA"]))
    shp["patch"] = rng.integers(0, 5, len(sel["RA_shape_sample"])).astype(np.int32)
    counter = LightconeCounter(kind, True, b.r_bins, 0.3, 25.0, b.pi_bins if kind == "w" else b.mu_r_bins)
    s1, c1 = counter.count(pos, shp, 5)
    s2, c2 = counter.count(pos, shp, 5)
    np.testing.assert_array_equal(s1, s2)
    np.testing.assert_array_equal(c1, c2)
    half = lambda d: dict(d, w=0.5 * d["w"])
    s3, c3 = counter.count(half(pos), half(shp), 5)
    np.testing.assert_array_equal(c3, c1)
    np.testing.assert_array_equal(s1, 4 * s3)
    assert c1[0].sum() > 0 and np.abs(s1[1, 0]).max() > 0


@pytest.mark.parametrize("kind", ["w", "m"])
def test_counter_wide_weight_range(kind):
    """Weights spanning ~10^8: the counter keeps its sums in 128-bit warp
    partials (the 64-bit ones hold a term only to 2^-46 of the largest), and
    every DD bin, however small its pairs' weights, is within 1e-10 of the
    oracle's relative to itself."""
    from measure_ia_gb300.cosmology import FlatLCDM
    from measure_ia_gb300.lightcone import LightconeCounter
    sel = _catalogue(91, 1500, 900, (10, 40), (-10, 10), (0.1, 0.3))
    rng = np.random.default_rng(8)
    sel["weight"] = np.exp(rng.normal(0.0, 3.0, len(sel["RA"])))
    sel["weight_shape_sample"] = np.exp(rng.normal(0.0, 3.0, len(sel["RA_shape_sample"])))
    cosmo = FlatLCDM()
    h = cosmo["h"]
    b = LO.LcBinning(0.3, 25.0, 6, 5, 30.0)
    chi_raw = lambda a: cosmo.comoving_radial_distance(a)
    chi = lambda zz: chi_raw(1 / (1 + zz))
    pos, shp = _prep(sel, chi, True)
    pp = rng.integers(0, 4, len(sel["RA"]))
    sp = rng.integers(0, 4, len(sel["RA_shape_sample"]))
    pos["patch"], shp["patch"] = pp, sp.astype(np.int32)
    counter = LightconeCounter(kind, True, b.r_bins, 0.3, 25.0, b.pi_bins if kind == "w" else b.mu_r_bins)
    assert counter._wide_sums(pos, shp)
    sums, counts = counter.count(pos, shp, 4)
    reals = [(np.ones(len(pp), bool), np.ones(len(sp), bool))] + [(pp != i, sp != i) for i in range(4)]
    for k, (mp, ms) in enumerate(reals):
        SP, SX, DD = LO.pair_counts(kind, True, b, _subset(sel, mp, ms), chi_raw, h, False, None)
        dd = sums[0, k].copy()
        dd[(dd == 0) | (counts[k] == 0)] = 1
        np.testing.assert_allclose(dd, DD, rtol=1e-10, atol=0, err_msg=f"DD {k}")
        _close(sums[1, k], SP, f"S+D {k}")
        _close(sums[2, k], SX, f"SxD {k}")


@pytest.mark.parametrize("shapes", [True, False])
@pytest.mark.parametrize("kind", ["w", "m"])
def test_partial_flushes(kind, shapes, monkeypatch):
    """The warp partials are flushed at patch changes and at least every
    2,000 half-steps; the small catalogues here never reach that, so the
    interval is cut to 2 (a flush after every step) and the counter must
    still match the oracle: counts per realisation exact, sums to 1e-10, and
    the same bits as with the default interval."""
    from measure_ia_gb300.cosmology import FlatLCDM
    from measure_ia_gb300.lightcone import LightconeCounter
    sel = _catalogue(33, 2500, 1500, (10, 40), (-10, 10), (0.1, 0.3))
    cosmo = FlatLCDM()
    h = cosmo["h"]
    b = LO.LcBinning(0.3, 25.0, 6, 5, 30.0)
    chi_raw = lambda a: cosmo.comoving_radial_distance(a)
    chi = lambda zz: chi_raw(1 / (1 + zz))
    rng = np.random.default_rng(4)
    pos, shp = _prep(sel, chi, shapes)
    pp = rng.integers(0, 3, len(sel["RA"]))
    sp = rng.integers(0, 3, len(sel["RA_shape_sample"]))
    pos["patch"], shp["patch"] = pp, sp.astype(np.int32)
    counter = LightconeCounter(kind, shapes, b.r_bins, 0.3, 25.0, b.pi_bins if kind == "w" else b.mu_r_bins)
    s_default, c_default = counter.count(pos, shp, 3)
    monkeypatch.setenv("MIA_LC_FLUSH_STEPS", "2")
    sums, counts = counter.count(pos, shp, 3)
    np.testing.assert_array_equal(counts, c_default)
    np.testing.assert_array_equal(sums, s_default)
    reals = [(np.ones(len(pp), bool), np.ones(len(sp), bool))] + [(pp != i, sp != i) for i in range(3)]
    for k, (mp, ms) in enumerate(reals):
        SP, SX, DD = LO.pair_counts(kind, shapes, b, _subset(sel, mp, ms), chi_raw, h, False, None)
        dd = sums[0, k].copy()
        dd[(dd == 0) | (counts[k] == 0)] = 1
        _close(dd, DD, f"DD {k}")
        if shapes:
            _close(sums[1, k], SP, f"S+D {k}")
            _close(sums[2, k], SX, f"SxD {k}")


def test_failing_counter_keeps_earlier_products(tmp_path):
    """The counters are enqueued ahead of their results; when a later one
    cannot start (here RD: a randoms shape redshift is NaN), the products of
    the counters before it are still written, as in the reference's
    one-after-the-other flow, and nothing of RD or RR is."""
    from measure_ia_gb300 import open_output
    meta, data, rnd, jk, outs, cosmo = load_lc_case("w_clusters_both")
    rnd = {k: np.array(v) for k, v in rnd.items()}
    if "Redshift_shape_sample" not in rnd:
        rnd.update(RA_shape_sample=rnd["RA"].copy(), DEC_shape_sample=rnd["DEC"].copy(),
                   Redshift_shape_sample=rnd["Redshift"].copy())
    rnd["Redshift_shape_sample"][0] = np.nan
    meta = dict(meta, measure_cov=False)
    out = str(tmp_path / "fail.hdf5")
    with pytest.raises(ValueError, match="finite"):   # the package's FlatLCDM refuses a NaN redshift
        _run_product(meta, data, rnd, jk, None, out)
    keys = set(open_output(out).keys())
    assert any(k.endswith("lc_SplusD") for k in keys), sorted(keys)[:10]
    assert any("randoms" in k and k.endswith("_SplusD") for k in keys), sorted(keys)[:10]
    assert not any(k.endswith("_RD") or k.endswith("_RR") for k in keys), sorted(keys)[:10]
