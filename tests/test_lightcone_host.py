"""Host side of the lightcone path (no GPU): distances, bin tables, patch
assignment and the reference's argument errors."""

import numpy as np
import pytest


def test_flat_lcdm_distance():
    from scipy.integrate import quad
    from measure_ia_gb300.cosmology import FlatLCDM, comoving_radial_distance, default_cosmology
    c = FlatLCDM(Omega_c=0.25, Omega_b=0.05, h=0.68)
    z = np.array([0.0, 0.01, 0.3, 1.0, 2.5, 8.0])
    want = np.array([quad(lambda x: 1.0 / float(c.E(x)), 0.0, zz, epsabs=0, epsrel=1e-13)[0] for zz in z])
    want *= 299792.458 / 68.0
    got = comoving_radial_distance(c, 1 / (1 + z))
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-9)
    assert default_cosmology()["h"] == 0.7
    # matter + radiation + Lambda = 1 (flat)
    assert abs(c.Omega_m + c.Omega_r + c.Omega_l - 1.0) < 1e-15


@pytest.mark.parametrize("clamp", [True, False])
def test_lightcone_tables_follow_the_reference_formula(clamp):
    from measure_ia_gb300 import binning as B
    rng = np.random.default_rng(3)
    r_min, r_max, n = 0.3, 25.0, 6
    rb = np.logspace(np.log10(r_min), np.log10(r_max), n + 1)
    tab = B.lc_r_table("w", rb, r_min, r_max, n, clamp)
    r = np.concatenate([rng.uniform(0.1, 30.0, 20000), rb, np.nextafter(rb, 0), np.nextafter(rb, 99)])
    q = r * r
    sep = np.sqrt(q)
    dlog = (np.log10(r_max) - np.log10(r_min)) / n
    ok = (sep >= rb[0]) & (sep < rb[-1])
    ind = np.floor(np.log10(sep) / dlog - np.log10(rb[0]) / dlog).astype(int)
    if clamp:
        ind[ind == n] = n - 1
    want = np.where(ok, np.where(ind >= n, -2, ind), -1)
    np.testing.assert_array_equal(tab.lookup(q), want)
    pb = np.linspace(-30.0, 30.0, 6)
    pt = B.lc_pi_table(pb, 5, clamp)
    x = np.concatenate([rng.uniform(-40, 40, 20000), pb, np.nextafter(pb, -99), np.nextafter(pb, 99)])
    step = (pb[-1] - pb[0]) / 5
    okp = (x >= pb[0]) & (x < pb[-1])
    indp = np.floor(x / step - pb[0] / step).astype(int)
    if clamp:
        indp[indp == 5] = 4
    np.testing.assert_array_equal(pt.lookup(x), np.where(okp, np.where(indp >= 5, -2, indp), -1))


def test_mu_table_has_no_clamp():
    from measure_ia_gb300 import binning as B
    mb = np.linspace(-1, 1, 9)
    t = B.lc_mu_table(mb, 8)
    assert t.lookup(np.array([1.0]))[0] == -2          # np.add.at would raise
    assert t.lookup(np.array([-1.0]))[0] == 0
    # just below 1 the reference's floor(mu / dmu - mu_0 / dmu) still rounds to n
    x = np.array([np.nextafter(1.0, 0), 0.9999, 0.99, 0.75, np.nextafter(0.75, 0)])
    ind = np.floor(x / 0.25 - (-1.0) / 0.25).astype(int)
    np.testing.assert_array_equal(t.lookup(x), np.where(ind >= 8, -2, ind))
    assert ind[0] == 8 and ind[1] == 7


def test_sky_kmeans_patches():
    from measure_ia_gb300.lightcone import assign_jackknife_patches
    rng = np.random.default_rng(0)
    rnd = {"RA": rng.uniform(10, 50, 3000), "DEC": rng.uniform(-10, 10, 3000)}
    rnd["RA_shape_sample"], rnd["DEC_shape_sample"] = rnd["RA"][:1000], rnd["DEC"][:1000]
    data = {"RA": rng.uniform(10, 50, 500), "DEC": rng.uniform(-10, 10, 500)}
    data["RA_shape_sample"], data["DEC_shape_sample"] = data["RA"][:200], data["DEC"][:200]
    a = assign_jackknife_patches(data, rnd, 6)
    b = assign_jackknife_patches(data, rnd, 6)
    assert set(a) == {"randoms_position", "randoms_shape", "position", "shape"}
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])             # seeded: reproducible
    assert set(np.unique(a["randoms_position"])) == set(range(6))
    np.testing.assert_array_equal(a["randoms_shape"], a["randoms_position"][:1000])


def test_reference_argument_errors():
    from measure_ia_gb300 import MeasureIALightcone
    data = {"RA": np.ones(3), "DEC": np.ones(3), "Redshift": np.ones(3), "RA_shape_sample": np.ones(2),
            "DEC_shape_sample": np.ones(2), "Redshift_shape_sample": np.ones(2), "e1": np.zeros(2), "e2": np.zeros(2)}
    with pytest.raises(ValueError):
        MeasureIALightcone(dict(data), None, None, pi_max=None)
    lc = MeasureIALightcone(dict(data), None, None, pi_max=10.0)
    assert np.array_equal(lc.data["weight"], np.ones(3))       # default weights, as the reference
    with pytest.raises(KeyError, match="add randoms"):
        lc.measure_xi_w("clusters", "d", "both")
    with pytest.raises(KeyError, match="No randoms given"):
        lc.measure_xi_w("galaxies", "d", "both")
    with pytest.raises(KeyError, match="Unknown input for IA_estimator"):
        lc.measure_xi_w("stars", "d", "both")
    lc = MeasureIALightcone(dict(data), {"RA": np.ones(4), "DEC": np.ones(4), "Redshift": np.ones(4)}, None,
                            pi_max=10.0)
    with pytest.raises(ValueError, match="provide either jk_patches or num_jk"):
        lc.measure_xi_w("clusters", "d", "both", measure_cov=True)
    with pytest.raises(KeyError, match="Unknown value for corr_type"):
        lc.measure_xi_multipoles("clusters", "d", "g-", calc_errors=False)


def test_distance_derivatives_from_the_node_table():
    """The Hermite derivatives c/H at the nodes come from a table built once;
    the distances are the same doubles as with E(z) evaluated per object."""
    from measure_ia_gb300.cosmology import FlatLCDM
    c = FlatLCDM()
    rng = np.random.default_rng(3)
    z = np.concatenate([rng.uniform(0.0, 3.0, 5000), rng.uniform(-0.05, 0.01, 200), [0.0, 1 / 2048, 2.5]])
    got = c.comoving_radial_distance(1 / (1 + z))
    # the same interpolation with the derivatives evaluated per object
    zz = 1 / (1 / (1 + z)) - 1
    k = np.floor(zz / c.DZ)
    k_lo, _, vals, _ = c._table(int(k.min()) - 1, int(k.max()) + 2)
    i = (k - k_lo).astype(np.int64)
    z0 = k * c.DZ
    t = (zz - z0) / c.DZ
    d0, d1 = c.DZ / c.E(z0), c.DZ / c.E(z0 + c.DZ)
    t2, t3 = t * t, t * t * t
    chi = (2 * t3 - 3 * t2 + 1) * vals[i] + (t3 - 2 * t2 + t) * d0 + (-2 * t3 + 3 * t2) * vals[i + 1] + (t3 - t2) * d1
    np.testing.assert_array_equal(got, chi * (299792.458 / (100.0 * c.h)))


def test_wide_sums_choice():
    """128-bit warp partials when the smallest weight product is below 2^-12
    of the largest possible term, 64-bit ones otherwise."""
    from measure_ia_gb300.lightcone import LightconeCounter
    c = LightconeCounter("w", True, np.logspace(-1, 1, 5), 0.1, 10.0, np.linspace(-10, 10, 5))
    n = 100
    pos = {"w": np.ones(n)}
    shp = {"w": np.ones(n), "e": np.full(n, 0.3)}
    assert not c._wide_sums(pos, shp)
    shp["w"] = np.linspace(0.1, 10.0, n)                   # products from 0.1 to 10: 2^-7
    assert not c._wide_sums(pos, shp)
    pos["w"] = np.r_[np.ones(n - 1), 1e-3]                 # 1e-4 of the largest: below 2^-12
    assert c._wide_sums(pos, shp)
    pos["w"] = np.r_[np.ones(n - 1), 0.0]                  # zero weights do not count
    assert not c._wide_sums(pos, shp)
    shp = {"w": np.ones(n), "e": np.r_[np.full(n - 1, 0.3), 5000.0]}   # |w e| sets the largest term
    pos["w"] = np.ones(n)
    assert c._wide_sums(pos, shp)
    assert not c._wide_sums({"w": np.array([])}, shp)


def test_grid_median_subsample():
    from measure_ia_gb300.lightcone import _median_abs
    assert _median_abs(np.array([])) == 1.0
    a = np.linspace(-3.0, 5.0, 1001)
    assert _median_abs(a) == np.median(np.abs(a))
    big = np.random.default_rng(1).uniform(100.0, 200.0, 1 << 20)
    assert abs(_median_abs(big) - np.median(big)) < 1.0


class _FakeCounter:
    """The GPU counter's interface with made-up results (host-side flow tests)."""

    def __init__(self, n_r, n_p, with_shapes, log):
        self.n_r, self.n_p, self.Q, self.log = n_r, n_p, 3 if with_shapes else 1, log

    def prepare(self, pos, shp, n_patch=0):
        self.log.append("prepare")
        return n_patch

    def run(self, job, stream=None):
        self.log.append("run")

    def fetch(self, job):
        self.log.append("fetch")
        return (np.ones((self.Q, 1 + job, self.n_r, self.n_p)), np.ones((1 + job, self.n_r, self.n_p), np.int64))


def _lc_inputs(n=300, seed=2):
    rng = np.random.default_rng(seed)
    data = {"RA": rng.uniform(10, 20, n), "DEC": rng.uniform(-5, 5, n), "Redshift": rng.uniform(0.1, 0.2, n),
            "e1": rng.uniform(-0.3, 0.3, n), "e2": rng.uniform(-0.3, 0.3, n)}
    data.update(RA_shape_sample=data["RA"], DEC_shape_sample=data["DEC"], Redshift_shape_sample=data["Redshift"])
    rnd = {"RA": rng.uniform(10, 20, 2 * n), "DEC": rng.uniform(-5, 5, 2 * n), "Redshift": rng.uniform(0.1, 0.2, 2 * n)}
    rnd.update(RA_shape_sample=rnd["RA"].copy(), DEC_shape_sample=rnd["DEC"].copy(),
               Redshift_shape_sample=rnd["Redshift"].copy())
    return data, rnd


def test_counters_enqueued_before_results(monkeypatch, tmp_path):
    """All four counters are prepared and run before the first result is
    fetched; the results are then taken in the reference's order."""
    from measure_ia_gb300 import lightcone as LC
    log = []
    monkeypatch.setattr(LC._Run, "_counter", lambda self, ws: _FakeCounter(
        len(self.o.r_bins) - 1, len(self.o.pi_bins) - 1, ws, log))
    data, rnd = _lc_inputs()
    lc = LC.MeasureIALightcone(data, rnd, str(tmp_path / "ok.hdf5"), separation_limits=[0.5, 10.0], num_bins_r=4,
                               num_bins_pi=4, pi_max=20.0)
    lc.measure_xi_w("clusters", "lc", "both", measure_cov=False)
    assert log == ["prepare", "run"] * 4 + ["fetch"] * 4


def test_failing_counter_keeps_earlier_products_host(monkeypatch, tmp_path):
    """When the third counter (RD) cannot start, the first two are still
    finished and written before the error propagates; nothing of RD or RR is
    written (the reference runs and writes them one after the other)."""
    from measure_ia_gb300 import lightcone as LC
    from measure_ia_gb300.output import open_output
    log = []
    monkeypatch.setattr(LC._Run, "_counter", lambda self, ws: _FakeCounter(
        len(self.o.r_bins) - 1, len(self.o.pi_bins) - 1, ws, log))
    data, rnd = _lc_inputs()
    rnd["Redshift_shape_sample"][0] = np.nan
    out = str(tmp_path / "fail.hdf5")
    lc = LC.MeasureIALightcone(data, rnd, out, separation_limits=[0.5, 10.0], num_bins_r=4, num_bins_pi=4,
                               pi_max=20.0)
    with pytest.raises(ValueError, match="finite"):
        lc.measure_xi_w("clusters", "lc", "both", measure_cov=False)
    assert log == ["prepare", "run"] * 2 + ["fetch"] * 2
    keys = set(open_output(out).keys())
    assert any(k.endswith("lc_SplusD") for k in keys), sorted(keys)
    assert any("randoms" in k and k.endswith("_SplusD") for k in keys), sorted(keys)
    assert not any(k.endswith("_RD") or k.endswith("_RR") for k in keys), sorted(keys)
