"""The lightcone oracle against the reference's own outputs
(``tests/golden/lc_*.npz``): every dataset MeasureIALightcone wrote, the
same dataset names, values within 1e-12 (only the order of the histogram
sums differs), and the reference's failure on gg jackknife covariances."""

import numpy as np
import pytest

from golden_io import assert_close, lc_case_names, lc_masks, load_lc_case
from oracle import lightcone_oracle as LO


def run_oracle(meta, data, rnd, jk, cosmo):
    b = LO.LcBinning(*meta["binning"]["separation_limits"], meta["binning"]["num_bins_r"],
                     meta["binning"]["num_bins_pi"], meta["binning"]["pi_max"])
    call = meta["call"]
    return LO.measure(meta["kind"], meta["estimator"], "lc", meta["corr_type"], dict(data), dict(rnd), b,
                      cosmo.comoving_radial_distance, cosmo["h"],
                      jk_patches={k: v for k, v in jk.items()} if meta["measure_cov"] else None,
                      measure_cov=meta["measure_cov"], over_h=call.get("over_h", False), rp_cut=call.get("rp_cut"),
                      masks=lc_masks(data) if call.get("masks") else None)


def test_fixtures_present():
    assert len(lc_case_names()) >= 8


@pytest.mark.parametrize("name", lc_case_names())
def test_oracle_matches_reference(name):
    meta, data, rnd, jk, outs, cosmo = load_lc_case(name)
    got = run_oracle(meta, data, rnd, jk, cosmo)
    assert set(got) == set(outs), sorted(set(got) ^ set(outs))[:10]
    for path, ref in outs.items():
        assert_close(got[path], ref, 1e-12, path)


def test_gg_covariance_fails_like_the_reference():
    meta, data, rnd, jk, outs, cosmo = load_lc_case("w_clusters_gg")
    meta = dict(meta, measure_cov=True)
    jk = {"position": np.zeros(len(data["RA"]), int), "shape": np.zeros(len(data["RA_shape_sample"]), int),
          "randoms": np.zeros(len(rnd["RA"]), int)}
    with pytest.raises(KeyError):
        run_oracle(meta, data, rnd, jk, cosmo)
