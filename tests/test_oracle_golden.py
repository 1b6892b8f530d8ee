"""The CPU oracle pinned against the reference's own outputs.

* every ``ref_*.npz`` case: the oracle re-runs the same measurement and must
  write the same datasets (names, shapes) with equal values, and its integer
  pair counts must equal the reference's unit-weight DD exactly;
* the reference's golden HDF5 files (``tng300_mock_outputs.npz``): the
  oracle's Pi integration, multipoles, xi assembly and jackknife covariance
  applied to the stored realisations reproduce the stored products;
* known answers from the reference's tests: jackknife labels [0, 5, 7, 3]
  (tests/test_w_jk.py:16-24) and the weight-scaling invariants
  (tests/test_weights.py:34-40).
"""

import os

import numpy as np
import pytest

from golden_io import GOLDEN, assert_close, box_params, case_names, layout_of, load_case, masks_for
from oracle import ia_oracle as O


def run_oracle_call(kw, call, inputs):
    b = O.Binning(**box_params(kw))
    data = {k: np.array(v) for k, v in inputs.items()}
    data["LOS"] = call["los"]
    masks = masks_for(inputs, call["mask"]) if call["mask"] else None
    return O.measure(call["kind"], b, data, call["dataset"], call["corr_type"], call["num_jk"], masks,
                     call["ellipticity"], layout_of(kw, call))


@pytest.mark.parametrize("name", case_names())
def test_oracle_matches_reference_case(name):
    meta, inputs, outs, cnts = load_case(name)
    kw = meta["kwargs"]
    produced = {}
    counts = {}
    for call in meta["calls"]:
        res = run_oracle_call(kw, call, inputs)
        c = res.pop("__counts__")
        produced.update(res)
        top = "w" if call["kind"] == "w" else "multipoles"
        counts[(top, call["dataset"], call["num_jk"])] = c
    assert set(produced) == set(outs), sorted(set(produced) ^ set(outs))[:10]
    for path, ref in outs.items():
        assert_close(produced[path], ref, 1e-12, path)
    # integer pair counts = the reference's unit-weight DD, total and per realisation
    for (top, d, njk), c in counts.items():
        sg = O.Binning(**box_params(kw)).snap_group
        tot = cnts[f"{sg}{top}/xi_gg/{d}_DD"]
        np.testing.assert_array_equal(c.npairs, tot)
        for i in range(njk):
            ri = cnts[f"{sg}{top}/xi_gg/{d}_jk{njk}/{d}_{i}_DD"]
            np.testing.assert_array_equal(c.npairs - c.npairs_jk[i], ri)


def test_corr_type_subsets_equal_both():
    """'g+' and 'gg' outputs are the matching parts of 'both'
    (reference tests/test_w_sim_internal_consistency.py:35-56)."""
    meta, inputs, _, _ = load_case("w_jk27_mp")
    kw = meta["kwargs"]
    call = dict(meta["calls"][0])
    both = run_oracle_call(kw, call, inputs)
    for ct, grp in (("g+", "w_g_plus"), ("gg", "w_gg")):
        call2 = dict(call, corr_type=ct)
        part = run_oracle_call(kw, call2, inputs)
        for k, v in part.items():
            if k == "__counts__":
                continue
            np.testing.assert_array_equal(v, both[k])
        assert any(grp in k for k in part)


def test_weight_scaling_invariants():
    """All weights 0.5: w_g+ and DD scale by 1/4, covariances by 1/16
    (reference tests/test_weights.py:34-40)."""
    meta, inputs, _, _ = load_case("w_clustered_jk27")
    kw = meta["kwargs"]
    call = dict(meta["calls"][0], num_jk=8)
    one = dict(inputs, weight=np.ones(len(inputs["Position"])),
               weight_shape_sample=np.ones(len(inputs["Position_shape_sample"])))
    half = dict(inputs, weight=np.full(len(inputs["Position"]), 0.5),
                weight_shape_sample=np.full(len(inputs["Position_shape_sample"]), 0.5))
    a = run_oracle_call(kw, call, one)
    h = run_oracle_call(kw, call, half)
    d = call["dataset"]
    np.testing.assert_allclose(a[f"w_g_plus/{d}"], 4 * h[f"w_g_plus/{d}"], rtol=1e-12)
    np.testing.assert_allclose(a[f"w/xi_gg/{d}_DD"], 4 * h[f"w/xi_gg/{d}_DD"], rtol=1e-12)
    np.testing.assert_allclose(a[f"w_g_plus/{d}_jackknife_cov_8"], 16 * h[f"w_g_plus/{d}_jackknife_cov_8"],
                               rtol=1e-9)
    np.testing.assert_allclose(a[f"w_gg/{d}_jackknife_cov_8"], 16 * h[f"w_gg/{d}_jackknife_cov_8"], rtol=1e-9)


def test_jackknife_labels_known_answer():
    com = np.array([[1, 1, 1], [2, 1, 2], [2.5, 2.5, 1.51], [1, 2, 2]], dtype=float)
    np.testing.assert_array_equal(O.jackknife_labels(com, 1.5, 2), [0, 5, 7, 3])


def test_jackknife_labels_faces_keep_zero():
    L = 205.0
    pts = np.array([[0.0, 10.0, 10.0], [L / 3, 10, 10], [2 * (L / 2.0 * 2.0 / 3), 100, 150], [100, 100, 100]])
    lab = O.jackknife_labels(pts, L / 2.0, 3)
    assert lab[0] == 0 and lab[1] == 0 and lab[2] == 0 and lab[3] == 13


# ---------------------------------------------------------------------------
# the reference's golden HDF5 outputs (TNG300 mock, 8 jackknife regions)
# ---------------------------------------------------------------------------

GOLD = os.path.join(GOLDEN, "tng300_mock_outputs.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


TNG = O.Binning(boxsize=205.0, r_min=0.1, r_max=20.0, num_bins_r=10, num_bins_pi=8, pi_max=None, snapshot=99)


@pytest.mark.parametrize("tag", ["small", "large"])
@pytest.mark.parametrize("d", ["All", "high", "low"])
def test_golden_w_and_covariance(gold, tag, d):
    g = lambda p: gold[f"{tag}/Snapshot_99/{p}"]
    np.testing.assert_array_equal(g(f"w/xi_g_plus/{d}_rp"), O.bin_centres(TNG.r_bins))
    np.testing.assert_array_equal(g(f"w/xi_g_plus/{d}_pi"), O.bin_centres(TNG.pi_bins))
    for xi_name, w_name in (("xi_g_plus", "w_g_plus"), ("xi_gg", "w_gg")):
        reals = []
        for i in [None] + list(range(8)):
            dn = d if i is None else f"{d}_{i}"
            w = O.w_from_xi(TNG, g(f"w/{xi_name}/{dn}"))
            assert_close(w, g(f"{w_name}/{dn}"), 1e-13, f"{tag} {w_name}/{dn}")
            if i is not None:
                reals.append(g(f"{w_name}/{dn}"))
        mean, std, cov = O.combine_jackknife(np.array(reals))
        assert_close(mean, g(f"{w_name}/{d}_mean_8"), 1e-12, "mean")
        assert_close(std, g(f"{w_name}/{d}_jackknife_8"), 1e-12, "std")
        assert_close(cov, g(f"{w_name}/{d}_jackknife_cov_8"), 1e-12, "cov")


@pytest.mark.parametrize("tag", ["small", "large"])
@pytest.mark.parametrize("d", ["All", "high", "low"])
def test_golden_multipoles_and_covariance(gold, tag, d):
    g = lambda p: gold[f"{tag}/Snapshot_99/{p}"]
    np.testing.assert_array_equal(g(f"multipoles/xi_g_plus/{d}_mu_r"), O.bin_centres(TNG.mu_r_bins))
    for xi_name, m_name, l in (("xi_g_plus", "multipoles_g_plus", 2), ("xi_gg", "multipoles_gg", 0)):
        reals = []
        for i in [None] + list(range(8)):
            dn = d if i is None else f"{d}_{i}"
            m = O.multipoles_from_xi(TNG, g(f"multipoles/{xi_name}/{dn}"), l)
            assert_close(m, g(f"{m_name}/{dn}"), 1e-12, f"{tag} {m_name}/{dn}")
            if i is not None:
                reals.append(g(f"{m_name}/{dn}"))
        mean, std, cov = O.combine_jackknife(np.array(reals))
        assert_close(cov, g(f"{m_name}/{d}_jackknife_cov_8"), 1e-12, "cov")
        assert_close(std, g(f"{m_name}/{d}_jackknife_8"), 1e-12, "std")


@pytest.mark.parametrize("tag", ["small", "large"])
@pytest.mark.parametrize("top", ["w", "multipoles"])
def test_golden_xi_assembly_and_randoms(gold, tag, top):
    g = lambda p: gold[f"{tag}/Snapshot_99/{top}/{p}"]
    for d in ("All", "high", "low"):
        assert_close(g(f"xi_g_plus/{d}_SplusD") / g(f"xi_g_plus/{d}_RR_g_plus"), g(f"xi_g_plus/{d}"), 1e-15, d)
        assert_close(g(f"xi_gg/{d}_DD") / g(f"xi_gg/{d}_RR_gg") - 1, g(f"xi_gg/{d}"), 1e-15, d)
        assert_close(g(f"xi_g_cross/{d}_ScrossD") / g(f"xi_g_cross/{d}_RR_g_cross"), g(f"xi_g_cross/{d}"), 1e-15, d)
        # analytic RR: one factor N_p*N_s (or (N_p-1)*N_s) times the bin volume over L^3
        rr = g(f"xi_g_plus/{d}_RR_g_plus")
        unit, _ = O.rr_tables(TNG, "w" if top == "w" else "m", 1 if top == "w" else 2, 1)
        scale = rr / unit
        assert np.allclose(scale, scale.flat[0], rtol=1e-12)
        n = scale.flat[0]
        assert abs(n - round(n)) < 1e-6 * n
