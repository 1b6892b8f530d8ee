"""GPU parity: the CUDA path (through the C ABI) against the reference's
fixtures and the CPU oracle on the same inputs.

Bar: integer pair counts per (bin, jackknife region) bit-exact; every
floating-point dataset within 1e-10 relative for the plain FP64 form (scale
floor: the array's max |value|, for bins that cancel to ~0).  The mixed form
keeps the counts bit-exact and stays within 2e-5 on these small catalogues
(few pairs per bin, so FP32 term errors do not average out).
"""

import numpy as np
import pytest

from golden_io import assert_close, box_params, case_names, layout_of, load_case, masks_for
from oracle import ia_oracle as O

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
MIXED_RTOL = 2e-5


def _box(kw, precision, outfile):
    from measure_ia_gb300 import MeasureIABox
    bp = box_params(kw)
    return MeasureIABox, dict(output_file_name=outfile, simulation=kw.get("simulation"), snapshot=kw.get("snapshot"),
                              separation_limits=kw["separation_limits"], num_bins_r=kw["num_bins_r"],
                              num_bins_pi=kw["num_bins_pi"], pi_max=kw.get("pi_max"), boxsize=kw.get("boxsize"),
                              num_nodes=kw.get("num_nodes", 1), precision=precision)


def run_product(meta, inputs, precision, outfile):
    from measure_ia_gb300 import open_output
    kw = meta["kwargs"]
    cls, ckw = _box(kw, precision, outfile)
    measurements = []
    for call in meta["calls"]:
        data = {k: np.array(v) for k, v in inputs.items()}
        data["LOS"] = call["los"]
        box = cls(data, **ckw)
        masks = masks_for(inputs, call["mask"]) if call["mask"] else None
        tpath = False if call["temp"] is False else "/tmp"
        fn = box.measure_xi_w if call["kind"] == "w" else box.measure_xi_multipoles
        fn(call["dataset"], call["corr_type"], call["num_jk"], temp_file_path=tpath, masks=masks,
           ellipticity=call["ellipticity"])
        measurements.append((call, box.last_measurement))
    store = open_output(outfile)
    return {k: store.read(k) for k in store.keys()}, measurements


def oracle_counts(meta, inputs, call):
    kw = meta["kwargs"]
    b = O.Binning(**box_params(kw))
    data = {k: np.array(v) for k, v in inputs.items()}
    data["LOS"] = call["los"]
    masks = masks_for(inputs, call["mask"]) if call["mask"] else None
    res = O.measure(call["kind"], b, data, call["dataset"], call["corr_type"], call["num_jk"], masks,
                    call["ellipticity"], layout_of(kw, call))
    return res


# cases whose floats were compared with the oracle on this host because the
# x86-made fixture's counts differ from the host oracle's (numpy's log10 is
# host dependent); reported at the end of the session
FALLBACKS = []
CHECKED = []


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", case_names())
def test_cases_match_reference(name, precision, tmp_path):
    meta, inputs, outs, cnts = load_case(name)
    produced, meas = run_product(meta, inputs, precision, str(tmp_path / f"{name}_{precision}.hdf5"))
    assert set(produced) == set(outs), sorted(set(produced) ^ set(outs))[:10]
    rtol = FP64_RTOL if precision == "fp64" else MIXED_RTOL
    CHECKED.append(f"{name}/{precision}")
    # integer counts: bit-exact against the oracle run on this host (same log10 as the bin tables),
    # and against the reference's unit-weight DD wherever the host oracle agrees with it
    host_agrees = True
    host_outs = {}
    for call, m in meas:
        res = oracle_counts(meta, inputs, call)
        c = res.pop("__counts__")
        host_outs.update(res)
        np.testing.assert_array_equal(m.npairs[0], c.npairs, err_msg=f"{call}")
        for i in range(call["num_jk"]):
            np.testing.assert_array_equal(m.npairs[0] - m.npairs[1 + i], c.npairs - c.npairs_jk[i])
        sg = "" if meta["kwargs"].get("snapshot") is None else f"Snapshot_{meta['kwargs']['snapshot']}/"
        top = "w" if call["kind"] == "w" else "multipoles"
        ref_tot = cnts[f"{sg}{top}/xi_gg/{call['dataset']}_DD"]
        host_agrees &= np.array_equal(c.npairs, ref_tot)
        if host_agrees:
            np.testing.assert_array_equal(m.npairs[0], ref_tot)
    if host_agrees:
        for path, ref in outs.items():
            assert_close(produced[path], ref, rtol, path)
    else:
        # the fixture's bin assignment is not this host's: every float dataset
        # against the oracle run here on the same inputs instead
        FALLBACKS.append(f"{name}/{precision}")
        assert set(host_outs) == set(outs), sorted(set(host_outs) ^ set(outs))[:10]
        for path, ref in host_outs.items():
            assert_close(produced[path], ref, rtol, path)


def test_config0_against_oracle():
    """10,000 uniform galaxies in a 205 Mpc/h box, w with 27 jackknife regions
    (the CPU-sized configuration): GPU FP64 vs the oracle on this host."""
    from measure_ia_gb300.catalogs import uniform_catalog
    from measure_ia_gb300 import MeasureIABox, open_output
    data = uniform_catalog(10000, 205.0, 2024)
    b = O.Binning(boxsize=205.0, r_min=0.1, r_max=20.0, num_bins_r=10, num_bins_pi=8, pi_max=20.0)
    ref = O.measure("w", b, {k: np.array(v) if k != "LOS" else v for k, v in data.items()}, "c0", "both", 27)
    c = ref.pop("__counts__")
    box = MeasureIABox(data, "/tmp/c0_gpu.hdf5", None, None, [0.1, 20.0], 10, 8, 20.0, boxsize=205.0, num_nodes=8)
    box.measure_xi_w("c0", "both", 27, temp_file_path="/tmp")
    m = box.last_measurement
    np.testing.assert_array_equal(m.npairs[0], c.npairs)
    np.testing.assert_array_equal(m.npairs[1:], c.npairs_jk)
    st = open_output("/tmp/c0_gpu.hdf5")
    for path, v in ref.items():
        assert_close(st.read(path), v, FP64_RTOL, path)
    assert m.stats["binned_pairs"] == int(c.npairs.sum())


def test_mixed_matches_fp64_clustered():
    """Clustered catalogue with lognormal weights: the mixed form's counts are
    bit-exact with the FP64 form; w_gg within 1e-6 relative per bin; w_g+
    within 1e-6 of the vector's scale.  (Per bin, w_g+ of the smallest r_p bin
    is a near-total cancellation here -- |sum e+| ~ 1e-3 sum|e+| -- so its
    relative error is bounded by 3e-5 instead.)"""
    from measure_ia_gb300.catalogs import neyman_scott_catalog
    from measure_ia_gb300.engine import PairCounter
    data = neyman_scott_catalog(2000, 205.0, 40000, 7, mean_children=50, sigma=1.0)
    r_bins = np.logspace(-1, np.log10(20.0), 11)
    pi_bins = np.linspace(-20.0, 20.0, 9)
    res = {}
    for prec in ("fp64", "mixed"):
        pc = PairCounter("w", boxsize=205.0, r_bins=r_bins, r_min=0.1, r_max=20.0, p_bins=pi_bins, l_subboxes=3,
                         precision=prec)
        res[prec] = pc.measure(data)
    a, m = res["fp64"], res["mixed"]
    np.testing.assert_array_equal(a.npairs, m.npairs)
    rel_gg = np.abs(m["proj_gg"] - a["proj_gg"]) / np.abs(a["proj_gg"])
    assert rel_gg.max() < 1e-6, rel_gg.max()
    gp_err = np.abs(m["proj_gp"] - a["proj_gp"])
    assert gp_err.max() / np.abs(a["proj_gp"]).max() < 1e-6
    assert (gp_err / np.abs(a["proj_gp"])).max() < 3e-5
    assert_close(m["DD_all"], a["DD_all"], 1e-6, "DD")
    assert m.stats["binned_pairs"] == a.stats["binned_pairs"]
