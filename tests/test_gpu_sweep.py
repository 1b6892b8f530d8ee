"""Randomised parity sweep: seeded configurations drawn across the space the
reference accepts (box size, r and Pi/mu_r binnings, pi_max including the
L/2 default, jackknife counts, line of sight, corr_type, ellipticity
definition, tree / multiprocessing / brute layouts, masks with and without
weight keys, unit and lognormal weights, uniform and clustered catalogues,
shape samples that are or are not the position sample), each run through
MeasureIABox in both forms and checked against the oracle on the same inputs.

Bar: the integer pair counts per (bin, jackknife region) bit-exact in both
forms; every dataset within 1e-10 relative (FP64 form) or 2e-5 (mixed form,
few pairs per bin), with the array's max |value| as the floor for bins that
cancel; non-finite entries (empty jackknife regions) at the same places.
"""

import numpy as np
import pytest

from oracle import ia_oracle as O

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
MIXED_RTOL = 2e-5
N_CASES = 40


def _catalogue(rng, L, los):
    n_pos = int(rng.integers(300, 6000))
    if rng.uniform() < 0.5:
        pos = rng.uniform(0.0, L, (n_pos, 3))
    else:
        n_par = max(4, n_pos // 30)
        cen = rng.uniform(0.0, L, (n_par, 3))
        pos = np.mod(cen[rng.integers(0, n_par, n_pos)] + rng.normal(0.0, L / 80.0, (n_pos, 3)), L)
    pos[pos >= L] = 0.0
    if rng.uniform() < 0.4:                       # shape sample = position sample
        spos = pos.copy()
    else:
        pick = np.sort(rng.choice(n_pos, int(rng.integers(50, n_pos)), replace=False))
        spos = pos[pick].copy()
    n_s = len(spos)
    ang = rng.uniform(0.0, np.pi, n_s)
    scale = rng.uniform(0.5, 2.0, n_s)            # unnormalised axes
    data = {"Position": pos, "Position_shape_sample": spos,
            "Axis_Direction": np.c_[scale * np.cos(ang), scale * np.sin(ang)],
            "q": rng.uniform(0.1, 1.0, n_s), "LOS": los}
    if rng.uniform() < 0.5:
        data["weight"] = np.exp(rng.normal(0.0, 0.4, n_pos))
        data["weight_shape_sample"] = np.exp(rng.normal(0.0, 0.4, n_s))
    else:
        data["weight"] = np.ones(n_pos)
        data["weight_shape_sample"] = np.ones(n_s)
    return data


def _masks(rng, data):
    if rng.uniform() < 0.6:
        return None
    sp = rng.uniform(size=len(data["Position"])) < 0.7
    ss = rng.uniform(size=len(data["Position_shape_sample"])) < 0.7
    m = {"Position": sp, "Position_shape_sample": ss, "Axis_Direction": ss, "q": ss}
    if rng.uniform() < 0.5:
        m["weight"] = sp
        m["weight_shape_sample"] = ss
    return m


def draw_case(i):
    rng = np.random.default_rng(7100 + i)
    L = float(rng.choice([40.0, 75.0, 150.0, 205.0, 300.0]))
    kind = "w" if i % 2 == 0 else "m"
    r_max = float(L * rng.uniform(0.04, 0.2))
    r_min = float(r_max * 10.0 ** -rng.uniform(0.4, 2.5))
    if rng.uniform() < 0.25:
        pi_max = None                             # the reference's default: L/2
    else:
        pi_max = float(min(L / 2.0, r_max * rng.uniform(0.3, 2.0)))
    case = dict(L=L, kind=kind, r_min=r_min, r_max=r_max, pi_max=pi_max,
                n_r=int(rng.integers(1, 16)), n_p=int(rng.integers(1, 13)),
                num_jk=int(rng.choice([0, 8, 27, 64, 125])), los=int(rng.integers(0, 3)),
                corr_type=str(rng.choice(["both", "g+", "gg"])),
                ellipticity=str(rng.choice(["distortion", "ellipticity"])),
                layout=str(rng.choice(["tree", "multiprocessing", "brute"])))
    data = _catalogue(rng, L, case["los"])
    return case, data, _masks(rng, data)


def _copy(data):
    return {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in data.items()}


def _copy_masks(m):
    return None if m is None else {k: v.copy() for k, v in m.items()}


def _close(got, ref, rtol, what):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    assert got.shape == ref.shape, (what, got.shape, ref.shape)
    fin = np.isfinite(ref)
    np.testing.assert_array_equal(np.isfinite(got), fin, err_msg=f"{what}: non-finite pattern")
    np.testing.assert_array_equal(np.isnan(got), np.isnan(ref), err_msg=f"{what}: nan pattern")
    if not fin.all():
        np.testing.assert_array_equal(got[~fin & ~np.isnan(ref)], ref[~fin & ~np.isnan(ref)], err_msg=what)
    g, r = got[fin], ref[fin]
    if r.size == 0:
        return
    lim = rtol * np.abs(r) + rtol * np.max(np.abs(r))
    err = np.abs(g - r)
    assert np.all(err <= lim), f"{what}: max err {err.max():.3e} (scale {np.max(np.abs(r)):.3e})"


_ORACLE = {}


def _oracle(i):
    if i not in _ORACLE:
        case, data, masks = draw_case(i)
        b = O.Binning(boxsize=case["L"], r_min=case["r_min"], r_max=case["r_max"], num_bins_r=case["n_r"],
                      num_bins_pi=case["n_p"], pi_max=case["pi_max"])
        _ORACLE[i] = O.measure(case["kind"], b, _copy(data), "s", case["corr_type"], case["num_jk"],
                               _copy_masks(masks), case["ellipticity"], case["layout"])
    return _ORACLE[i]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("i", range(N_CASES))
def test_random_configuration(i, precision, tmp_path):
    from measure_ia_gb300 import MeasureIABox, open_output, read_output
    case, data, masks = draw_case(i)
    ref = dict(_oracle(i))
    c = ref.pop("__counts__")
    out = str(tmp_path / "sweep.hdf5")
    box = MeasureIABox(_copy(data), out, None, None, [case["r_min"], case["r_max"]], case["n_r"], case["n_p"],
                       case["pi_max"], boxsize=case["L"], num_nodes=4 if case["layout"] == "multiprocessing" else 1,
                       precision=precision)
    fn = box.measure_xi_w if case["kind"] == "w" else box.measure_xi_multipoles
    fn("s", case["corr_type"], case["num_jk"], temp_file_path=False if case["layout"] == "brute" else str(tmp_path),
       masks=_copy_masks(masks), ellipticity=case["ellipticity"])
    m = box.last_measurement
    np.testing.assert_array_equal(m.npairs[0], c.npairs, err_msg=str(case))
    if case["num_jk"]:
        np.testing.assert_array_equal(m.npairs[1:], c.npairs_jk, err_msg=str(case))
    store = open_output(out)
    assert set(store.keys()) == set(ref), sorted(set(store.keys()) ^ set(ref))[:10]
    rtol = FP64_RTOL if precision == "fp64" else MIXED_RTOL
    for path, v in ref.items():
        _close(store.read(path), v, rtol, f"{path} {case}")
    on_disk = read_output(out)                    # the HDF5 file holds exactly the store
    assert set(on_disk) == set(ref)
    for path in ref:
        np.testing.assert_array_equal(on_disk[path], store.read(path))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("i", range(6))
def test_multipoles_rp_cut(i, precision):
    """The pair counter's projected-separation cut for multipoles (pairs with
    r_p <= rp_cut dropped, measure_m_box_jk.py's rp_cut branch): counts per
    region bit-exact, DD and S+D against the oracle's histograms."""
    from measure_ia_gb300.engine import PairCounter
    case, data, _ = draw_case(2 * i + 1)
    rng = np.random.default_rng(300 + i)
    rp_cut = float(case["r_max"] * rng.uniform(0.05, 0.6))
    b = O.Binning(boxsize=case["L"], r_min=case["r_min"], r_max=case["r_max"], num_bins_r=case["n_r"],
                  num_bins_pi=case["n_p"], pi_max=case["pi_max"])
    L_sub = round(case["num_jk"] ** (1 / 3)) if case["num_jk"] else 0
    pos, spos, axis, q, w, ws = O.select_inputs(data, None)
    e = O.ellipticity_size(q, case["ellipticity"])
    R = O.responsivity(ws, e)
    lab_p = lab_s = None
    if L_sub:
        lab_p = O.jackknife_labels(pos, b.L_0p5, L_sub)
        lab_s = O.jackknife_labels(spos, b.L_0p5, L_sub)
    c = O.count_pairs("m", b, case["los"], pos, w, spos, axis, e, ws, R, lab_p, lab_s, L_sub ** 3 if L_sub else 0,
                      "tree", rp_cut)
    pc = PairCounter("m", boxsize=case["L"], r_bins=b.r_bins, r_min=case["r_min"], r_max=case["r_max"],
                     p_bins=b.mu_r_bins, los=case["los"], l_subboxes=L_sub, precision=precision,
                     ellipticity=case["ellipticity"], rp_cut=rp_cut)
    m = pc.measure(data)
    np.testing.assert_array_equal(m.npairs[0], c.npairs)
    if L_sub:
        np.testing.assert_array_equal(m.npairs[1:], c.npairs_jk)
    rtol = FP64_RTOL if precision == "fp64" else MIXED_RTOL
    _close(m["DD"], c.DD, rtol, "DD")
    _close(m["splusd"], c.SplusD, rtol, "S+D")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["w", "m"])
def test_positions_on_subbox_faces(kind, precision, tmp_path):
    """Galaxies exactly on jackknife sub-box faces carry region 0 wherever
    they are (measure_IA_base.py:428-451); a quarter of the positions and of
    the shapes sit on a face here.  Counts per region bit-exact, values as in
    the sweep."""
    from measure_ia_gb300 import MeasureIABox, open_output
    rng = np.random.default_rng(4242)
    L, n_sub = 120.0, 2
    faces = np.array([0.0, L / n_sub])
    pos = rng.uniform(0.0, L, (5000, 3))
    on = rng.uniform(size=len(pos)) < 0.25
    pos[on, rng.integers(0, 3, on.sum())] = faces[rng.integers(0, 2, on.sum())]
    pick = np.sort(rng.choice(len(pos), 2000, replace=False))
    spos = pos[pick].copy()
    on_s = rng.uniform(size=len(spos)) < 0.25
    spos[on_s, rng.integers(0, 3, on_s.sum())] = faces[rng.integers(0, 2, on_s.sum())]
    ang = rng.uniform(0.0, np.pi, len(spos))
    data = {"Position": pos, "Position_shape_sample": spos, "Axis_Direction": np.c_[np.cos(ang), np.sin(ang)],
            "q": rng.uniform(0.2, 1.0, len(spos)), "weight": np.exp(rng.normal(0.0, 0.3, len(pos))),
            "weight_shape_sample": np.exp(rng.normal(0.0, 0.3, len(spos))), "LOS": 2}
    r_min, r_max, n_r, n_p, pi_max = 0.2, 15.0, 8, 6, 15.0
    b = O.Binning(boxsize=L, r_min=r_min, r_max=r_max, num_bins_r=n_r, num_bins_pi=n_p, pi_max=pi_max)
    ref = dict(O.measure(kind, b, _copy(data), "f", "both", n_sub ** 3, None, "distortion", "tree"))
    c = ref.pop("__counts__")
    out = str(tmp_path / "faces.hdf5")
    box = MeasureIABox(_copy(data), out, None, None, [r_min, r_max], n_r, n_p, pi_max, boxsize=L,
                       precision=precision)
    fn = box.measure_xi_w if kind == "w" else box.measure_xi_multipoles
    fn("f", "both", n_sub ** 3, temp_file_path=str(tmp_path), ellipticity="distortion")
    m = box.last_measurement
    np.testing.assert_array_equal(m.npairs[0], c.npairs)
    np.testing.assert_array_equal(m.npairs[1:], c.npairs_jk)
    store = open_output(out)
    rtol = FP64_RTOL if precision == "fp64" else MIXED_RTOL
    for path, v in ref.items():
        _close(store.read(path), v, rtol, path)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nan_axis_directions(precision, tmp_path):
    """A shape with a NaN axis contributes e+ = ex = 0 (the reference's NaN -> 0,
    measure_w_box_jk.py:599-600) and still counts in DD; the mixed form hands
    such a catalogue to the FP64 form with a warning."""
    from measure_ia_gb300 import MeasureIABox, open_output
    rng = np.random.default_rng(77)
    L, n = 100.0, 3000
    pos = rng.uniform(0, L, (n, 3))
    ang = rng.uniform(0, np.pi, n)
    ax = np.c_[np.cos(ang), np.sin(ang)]
    ax[::17] = np.nan
    data = {"Position": pos, "Position_shape_sample": pos.copy(), "Axis_Direction": ax,
            "q": rng.uniform(0.2, 1, n), "LOS": 2, "weight": np.exp(rng.normal(0, 0.3, n)),
            "weight_shape_sample": np.exp(rng.normal(0, 0.3, n))}
    b = O.Binning(boxsize=L, r_min=0.1, r_max=10.0, num_bins_r=6, num_bins_pi=4, pi_max=10.0)
    ref = dict(O.measure("w", b, _copy(data), "a", "both", 8, None, "distortion", "tree"))
    ref.pop("__counts__")
    out = str(tmp_path / "nan_axis.hdf5")
    box = MeasureIABox(_copy(data), out, None, None, [0.1, 10.0], 6, 4, 10.0, boxsize=L, precision=precision)
    if precision == "mixed":
        with pytest.warns(RuntimeWarning, match="Axis_Direction"):
            box.measure_xi_w("a", "both", 8, temp_file_path=str(tmp_path))
    else:
        box.measure_xi_w("a", "both", 8, temp_file_path=str(tmp_path))
    store = open_output(out)
    for path, v in ref.items():
        _close(store.read(path), v, FP64_RTOL, path)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["w", "m"])
def test_large_box_geometry_jk125(kind, precision, tmp_path):
    """The large-box configuration's geometry scaled down: a 1000 Mpc/h box,
    15 log r bins 0.1-60, 20 Pi bins over |Pi| <= 60 (or 20 mu_r bins), 125
    jackknife regions (5 x 5 x 5 sub-boxes, measure_IA_base.py:404-452, and
    the RR_jk loop of measure_w_box_jk.py:798-807), on a clustered catalogue
    of ~24,000 positions and 6,000 shapes, plus 600 pairs placed on bin
    edges (r_p or Pi equal to an edge up to the FP64 subtraction, r_max = 60
    and |Pi| = 60 among them): in this box the FP64 form's FP32 range test has
    its largest absolute margin.  At 125 regions a work unit's neighbourhood
    spans more regions than at 27.  Every dataset against the oracle: counts
    per (bin, region) bit-exact, values as in the sweep."""
    from measure_ia_gb300 import MeasureIABox, open_output
    from measure_ia_gb300.catalogs import add_edge_pairs, neyman_scott_catalog
    L = 1000.0
    r_min, r_max, n_r, n_p, pi_max = 0.1, 60.0, 15, 20, 60.0
    data = neyman_scott_catalog(600, L, 6000, 125, mean_children=40, sigma=1.5)
    data = add_edge_pairs(data, L, 126, np.logspace(np.log10(r_min), np.log10(r_max), n_r + 1),
                          np.linspace(-pi_max, pi_max, n_p + 1), 600)
    b = O.Binning(boxsize=L, r_min=r_min, r_max=r_max, num_bins_r=n_r, num_bins_pi=n_p, pi_max=pi_max)
    ref = dict(O.measure(kind, b, _copy(data), "big", "both", 125, None, "distortion", "multiprocessing"))
    c = ref.pop("__counts__")
    out = str(tmp_path / "big.hdf5")
    box = MeasureIABox(_copy(data), out, None, None, [r_min, r_max], n_r, n_p, pi_max, boxsize=L, num_nodes=4,
                       precision=precision)
    fn = box.measure_xi_w if kind == "w" else box.measure_xi_multipoles
    fn("big", "both", 125, temp_file_path=str(tmp_path))
    m = box.last_measurement
    assert c.npairs.sum() > 10000
    np.testing.assert_array_equal(m.npairs[0], c.npairs)
    np.testing.assert_array_equal(m.npairs[1:], c.npairs_jk)
    store = open_output(out)
    assert set(store.keys()) == set(ref)
    rtol = FP64_RTOL if precision == "fp64" else MIXED_RTOL
    for path, v in ref.items():
        _close(store.read(path), v, rtol, path)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["w", "m"])
def test_narrow_r_bins(kind, precision, tmp_path):
    """60 log r bins over 1.0-1.2 Mpc/h: adjacent breakpoints of q = r^2 lie
    0.6% apart, so a 1/64-octave bucket of the mixed form's lookup table can
    hold the guard bands of two of them, and r_min / r_max coincide with the
    first and last bin edges (tree membership).  The short pair path merges
    the bands that meet a bucket into one; a q inside it goes to the FP64
    re-test.  Counts per (bin, region) bit-exact against the oracle, values as
    in the sweep."""
    from measure_ia_gb300 import MeasureIABox, open_output
    from measure_ia_gb300.catalogs import neyman_scott_catalog
    L = 60.0
    r_min, r_max, n_r, n_p, pi_max = 1.0, 1.2, 60, 4, 3.0
    data = neyman_scott_catalog(600, L, 8000, 61, mean_children=60, sigma=1.0)
    b = O.Binning(boxsize=L, r_min=r_min, r_max=r_max, num_bins_r=n_r, num_bins_pi=n_p, pi_max=pi_max)
    ref = dict(O.measure(kind, b, _copy(data), "nb", "both", 8, None, "distortion", "tree"))
    c = ref.pop("__counts__")
    out = str(tmp_path / "nb.hdf5")
    box = MeasureIABox(_copy(data), out, None, None, [r_min, r_max], n_r, n_p, pi_max, boxsize=L, num_nodes=1,
                       precision=precision)
    fn = box.measure_xi_w if kind == "w" else box.measure_xi_multipoles
    fn("nb", "both", 8, temp_file_path=str(tmp_path))
    m = box.last_measurement
    assert c.npairs.sum() > 20000
    np.testing.assert_array_equal(m.npairs[0], c.npairs)
    np.testing.assert_array_equal(m.npairs[1:], c.npairs_jk)
    store = open_output(out)
    assert set(store.keys()) == set(ref)
    rtol = FP64_RTOL if precision == "fp64" else MIXED_RTOL
    for path, v in ref.items():
        _close(store.read(path), v, rtol, path)


def test_default_pi_max_medium():
    """w with the reference's default pi_max = L/2 (the line-of-sight reach
    spans the box, so the mixed form's short path brings Pi to the minimum
    image per pair) on ~60,000 clustered positions and 15,000 shapes with 27
    jackknife regions: the mixed form against the FP64 form, pair counts per
    (bin, region) bit-exact, w_g+ and w_gg within 1e-5 of their scale."""
    from measure_ia_gb300.catalogs import neyman_scott_catalog
    from measure_ia_gb300.engine import PairCounter
    L = 100.0
    data = neyman_scott_catalog(1200, L, 15000, 77, mean_children=50, sigma=1.0, kappa=2.0)
    common = dict(boxsize=L, r_bins=np.logspace(-1, 1, 9), r_min=0.1, r_max=10.0,
                  p_bins=np.linspace(-L / 2, L / 2, 11), l_subboxes=3, device=0)
    mixed = PairCounter("w", precision="mixed", **common).measure(data)
    fp64 = PairCounter("w", precision="fp64", **common).measure(data)
    assert mixed.stats["binned_pairs"] > 1_000_000
    np.testing.assert_array_equal(mixed.npairs, fp64.npairs)
    for key in ("proj_gp", "proj_gg"):
        ref = np.asarray(fp64[key])
        err = np.max(np.abs(np.asarray(mixed[key]) - ref)) / np.max(np.abs(ref))
        assert err < 1e-5, (key, err)
