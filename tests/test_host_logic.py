"""Host-side logic that needs no GPU: the C ABI library and its exports, the
exact bin tables against the reference's formulas, and the API's validation."""

import ctypes
import os
import re

import numpy as np
import pytest

from measure_ia_gb300 import binning as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_header_symbol():
    from measure_ia_gb300 import _lib
    lib = _lib.load()
    hdr = open(os.path.join(ROOT, "include", "measure_ia_gb300.h")).read()
    declared = set(re.findall(r"MIA_API\s+[\w\s\*]+?\b(mia_\w+)\s*\(", hdr))
    assert declared == set(_lib.EXPORTED)
    for name in declared:
        assert hasattr(lib, name)
    assert lib.mia_version() >= 1


def test_layout_and_workspace_sizes():
    from measure_ia_gb300.engine import PairCounter
    pc = PairCounter("w", boxsize=205.0, r_bins=np.logspace(-1, np.log10(20), 11), r_min=0.1, r_max=20.0,
                     p_bins=np.linspace(-20, 20, 9), l_subboxes=3)
    lay = pc.layout
    assert lay.dd == 0 and lay.splus == 28 * 80 and lay.total > lay.stats
    assert pc.workspace_bytes(10000, 10000) > 10000 * 60
    mixed = PairCounter("w", boxsize=205.0, r_bins=np.logspace(-1, np.log10(20), 11), r_min=0.1, r_max=20.0,
                        p_bins=np.linspace(-20, 20, 9), l_subboxes=3, precision="mixed")
    assert mixed.workspace_bytes(10000, 10000) > pc.workspace_bytes(10000, 10000)


def _ref_r_bin(rp, r_bins, r_min, r_max, n):
    dlog = (np.log10(r_max) - np.log10(r_min)) / n
    mask = (rp >= r_bins[0]) * (rp < r_bins[-1])
    ind = np.floor(np.log10(rp[mask]) / dlog - np.log10(r_bins[0]) / dlog).astype(int)
    if np.any(ind == n):
        ind[ind >= n] -= 1
    out = np.full(len(rp), -1)
    out[mask] = np.where(ind < 0, ind + n, ind)
    return out


@pytest.mark.parametrize("r_min,r_max,n", [(0.1, 20.0, 10), (0.2, 15.0, 7), (0.1, 60.0, 15)])
def test_r_table_matches_reference_formula(r_min, r_max, n):
    r_bins = np.logspace(np.log10(r_min), np.log10(r_max), n + 1)
    t = B.r_table("w", r_bins, r_min, r_max, n, "brute")
    rng = np.random.default_rng(5)
    rp = np.concatenate([np.exp(rng.uniform(np.log(r_min / 2), np.log(r_max * 2), 200000)), r_bins,
                         np.nextafter(r_bins, 0), np.nextafter(r_bins, 1)])
    q = rp * rp
    rp_exact = np.sqrt(q)
    np.testing.assert_array_equal(t.lookup(q), _ref_r_bin(rp_exact, r_bins, r_min, r_max, n))


def test_tree_membership_uses_squared_radii():
    r_bins = np.logspace(-1, np.log10(20.0), 11)
    t = B.r_table("w", r_bins, 0.1, 20.0, 10, "tree")
    rmax2 = 20.0 * 20.0
    assert t.lookup(np.array([rmax2]))[0] >= 0
    assert t.lookup(np.array([np.nextafter(rmax2, np.inf)]))[0] == -1
    assert t.lookup(np.array([0.1 * 0.1]))[0] == -1


def test_pi_and_mu_tables_match_reference_formula():
    pi_bins = np.linspace(-20.0, 20.0, 9)
    t = B.pi_table(pi_bins, 8)
    rng = np.random.default_rng(6)
    x = np.concatenate([rng.uniform(-30, 30, 100000), pi_bins, np.nextafter(pi_bins, -1), np.nextafter(pi_bins, 1),
                        [-1e-15, -1e-16, 0.0, -0.0]])
    step = (pi_bins[-1] - pi_bins[0]) / 8
    mask = (x >= pi_bins[0]) & (x < pi_bins[-1])
    ind = np.floor(x[mask] / step - pi_bins[0] / step).astype(int)
    ind[ind >= 8] -= 1
    want = np.full(len(x), -1)
    want[mask] = ind
    np.testing.assert_array_equal(t.lookup(x), want)
    mu_bins = np.linspace(-1, 1, 21)
    tm = B.mu_table(mu_bins, 20)
    mu = np.concatenate([rng.uniform(-1, 1, 100000), mu_bins])
    ind = np.floor(mu / 0.1 - mu_bins[0] / 0.1).astype(int)
    ind[ind >= 20] -= 1
    np.testing.assert_array_equal(tm.lookup(mu), ind)


def test_order_key_roundtrip_and_order():
    x = np.array([-np.inf, -3.5, -1e-300, -0.0, 0.0, 1e-300, 2.0, np.inf])
    k = B.order_key(x)
    assert np.all(np.diff(k) > 0)
    np.testing.assert_array_equal(B.from_key(k).view(np.int64), x.view(np.int64))


def test_validation_errors_match_reference():
    from measure_ia_gb300 import MeasureIABox
    from measure_ia_gb300.catalogs import uniform_catalog
    d = uniform_catalog(100, 50.0, 1)
    box = MeasureIABox(d, None, None, None, [0.1, 5.0], 5, 4, 5.0, boxsize=50.0)
    with pytest.raises(ValueError, match="x\\^3"):
        box.measure_xi_w("x", "both", 10, temp_file_path="/tmp")
    with pytest.raises(ValueError, match="temp_file_path"):
        box.measure_xi_w("x", "both", 8, temp_file_path=None)
    with pytest.raises(KeyError, match="corr_type"):
        box.measure_xi_w("x", "bad", 8, temp_file_path="/tmp")
    with pytest.raises(ValueError, match="ellipticity"):
        box.measure_xi_multipoles("x", "both", 8, temp_file_path="/tmp", ellipticity="nope")
    with pytest.raises(ValueError, match="pi_max"):
        MeasureIABox(d, None, None, None)


def test_default_weights_written_into_callers_dict_and_siminfo():
    from measure_ia_gb300 import MeasureIABox
    d = {"Position": np.zeros((3, 3)), "Position_shape_sample": np.zeros((2, 3))}
    MeasureIABox(d, None, "TNG300", 99)
    np.testing.assert_array_equal(d["weight"], np.ones(3))
    np.testing.assert_array_equal(d["weight_shape_sample"], np.ones(2))
    b = MeasureIABox(None, None, "TNG300", 30)
    assert b.boxsize == 205.0 and b.snap_group == "Snapshot_30/" and b.L_0p5 == 102.5
    b = MeasureIABox(None, None, None, None, boxsize=300.0)
    assert b.snap_group == "" and b.boxsize == 300.0
    assert MeasureIABox(None, None, pi_max=20.0).boxsize is None


def test_mask_weight_quirk_mutates_masks():
    """Without weight keys the first sum(mask) weights are selected
    (measure_w_box_jk.py:701-712)."""
    from measure_ia_gb300 import MeasureIABox
    from measure_ia_gb300.catalogs import uniform_catalog
    d = uniform_catalog(10, 50.0, 2)
    d["weight"] = np.arange(10.0)
    box = MeasureIABox(d, None, None, None, [0.1, 5.0], 5, 4, 5.0, boxsize=50.0)
    sel = np.zeros(10, bool)
    sel[[2, 5, 7]] = True
    masks = {"Position": sel, "Position_shape_sample": sel, "Axis_Direction": sel, "q": sel}
    got = box._select(masks)
    np.testing.assert_array_equal(got["weight"], [0.0, 1.0, 2.0])
    assert "weight" in masks and "weight_shape_sample" in masks


def test_autotune_cache_roundtrip(tmp_path, monkeypatch):
    from measure_ia_gb300 import autotune
    path = str(tmp_path / "tune.json")
    monkeypatch.setenv("MIA_TUNE_CACHE", path)
    k1 = autotune.workload_key("w", "mixed", 4_000_000, 1_000_000, 205.0, 10, 8, 20.0, 20.0, 3, "tree", "GB300")
    k2 = autotune.workload_key("w", "mixed", 4_100_000, 1_000_000, 205.0, 10, 8, 20.0, 20.0, 3, "tree", "GB300")
    k3 = autotune.workload_key("w", "mixed", 8_000_000, 1_000_000, 205.0, 10, 8, 20.0, 20.0, 3, "tree", "GB300")
    assert k1 == k2 and k1 != k3
    assert autotune.load_cache() == {}
    autotune.store(k1, {"cell_size": 2.5, "cell_refine": 2, "shapes_per_unit": 128, "cell_size_los": 20.0,
                        "cell_refine_los": 1, "ms": 1.0})
    assert autotune.load_cache()[k1]["cell_refine"] == 2
    assert set(autotune.KNOBS) <= set(autotune.load_cache()[k1])
    sides, los_sides, refines, units = autotune.candidates(20.0, 40.0)
    assert len(sides) == 8 and 40.0 in los_sides and 2 in refines and 128 in units


@pytest.mark.parametrize("key,value", [("q", np.nan), ("weight", np.inf), ("weight_shape_sample", np.nan)])
def test_box_rejects_non_finite_weights_and_q(key, value):
    """A non-finite weight or q makes the reference's sums (through the
    responsivity, every S+D bin) NaN; the box path refuses them before any
    GPU work."""
    from measure_ia_gb300 import MeasureIABox
    rng = np.random.default_rng(0)
    n = 200
    pos = rng.uniform(0, 100.0, (n, 3))
    ang = rng.uniform(0, np.pi, n)
    data = {"Position": pos, "Position_shape_sample": pos.copy(), "Axis_Direction": np.c_[np.cos(ang), np.sin(ang)],
            "q": rng.uniform(0.2, 1, n), "LOS": 2, "weight": np.ones(n), "weight_shape_sample": np.ones(n)}
    data[key] = data[key].copy()
    data[key][3] = value
    box = MeasureIABox(data, None, None, None, [0.1, 10.0], 6, 4, 10.0, boxsize=100.0)
    with pytest.raises(ValueError, match="finite"):
        box.measure_xi_w("a", "both", 0, temp_file_path="/tmp")


@pytest.mark.parametrize("which", ["Position", "Position_shape_sample"])
def test_box_rejects_empty_samples(which):
    """A sample left empty by the masks is refused before any GPU work (the
    reference divides by zero for an empty shape sample and returns NaN
    correlations for an empty position sample)."""
    from measure_ia_gb300 import MeasureIABox
    rng = np.random.default_rng(0)
    n = 50
    pos = rng.uniform(0, 100.0, (n, 3))
    ang = rng.uniform(0, np.pi, n)
    data = {"Position": pos, "Position_shape_sample": pos.copy(), "Axis_Direction": np.c_[np.cos(ang), np.sin(ang)],
            "q": rng.uniform(0.2, 1, n), "LOS": 2, "weight": np.ones(n), "weight_shape_sample": np.ones(n)}
    keep = np.ones(n, dtype=bool)
    masks = {"Position": keep.copy(), "Position_shape_sample": keep.copy(), "Axis_Direction": keep.copy(),
             "q": keep.copy()}
    for k in ((which,) if which == "Position" else ("Position_shape_sample", "Axis_Direction", "q")):
        masks[k][:] = False
    box = MeasureIABox(data, None, None, None, [0.1, 10.0], 6, 4, 10.0, boxsize=100.0)
    with pytest.raises(ValueError, match="empty position or shape sample"):
        box.measure_xi_w("a", "both", 0, temp_file_path="/tmp", masks=masks)


def test_mixed_form_hands_nan_axes_to_fp64(monkeypatch):
    """A non-finite Axis_Direction: the mixed form's FP32 terms would not give
    the reference's e+ = ex = 0, so the measurement runs in the FP64 form,
    with a warning (the counter itself is replaced here: no GPU)."""
    import warnings
    from measure_ia_gb300 import measure_ia as M
    seen = []

    class Stop(Exception):
        pass

    class FakeCounter:
        def __init__(self, kind, **kw):
            seen.append(kw["precision"])
            raise Stop()

    monkeypatch.setattr(M, "PairCounter", FakeCounter)
    rng = np.random.default_rng(0)
    n = 100
    pos = rng.uniform(0, 100.0, (n, 3))
    ang = rng.uniform(0, np.pi, n)
    ax = np.c_[np.cos(ang), np.sin(ang)]
    data = {"Position": pos, "Position_shape_sample": pos.copy(), "Axis_Direction": ax, "q": rng.uniform(0.2, 1, n),
            "LOS": 2, "weight": np.ones(n), "weight_shape_sample": np.ones(n)}
    for bad, want in ((False, "mixed"), (True, "fp64")):
        d = dict(data, Axis_Direction=ax.copy())
        if bad:
            d["Axis_Direction"][7] = np.nan
        box = M.MeasureIABox(d, None, None, None, [0.1, 10.0], 6, 4, 10.0, boxsize=100.0, precision="mixed")
        with warnings.catch_warnings(record=True) as w:
            warnings.simplefilter("always")
            with pytest.raises(Stop):
                box.measure_xi_w("a", "both", 0, temp_file_path="/tmp")
        assert seen[-1] == want
        assert any("Axis_Direction" in str(x.message) for x in w) == bad


def _header_structs():
    """Field (name, kind) lists of the header's typedef structs, kind one of
    pointer / int / int64 / double."""
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "measure_ia_gb300.h")
    text = re.sub(r"/\*.*?\*/", " ", open(path).read(), flags=re.S)
    scalar = {"int": "int", "int64_t": "int64", "double": "double"}
    out = {}
    for body, name in re.findall(r"typedef struct\s*\{(.*?)\}\s*(\w+)\s*;", text, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = re.sub(r"\s+", " ", decl).strip()
            if not decl:
                continue
            # "<type words>[*] name, [*]name, ...": the type ends before the first declarator
            m = re.match(r"((?:const |unsigned |long )*\w+)(\s*\*)?\s*(.*)", decl)
            base, star, rest = m.group(1), bool(m.group(2)), m.group(3)
            for item in rest.split(","):
                item = item.strip()
                ptr = star or item.startswith("*")
                fields.append((item.lstrip("*").strip(), "pointer" if ptr else scalar[base.split()[-1]]))
        out[name] = fields
    return out


def test_ctypes_structs_mirror_the_header():
    """Every C-ABI struct the package passes by pointer has the header's
    fields, in the header's order, with the same kinds."""
    import ctypes as C
    from measure_ia_gb300 import _lib as L
    hdr = _header_structs()

    def kind(t):
        if t is C.c_void_p or (isinstance(t, type) and issubclass(t, C._Pointer)):
            return "pointer"
        return {C.c_int: "int", C.c_int64: "int64", C.c_double: "double"}[t]

    for cname, cls in (("mia_catalog", L.Catalog), ("mia_config", L.Config), ("mia_layout", L.Layout),
                       ("mia_result", L.Result), ("mia_lc_config", L.LcConfig), ("mia_lc_sample", L.LcSample)):
        want = hdr[cname]
        got = [(n, kind(t)) for n, t in cls._fields_]
        assert got == want, (cname, [x for x in zip(got, want) if x[0] != x[1]][:3], len(got), len(want))


def test_reference_base_helpers():
    """The public helpers of the reference's base classes on both drop-in
    classes (measure_IA_base.py:186-402), against closed forms."""
    from measure_ia_gb300 import MeasureIABox, MeasureIALightcone
    from measure_ia_gb300.sim_info import SimInfo
    box = MeasureIABox(None, None, None, None, boxsize=100.0)
    lc_cls = MeasureIALightcone
    rng = np.random.default_rng(5)
    a, b = rng.normal(size=(7, 3)), rng.normal(size=(7, 3))
    np.testing.assert_allclose(box.calculate_dot_product_arrays(a, b), np.einsum("ij,ij->i", a, b), rtol=1e-14)
    e, phi = rng.uniform(0, 1, 5), rng.uniform(0, np.pi, 5)
    ep, ex = lc_cls.get_ellipticity(e, phi)
    np.testing.assert_allclose(ep ** 2 + ex ** 2, e ** 2, rtol=1e-12)
    # analytic random pairs: cylinder shell over the box; 'auto' counts a pair once
    L3, n_p, n_s = 1e6, 1000, 400
    cross = box.get_random_pairs(2.0, 1.0, 5.0, -5.0, L3, "cross", n_p, n_s)
    assert np.isclose(cross, n_p * n_s * np.pi * 3.0 * 10.0 / L3)
    assert np.isclose(box.get_random_pairs(2.0, 1.0, 5.0, -5.0, L3, "auto", n_p, n_s), cross * (n_p - 1) / (2 * n_p))
    with pytest.raises(ValueError, match="auto or cross"):
        box.get_random_pairs(2.0, 1.0, 5.0, -5.0, L3, "nope", n_p, n_s)
    # caps: mu = -1 is the whole sphere, mu = 1 nothing; over mu in [-1, 1] the
    # (r, mu) count is the spherical shell's
    assert np.isclose(box.get_volume_spherical_cap(-1.0, 3.0), 4.0 / 3.0 * np.pi * 27.0)
    assert box.get_volume_spherical_cap(1.0, 3.0) == 0.0
    shell = 4.0 / 3.0 * np.pi * (3.0 ** 3 - 1.0 ** 3)
    assert np.isclose(box.get_random_pairs_r_mur(3.0, 1.0, 1.0, -1.0, L3, "cross", n_p, n_s),
                      (n_p - 1.0) * n_s * shell / L3)
    assert np.isclose(box.get_random_pairs_r_mur(3.0, 1.0, 1.0, -1.0, L3, "auto", n_p, n_s),
                      (n_p - 1.0) / 2.0 * n_s * shell / L3)
    # row-wise set differences
    d = box.setdiff2D([[1, 2, 3], [4, 5]], [[2], [4, 5]])
    assert [list(x) for x in d] == [[1, 3], []]
    d = box.setdiff_omit([[1, 2, 3], [4, 5], [6]], [2, 6], [0, 2])
    assert [list(x) for x in d] == [[1, 3], []]
    with pytest.raises(AssertionError):
        box.setdiff2D([[1]], [[1], [2]])
    # SimInfo.get_specs
    s = SimInfo("TNG100", 99)
    s.boxsize = None
    s.get_specs()
    assert s.boxsize == 75.0 and s.h == 0.6774
    for name in ("measure_covariance_multiple_datasets", "create_full_cov_matrix_projections",
                 "assign_jackknife_patches", "get_random_pairs_r_mur"):
        assert callable(getattr(lc_cls, name)) and callable(getattr(MeasureIABox, name))
