"""Loading helpers for the fixtures in tests/golden."""

import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def reference_file(rel):
    """A file of the reference's source tree, found under the directory that
    ``MIA_REFERENCE_ROOT`` names; None when the variable is unset or the file
    is absent (tests that need it skip)."""
    root = os.environ.get("MIA_REFERENCE_ROOT")
    if not root:
        return None
    p = os.path.join(root, rel)
    return p if os.path.exists(p) else None


def case_names():
    return sorted(os.path.basename(p)[4:-4] for p in glob.glob(os.path.join(GOLDEN, "ref_*.npz")))


def load_case(name):
    z = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    meta = json.loads(bytes(z["meta"]).decode())
    inputs = {k[3:]: z[k] for k in z.files if k.startswith("in/")}
    outs = {k[4:]: z[k] for k in z.files if k.startswith("out/")}
    cnts = {k[4:]: z[k] for k in z.files if k.startswith("cnt/")}
    return meta, inputs, outs, cnts


def box_params(kw):
    """(boxsize, snapshot, r_min, r_max, n_r, n_pi, pi_max) from MeasureIABox kwargs."""
    sims = {"TNG300": 205.0}
    L = sims[kw["simulation"]] if kw.get("simulation") else kw["boxsize"]
    return dict(boxsize=L, snapshot=kw.get("snapshot"), r_min=kw["separation_limits"][0],
                r_max=kw["separation_limits"][1], num_bins_r=kw["num_bins_r"], num_bins_pi=kw["num_bins_pi"],
                pi_max=kw.get("pi_max"))


def layout_of(kw, call):
    if call["temp"] is False:
        return "brute"
    return "multiprocessing" if kw.get("num_nodes", 1) > 1 else "tree"


def masks_for(inputs, kind):
    """Recreates the masks make_golden.py used (same seed)."""
    rng = np.random.default_rng(99)
    sel_p = rng.uniform(size=len(inputs["Position"])) < 0.6
    sel_s = rng.uniform(size=len(inputs["Position_shape_sample"])) < 0.6
    m = {"Position": sel_p, "Position_shape_sample": sel_s, "Axis_Direction": sel_s, "q": sel_s}
    if kind == "full":
        m["weight"] = sel_p
        m["weight_shape_sample"] = sel_s
    return m


def assert_close(a, b, rtol, what=""):
    """|a-b| <= rtol*|b| + rtol*max|b|: relative per element, with the
    array's own scale as the floor for elements that cancel to ~0."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    scale = np.max(np.abs(b)) if b.size else 0.0
    err = np.abs(a - b)
    lim = rtol * np.abs(b) + rtol * scale
    bad = err > lim
    assert not np.any(bad), f"{what}: max err {err.max():.3e} (scale {scale:.3e}) at {np.argwhere(bad)[:3].tolist()}"


# ---- lightcone fixtures (lc_<case>.npz) ----------------------------------------

def lc_case_names():
    return sorted(os.path.basename(p)[3:-4] for p in glob.glob(os.path.join(GOLDEN, "lc_*.npz")))


class TableCosmology:
    """Replays the distances a fixture's reference run saw: chi(a) looked up
    by the exact float64 scale factor, h as given."""

    def __init__(self, a, chi, h):
        self.table = dict(zip(np.asarray(a, dtype=np.float64).tolist(), np.asarray(chi, dtype=np.float64).tolist()))
        self.h = h

    def __getitem__(self, key):
        if key == "h":
            return self.h
        raise KeyError(key)

    def comoving_radial_distance(self, a):
        a = np.asarray(a, dtype=np.float64)
        return np.array([self.table[x] for x in a.ravel().tolist()]).reshape(a.shape)


def load_lc_case(name):
    z = np.load(os.path.join(GOLDEN, f"lc_{name}.npz"))
    meta = json.loads(bytes(z["meta"]).decode())
    data = {k[3:]: z[k] for k in z.files if k.startswith("in/")}
    rnd = {k[4:]: z[k] for k in z.files if k.startswith("rnd/")}
    jk = {k[3:]: z[k] for k in z.files if k.startswith("jk/")}
    outs = {k[4:]: z[k] for k in z.files if k.startswith("out/")}
    ckw = meta["call"].get("cosmology")
    h = ckw["h"] if ckw else 0.7
    return meta, data, rnd, jk, outs, TableCosmology(z["chi/a"], z["chi/chi"], h)


def lc_masks(data, seed=99):
    """The masks make_golden.py used for a lightcone case with call['masks']."""
    rng = np.random.default_rng(seed)
    mp = rng.uniform(size=len(data["RA"])) < 0.75
    ms = rng.uniform(size=len(data["RA_shape_sample"])) < 0.75
    m = {k: mp for k in ("Redshift", "RA", "DEC", "weight")}
    m.update({k: ms for k in ("Redshift_shape_sample", "RA_shape_sample", "DEC_shape_sample", "e1", "e2",
                              "weight_shape_sample")})
    return m
