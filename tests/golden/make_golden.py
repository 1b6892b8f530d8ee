"""Generate the golden fixtures in this folder.

Runs only where the reference sources exist (the build host), never on the
GPU host and never from the test suite.  Two kinds of fixture:

1. ``ref_<case>.npz`` -- the reference's own ``MeasureIABox.measure_xi_w`` /
   ``measure_xi_multipoles`` run on small seeded catalogues.  The reference
   is imported from ``$MIA_REFERENCE_ROOT/src`` with stand-ins for modules that
   are absent here and unused by the box path (kmeans_radec, astropy,
   pathos, pyccl), an in-memory replacement for h5py, and ``lpmn`` mapped to
   ``scipy.special.assoc_legendre_p`` (scipy 1.18 removed ``lpmn``).  Each
   file stores the inputs (``in/<key>``), the call parameters (``meta``) and
   every dataset the reference wrote (``out/<hdf5 path>``).  Integer pair
   counts come from a second reference run with unit weights
   (``cnt/<path>`` = that run's DD datasets).

2. ``tng300_mock_outputs.npz`` -- every dataset of the reference's golden
   output files ``tests/data/processed/TNG300/mock_IA_TNG300*.hdf5``, read
   with the minimal HDF5 reader in ``h5read.py``.

3. ``crosscov_los3.npz`` -- three line-of-sight projections of one catalogue
   measured by the reference, then its cross-dataset jackknife covariance
   functions on that output (``run_crosscov``).

4. ``lc_<case>.npz`` -- the reference's ``MeasureIALightcone.measure_xi_w`` /
   ``measure_xi_multipoles`` on small seeded lightcone catalogues with
   randoms and jackknife patches (``run_lightcone``).  pyccl is replaced by a
   module whose ``comoving_radial_distance`` is the package's ``FlatLCDM``;
   the distances it returned are stored (``chi/z``, ``chi/chi``) so that tests
   replay them exactly.  pathos's pool is replaced by a serial map (the
   pooled realisation driver runs unchanged, one patch after another).

Usage:  MIA_REFERENCE_ROOT=<reference checkout> python tests/golden/make_golden.py
"""

from __future__ import annotations

import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference's source tree (MarloesvL/measure_IA), e.g. a clone of it
REF = os.environ.get("MIA_REFERENCE_ROOT", "")
sys.path.insert(0, os.path.join(HERE, "..", ".."))


# --------------------------------------------------------------------------
# Import shims for the reference
# --------------------------------------------------------------------------

class _Dataset:
    """A stored array; like h5py, reading it (``ds[:]``, ``np.asarray(ds)``)
    returns a copy, so in-place arithmetic on what was read leaves the file
    unchanged."""

    def __init__(self, v):
        self.v = np.array(v)

    def __getitem__(self, key):
        return np.array(self.v[key])

    def __array__(self, dtype=None, copy=None):
        return np.array(self.v, dtype=dtype)

    def __len__(self):
        return len(self.v)

    @property
    def shape(self):
        return self.v.shape


class _Group(dict):
    def _walk(self, path, create=False):
        node = self
        for part in [p for p in path.split("/") if p]:
            if part not in node:
                if not create:
                    raise KeyError(path)
                dict.__setitem__(node, part, _Group())
            node = dict.__getitem__(node, part)
        return node

    def __getitem__(self, k):
        return self._walk(k)

    def __delitem__(self, k):
        parts = [p for p in k.split("/") if p]
        dict.__delitem__(self._walk("/".join(parts[:-1])), parts[-1])

    def create_group(self, k):
        return self._walk(k, create=True)

    def create_dataset(self, k, data=None, **kw):
        parts = [p for p in k.split("/") if p]
        g = self._walk("/".join(parts[:-1]), create=True)
        dict.__setitem__(g, parts[-1], _Dataset(np.asarray(data)))
        return dict.__getitem__(g, parts[-1])

    def keys(self):
        return dict.keys(self)

    def close(self):
        pass


_FILES: dict = {}


class _File(_Group):
    def __new__(cls, name, mode="r"):
        if mode == "w" or name not in _FILES:
            _FILES[name] = _Group()
            open(name, "a").close()  # the reference deletes its temp file afterwards
        return _FILES[name]

    def __init__(self, *a, **k):
        pass


class _SerialPool:
    def __init__(self, nodes=1):
        pass

    def map(self, f, *its):
        return list(map(f, *its))


_CHI_SEEN: dict = {}


def _ccl_cosmology(Omega_c=0.225, Omega_b=0.045, h=0.7, **_):
    from measure_ia_gb300.cosmology import FlatLCDM
    return FlatLCDM(Omega_c=Omega_c, Omega_b=Omega_b, h=h)


def _ccl_distance(cosmo, a):
    chi = cosmo.comoving_radial_distance(a)
    for x, c in zip(np.ravel(a), np.ravel(chi)):
        _CHI_SEEN[float(x)] = float(c)
    return chi


def install_shims():
    sys.modules["kmeans_radec"] = types.SimpleNamespace(kmeans_sample=None)
    astro = types.ModuleType("astropy")
    cosmo = types.ModuleType("astropy.cosmology")
    cosmo.LambdaCDM = lambda **k: None
    astro.cosmology = cosmo
    sys.modules["astropy"] = astro
    sys.modules["astropy.cosmology"] = cosmo
    pth = types.ModuleType("pathos")
    pm = types.ModuleType("pathos.multiprocessing")
    pm.ProcessingPool = _SerialPool
    pth.multiprocessing = pm
    sys.modules["pathos"] = pth
    sys.modules["pathos.multiprocessing"] = pm
    ccl = types.ModuleType("pyccl")
    ccl.Cosmology = _ccl_cosmology
    ccl.comoving_radial_distance = _ccl_distance
    sys.modules["pyccl"] = ccl
    h5 = types.ModuleType("h5py")
    h5.File = _File
    sys.modules["h5py"] = h5
    import scipy.special as ss
    if not hasattr(ss, "lpmn"):
        def lpmn(m, n, z):
            out = np.zeros((m + 1, n + 1))
            out[m, n] = float(np.squeeze(ss.assoc_legendre_p(n, m, z)))
            return out, None
        ss.lpmn = lpmn
    sys.path.insert(0, os.path.join(REF, "src"))


def walk(g, prefix=""):
    for k in g.keys():
        v = dict.__getitem__(g, k)
        p = f"{prefix}/{k}" if prefix else k
        if isinstance(v, _Group):
            yield from walk(v, p)
        else:
            yield p, np.asarray(v)


# --------------------------------------------------------------------------
# Cases
# --------------------------------------------------------------------------

def uniform_case(seed, n, L):
    from measure_ia_gb300.catalogs import uniform_catalog
    return uniform_catalog(n, L, seed)


def clustered_case(seed, n_centres, L, n_shape, mean_children=10, sigma=1.0):
    from measure_ia_gb300.catalogs import neyman_scott_catalog
    return neyman_scott_catalog(n_centres, L, n_shape, seed, mean_children=mean_children, sigma=sigma)


def edge_case(seed, L):
    """Uniform points plus pairs placed exactly on r_min, r_max, r-bin edges,
    Pi-bin edges and jackknife faces, and points at coordinate 0."""
    from measure_ia_gb300.catalogs import uniform_catalog, inject_edge_pairs
    d = uniform_catalog(1500, L, seed)
    return inject_edge_pairs(d, L, seed + 1, r_edges=np.logspace(-1, np.log10(20.0), 11),
                             pi_edges=np.linspace(-20.0, 20.0, 9), n_sub=3)


CASES = {
    # name: (catalogue builder, MeasureIABox kwargs, calls)
    "w_jk27_mp": (lambda: uniform_case(11, 2500, 205.0),
                  dict(simulation=None, snapshot=None, separation_limits=[0.1, 20.0], num_bins_r=10,
                       num_bins_pi=8, pi_max=20.0, boxsize=205.0, num_nodes=2),
                  [("w", "All", "both", 27, "tmp")]),
    "m_jk27_mp": (lambda: uniform_case(12, 2500, 205.0),
                  dict(simulation=None, snapshot=None, separation_limits=[0.1, 20.0], num_bins_r=10,
                       num_bins_pi=20, pi_max=20.0, boxsize=205.0, num_nodes=2),
                  [("m", "All", "both", 27, "tmp")]),
    "w_clustered_jk27": (lambda: clustered_case(13, 300, 205.0, 1800),
                         dict(simulation=None, snapshot=None, separation_limits=[0.1, 20.0], num_bins_r=10,
                              num_bins_pi=8, pi_max=20.0, boxsize=205.0, num_nodes=2),
                         [("w", "clu", "both", 27, "tmp")]),
    "m_clustered_jk27": (lambda: clustered_case(14, 300, 205.0, 1800),
                         dict(simulation=None, snapshot=None, separation_limits=[0.1, 20.0], num_bins_r=10,
                              num_bins_pi=20, pi_max=20.0, boxsize=205.0, num_nodes=2),
                         [("m", "clu", "both", 27, "tmp")]),
    "w_tng_default_jk8": (lambda: uniform_case(15, 2000, 205.0),
                          dict(simulation="TNG300", snapshot=99, separation_limits=[0.1, 20.0], num_bins_r=10,
                               num_bins_pi=8, pi_max=None, num_nodes=1),
                          [("w", "All", "both", 8, "tmp"), ("m", "All", "both", 8, "tmp")]),
    "w_nojk_tree": (lambda: uniform_case(16, 2500, 150.0),
                    dict(simulation=None, snapshot=3, separation_limits=[0.2, 15.0], num_bins_r=7,
                         num_bins_pi=6, pi_max=15.0, boxsize=150.0, num_nodes=1),
                    [("w", "nojk", "both", 0, "tmp"), ("m", "nojk", "g+", 0, "tmp")]),
    "w_brute_jk8": (lambda: uniform_case(17, 1200, 100.0),
                    dict(simulation=None, snapshot=None, separation_limits=[0.1, 20.0], num_bins_r=10,
                         num_bins_pi=8, pi_max=20.0, boxsize=100.0, num_nodes=1),
                    [("w", "br", "both", 8, False), ("m", "br", "gg", 8, False)]),
    "edges_jk27": (lambda: edge_case(18, 205.0),
                   dict(simulation=None, snapshot=None, separation_limits=[0.1, 20.0], num_bins_r=10,
                        num_bins_pi=8, pi_max=20.0, boxsize=205.0, num_nodes=2),
                   [("w", "edge", "both", 27, "tmp"), ("m", "edge", "both", 27, "tmp")]),
    "los0_ellipticity": (lambda: clustered_case(19, 250, 120.0, 1500),
                         dict(simulation=None, snapshot=None, separation_limits=[0.1, 20.0], num_bins_r=10,
                              num_bins_pi=8, pi_max=20.0, boxsize=120.0, num_nodes=2),
                         [("w", "l0", "both", 8, "tmp", dict(ellipticity="ellipticity", los=0)),
                          ("m", "l0", "both", 8, "tmp", dict(ellipticity="ellipticity", los=0))]),
    "masks_jk8": (lambda: clustered_case(20, 250, 205.0, 2000),
                  dict(simulation=None, snapshot=None, separation_limits=[0.1, 20.0], num_bins_r=10,
                       num_bins_pi=8, pi_max=20.0, boxsize=205.0, num_nodes=2),
                  [("w", "msk", "both", 8, "tmp", dict(mask="quirk")),
                   ("w", "mskw", "both", 8, "tmp", dict(mask="full"))]),
}


def _masks(data, kind):
    rng = np.random.default_rng(99)
    sel_p = rng.uniform(size=len(data["Position"])) < 0.6
    sel_s = rng.uniform(size=len(data["Position_shape_sample"])) < 0.6
    masks = {"Position": sel_p, "Position_shape_sample": sel_s, "Axis_Direction": sel_s, "q": sel_s}
    if kind == "full":
        masks["weight"] = sel_p
        masks["weight_shape_sample"] = sel_s
    return masks


def run_case(name, builder, kw, calls):
    from measureia import MeasureIABox
    base = builder()
    arrays = {}
    meta = {"kwargs": kw, "calls": []}
    for key in ("Position", "Position_shape_sample", "Axis_Direction", "q", "weight", "weight_shape_sample"):
        if key in base:
            arrays[f"in/{key}"] = np.asarray(base[key])
    outfile = f"/tmp/golden_{name}.hdf5"
    cntfile = f"/tmp/golden_{name}_cnt.hdf5"
    _FILES.pop(outfile, None)
    _FILES.pop(cntfile, None)
    for call in calls:
        kind, dname, corr, num_jk, tmp = call[:5]
        extra = call[5] if len(call) > 5 else {}
        los = extra.get("los", 2)
        ell = extra.get("ellipticity", "distortion")
        mkind = extra.get("mask")
        meta["calls"].append(dict(kind=kind, dataset=dname, corr_type=corr, num_jk=num_jk,
                                  temp=(tmp if tmp is False else "path"), los=los, ellipticity=ell, mask=mkind))
        for weighted, fname in ((True, outfile), (False, cntfile)):
            data = {k: np.array(v) for k, v in base.items()}
            data["LOS"] = los
            if not weighted:
                data["weight"] = np.ones(len(data["Position"]))
                data["weight_shape_sample"] = np.ones(len(data["Position_shape_sample"]))
            masks = _masks(data, mkind) if mkind else None
            box = MeasureIABox(data, fname, **kw)
            tpath = "/tmp" if tmp == "tmp" else False
            if kind == "w":
                box.measure_xi_w(dname, corr, num_jk, temp_file_path=tpath, masks=masks, ellipticity=ell)
            else:
                box.measure_xi_multipoles(dname, corr, num_jk, temp_file_path=tpath, masks=masks, ellipticity=ell)
    for p, v in walk(_FILES[outfile]):
        arrays[f"out/{p}"] = np.asarray(v)
    for p, v in walk(_FILES[cntfile]):
        if p.endswith("_DD"):
            arrays[f"cnt/{p}"] = np.rint(np.asarray(v)).astype(np.int64)
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **arrays)
    print(name, "datasets:", sum(1 for k in arrays if k.startswith("out/")))


def run_crosscov():
    """Cross-dataset jackknife covariance: three projections (LOS = 0, 1, 2) of
    one clustered catalogue measured by the reference (w, jk8, multiprocessing
    backend), then the reference's own
    ``MeasureJackknife.measure_covariance_multiple_datasets`` and
    ``create_full_cov_matrix_projections`` (measure_jackknife.py:485-652) on
    that output, called on the box object (they use only the output file,
    ``snap_group`` and ``num_bins_r``).  Returned arrays go to ``res/...``."""
    from measureia import MeasureIABox
    from measureia.measure_jackknife import MeasureJackknife
    base = clustered_case(21, 250, 205.0, 2000)
    kw = dict(simulation=None, snapshot=None, separation_limits=[0.1, 20.0], num_bins_r=10, num_bins_pi=8,
              pi_max=20.0, boxsize=205.0, num_nodes=2)
    outfile = "/tmp/golden_crosscov.hdf5"
    _FILES.pop(outfile, None)
    names = ["LOS_x", "LOS_y", "LOS_z"]
    arrays = {f"in/{k}": np.asarray(v) for k, v in base.items() if k != "LOS"}
    box = None
    for los, dname in enumerate(names):
        data = {k: np.array(v) for k, v in base.items()}
        data["LOS"] = los
        box = MeasureIABox(data, outfile, **kw)
        box.measure_xi_w(dname, "both", 8, temp_file_path="/tmp")
    # the reference's methods, bound to the box (create_full_cov_matrix_projections calls the other on self)
    box.measure_covariance_multiple_datasets = types.MethodType(
        MeasureJackknife.measure_covariance_multiple_datasets, box)
    for ct in ("w_g_plus", "w_gg"):
        c, sd = MeasureJackknife.measure_covariance_multiple_datasets(box, ct, ["LOS_y"], num_box=8, return_output=True)
        arrays[f"res/{ct}/single_cov"], arrays[f"res/{ct}/single_std"] = c, sd
        c, sd = MeasureJackknife.measure_covariance_multiple_datasets(box, ct, ["LOS_x", "LOS_z"], num_box=8,
                                                                      return_output=True)
        arrays[f"res/{ct}/pair_cov"], arrays[f"res/{ct}/pair_std"] = c, sd
        MeasureJackknife.measure_covariance_multiple_datasets(box, ct, ["LOS_z"], num_box=8)
        full = MeasureJackknife.create_full_cov_matrix_projections(box, ct, names, num_box=8, return_output=True)
        for tag, m in zip(("cov3", "cov2xy", "cov2xz", "cov2yz"), full):
            arrays[f"res/{ct}/{tag}"] = m
        MeasureJackknife.create_full_cov_matrix_projections(box, ct, names, num_box=8)
    for p, v in walk(_FILES[outfile]):
        arrays[f"out/{p}"] = np.asarray(v)
    meta = {"kwargs": kw, "names": names, "num_jk": 8, "seed": 21}
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "crosscov_los3.npz"), **arrays)
    print("crosscov datasets:", sum(1 for k in arrays if k.startswith("out/")))


def lightcone_catalogue(seed, n_pos, n_shape, n_rand, n_rand_shape=None, ra=(10.0, 40.0), dec=(-10.0, 10.0),
                        z=(0.1, 0.3), weights=False):
    """Clustered points in an RA/DEC/z window, shapes a subset of the
    positions, uniform randoms (one sample, or separate position and shape
    randoms), and RA-stripe jackknife patches 0..3."""
    rng = np.random.default_rng(seed)
    n_par = max(4, n_pos // 20)
    cen = np.c_[rng.uniform(*ra, n_par), rng.uniform(*dec, n_par), rng.uniform(*z, n_par)]
    pick = rng.integers(0, n_par, n_pos)
    RA = cen[pick, 0] + rng.normal(0.0, 0.15, n_pos)
    DEC = cen[pick, 1] + rng.normal(0.0, 0.15, n_pos)
    Z = np.abs(cen[pick, 2] + rng.normal(0.0, 0.002, n_pos))
    sh = np.sort(rng.choice(n_pos, n_shape, replace=False))
    eps = rng.uniform(0.0, 0.6, n_shape)
    ang = rng.uniform(0.0, np.pi, n_shape)
    data = {"RA": RA, "DEC": DEC, "Redshift": Z, "RA_shape_sample": RA[sh], "DEC_shape_sample": DEC[sh],
            "Redshift_shape_sample": Z[sh], "e1": eps * np.cos(2 * ang), "e2": eps * np.sin(2 * ang)}
    if weights:
        data["weight"] = np.exp(rng.normal(0.0, 0.3, n_pos))
        data["weight_shape_sample"] = data["weight"][sh]
    rnd = {"RA": rng.uniform(*ra, n_rand), "DEC": rng.uniform(*dec, n_rand), "Redshift": rng.uniform(*z, n_rand)}
    if n_rand_shape:
        rnd.update(RA_shape_sample=rng.uniform(*ra, n_rand_shape), DEC_shape_sample=rng.uniform(*dec, n_rand_shape),
                   Redshift_shape_sample=rng.uniform(*z, n_rand_shape))
    stripe = lambda x: np.clip(np.floor((x - ra[0]) / ((ra[1] - ra[0]) / 4)), 0, 3).astype(int)
    patches = {"position": stripe(data["RA"]), "shape": stripe(data["RA_shape_sample"])}
    if n_rand_shape:
        patches.update(randoms_position=stripe(rnd["RA"]), randoms_shape=stripe(rnd["RA_shape_sample"]))
    else:
        patches["randoms"] = stripe(rnd["RA"])
    return data, rnd, patches


LC_CASES = {
    # name: (kind, estimator, corr_type, catalogue kwargs, call kwargs, binning)
    "w_clusters_both": ("w", "clusters", "both", dict(seed=31, n_pos=500, n_shape=300, n_rand=900), {},
                        dict(separation_limits=[0.3, 25.0], num_bins_r=6, num_bins_pi=5, pi_max=30.0)),
    "w_galaxies_gplus_overh": ("w", "galaxies", "g+", dict(seed=32, n_pos=450, n_shape=250, n_rand=700,
                                                           n_rand_shape=500, weights=True),
                               dict(over_h=True, cosmology=dict(Omega_c=0.25, Omega_b=0.05, h=0.68)),
                               dict(separation_limits=[0.2, 15.0], num_bins_r=5, num_bins_pi=4, pi_max=20.0)),
    "w_clusters_gg": ("w", "clusters", "gg", dict(seed=33, n_pos=400, n_shape=400, n_rand=800),
                      dict(measure_cov=False),
                      dict(separation_limits=[0.5, 30.0], num_bins_r=7, num_bins_pi=6, pi_max=40.0)),
    "w_galaxies_both_nocov": ("w", "galaxies", "both", dict(seed=34, n_pos=400, n_shape=300, n_rand=600),
                              dict(measure_cov=False),
                              dict(separation_limits=[0.3, 20.0], num_bins_r=6, num_bins_pi=6, pi_max=25.0)),
    "m_clusters_both": ("m", "clusters", "both", dict(seed=35, n_pos=500, n_shape=300, n_rand=900), {},
                        dict(separation_limits=[0.3, 25.0], num_bins_r=6, num_bins_pi=8, pi_max=30.0)),
    "m_galaxies_gg_rpcut": ("m", "galaxies", "gg", dict(seed=36, n_pos=450, n_shape=350, n_rand=800,
                                                        n_rand_shape=600, weights=True),
                            dict(rp_cut=1.0, over_h=True, measure_cov=False),
                            dict(separation_limits=[0.4, 20.0], num_bins_r=5, num_bins_pi=6, pi_max=20.0)),
    "m_galaxies_gplus": ("m", "galaxies", "g+", dict(seed=37, n_pos=400, n_shape=250, n_rand=700), {},
                         dict(separation_limits=[0.3, 18.0], num_bins_r=6, num_bins_pi=10, pi_max=20.0)),
    # masks: the reference applies the data's masks to the randoms' arrays too, so
    # randoms and data have the same lengths here (shape sample = position sample)
    "w_clusters_both_masks": ("w", "clusters", "both", dict(seed=38, n_pos=500, n_shape=500, n_rand=500,
                                                            weights=True), dict(masks=True),
                              dict(separation_limits=[0.3, 25.0], num_bins_r=6, num_bins_pi=5, pi_max=30.0)),
}


def lightcone_masks(data, seed=99):
    rng = np.random.default_rng(seed)
    mp = rng.uniform(size=len(data["RA"])) < 0.75
    ms = rng.uniform(size=len(data["RA_shape_sample"])) < 0.75
    m = {k: mp for k in ("Redshift", "RA", "DEC", "weight")}
    m.update({k: ms for k in ("Redshift_shape_sample", "RA_shape_sample", "DEC_shape_sample", "e1", "e2",
                              "weight_shape_sample")})
    return m


def run_lightcone(name):
    """One lightcone case through the reference's MeasureIALightcone with
    num_nodes = 2 (the pooled realisation driver; the serial one,
    num_nodes = 1, passes its arguments out of order and raises)."""
    from measureia.measure_IA import MeasureIALightcone
    kind, est, corr, ckw, call, bkw = LC_CASES[name]
    data, rnd, patches = lightcone_catalogue(**ckw)
    arrays = {f"in/{k}": np.asarray(v) for k, v in data.items()}
    arrays.update({f"rnd/{k}": np.asarray(v) for k, v in rnd.items()})
    arrays.update({f"jk/{k}": np.asarray(v) for k, v in patches.items()})
    outfile = f"/tmp/golden_lc_{name}.hdf5"
    _FILES.pop(outfile, None)
    _CHI_SEEN.clear()
    call = dict(call)
    cosmo_kw = call.pop("cosmology", None)
    cosmology = _ccl_cosmology(**cosmo_kw) if cosmo_kw else None
    measure_cov = call.pop("measure_cov", True)
    if call.pop("masks", False):
        call["masks"] = lightcone_masks(data)
    lc = MeasureIALightcone({k: np.array(v) for k, v in data.items()}, {k: np.array(v) for k, v in rnd.items()},
                            outfile, num_nodes=2, **bkw)
    jk = {k: np.array(v) for k, v in patches.items()} if measure_cov else None
    if kind == "w":
        lc.measure_xi_w(est, "lc", corr, jk_patches=jk, measure_cov=measure_cov, cosmology=cosmology, **call)
    else:
        lc.measure_xi_multipoles(est, "lc", corr, jk_patches=jk, calc_errors=measure_cov, cosmology=cosmology,
                                 **call)
    for p, v in walk(_FILES[outfile]):
        arrays[f"out/{p}"] = np.asarray(v)
    zs = np.array(sorted(_CHI_SEEN))
    arrays["chi/a"] = zs
    arrays["chi/chi"] = np.array([_CHI_SEEN[a] for a in zs])
    meta = {"kind": kind, "estimator": est, "corr_type": corr, "binning": bkw, "call": LC_CASES[name][4],
            "measure_cov": measure_cov}
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, f"lc_{name}.npz"), **arrays)
    print("lightcone", name, "datasets:", sum(1 for k in arrays if k.startswith("out/")))


def extract_reference_golden_files():
    from h5read import read_all
    out = {}
    for tag, fn in (("small", "mock_IA_TNG300.hdf5"), ("large", "mock_IA_TNG300_large.hdf5")):
        for path, arr in read_all(os.path.join(REF, "tests/data/processed/TNG300", fn)).items():
            out[f"{tag}/{path}"] = arr
    np.savez_compressed(os.path.join(HERE, "tng300_mock_outputs.npz"), **out)
    print("golden hdf5 datasets:", len(out))


if __name__ == "__main__":
    if not REF or not os.path.isdir(os.path.join(REF, "src", "measureia")):
        sys.exit("set MIA_REFERENCE_ROOT to a checkout of the reference (with src/measureia)")
    sys.path.insert(0, HERE)
    install_shims()
    import io, contextlib
    only = sys.argv[1:]
    if not only or "hdf5" in only:
        extract_reference_golden_files()
    for name, (builder, kw, calls) in CASES.items():
        if only and name not in only:
            continue
        with contextlib.redirect_stdout(io.StringIO()):
            run_case(name, builder, kw, calls)
        print("done", name)
    if not only or "crosscov" in only:
        with contextlib.redirect_stdout(io.StringIO()):
            run_crosscov()
        print("done crosscov")
    for name in LC_CASES:
        if only and name not in only and "lightcone" not in only:
            continue
        with contextlib.redirect_stdout(io.StringIO()):
            run_lightcone(name)
        print("done", name)
