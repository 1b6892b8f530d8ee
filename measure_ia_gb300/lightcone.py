"""Lightcone measurements: MeasureIALightcone (measure_IA.py:265-1060).

The reference measures xi_g+ and xi_gg of lightcone data (RA, DEC, redshift)
against randoms, with four brute-force pair counters (S+D and S+R with
shapes; SD, SR, RD, RR counts only) and jackknife patches it re-counts one at
a time.  Here each counter is one call of the C ABI's ``mia_lc_count``, which
returns the full-sample sums and every patch realisation from one pass on the
GPU; the host keeps the reference's flow: input selection with its mask
behaviour, distances from the cosmology, the estimator
(``measure_IA_base.py:670-743``), the Pi integration / multipoles
(``measure_IA_base.py:515-668``) and the jackknife covariance
(``measure_jackknife.py:172-263``), all written under the reference's dataset
names.

Behaviour kept from the reference on purpose: empty DD bins are set to 1
before anything divides by them; the w counter with shapes clamps an index
equal to the bin count, the other counters raise IndexError instead; the
estimator uses '-1' for clusters and '+1' for galaxies in xi_gg; with
corr_type 'gg' and jackknife errors the reference stops with a KeyError
(its estimator opens the randoms realisation group that only the g+ flow
creates) after writing the full-sample products and the realisation counts,
and so does this class.  One difference: ``num_nodes = 1`` runs the same
one-pass realisations as ``num_nodes > 1`` (the reference's serial driver
passes its arguments out of order and raises TypeError), and writes the
pooled driver's datasets.
"""

from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L
from . import binning as B
from .base import BaseHelpers, JackknifeCovariance
from .cosmology import comoving_radial_distance, default_cosmology
from .output import norm_path, store_for


def _centres(edges):
    return edges[:-1] + abs((edges[1:] - edges[:-1]) / 2.0)


# ----------------------------------------------------------------------------
# one counter on the GPU
# ----------------------------------------------------------------------------

def _median_abs(a):
    """Median of |a| (1 for an empty array), over an evenly strided subsample
    of ~32k values for large arrays: it only sizes the cell grid."""
    a = np.asarray(a, dtype=np.float64)
    if not len(a):
        return 1.0
    if len(a) > (1 << 16):
        a = a[:: len(a) >> 15]
    return float(np.median(np.abs(a)))


class LightconeCounter:
    """One of the reference's four lightcone pair counters, with patch
    realisations, through ``mia_lc_count``."""

    # cells per window half-width along RA and DEC and per distance window,
    # from sweeps on the 1000 deg^2 / 1M-random workload
    CELL_DIV = {"w": (8.0, 3.0, 4.0), "m": (8.0, 3.0, 6.0)}

    def __init__(self, kind, with_shapes, r_bins, r_min, r_max, p_bins, h_extra=1.0, rp_cut=0.0, device=0,
                 cell_div=None):
        if kind not in ("w", "m"):
            raise ValueError(kind)
        if cell_div is None:
            cell_div = self.CELL_DIV[kind]
        self.kind, self.with_shapes, self.device = kind, bool(with_shapes), device
        self.n_r, self.n_p = len(r_bins) - 1, len(p_bins) - 1
        if self.n_r > L.MAX_BINS_R or self.n_p > L.MAX_BINS_P:
            raise ValueError(f"at most {L.MAX_BINS_R} r bins and {L.MAX_BINS_P} pi/mu bins are supported")
        clamp = kind == "w" and self.with_shapes
        self.q_table = B.lc_r_table(kind, np.asarray(r_bins, dtype=np.float64), r_min, r_max, self.n_r, clamp)
        if kind == "w":
            self.p_table = B.lc_pi_table(np.asarray(p_bins, dtype=np.float64), self.n_p, clamp)
        else:
            self.p_table = B.lc_mu_table(np.asarray(p_bins, dtype=np.float64), self.n_p)
        self._qb = np.ascontiguousarray(self.q_table.breaks, dtype=np.float64)
        self._qn = np.ascontiguousarray(self.q_table.bins, dtype=np.int32)
        self._pb = np.ascontiguousarray(self.p_table.breaks, dtype=np.float64)
        self._pn = np.ascontiguousarray(self.p_table.bins, dtype=np.int32)
        self.r_lim = float(r_bins[-1])
        self.pi_lo, self.pi_hi = (float(p_bins[0]), float(p_bins[-1])) if kind == "w" else (0.0, 0.0)
        self.h_extra = float(h_extra)
        self.rp_cut = float(rp_cut)
        # launch geometry (results do not depend on it): cells per separation
        # window half-width along RA, DEC and the comoving distance
        self.cell_div = tuple(float(x) for x in cell_div)

    def _grid(self, cfg, pos, shp):
        """Cells of 1/cell_div of the separation window's half-width (RA,
        DEC) and of the line-of-sight window (distance) at the median position
        distance, at most ~2^22 cells."""
        ra, dec, chi = shp["ra"], shp["dec"], shp["chi"]
        lo = np.array([ra.min(), dec.min(), chi.min()])
        hi = np.array([ra.max(), dec.max(), chi.max()])
        hx = self.h_extra if self.kind == "w" else 1.0
        chi_med = _median_abs(pos["chi"])
        cos_med = _median_abs(pos["cos_dec"])
        span = self.r_lim / max(hx * chi_med, 1e-12) / (np.pi / 180.0)
        chi_span = (self.pi_hi - self.pi_lo) if self.kind == "w" else 2.0 * self.r_lim
        dv = self.cell_div
        want = np.array([span / max(cos_med, 1e-3) / dv[0], span / dv[1], chi_span / dv[2]])
        ext = np.maximum(hi - lo, 1e-9)
        want = np.maximum(want, ext / 4096.0)
        n = np.maximum(1, np.ceil(ext / want)).astype(np.int64)
        while n.prod() > (1 << 22):
            n = np.maximum(1, n // 2)
        cell = ext / n * (1.0 + 1e-12)
        cfg.ra0, cfg.dec0, cfg.chi0 = (float(x) for x in lo)
        cfg.ra_cell, cfg.dec_cell, cfg.chi_cell = (float(x) for x in cell)
        cfg.n_ra, cfg.n_dec, cfg.n_chi = (int(x) for x in n)

    def _wide_sums(self, pos, shp):
        """128-bit warp partials when the smallest weight product is below
        2^-12 of the largest possible term: the 64-bit partials keep every
        bit of a term down to 2^-46 of that term only, too coarse for a bin
        that holds nothing but small-weight pairs."""
        wp, ws = np.abs(np.asarray(pos["w"], float)), np.abs(np.asarray(shp["w"], float))
        if not len(wp) or not len(ws):
            return False
        top = ws.max()
        if self.with_shapes and "e" in shp:
            top = max(top, float(np.max(np.abs(ws * np.asarray(shp["e"], float)))))
        big = wp.max() * top
        nzp, nzs = wp[wp > 0], ws[ws > 0]
        if not len(nzp) or not len(nzs) or not (big > 0):
            return False
        return bool(nzp.min() * nzs.min() < big * 2.0 ** -12)

    def prepare(self, pos, shp, n_patch=0):
        """Upload one pair of samples and size the launch: pos holds ra, dec,
        chi, w, cos_dec (and patch); shp holds ra, dec, chi, w (and e, c2a,
        s2a with shapes; patch).  Host float64 arrays."""
        import torch
        dev = torch.device("cuda", self.device)
        cfg = L.LcConfig()
        cfg.kind = L.MIA_KIND_W if self.kind == "w" else L.MIA_KIND_MULTIPOLES
        cfg.with_shapes = int(self.with_shapes)
        cfg.n_r, cfg.n_p, cfg.n_patch = self.n_r, self.n_p, int(n_patch)
        cfg.n_qbreak, cfg.n_pbreak = len(self._qb), len(self._pb)
        cfg.q_break = self._qb.ctypes.data_as(C.POINTER(C.c_double))
        cfg.q_bin = self._qn.ctypes.data_as(C.POINTER(C.c_int))
        cfg.p_break = self._pb.ctypes.data_as(C.POINTER(C.c_double))
        cfg.p_bin = self._pn.ctypes.data_as(C.POINTER(C.c_int))
        cfg.h_extra, cfg.rp_cut, cfg.r_lim = self.h_extra, self.rp_cut, self.r_lim
        cfg.pi_lo, cfg.pi_hi = self.pi_lo, self.pi_hi
        n_pos, n_shp = len(pos["ra"]), len(shp["ra"])
        for k in ("ra", "dec", "chi", "w"):
            for smp in (pos, shp):
                if not np.all(np.isfinite(smp[k])):
                    raise ValueError(f"lightcone {k} values must be finite")
        cfg.unit_weights = int(bool(np.all(np.asarray(pos["w"]) == 1.0) and np.all(np.asarray(shp["w"]) == 1.0)))
        cfg.wide_sums = int(self._wide_sums(pos, shp))
        if n_shp:
            self._grid(cfg, pos, shp)
        else:
            cfg.ra0 = cfg.dec0 = cfg.chi0 = 0.0
            cfg.ra_cell = cfg.dec_cell = cfg.chi_cell = 1.0
            cfg.n_ra = cfg.n_dec = cfg.n_chi = 1
        keep = []

        def dptr(a, dtype=torch.float64):
            t = torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)
            keep.append(t)
            return t.data_ptr()

        sp = L.LcSample()
        sp.n = n_pos
        if n_pos:
            sp.ra, sp.dec, sp.chi, sp.w = (dptr(pos[k]) for k in ("ra", "dec", "chi", "w"))
            sp.cos_dec = dptr(pos["cos_dec"])
            if n_patch:
                sp.patch = dptr(pos["patch"], torch.int32)
        ss = L.LcSample()
        ss.n = n_shp
        if n_shp:
            ss.ra, ss.dec, ss.chi, ss.w = (dptr(shp[k]) for k in ("ra", "dec", "chi", "w"))
            if self.with_shapes:
                ss.e, ss.c2a, ss.s2a = (dptr(shp[k]) for k in ("e", "c2a", "s2a"))
            if n_patch:
                ss.patch = dptr(shp["patch"], torch.int32)
        lib = L.load()
        nbytes = C.c_size_t()
        rc = lib.mia_lc_workspace_size(C.byref(cfg), n_pos, n_shp, C.byref(nbytes))
        if rc != L.MIA_OK:
            raise L.MiaError(rc, "invalid lightcone configuration")
        Q = 3 if self.with_shapes else 1
        nb = self.n_r * self.n_p
        ws = torch.empty(nbytes.value + 256, dtype=torch.uint8, device=dev)
        base = ws.data_ptr()
        base += (-base) % 256
        job = _LcJob(cfg=cfg, pos=sp, shp=ss, keep=keep + [ws], ws=base, ws_bytes=nbytes.value, n_patch=int(n_patch),
                     Q=Q, h2d=sum(t.numel() * t.element_size() for t in keep))
        job.out = torch.empty(Q * (1 + n_patch) * nb, dtype=torch.float64, device=dev)
        job.cnt = torch.empty((1 + n_patch) * nb, dtype=torch.int64, device=dev)
        job.status = torch.zeros(1, dtype=torch.int32, device=dev)
        return job

    def run(self, job, stream=None):
        """Enqueue the count on ``stream`` (default: torch's current stream)."""
        import torch
        from .engine import context
        lib = L.load()
        ctx = context(self.device)
        if stream is None:
            stream = torch.cuda.current_stream(torch.device("cuda", self.device)).cuda_stream
        rc = lib.mia_lc_count(ctx, C.byref(job.cfg), C.byref(job.pos), C.byref(job.shp), C.c_void_p(job.ws),
                              job.ws_bytes, C.c_void_p(job.out.data_ptr()), C.c_void_p(job.cnt.data_ptr()),
                              C.c_void_p(job.status.data_ptr()), C.c_void_p(stream))
        if rc != L.MIA_OK:
            raise L.MiaError(rc, lib.mia_last_error(ctx).decode())

    def fetch(self, job):
        """(sums (Q, 1 + n_patch, n_r, n_p), counts (1 + n_patch, n_r, n_p))
        with Q = 3 (DD, S+D, SxD) or 1 (DD); raises what the reference raises."""
        sums = job.out.cpu().numpy().reshape(job.Q, 1 + job.n_patch, self.n_r, self.n_p)
        counts = job.cnt.cpu().numpy().reshape(1 + job.n_patch, self.n_r, self.n_p)
        flags = int(job.status.cpu().item())
        if flags & L.MIA_LC_BAD_PATCH:
            raise ValueError(f"jackknife patch labels must lie in 0..{job.n_patch - 1} (positions) or be -1 (shapes)")
        if flags & L.MIA_LC_INDEX_ERROR:
            n = self.n_r
            raise IndexError(f"index {n} is out of bounds for axis 0 with size {n}")
        return sums, counts

    def count(self, pos, shp, n_patch=0):
        """prepare + run + fetch."""
        job = self.prepare(pos, shp, n_patch)
        self.run(job)
        return self.fetch(job)


class _LcJob:
    def __init__(self, **kw):
        self.__dict__.update(kw)


# ----------------------------------------------------------------------------
# jackknife patches (assign_jackknife_patches, measure_IA_base.py:745-800)
# ----------------------------------------------------------------------------

def _unit(ra, dec):
    r, d = np.radians(ra), np.radians(dec)
    return np.c_[np.cos(d) * np.cos(r), np.cos(d) * np.sin(r), np.sin(d)]


class SkyKMeans:
    """k-means on the sphere (unit vectors, centres renormalised), seeded.
    The reference uses kmeans_radec (random initialisation, no seed); its
    labels cannot be reproduced, so this is a stand-in of the same kind."""

    def __init__(self, ra, dec, k, maxiter=100, tol=1.0e-5, seed=0):
        x = _unit(ra, dec)
        rng = np.random.default_rng(seed)
        c = x[rng.choice(len(x), 1)]
        for _ in range(1, k):           # k-means++ seeding
            d2 = np.min(((x[:, None, :] - c[None, :, :]) ** 2).sum(-1), axis=1)
            c = np.vstack([c, x[rng.choice(len(x), 1, p=d2 / d2.sum())]])
        for _ in range(maxiter):
            lab = self._nearest(x, c)
            new = np.array([x[lab == j].mean(axis=0) if np.any(lab == j) else c[j] for j in range(k)])
            new /= np.linalg.norm(new, axis=1)[:, None]
            shift = np.max(np.linalg.norm(new - c, axis=1))
            c = new
            if shift < tol:
                break
        self.centres = c
        self.labels = self._nearest(x, c)

    @staticmethod
    def _nearest(x, c):
        return np.argmax(x @ c.T, axis=1)

    def find_nearest(self, radec):
        radec = np.asarray(radec)
        return self._nearest(_unit(radec[:, 0], radec[:, 1]), self.centres)


def assign_jackknife_patches(data, randoms_data, num_jk):
    km = SkyKMeans(randoms_data["RA"], randoms_data["DEC"], num_jk)
    return {"randoms_position": km.labels,
            "randoms_shape": km.find_nearest(np.c_[randoms_data["RA_shape_sample"], randoms_data["DEC_shape_sample"]]),
            "position": km.find_nearest(np.c_[data["RA"], data["DEC"]]),
            "shape": km.find_nearest(np.c_[data["RA_shape_sample"], data["DEC_shape_sample"]])}


# ----------------------------------------------------------------------------
# the measurement class
# ----------------------------------------------------------------------------

_POS_KEYS = ("Redshift", "RA", "DEC", "weight")
_SHAPE_KEYS = ("Redshift_shape_sample", "RA_shape_sample", "DEC_shape_sample", "weight_shape_sample")


class MeasureIALightcone(BaseHelpers, JackknifeCovariance):
    """Drop-in for the reference's ``MeasureIALightcone``: same constructor,
    ``measure_xi_w`` and ``measure_xi_multipoles``, same datasets; the
    jackknife covariance methods and helpers of the reference's base classes."""

    def __init__(self, data, randoms_data, output_file_name, separation_limits=[0.1, 20.0], num_bins_r=8,
                 num_bins_pi=20, pi_max=None, num_nodes=1, device=0):
        self.data = data
        self.randoms_data = randoms_data
        self.output_file_name = output_file_name
        self.num_nodes = num_nodes
        self.device = device
        self.snap_group = ""
        try:
            self.Num_position = len(data["RA"])
            self.Num_shape = len(data["RA_shape_sample"])
        except Exception:
            self.Num_position = self.Num_shape = 0
        if self.Num_position > 0:
            if "weight" not in self.data:
                self.data["weight"] = np.ones(self.Num_position)
            if "weight_shape_sample" not in self.data:
                self.data["weight_shape_sample"] = np.ones(self.Num_shape)
        self.r_min, self.r_max = separation_limits[0], separation_limits[1]
        self.num_bins_r, self.num_bins_pi = num_bins_r, num_bins_pi
        self.r_bins = np.logspace(np.log10(self.r_min), np.log10(self.r_max), self.num_bins_r + 1)
        if pi_max is None:
            raise ValueError("Both pi_max and boxsize are None. Provide input on one of them to determine the "
                             "integration limit pi_max.")
        self.pi_max = pi_max
        self.pi_bins = np.linspace(-pi_max, pi_max, self.num_bins_pi + 1)
        self.mu_r_bins = np.linspace(-1, 1, self.num_bins_pi + 1)
        self.data_dir = None
        self.num_samples = None

    # ------------------------------------------------------------------ API
    def measure_xi_w(self, IA_estimator, dataset_name, corr_type, jk_patches=None, num_jk=None, measure_cov=True,
                     masks=None, masks_randoms=None, cosmology=None, over_h=False):
        """xi_gg, xi_g+ and w_gg, w_g+ of lightcone data with randoms, and the
        jackknife covariance (measure_IA.py:336-688)."""
        self._measure("w", IA_estimator, dataset_name, corr_type, jk_patches, num_jk, measure_cov, masks,
                      masks_randoms, cosmology, over_h, None)

    def measure_xi_multipoles(self, IA_estimator, dataset_name, corr_type, jk_patches=None, num_jk=None,
                              calc_errors=True, masks=None, masks_randoms=None, cosmology=None, over_h=False,
                              rp_cut=None):
        """Multipoles of xi_gg and xi_g+ of lightcone data with randoms, and
        the jackknife covariance (measure_IA.py:690-1060)."""
        self._measure("m", IA_estimator, dataset_name, corr_type, jk_patches, num_jk, calc_errors, masks,
                      masks_randoms, cosmology, over_h, rp_cut)

    assign_jackknife_patches = staticmethod(assign_jackknife_patches)

    # ------------------------------------------------------------------ flow
    def _measure(self, kind, est, d, corr_type, jk_patches, num_jk, measure_cov, masks, masks_randoms, cosmology,
                 over_h, rp_cut):
        if est == "clusters":
            if self.randoms_data is None:
                raise KeyError("This version does not work yet, add randoms.")
        elif est == "galaxies":
            if self.randoms_data is None:
                raise KeyError("No randoms given. Please provide input.")
        else:
            raise KeyError("Unknown input for IA_estimator, choose from [clusters, galaxies].")
        if corr_type not in ("g+", "gg", "both"):
            raise KeyError("Unknown value for corr_type. Choose from [g+, gg, both]")
        data, rnd = self.data, self.randoms_data
        one_random = "RA_shape_sample" not in rnd
        if one_random:
            rnd["RA_shape_sample"] = rnd["RA"]
            rnd["DEC_shape_sample"] = rnd["DEC"]
            rnd["Redshift_shape_sample"] = rnd["Redshift"]
        if "weight" not in rnd:
            rnd["weight"] = np.ones(len(rnd["RA"]))
        if "weight_shape_sample" not in rnd:
            rnd["weight_shape_sample"] = rnd["weight"] if one_random else np.ones(len(rnd["RA_shape_sample"]))
        if measure_cov:
            if jk_patches is None:
                if num_jk is None:
                    raise ValueError("Set calc_errors to False, or provide either jk_patches or num_jk input.")
                jk_patches = assign_jackknife_patches(data, rnd, num_jk)
            elif one_random:
                jk_patches["randoms_position"] = jk_patches["randoms"]
                jk_patches["randoms_shape"] = jk_patches["randoms"]
        self.data_dir = data
        if "weight" not in data:
            data["weight"] = np.ones(len(data["RA"]))
        if "weight_shape_sample" not in data:
            data["weight_shape_sample"] = np.ones(len(data["RA_shape_sample"]))
        ns = {"D": len(data["RA"]) if masks is None else len(data["RA"][masks["RA"]]),
              "S": len(data["RA_shape_sample"]) if masks is None else
              len(data["RA_shape_sample"][masks["RA_shape_sample"]]),
              "R_D": len(rnd["RA"]) if masks_randoms is None else len(rnd["RA"][masks_randoms["RA"]]),
              "R_S": len(rnd["RA_shape_sample"]) if masks_randoms is None else
              len(rnd["RA_shape_sample"][masks_randoms["RA_shape_sample"]])}
        if cosmology is None:
            cosmology = default_cosmology()
        h = cosmology["h"]
        chi = lambda z: comoving_radial_distance(cosmology, 1 / (1 + z)) * (h if over_h else 1.0)
        run = _Run(self, kind, est, d, corr_type, data, rnd, chi, h, over_h, rp_cut, masks, jk_patches if measure_cov
                   else None)
        store = store_for(self)
        try:
            run.full_and_realisations(ns)
        finally:
            run.write(store)
            if self.output_file_name is not None:
                store.flush()
        self.num_samples = run.nsj


class _Run:
    """One measure_xi_w / measure_xi_multipoles call."""

    def __init__(self, owner, kind, est, d, corr_type, data, rnd, chi, h, over_h, rp_cut, masks, jk):
        self.o, self.kind, self.est, self.d, self.corr = owner, kind, est, d, corr_type
        self.data, self.rnd, self.chi, self.h, self.over_h = data, rnd, chi, h, over_h
        self.rp_cut = 0.0 if rp_cut is None else rp_cut
        self.masks, self.jk = masks, jk
        self.top = "w" if kind == "w" else "multipoles"
        self.rs, self.ps = ("_rp", "_pi") if kind == "w" else ("_r", "_mu_r")
        self.rc = _centres(owner.r_bins)
        self.pc = _centres(owner.pi_bins if kind == "w" else owner.mu_r_bins)
        self.out = {}
        self.nsj = {}
        self._gs = set()          # every group that holds a stored dataset (path prefixes)
        self._chi_memo = []       # (redshift array, distances): unmasked samples recur across counters

    def put(self, path, v):
        p = norm_path(self.o.snap_group, path)
        self.out[p] = np.asarray(v)
        parts = p.split("/")
        for k in range(1, len(parts)):
            self._gs.add("/".join(parts[:k]))

    def _chi(self, z):
        """Distances of a redshift array, reused when the same array object
        comes back (the distance is element-wise, so a masked copy would get
        the same values; only the identical object is reused)."""
        for a, c in self._chi_memo:
            if a is z:
                return c
        c = self.chi(np.asarray(z, dtype=np.float64))
        self._chi_memo.append((z, c))
        return c

    def get(self, path):
        return self.out[norm_path(self.o.snap_group, path)]

    def write(self, store):
        for path, v in self.out.items():
            store.write("", path, v)

    # ---- inputs -------------------------------------------------------------
    def _combo(self, pos_from, shape_from, with_shapes):
        src = {"D": self.data, "R": self.rnd}
        p, s = src[pos_from], src[shape_from]
        out = {k: p[k] for k in _POS_KEYS}
        out.update({k: s[k] for k in _SHAPE_KEYS})
        if with_shapes:
            out["e1"], out["e2"] = s["e1"], s["e2"]
        return out

    def _select(self, combo, masks, with_shapes):
        """measure_w_lightcone.py:73-107 (the same in the other counters)."""
        keys = list(_POS_KEYS[:3]) + list(_SHAPE_KEYS[:3]) + (["e1", "e2"] if with_shapes else [])
        if masks is None:
            sel = {k: combo[k] for k in keys}
            sel["weight"], sel["weight_shape_sample"] = combo["weight"], combo["weight_shape_sample"]
            return sel
        sel = {k: combo[k][masks[k]] for k in keys}
        if "weight" not in masks:
            masks["weight"] = np.ones(self.o.Num_position, dtype=bool)
        if "weight_shape_sample" not in masks:
            masks["weight_shape_sample"] = np.ones(self.o.Num_shape, dtype=bool)
        sel["weight"] = combo["weight"][masks["weight"]]
        sel["weight_shape_sample"] = combo["weight_shape_sample"][masks["weight_shape_sample"]]
        return sel

    def _samples(self, sel, with_shapes, pos_patch=None, shape_patch=None):
        n_p, n_s = len(sel["RA"]), len(sel["RA_shape_sample"])
        w = np.asarray(sel["weight"], dtype=np.float64)
        ws = np.asarray(sel["weight_shape_sample"], dtype=np.float64)
        if len(w) < n_p:     # weight[n] for every position n of the loop
            raise IndexError(f"index {len(w)} is out of bounds for axis 0 with size {len(w)}")
        if len(ws) != n_s:   # weight_shape[mask] with a mask of the shape sample's length
            raise IndexError(f"boolean index did not match indexed array along axis 0; size of axis is {len(ws)} "
                             f"but size of corresponding boolean axis is {n_s}")
        dec = np.asarray(sel["DEC"], dtype=np.float64)
        pos = {"ra": np.asarray(sel["RA"], dtype=np.float64), "dec": dec,
               "chi": self._chi(sel["Redshift"]), "w": w[:n_p],
               "cos_dec": np.cos(dec / 180 * np.pi)}
        shp = {"ra": np.asarray(sel["RA_shape_sample"], dtype=np.float64),
               "dec": np.asarray(sel["DEC_shape_sample"], dtype=np.float64),
               "chi": self._chi(sel["Redshift_shape_sample"]), "w": ws}
        if with_shapes:
            e1, e2 = np.asarray(sel["e1"], dtype=np.float64), np.asarray(sel["e2"], dtype=np.float64)
            theta = 1. / 2 * np.arctan2(e2, e1)
            semi = np.array([np.cos(theta), np.sin(theta)])
            axis = semi / np.sqrt(np.sum(semi ** 2, axis=0))
            phi_axis = np.arctan2(axis[1], axis[0])
            shp["e"] = np.sqrt(e1 ** 2 + e2 ** 2)
            shp["c2a"], shp["s2a"] = np.cos(2 * phi_axis), np.sin(2 * phi_axis)
        if pos_patch is not None:
            pos["patch"], shp["patch"] = pos_patch, shape_patch
        return pos, shp

    def _counter(self, with_shapes):
        o = self.o
        return LightconeCounter(self.kind, with_shapes, o.r_bins, o.r_min, o.r_max,
                                o.pi_bins if self.kind == "w" else o.mu_r_bins,
                                h_extra=self.h if self.over_h else 1.0, rp_cut=self.rp_cut, device=o.device)

    @staticmethod
    def _dd(dd, cnt):
        dd = np.array(dd)
        dd[(dd == 0) | (cnt == 0)] = 1     # DD[np.where(DD == 0)] = 1 (measure_w_lightcone.py:186)
        return dd

    # ---- one counter: full sample (+ realisations) --------------------------
    def launch(self, pos_from, shape_from, with_shapes, name, suffix, patches=None, real_name=None,
               real_suffix=None, names=None):
        """Enqueue the full-sample counter (with ``patches`` = (position
        patches, shape patches) and no masks, the pooled driver's realisations
        in the same pass) and return the function that fetches its result and
        writes the products.  The host work of the next counter then overlaps
        this one on the GPU."""
        combo = self._combo(pos_from, shape_from, with_shapes)
        counter = self._counter(with_shapes)
        sel = self._select(combo, self.masks, with_shapes)
        # the reference hands the masks to the S+D and S+R realisations only
        # (measure_IA.py:562-590); the count realisations use every object
        rmasks = self.masks if with_shapes else None
        one_pass = patches is not None and self.masks is None
        if one_pass:
            pp, sp = patches
            lo, hi = int(np.min(pp)), int(np.max(pp))
            pos, shp = self._samples(sel, with_shapes, np.asarray(pp) - lo, self._shape_labels(sp, lo, hi))
            job = counter.prepare(pos, shp, hi - lo + 1)
        else:
            pos, shp = self._samples(sel, with_shapes)
            job = counter.prepare(pos, shp, 0)
        counter.run(job)
        del pos, shp

        def finish():
            sums, cnt = counter.fetch(job)
            real = (lo, hi, sums, cnt) if one_pass else None
            self._finish(combo, counter, with_shapes, rmasks, sums, cnt, real, name, suffix, patches, real_name,
                         real_suffix, names)
        return finish

    def _finish(self, combo, counter, with_shapes, rmasks, sums, cnt, real, name, suffix, patches, real_name,
                real_suffix, names):
        self._write_full(sums[:, 0], cnt[0], with_shapes, name, suffix)
        if patches is None:
            return
        pp, sp = patches
        lo, hi = int(np.min(pp)), int(np.max(pp))
        if real is None:   # masks: the realisations select with the 'Redshift' masks (measure_jackknife.py:346-356)
            if rmasks is None:
                mp = np.ones(len(pp), dtype=bool)
                ms = np.ones(len(sp), dtype=bool)
                rsel = self._select(combo, None, with_shapes)
            else:
                mp = np.asarray(rmasks["Redshift"], dtype=bool)
                ms = np.asarray(rmasks["Redshift_shape_sample"], dtype=bool)
                mt = {k: mp for k in _POS_KEYS}
                mt.update({k: ms for k in _SHAPE_KEYS})
                mt["e1"] = mt["e2"] = ms
                rsel = self._select(combo, mt, with_shapes)
            pos, shp = self._samples(rsel, with_shapes, (np.asarray(pp) - lo)[mp],
                                     self._shape_labels(sp, lo, hi)[ms])
            sums, cnt = counter.count(pos, shp, hi - lo + 1)
            real = (lo, hi, sums, cnt)
        self._write_realisations(real, with_shapes, real_name, real_suffix, names, patches, rmasks)

    @staticmethod
    def _shape_labels(sp, lo, hi):
        lab = np.asarray(sp).astype(np.int64) - lo
        return np.where((lab >= 0) & (lab <= hi - lo), lab, -1).astype(np.int32)

    def _write_full(self, sums, cnt, with_shapes, name, suffix):
        top, rs, ps = self.top, self.rs, self.ps
        dd = self._dd(sums[0], cnt)
        if with_shapes:
            sp, sx = sums[1], sums[2]
            self.put(f"{top}/xi_g_plus/{name}", sp / dd)
            self.put(f"{top}/xi_g_plus/{name}_SplusD", sp)
            self.put(f"{top}/xi_g_cross/{name}_ScrossD", sx)
            self.put(f"{top}/xi_gg/{name}_DD", dd)
            for grp in ("xi_g_plus", "xi_g_cross", "xi_gg"):
                self.put(f"{top}/{grp}/{name}{rs}", self.rc)
                self.put(f"{top}/{grp}/{name}{ps}", self.pc)
        else:
            self.put(f"{top}/xi_gg/{name}{suffix}", dd)
            self.put(f"{top}/xi_gg/{name}{rs}", self.rc)
            self.put(f"{top}/xi_gg/{name}{ps}", self.pc)

    def _write_realisations(self, real, with_shapes, name, suffix, names, patches, masks):
        """measure_jackknife.py:340-470 (pooled driver): datasets of each
        realisation, and the per-realisation sample sizes."""
        lo, hi, sums, cnt = real
        top, rs, ps = self.top, self.rs, self.ps
        grp = f"{name}_jk{hi - lo + 1}"
        pp, sp = patches
        mp = np.ones(len(pp), dtype=bool) if masks is None else np.asarray(masks["Redshift"], dtype=bool)
        ms = np.ones(len(sp), dtype=bool) if masks is None else np.asarray(masks["Redshift_shape_sample"], dtype=bool)
        # objects outside patch i: the (masked) total less those in i
        def outside(lab, m):
            lab = np.asarray(lab).astype(np.int64)[m] - lo
            inside = np.bincount(lab[(lab >= 0) & (lab <= hi - lo)], minlength=hi - lo + 1)
            return int(np.count_nonzero(m)) - inside

        out_s, out_p = outside(sp, ms), outside(pp, mp)
        for k, i in enumerate(range(lo, hi + 1)):
            self.nsj.setdefault(f"{i}", {})[names[0]] = int(out_s[k])
            self.nsj[f"{i}"][names[1]] = int(out_p[k])
            dd = self._dd(sums[0, 1 + k], cnt[1 + k])
            if with_shapes:
                for sub, tag, v in (("xi_g_plus", "SplusD", sums[1, 1 + k]), ("xi_gg", "DD", dd)):
                    self.put(f"{top}/{sub}/{grp}/{name}_{i}_{tag}", v)
                    self.put(f"{top}/{sub}/{grp}/{name}_{i}{rs}", self.rc)
                    self.put(f"{top}/{sub}/{grp}/{name}_{i}{ps}", self.pc)
            else:
                self.put(f"{top}/xi_gg/{grp}/{name}_{i}{suffix}", dd)
                self.put(f"{top}/xi_gg/{grp}/{name}_{i}{rs}", self.rc)
                self.put(f"{top}/xi_gg/{grp}/{name}_{i}{ps}", self.pc)

    # ---- estimator and integrals ---------------------------------------------
    def obs(self, name, rname, ns, grp="", grp_r=""):
        """measure_IA_base.py:670-743"""
        top, corr, est = self.top, self.corr, self.est
        g = f"{grp}/" if grp else ""
        gr = f"{grp_r}/" if grp_r else ""
        if grp_r and f"{top}/xi_gg/{grp_r}" not in self._groups():
            raise KeyError(f"Unable to open object '{grp_r}' in '{norm_path(self.o.snap_group, top, 'xi_gg')}'")
        SpD = SpR = SR = RD = RR = None
        if corr in ("g+", "both"):
            SpD = self.get(f"{top}/xi_g_plus/{g}{name}_SplusD")
            SpR = self.get(f"{top}/xi_g_plus/{gr}{rname}_SplusD")
        DD = self.get(f"{top}/xi_gg/{g}{name}_DD")
        if est == "clusters" or corr in ("gg", "both"):
            SR = self.get(f"{top}/xi_gg/{g}{name}_SR") if corr == "gg" else self.get(f"{top}/xi_gg/{gr}{rname}_DD")
        if corr in ("gg", "both"):
            RD = self.get(f"{top}/xi_gg/{g}{name}_RD")
        if est == "galaxies" or corr in ("gg", "both"):
            RR = self.get(f"{top}/xi_gg/{g}{name}_RR")
        if est == "clusters":
            SR = SR * (ns["D"] / ns["R_D"])
            if corr in ("g+", "both"):
                SpR = SpR * (ns["D"] / ns["R_D"])
                self.put(f"{top}/xi_g_plus/{g}{name}", SpD / DD - SpR / SR)
            if corr in ("gg", "both"):
                RD = RD * (ns["S"] / ns["R_S"])
                RR = RR * ((ns["S"] / ns["R_S"]) * (ns["D"] / ns["R_D"]))
                self.put(f"{top}/xi_gg/{g}{name}", (DD - RD - SR) / RR - 1)
        else:
            RR = RR * ((ns["S"] / ns["R_S"]) * (ns["D"] / ns["R_D"]))
            if corr in ("g+", "both"):
                SpR = SpR * (ns["D"] / ns["R_D"])
                self.put(f"{top}/xi_g_plus/{g}{name}", (SpD - SpR) / RR)
            if corr in ("gg", "both"):
                RD = RD * (ns["S"] / ns["R_S"])
                SR = SR * (ns["D"] / ns["R_D"])
                self.put(f"{top}/xi_gg/{g}{name}", (DD - RD - SR) / RR + 1)

    def _groups(self):
        return {g[len(self.o.snap_group):] if g.startswith(self.o.snap_group) else g for g in self._gs}

    def integrate(self, name, grp=""):
        """measure_IA_base.py:515-668 for this corr_type."""
        o = self.o
        g = f"{grp}/" if grp else ""
        todo = {"both": [("g_plus", 2), ("gg", 0)], "g+": [("g_plus", 2)], "gg": [("gg", 0)]}[self.corr]
        for suff, l in todo:
            xi = self.get(f"{self.top}/xi_{suff}/{g}{name}")
            if self.kind == "w":
                dpi = o.pi_bins[1:] - o.pi_bins[:-1]
                val = np.sum(xi * abs(np.array([dpi] * len(xi[:, 0]))), axis=1)
                dst = f"w_{suff}"
            else:
                mu_c = _centres(o.mu_r_bins)
                leg = 3.0 * (1.0 - mu_c ** 2) if l == 2 else np.ones_like(mu_c)
                dmu = o.mu_r_bins[1:] - o.mu_r_bins[:-1]
                fac = (2 * l + 1) / 2.0 * math.factorial(0) / math.factorial(2 * l)
                val = np.sum(fac * np.array([leg] * xi.shape[0]) * xi * np.array([dmu] * xi.shape[0]), axis=1)
                dst = f"multipoles_{suff}"
            self.put(f"{dst}/{g}{name}{self.rs}", self.rc)
            self.put(f"{dst}/{g}{name}", val)

    # ---- the flow ------------------------------------------------------------
    def full_and_realisations(self, ns):
        d, dr, corr, est, jk = self.d, f"{self.d}_randoms", self.corr, self.est, self.jk
        P = (lambda a, b: (jk[a], jk[b])) if jk is not None else (lambda a, b: None)
        steps = []
        if corr in ("g+", "both"):
            steps.append(("D", "D", True, d, "", P("position", "shape"), d, "", ["S", "D"]))
            steps.append(("R", "D", True, dr, "", P("randoms_position", "shape"), dr, "", ["S", "R_D"]))
        if corr == "gg":
            steps.append(("D", "D", False, d, "_DD", P("position", "shape"), d, "_DD", ["S", "D"]))
            steps.append(("R", "D", False, d, "_SR", P("randoms_position", "shape"), d, "_SR", ["S", "R_D"]))
        if corr in ("gg", "both"):
            steps.append(("D", "R", False, d, "_RD", P("position", "randoms_shape"), d, "_RD", ["R_S", "D"]))
        if est == "galaxies" or corr in ("gg", "both"):
            steps.append(("R", "R", False, d, "_RR", P("randoms_position", "randoms_shape"), d, "_RR",
                          ["R_S", "R_D"]))
        # every counter is enqueued first, then finished in the reference's
        # order; if enqueuing one fails, those before it are finished (and
        # their products kept) before the error propagates, as in the
        # reference's one-after-the-other flow
        pending = []
        try:
            for step in steps:
                pending.append(self.launch(*step))
        except BaseException:
            for fin in pending:
                fin()
            raise
        for fin in pending:
            fin()
        self.obs(d, dr, ns)
        self.integrate(d)
        if jk is None:
            return
        lo, hi = int(np.min(jk["shape"])), int(np.max(jk["shape"]))
        n_p = hi - lo + 1
        grp, grp_r = f"{d}_jk{n_p}", f"{dr}_jk{n_p}"
        for i in range(lo, hi + 1):
            self.obs(f"{d}_{i}", f"{dr}_{i}", self.nsj[f"{i}"], grp, grp_r)
            self.integrate(f"{d}_{i}", grp)
        for suff in {"both": ["g_plus", "gg"], "g+": ["g_plus"], "gg": ["gg"]}[corr]:
            dst = f"w_{suff}" if self.kind == "w" else f"multipoles_{suff}"
            reals = np.array([self.get(f"{dst}/{grp}/{d}_{i}") for i in range(lo, hi + 1)])
            n = len(reals)
            mean = np.zeros(reals.shape[1])
            for x in reals:
                mean += x
            mean /= n
            cov = np.zeros((reals.shape[1],) * 2)
            std = np.zeros(reals.shape[1])
            for x in reals:
                std += (x - mean) ** 2
                for k in range(reals.shape[1]):
                    cov[:, k] += (x - mean) * (x[k] - mean[k])
            std *= (n - 1) / n
            self.put(f"{dst}/{d}_mean_{n_p}", mean)
            self.put(f"{dst}/{d}_jackknife_{n_p}", np.sqrt(std))
            self.put(f"{dst}/{d}_jackknife_cov_{n_p}", cov * ((n - 1) / n))
