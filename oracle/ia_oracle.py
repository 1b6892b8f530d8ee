"""CPU oracle for the periodic-box IA pair-counting path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``measure_ia_gb300``)
imports this module; only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` use it, and only as the checker or as the
timed CPU reference.

This is a restatement, in vectorised numpy, of the reference algorithm of
MeasureIA's box path (``src/measureia`` of MarloesvL/measure_IA).  Every
function names the reference lines it follows.  The per-pair arithmetic is
written as the same sequence of numpy operations as the reference (same
operand order, same ufuncs: ``sqrt``, ``log10``, ``arccos``, ``cos``,
``sin``), so on the same host the oracle reproduces the reference's bin
assignment bit for bit; only the order of the floating-point sums differs
(the reference scatters with ``np.add.at`` shape by shape, the oracle uses
``np.bincount`` over all pairs of a chunk).

Neighbour pre-selection follows the reference's tree path: scipy's periodic
``KDTree.query_ball_tree`` at ``r_min`` and ``r_max`` and the set difference
of the two (``measure_w_box_jk.py:577-580``), i.e. ``r_min < d <= r_max`` in
the projected plane for (r_p, Pi) and in 3-D for (r, mu_r).  The brute-force
path (``temp_file_path=False``) takes every pair.

The pins for this module are the fixtures in ``tests/golden`` made by
``tests/golden/make_golden.py``: outputs of the reference itself on seeded
catalogues, and datasets read from the reference's own golden HDF5 files.
"""

from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

try:  # scipy is present on both the build host and the GPU host
    from scipy.spatial import KDTree
except Exception:  # pragma: no cover
    KDTree = None


# ----------------------------------------------------------------------------
# Binning state  (measure_IA_base.py:155-167, Sim_info.py:64-80)
# ----------------------------------------------------------------------------

@dataclass
class Binning:
    boxsize: float
    r_min: float
    r_max: float
    num_bins_r: int
    num_bins_pi: int
    pi_max: float | None = None
    snapshot: object = None
    r_bins: np.ndarray = field(init=False)
    pi_bins: np.ndarray = field(init=False)
    mu_r_bins: np.ndarray = field(init=False)

    def __post_init__(self):
        self.L_0p5 = self.boxsize / 2.0
        pi_max = self.L_0p5 if self.pi_max is None else self.pi_max
        self.r_bins = np.logspace(np.log10(self.r_min), np.log10(self.r_max), self.num_bins_r + 1)
        self.pi_bins = np.linspace(-pi_max, pi_max, self.num_bins_pi + 1)
        self.mu_r_bins = np.linspace(-1, 1, self.num_bins_pi + 1)
        self.snap_group = "" if self.snapshot is None else f"Snapshot_{self.snapshot}/"


# ----------------------------------------------------------------------------
# Input preparation  (measure_w_box_jk.py:685-748, measure_m_box_jk.py:722-788)
# ----------------------------------------------------------------------------

def select_inputs(data, masks):
    """Masking and axis normalisation, including the reference's weight-mask
    quirk: without a ``weight`` key in ``masks`` the first ``sum(mask)``
    weights are taken (measure_w_box_jk.py:694-712).  Mutates ``masks`` the
    same way the reference does."""
    n_pos_all = len(data["Position"])
    n_shape_all = len(data["Position_shape_sample"])
    if masks is None:
        pos = data["Position"]
        spos = data["Position_shape_sample"]
        axis_raw = data["Axis_Direction"]
        q = data["q"]
        w = data["weight"]
        ws = data["weight_shape_sample"]
    else:
        pos = data["Position"][masks["Position"]]
        spos = data["Position_shape_sample"][masks["Position_shape_sample"]]
        axis_raw = data["Axis_Direction"][masks["Axis_Direction"]]
        q = data["q"][masks["q"]]
        if "weight" not in masks:
            m = np.ones(n_pos_all, dtype=bool)
            m[sum(masks["Position"]):n_pos_all] = 0
            masks["weight"] = m
        if "weight_shape_sample" not in masks:
            m = np.ones(n_shape_all, dtype=bool)
            m[sum(masks["Position_shape_sample"]):n_shape_all] = 0
            masks["weight_shape_sample"] = m
        w = data["weight"][masks["weight"]]
        ws = data["weight_shape_sample"][masks["weight_shape_sample"]]
    norm = np.sqrt(np.sum(axis_raw ** 2, axis=1))
    axis = (axis_raw.transpose() / norm).transpose()
    return pos, spos, axis, q, w, ws


def ellipticity_size(q, ellipticity="distortion"):
    """measure_w_box_jk.py:737-742"""
    if ellipticity == "distortion":
        return (1 - q ** 2) / (1 + q ** 2)
    if ellipticity == "ellipticity":
        return (1 - q) / (1 + q)
    raise ValueError("Invalid value for ellipticity. Choose 'distortion' or 'ellipticity'.")


def responsivity(ws, e):
    """R = sum(w_s (1 - e^2/2)) / sum(w_s) with Python's sequential sum
    (measure_w_box_jk.py:744)."""
    return sum(ws * (1 - e ** 2 / 2.0)) / sum(ws)


def responsivity_jk(ws, e, labels, n_box):
    """R without region i (measure_w_box_jk.py:782-785)."""
    out = np.zeros(n_box)
    for i in range(n_box):
        keep = np.where(labels != i)
        out[i] = sum(ws[keep] * (1 - e[keep] ** 2 / 2.0)) / sum(ws[keep])
    return out


def jackknife_labels(points, L_0p5, L_subboxes):
    """Sub-box label i*L^2 + j*L + k of each point, strict bounds, points on a
    face keep label 0 (measure_IA_base.py:404-452)."""
    L_sub = L_0p5 * 2.0 / L_subboxes
    edges = np.arange(0, L_subboxes + 1) * L_sub        # i * L_sub, as the reference forms it
    idx = []
    inside = np.ones(len(points), dtype=bool)
    for d in range(3):
        x = points[:, d]
        k = np.searchsorted(edges, x, side="left") - 1
        k = np.clip(k, 0, L_subboxes - 1)
        ok = (x > edges[k]) & (x < edges[k + 1])
        inside &= ok
        idx.append(k)
    lab = (idx[0] * L_subboxes + idx[1]) * L_subboxes + idx[2]
    return np.where(inside, lab, 0).astype(np.int64)


# ----------------------------------------------------------------------------
# Analytic randoms  (measure_IA_base.py:230-351)
# ----------------------------------------------------------------------------

def random_pairs_rp_pi(rp_max, rp_min, pi_max, pi_min, L3, n_pos, n_shape):
    """'cross' branch of get_random_pairs (measure_IA_base.py:268-269)."""
    return n_pos * n_shape * np.pi * (rp_max ** 2 - rp_min ** 2) * abs(pi_max - pi_min) / L3


def _cap_volume(mur, r):
    """measure_IA_base.py:291"""
    return np.pi / 3.0 * r ** 3 * (2 + mur) * (1 - mur) ** 2


def random_pairs_r_mur(r_max, r_min, mur_max, mur_min, L3, n_pos, n_shape):
    """'cross' branch of get_random_pairs_r_mur, with its (N_p - 1) factor
    and the final abs (measure_IA_base.py:337-351)."""
    rr = (n_pos - 1.0) * n_shape * (
        _cap_volume(mur_min, r_max) - _cap_volume(mur_max, r_max)
        - (_cap_volume(mur_min, r_min) - _cap_volume(mur_max, r_min))) / L3
    return abs(rr)


def rr_tables(b: Binning, kind, n_pos, n_shape, n_pos_jk=None, n_shape_jk=None):
    """RR and RR_jk grids (measure_w_box_jk.py:789-807, measure_m_box_jk.py:829-848)."""
    L3 = b.boxsize ** 3
    nr, npi = b.num_bins_r, b.num_bins_pi
    edges = b.pi_bins if kind == "w" else b.mu_r_bins
    fn = random_pairs_rp_pi if kind == "w" else random_pairs_r_mur
    rr = np.zeros((nr, npi))
    for i in range(nr):
        for p in range(npi):
            rr[i, p] = fn(b.r_bins[i + 1], b.r_bins[i], edges[p + 1], edges[p], L3, n_pos, n_shape)
    rr_jk = None
    if n_pos_jk is not None:
        nbox = len(n_pos_jk)
        vol = L3 * (nbox - 1) / nbox
        rr_jk = np.zeros((nbox, nr, npi))
        for jk in range(nbox):
            for i in range(nr):
                for p in range(npi):
                    rr_jk[jk, i, p] = fn(b.r_bins[i + 1], b.r_bins[i], edges[p + 1], edges[p], vol,
                                         int(n_pos_jk[jk]), int(n_shape_jk[jk]))
    return rr, rr_jk


# ----------------------------------------------------------------------------
# Candidate pairs
# ----------------------------------------------------------------------------

def _flatten(lists):
    lens = np.fromiter((len(x) for x in lists), dtype=np.int64, count=len(lists))
    if lens.sum() == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    flat = np.concatenate([np.asarray(x, dtype=np.int64) for x in lists if len(x)])
    owner = np.repeat(np.arange(len(lists), dtype=np.int64), lens)
    return owner, flat


def tree_candidates(shape_pts, pos_tree, r_min, r_max, boxsize):
    """(shape, position) index pairs with r_min < d <= r_max under scipy's
    periodic metric: two ``query_ball_tree`` calls and their per-row set
    difference (measure_w_box_jk.py:577-580, measure_IA_base.py:354-375)."""
    shape_tree = KDTree(shape_pts, boxsize=boxsize)
    s_out, p_out = _flatten(shape_tree.query_ball_tree(pos_tree, r_max))
    s_in, p_in = _flatten(shape_tree.query_ball_tree(pos_tree, r_min))
    if len(s_in):
        n = pos_tree.n
        drop = np.isin(s_out * n + p_out, s_in * n + p_in)
        s_out, p_out = s_out[~drop], p_out[~drop]
    return s_out, p_out


# ----------------------------------------------------------------------------
# Per-pair binning  (measure_w_box_jk.py:584-617, measure_m_box_jk.py:611-653)
# ----------------------------------------------------------------------------

def _not_los(los):
    return np.array([0, 1, 2])[np.isin([0, 1, 2], los, invert=True)]


def _clamp_top(ind, n):
    """'if any(ind == n): ind[ind >= n] -= 1' (measure_w_box_jk.py:614-617)."""
    if np.any(ind == n):
        ind = ind.copy()
        ind[ind >= n] -= 1
    return ind


def pair_terms(kind, b: Binning, los, spos, axis, e, pos, si, pj, rp_cut=0.0, periodic=True):
    """Shared per-pair arithmetic of the w and multipole kernels.  Returns
    (mask, ind_r, ind_p, e_plus, e_cross) with ind_* for the masked pairs."""
    nl = _not_los(los)
    sep = spos[si] - pos[pj]                               # shape minus position
    if periodic:
        sep[sep > b.L_0p5] -= b.boxsize
        sep[sep < -b.L_0p5] += b.boxsize
    proj = sep[:, nl]
    los_sep = sep[:, los]
    rp = np.sqrt(np.sum(proj ** 2, axis=1))
    with np.errstate(invalid="ignore", divide="ignore"):
        sdir = (proj.transpose() / rp).transpose()
        if kind == "m":
            r3 = np.sqrt(np.sum(sep ** 2, axis=1))
            mu = los_sep / r3
        phi = np.arccos(sdir[:, 0] * axis[si, 0] + sdir[:, 1] * axis[si, 1])
    ep = e[si] * np.cos(2 * phi)
    ex = e[si] * np.sin(2 * phi)
    ep[np.isnan(ep)] = 0.0
    ex[np.isnan(ex)] = 0.0
    dlog = (np.log10(b.r_max) - np.log10(b.r_min)) / b.num_bins_r
    if kind == "w":
        dpi = (b.pi_bins[-1] - b.pi_bins[0]) / b.num_bins_pi
        mask = (rp >= b.r_bins[0]) * (rp < b.r_bins[-1]) * (los_sep >= b.pi_bins[0]) * (los_sep < b.pi_bins[-1])
        ind_r = np.floor(np.log10(rp[mask]) / dlog - np.log10(b.r_bins[0]) / dlog)
        ind_p = np.floor(los_sep[mask] / dpi - b.pi_bins[0] / dpi)
    else:
        dmu = 2.0 / b.num_bins_pi
        mask = (rp > rp_cut) * (r3 >= b.r_bins[0]) * (r3 < b.r_bins[-1])
        ind_r = np.floor(np.log10(r3[mask]) / dlog - np.log10(b.r_bins[0]) / dlog)
        ind_p = np.floor(mu[mask] / dmu - b.mu_r_bins[0] / dmu)
    ind_r = _clamp_top(np.array(ind_r, dtype=int), b.num_bins_r)
    ind_p = _clamp_top(np.array(ind_p, dtype=int), b.num_bins_pi)
    # numpy index semantics of np.add.at: -k addresses n-k
    ind_r = np.where(ind_r < 0, ind_r + b.num_bins_r, ind_r)
    ind_p = np.where(ind_p < 0, ind_p + b.num_bins_pi, ind_p)
    return mask, ind_r, ind_p, ep, ex


@dataclass
class Counts:
    """Raw histograms of one measurement (all shaped (n_r, n_pi) or (n_jk, n_r, n_pi))."""
    DD: np.ndarray
    SplusD: np.ndarray      # already divided by 2R
    ScrossD: np.ndarray     # already divided by 2R
    variance: np.ndarray    # sum of squared S+D terms (brute path only)
    npairs: np.ndarray      # integer pair counts
    DD_jk: np.ndarray | None = None
    SplusD_jk: np.ndarray | None = None
    npairs_jk: np.ndarray | None = None


def position_tree(kind, b: Binning, los, pos):
    """The periodic KD-tree over the positions that the tree backends query:
    2-D over the projected plane for (r_p, Pi), 3-D for (r, mu_r)
    (measure_w_box_jk.py:764, measure_m_box_jk.py:804)."""
    return KDTree(pos[:, _not_los(los)] if kind == "w" else pos, boxsize=b.boxsize)


def count_pairs(kind, b: Binning, los, pos, w, spos, axis, e, ws, R, lab_pos=None, lab_shape=None,
                n_box=0, membership="tree", rp_cut=0.0, chunk=2000, periodic=True, shape_range=None,
                pos_tree=None):
    """Histograms DD, S+D, SxD (+ jackknife parts) over all binned pairs.

    Follows ``_measure_xi_rp_pi_box_jk_batch`` (measure_w_box_jk.py:543-646)
    for ``kind='w'`` and ``_measure_xi_r_mur_box_jk_batch``
    (measure_m_box_jk.py:570-682) for ``kind='m'``; ``membership='brute'``
    follows the brute variants (measure_w_box_jk.py:157-211,
    measure_m_box_jk.py:164-223), which also accumulate the S+D variance.
    ``pos_tree`` (from ``position_tree``) is reused when given, as the
    reference's Pool workers reuse the parent's ``self.pos_tree``; ``chunk``
    bounds the shapes whose candidate pairs are held in memory at once."""
    nr, npi = b.num_bins_r, b.num_bins_pi
    nb = nr * npi
    DD = np.zeros(nb); SP = np.zeros(nb); SX = np.zeros(nb); VAR = np.zeros(nb)
    CNT = np.zeros(nb, dtype=np.int64)
    jk = n_box > 0
    if jk:
        DDj = np.zeros(n_box * nb); SPj = np.zeros(n_box * nb); CNTj = np.zeros(n_box * nb, dtype=np.int64)
    nl = _not_los(los)
    if membership == "tree" and pos_tree is None:
        pos_tree = position_tree(kind, b, los, pos)
    s_lo, s_hi = (0, len(spos)) if shape_range is None else shape_range
    for c0 in range(s_lo, s_hi, chunk):
        c1 = min(s_hi, c0 + chunk)
        if membership == "tree":
            pts = spos[c0:c1][:, nl] if kind == "w" else spos[c0:c1]
            si, pj = tree_candidates(pts, pos_tree, b.r_min, b.r_max, b.boxsize)
            si = si + c0
        else:
            si = np.repeat(np.arange(c0, c1, dtype=np.int64), len(pos))
            pj = np.tile(np.arange(len(pos), dtype=np.int64), c1 - c0)
        if len(si) == 0:
            continue
        mask, ir, ip, ep, ex = pair_terms(kind, b, los, spos, axis, e, pos, si, pj, rp_cut, periodic)
        si, pj = si[mask], pj[mask]
        flat = ir * npi + ip
        ww = w[pj] * ws[si]
        sp = ww * ep[mask]
        DD += np.bincount(flat, weights=ww, minlength=nb)
        SP += np.bincount(flat, weights=sp / (2 * R), minlength=nb)
        SX += np.bincount(flat, weights=ww * ex[mask] / (2 * R), minlength=nb)
        if membership == "brute":
            VAR += np.bincount(flat, weights=(sp / (2 * R)) ** 2, minlength=nb)
        CNT += np.bincount(flat, minlength=nb)
        if jk:
            a = lab_shape[si]
            bb = lab_pos[pj]
            other = bb != a
            for lab, sel in ((a, slice(None)), (bb[other], other)):
                idx = lab * nb + flat[sel]
                DDj += np.bincount(idx, weights=ww[sel], minlength=n_box * nb)
                SPj += np.bincount(idx, weights=sp[sel], minlength=n_box * nb)
                CNTj += np.bincount(idx, minlength=n_box * nb)
    shp = (nr, npi)
    out = Counts(DD.reshape(shp), SP.reshape(shp), SX.reshape(shp), VAR.reshape(shp), CNT.reshape(shp))
    if jk:
        out.DD_jk = DDj.reshape((n_box,) + shp)
        out.SplusD_jk = SPj.reshape((n_box,) + shp)
        out.npairs_jk = CNTj.reshape((n_box,) + shp)
    return out


# ----------------------------------------------------------------------------
# Post-processing  (measure_IA_base.py:454-668; measure_w_box_jk.py:809-854)
# ----------------------------------------------------------------------------

def bin_centres(edges):
    """edges[:-1] + |diff/2| (measure_w_box_jk.py:811-814)."""
    return edges[:-1] + abs((edges[1:] - edges[:-1]) / 2.0)


def w_from_xi(b: Binning, xi):
    """Pi integration sum(xi * |dpi|) (measure_IA_base.py:553-562)."""
    dpi = b.pi_bins[1:] - b.pi_bins[:-1]
    dpi = np.array([dpi] * len(xi[:, 0]))
    return np.sum(xi * abs(dpi), axis=1)


def assoc_legendre_mm(l, x):
    """P_l^l(x) for l in {0, 2}, the two orders the multipoles use
    (P_0^0 = 1, P_2^2 = 3 (1 - x^2), scipy's lpmn convention)."""
    if l == 0:
        return np.ones_like(x)
    if l == 2:
        return 3.0 * (1.0 - x * x)
    raise ValueError(l)


def multipoles_from_xi(b: Binning, xi, l):
    """(2l+1)/2 (l-m)!/(l+m)! sum_mu P_l^m(mu) xi dmu with m = l
    (measure_IA_base.py:628-655)."""
    mu_c = bin_centres(b.mu_r_bins)
    Lg = np.array([assoc_legendre_mm(l, mu_c)] * xi.shape[0])
    dmu = b.mu_r_bins[1:] - b.mu_r_bins[:-1]
    dmu = np.array([dmu] * xi.shape[0])
    fac = (2 * l + 1) / 2.0 * math.factorial(0) / math.factorial(2 * l)
    return np.sum(fac * Lg * xi * dmu, axis=1)


def combine_jackknife(realisations):
    """mean, jackknife std and covariance over realisations (n_box, n_r)
    (measure_IA_base.py:481-498)."""
    n_box, nr = realisations.shape
    mean = np.zeros(nr)
    for x in realisations:
        mean += x
    mean /= n_box
    cov = np.zeros((nr, nr))
    std = np.zeros(nr)
    for x in realisations:
        std += (x - mean) ** 2
        for i in range(nr):
            cov[:, i] += (x - mean) * (x[i] - mean[i])
    std *= (n_box - 1) / n_box
    std = np.sqrt(std)
    cov *= (n_box - 1) / n_box
    return mean, std, cov


def jackknife_cross_cov(real_a, real_b):
    """Jackknife covariance of two datasets' realisations (n_box, n_r) each
    (``MeasureJackknife.measure_covariance_multiple_datasets``,
    measure_jackknife.py:519-555): means in realisation order, then
    cov[:, i] += (a_b - mean_a) * (b_b[i] - mean_b[i]) and
    std += (a_b - mean_a) * (b_b - mean_b), both times (n - 1) / n, std
    square-rooted (NaN where the cross sum is negative).  With real_a is
    real_b it is the single-dataset branch (:533-539)."""
    real_a = np.asarray(real_a, dtype=np.float64)
    real_b = np.asarray(real_b, dtype=np.float64)
    n_box, nr = real_a.shape
    ma = np.zeros(nr)
    mb = np.zeros(nr)
    for x in real_a:
        ma += x
    ma /= n_box
    for x in real_b:
        mb += x
    mb /= n_box
    cov = np.zeros((nr, nr))
    std = np.zeros(nr)
    for xa, xb in zip(real_a, real_b):
        std += (xa - ma) * (xb - mb)
        for i in range(nr):
            cov[:, i] += (xa - ma) * (xb[i] - mb[i])
    std *= (n_box - 1) / n_box
    with np.errstate(invalid="ignore"):
        std = np.sqrt(std)
    cov *= (n_box - 1) / n_box
    return cov, std


def full_projection_cov(cov_00, cov_11, cov_22, cov_01, cov_02, cov_12):
    """The combined covariances of three projections
    (``create_full_cov_matrix_projections``, measure_jackknife.py:604-635):
    returns (cov3, cov2 of 0-1, cov2 of 0-2, cov2 of 1-2).  The reference
    reads its 'cov_yz' from the (0, 2) pair dataset and its 'cov_xz' from the
    (1, 2) one (:611-612) and assembles with those names; this follows it."""
    cov_xx, cov_yy, cov_zz, cov_xy = cov_00, cov_11, cov_22, cov_01
    cov_yz, cov_xz = cov_02, cov_12
    cov3 = np.concatenate((np.concatenate((cov_xx, cov_xy, cov_xz), axis=1),
                           np.concatenate((cov_xy.T, cov_yy, cov_yz), axis=1),
                           np.concatenate((cov_xz.T, cov_yz.T, cov_zz), axis=1)), axis=0)
    cov2xy = np.concatenate((np.concatenate((cov_xx, cov_xy), axis=1),
                             np.concatenate((cov_xy.T, cov_yy), axis=1)), axis=0)
    cov2xz = np.concatenate((np.concatenate((cov_xx, cov_xz), axis=1),
                             np.concatenate((cov_xz.T, cov_zz), axis=1)), axis=0)
    cov2yz = np.concatenate((np.concatenate((cov_yy, cov_yz), axis=1),
                             np.concatenate((cov_yz.T, cov_zz), axis=1)), axis=0)
    return cov3, cov2xy, cov2xz, cov2yz


def _sub(a, b):
    return "/".join(x for x in (a + "/" + b).split("/") if x)


def measure(kind, b: Binning, data, dataset_name, corr_type="both", num_jk=0, masks=None,
            ellipticity="distortion", layout="multiprocessing", rp_cut=0.0, chunk=2000, processes=1):
    """Whole measurement as ``MeasureIABox.measure_xi_w`` (kind='w') or
    ``measure_xi_multipoles`` (kind='m') writes it (measure_IA.py:68-262):
    returns {hdf5 path: array} with the reference's dataset names, plus
    '__counts__' with the raw histograms.

    ``layout`` selects the backend whose datasets are mirrored:
    'multiprocessing' (num_nodes > 1), 'tree' (num_nodes == 1) or 'brute'
    (temp_file_path=False).  ``processes > 1`` counts the pairs of a tree
    layout in a spawned process pool (``count_pairs_parallel``; large
    catalogues), with ``chunk`` shapes per task."""
    if corr_type not in ("both", "g+", "gg"):
        raise KeyError("Unknown value for corr_type. Choose from [g+, gg, both]")
    L_sub = 0
    if num_jk > 0:
        L_sub = round(num_jk ** (1.0 / 3.0))
        if L_sub ** 3 != num_jk:
            raise ValueError("Use x^3 as input for num_jk, with x as an int.")
    los = data["LOS"]
    pos, spos, axis, q, w, ws = select_inputs(data, masks)
    e = ellipticity_size(q, ellipticity)
    R = responsivity(ws, e)
    n_pos, n_shape = len(pos), len(spos)
    lab_p = lab_s = None
    n_box = L_sub ** 3 if num_jk > 0 else 0
    if n_box:
        lab_p = jackknife_labels(pos, b.L_0p5, L_sub)
        lab_s = jackknife_labels(spos, b.L_0p5, L_sub)
    membership = "brute" if layout == "brute" else "tree"
    if processes > 1 and membership == "tree" and rp_cut == 0.0:
        c, _ = count_pairs_parallel(kind, b, los, pos, w, spos, axis, e, ws, R, lab_p, lab_s, n_box,
                                    (0, n_shape), processes=processes, chunk=chunk, context="spawn")
    else:
        c = count_pairs(kind, b, los, pos, w, spos, axis, e, ws, R, lab_p, lab_s, n_box, membership, rp_cut, chunk)
    out = {"__counts__": c}
    sg = b.snap_group
    top = "w" if kind == "w" else "multipoles"
    rsuf, psuf = ("_rp", "_pi") if kind == "w" else ("_r", "_mu_r")
    rc = bin_centres(b.r_bins)
    pc = bin_centres(b.pi_bins if kind == "w" else b.mu_r_bins)
    d = dataset_name
    jkg = f"{d}_jk{num_jk}" if n_box else ""
    if n_box:
        npj = np.array([np.sum(lab_p != i) for i in range(n_box)])
        nsj = np.array([np.sum(lab_s != i) for i in range(n_box)])
        rr, rr_jk = rr_tables(b, kind, n_pos, n_shape, npj, nsj)
        Rj = responsivity_jk(ws, e, lab_s, n_box)
    else:
        rr, _ = rr_tables(b, kind, n_pos, n_shape)
    xi_gp = c.SplusD / rr
    xi_gx = c.ScrossD / rr
    xi_gg = (c.DD / rr) - 1

    def put(group, name, arr):
        out[_sub(_sub(sg, group), name)] = np.asarray(arr)

    with_sig = n_box and layout in ("tree", "brute")
    sig = c.variance / rr ** 2
    g = f"{top}/xi_g_plus"
    put(g, d, xi_gp); put(g, d + "_SplusD", c.SplusD); put(g, d + "_RR_g_plus", rr)
    if with_sig:
        put(g, d + "_sigmasq", sig)
    put(g, d + rsuf, rc); put(g, d + psuf, pc)
    if n_box:
        for i in range(n_box):
            gj = f"{top}/xi_g_plus/{jkg}"
            num = c.SplusD * (2 * R) - c.SplusD_jk[i]
            put(gj, f"{d}_{i}", num / (rr_jk[i] * 2 * Rj[i]))
            put(gj, f"{d}_{i}_SplusD", num / (2 * Rj[i]))
            put(gj, f"{d}_{i}_RR", rr_jk[i])
            put(gj, f"{d}_{i}{rsuf}", rc); put(gj, f"{d}_{i}{psuf}", pc)
    g = f"{top}/xi_g_cross/{jkg}"
    put(g, d + "_ScrossD", c.ScrossD); put(g, d, xi_gx); put(g, d + "_RR_g_cross", rr)
    if with_sig:
        put(g, d + "_sigmasq", sig)
    put(g, d + rsuf, rc); put(g, d + psuf, pc)
    g = f"{top}/xi_gg"
    put(g, d, xi_gg); put(g, d + "_DD", c.DD); put(g, d + "_RR_gg", rr)
    if with_sig:
        put(g, d + "_sigmasq", sig)
    put(g, d + rsuf, rc); put(g, d + psuf, pc)
    if n_box:
        for i in range(n_box):
            gj = f"{top}/xi_gg/{jkg}"
            put(gj, f"{d}_{i}", ((c.DD - c.DD_jk[i]) / rr_jk[i]) - 1)
            put(gj, f"{d}_{i}_DD", c.DD - c.DD_jk[i])
            put(gj, f"{d}_{i}_RR", rr_jk[i])
            put(gj, f"{d}_{i}{rsuf}", rc); put(gj, f"{d}_{i}{psuf}", pc)

    # second stage: w or multipoles per realisation, then the covariance
    types = {"both": [("g_plus", 2), ("gg", 0)], "g+": [("g_plus", 2)], "gg": [("gg", 0)]}[corr_type]
    for name, l in types:
        src = f"{top}/xi_{name}"
        dst = f"w_{name}" if kind == "w" else f"multipoles_{name}"
        series = [(d, "")] + [(f"{d}_{i}", jkg) for i in range(n_box)]
        reals = []
        for dn, grp in series:
            xi = out[_sub(_sub(sg, _sub(src, grp)), dn)]
            val = w_from_xi(b, xi) if kind == "w" else multipoles_from_xi(b, xi, l)
            put(_sub(dst, grp), dn + rsuf, rc)
            put(_sub(dst, grp), dn, val)
            if grp:
                reals.append(val)
        if n_box:
            mean, std, cov = combine_jackknife(np.array(reals))
            put(dst, f"{d}_mean_{n_box}", mean)
            put(dst, f"{d}_jackknife_{n_box}", std)
            put(dst, f"{d}_jackknife_cov_{n_box}", cov)
    return out


# ----------------------------------------------------------------------------
# Parallel driver for the timed CPU reference (the reference's Pool.map over
# shape chunks, measure_w_box_jk.py:761-780)
# ----------------------------------------------------------------------------

_G = {}


def _worker(args):
    c0, c1 = args
    g = _G
    return count_pairs(g["kind"], g["b"], g["los"], g["pos"], g["w"], g["spos"], g["axis"], g["e"], g["ws"],
                       g["R"], g["lab_p"], g["lab_s"], g["n_box"], "tree", 0.0, g["sub_chunk"], True, (c0, c1),
                       pos_tree=g["tree"])


def _init_spawned(state):
    """Pool initializer of a spawned worker: the inputs, and its own copy of
    the position tree (a spawned process shares nothing with the parent)."""
    _G.update(state)
    _G["tree"] = position_tree(state["kind"], state["b"], state["los"], state["pos"])


def count_pairs_parallel(kind, b, los, pos, w, spos, axis, e, ws, R, lab_p, lab_s, n_box, shape_range,
                         processes=None, chunk=1000, sub_chunk=4, context="fork"):
    """The reference's multiprocessing driver (measure_w_box_jk.py:764-780,
    measure_m_box_jk.py:804-820): the position tree is built once, in the
    parent, then a fork Pool maps chunks of ``chunk`` shapes (the reference's
    ``chunk_size``) over ``processes`` workers that query that tree, and the
    parent sums the partial histograms.  Inside a chunk, ``sub_chunk`` shapes
    at a time hold their candidate pairs in memory (the reference loops shape
    by shape).  A fork Pool must start before any GPU work; ``context =
    'spawn'`` (for callers that already use the GPU) starts fresh workers that
    each build the tree once; ``processes == 1`` runs in this process.
    Returns (Counts, seconds the parent spent building the tree)."""
    import multiprocessing as mp
    import time
    processes = processes or os.cpu_count()
    state = dict(kind=kind, b=b, los=los, pos=pos, w=w, spos=spos, axis=axis, e=e, ws=ws, R=R,
                 lab_p=lab_p, lab_s=lab_s, n_box=n_box, sub_chunk=sub_chunk)
    lo, hi = shape_range
    jobs = [(c, min(hi, c + chunk)) for c in range(lo, hi, chunk)]
    t_tree = 0.0
    try:
        if context == "spawn" and processes > 1:
            ctx = mp.get_context("spawn")
            with ctx.Pool(processes, initializer=_init_spawned, initargs=(state,)) as pool:
                parts = pool.map(_worker, jobs)
        else:
            t0 = time.perf_counter()
            tree = position_tree(kind, b, los, pos)
            t_tree = time.perf_counter() - t0
            _G.update(state, tree=tree)
            if processes == 1:
                parts = [_worker(j) for j in jobs]
            else:
                with mp.get_context("fork").Pool(processes) as pool:
                    parts = pool.map(_worker, jobs)
    finally:
        _G.clear()
    tot = parts[0]
    for p in parts[1:]:
        tot.DD += p.DD; tot.SplusD += p.SplusD; tot.ScrossD += p.ScrossD; tot.npairs += p.npairs
        if n_box:
            tot.DD_jk += p.DD_jk; tot.SplusD_jk += p.SplusD_jk; tot.npairs_jk += p.npairs_jk
    return tot, t_tree
