"""``MeasureIABox`` -- drop-in for the reference's periodic-box measurement API.

Same constructor, same ``measure_xi_w`` / ``measure_xi_multipoles`` signatures,
same validation errors, same output datasets (``measure_IA.py:10-262``); the
pair counting and everything after it run on the GPU through the C ABI
(``include/measure_ia_gb300.h``).

Backend choice mirrors the reference's dispatch (measure_IA.py:103-161):

* ``temp_file_path=False``           -> brute-force membership (every pair in
  the bin range) and the brute backends' datasets (with ``_sigmasq``);
* a path and ``num_nodes == 1``      -> KD-tree membership (r_min < d <= r_max)
  and the tree backends' datasets (``_sigmasq`` of zeros with jackknife);
* a path and ``num_nodes > 1``       -> KD-tree membership and the
  multiprocessing backends' datasets (the reference default for big runs).

The temporary file the reference writes is not needed: catalogues stay in
device memory.  Extra keyword arguments: ``precision`` ('fp64' for the plain
FP64 form, 'mixed' for FP32 pair arithmetic with FP64 edge re-tests),
``device``, ``autotune`` (search the launch knobs on first use of a
workload shape; results are identical, only speed changes) and
``launch_knobs`` (fixed knobs instead: a dict with any of ``cell_size``,
``cell_refine``, ``shapes_per_unit``, ``cell_size_los``, ``cell_refine_los``).
"""

from __future__ import annotations

import warnings

import numpy as np

from ._lib import MIA_ERR_OVERFLOW, MiaError
from .engine import PairCounter
from .output import norm_path, store_for
from .base import BaseHelpers, JackknifeCovariance
from .sim_info import SimInfo


def _all_finite(a) -> bool:
    """No NaN or infinity in ``a``: the dot product of ``a`` with itself is
    finite when every element is (one BLAS pass, no temporary array); only a
    non-finite result, which large finite elements can also give by
    overflowing, needs the element-wise test."""
    if hasattr(a, "is_cuda"):  # a torch tensor
        import torch
        return bool(torch.isfinite(a).all())
    a = np.ascontiguousarray(a, dtype=np.float64).ravel()
    with np.errstate(over="ignore", invalid="ignore"):
        if np.isfinite(np.dot(a, a)):
            return True
    return bool(np.all(np.isfinite(a)))


def _cube_root_exact(n):
    """(root, exact) like sympy.integer_nthroot(n, 3)."""
    r = int(round(n ** (1.0 / 3.0)))
    for c in (r - 1, r, r + 1):
        if c >= 0 and c ** 3 == n:
            return c, True
    while (r + 1) ** 3 <= n:
        r += 1
    while r ** 3 > n:
        r -= 1
    return r, False


def _centres(edges):
    return edges[:-1] + abs((edges[1:] - edges[:-1]) / 2.0)


class MeasureIABox(SimInfo, BaseHelpers, JackknifeCovariance):
    """Measurements of w_gg, w_g+ and multipoles (with jackknife covariance)
    for a periodic simulation box.  ``data`` keys: 'Position' (N_p, 3),
    'Position_shape_sample' (N_s, 3), 'Axis_Direction' (N_s, 2), 'LOS',
    'q' (N_s) and optionally 'weight', 'weight_shape_sample'."""

    def __init__(self, data, output_file_name, simulation=None, snapshot=None, separation_limits=[0.1, 20.0],
                 num_bins_r=8, num_bins_pi=20, pi_max=None, boxsize=None, periodicity=True, num_nodes=1,
                 precision="fp64", device=0, autotune=False, launch_knobs=None):
        SimInfo.__init__(self, simulation, snapshot, boxsize)
        self.data = data
        self.output_file_name = output_file_name
        self.periodicity = periodicity
        self.num_nodes = num_nodes
        self.precision = precision
        self.device = device
        self.autotune = autotune
        self.launch_knobs = dict(launch_knobs or {})
        try:
            self.Num_position = len(data["Position"])
            self.Num_shape = len(data["Position_shape_sample"])
        except Exception:
            self.Num_position = 0
            self.Num_shape = 0
        if self.Num_position > 0:  # default unit weights, written into the caller's dict like the reference
            if "weight" not in self.data:
                self.data["weight"] = np.ones(self.Num_position)
            if "weight_shape_sample" not in self.data:
                self.data["weight_shape_sample"] = np.ones(self.Num_shape)
        self.r_min = separation_limits[0]
        self.r_max = separation_limits[1]
        self.num_bins_r = num_bins_r
        self.num_bins_pi = num_bins_pi
        self.r_bins = np.logspace(np.log10(self.r_min), np.log10(self.r_max), self.num_bins_r + 1)
        if pi_max is None:
            if self.L_0p5 is None:
                raise ValueError("Both pi_max and boxsize are None. Provide input on one of them to determine the "
                                 "integration limit pi_max.")
            pi_max = self.L_0p5
        self.pi_max = pi_max
        self.pi_bins = np.linspace(-pi_max, pi_max, self.num_bins_pi + 1)
        self.mu_r_bins = np.linspace(-1, 1, self.num_bins_pi + 1)
        self.last_measurement = None

    # ------------------------------------------------------------------ inputs
    def _select(self, masks):
        """Masked inputs with the reference's weight-mask behaviour
        (measure_w_box_jk.py:685-712): without 'weight' keys in ``masks`` the
        first sum(mask) weights are used, and ``masks`` gains those keys."""
        d = self.data
        if masks is None:
            return {k: d[k] for k in ("Position", "Position_shape_sample", "Axis_Direction", "q", "weight",
                                      "weight_shape_sample")}
        out = {"Position": d["Position"][masks["Position"]],
               "Position_shape_sample": d["Position_shape_sample"][masks["Position_shape_sample"]],
               "Axis_Direction": d["Axis_Direction"][masks["Axis_Direction"]],
               "q": d["q"][masks["q"]]}
        if "weight" not in masks:
            m = np.ones(self.Num_position, dtype=bool)
            m[sum(masks["Position"]):self.Num_position] = 0
            masks["weight"] = m
        if "weight_shape_sample" not in masks:
            m = np.ones(self.Num_shape, dtype=bool)
            m[sum(masks["Position_shape_sample"]):self.Num_shape] = 0
            masks["weight_shape_sample"] = m
        out["weight"] = d["weight"][masks["weight"]]
        out["weight_shape_sample"] = d["weight_shape_sample"][masks["weight_shape_sample"]]
        return out

    def _validate(self, corr_type, num_jk, temp_file_path):
        L = 0
        if num_jk > 0:
            root, exact = _cube_root_exact(num_jk)
            if not exact:
                raise ValueError(
                    f"Use x^3 as input for num_jk, with x as an int. {float(int(num_jk ** (1. / 3)))},"
                    f"{num_jk ** (1. / 3)}")
            L = root
        if temp_file_path is False:
            temp_storage = False
        else:
            temp_storage = True
            if temp_file_path is None:
                raise ValueError("Input temp_file_path for faster computation. Do not want to save data "
                                 "temporarily? Input file_path_tree=False.")
        if self.data is not None and "RA" in self.data:
            print("Given data is lightcone, use measure_xi_w_lightcone method instead.")
        if corr_type not in ("both", "g+", "gg"):
            raise KeyError("Unknown value for corr_type. Choose from [g+, gg, both]")
        if not self.periodicity:
            raise NotImplementedError("only periodic boxes are supported (periodicity=True)")
        if not temp_storage:
            layout = "brute"
        elif self.num_nodes > 1:
            layout = "multiprocessing"
        else:
            layout = "tree"
        return L, layout

    # ------------------------------------------------------------------ run
    def _run(self, kind, dataset_name, corr_type, num_jk, temp_file_path, masks, ellipticity, rp_cut=None):
        if ellipticity not in ("distortion", "ellipticity"):
            raise ValueError("Invalid value for ellipticity. Choose 'distortion' or 'ellipticity'.")
        L_sub, layout = self._validate(corr_type, num_jk, temp_file_path)
        cat = self._select(masks)
        if len(cat["Position"]) == 0 or len(cat["Position_shape_sample"]) == 0:
            raise ValueError("empty position or shape sample")
        for key in ("weight", "weight_shape_sample", "q"):
            if not _all_finite(cat[key]):
                # the reference carries these into NaN sums (a NaN q or shape
                # weight makes its responsivity, and so every S+D bin, NaN)
                raise ValueError(f"'{key}' values must be finite")
        precision = self.precision
        if precision == "mixed" and not _all_finite(cat["Axis_Direction"]):
            # a non-finite axis gives e+ = ex = 0 in the reference (NaN -> 0,
            # measure_w_box_jk.py:599-600); the FP64 form repeats that exactly
            warnings.warn("mixed form: non-finite Axis_Direction, measuring in the FP64 form", RuntimeWarning)
            precision = "fp64"
        los = self.data["LOS"]
        args = dict(boxsize=self.boxsize, r_bins=self.r_bins, r_min=self.r_min, r_max=self.r_max,
                    p_bins=self.pi_bins if kind == "w" else self.mu_r_bins, los=los, l_subboxes=L_sub,
                    precision=precision, membership="brute" if layout == "brute" else "tree",
                    ellipticity=ellipticity, want_variance=(layout == "brute" and L_sub > 0),
                    volume=self.boxsize ** 3, rp_cut=0.0 if rp_cut is None else rp_cut, device=self.device)
        counter = PairCounter(kind, **args, **self.launch_knobs)
        dcat = counter.to_device(cat)
        if self.autotune:
            counter = counter.tuned(dcat)
        n_pos, n_shape = dcat["Position"].shape[0], dcat["Position_shape_sample"].shape[0]
        bufs = counter.allocate(n_pos, n_shape)
        try:
            counter.run(dcat, bufs)
        except MiaError as exc:
            # more pairs near a bin edge than the FP64 re-test queue holds:
            # the mixed form cannot finish exactly, the FP64 form always can
            if exc.code != MIA_ERR_OVERFLOW or precision != "mixed":
                raise
            warnings.warn("mixed form: edge re-test queue overflow, measuring in the FP64 form", RuntimeWarning)
            del bufs
            counter = PairCounter(kind, **{**args, "precision": "fp64"}, **self.launch_knobs)
            bufs = counter.allocate(n_pos, n_shape)
            counter.run(dcat, bufs)
        meas = counter.fetch(bufs)
        self.last_measurement = meas
        self._write(kind, dataset_name, corr_type, num_jk, meas, layout)
        return meas

    def measure_xi_w(self, dataset_name, corr_type, num_jk=0, temp_file_path=None, masks=None,
                     ellipticity="distortion", chunk_size=1000):
        """xi_gg, xi_g+ in (r_p, Pi) bins, w_gg and w_g+ and, with num_jk = x^3,
        the jackknife realisations and covariance (measure_IA.py:68-163)."""
        self._run("w", dataset_name, corr_type, num_jk, temp_file_path, masks, ellipticity)

    def measure_xi_multipoles(self, dataset_name, corr_type, num_jk=0, temp_file_path=None, masks=None, rp_cut=None,
                              ellipticity="distortion", chunk_size=1000):
        """xi_gg, xi_g+ in (r, mu_r) bins and their multipoles (l = 0 for gg,
        l = m = 2 for g+) with optional jackknife covariance
        (measure_IA.py:165-262).  Like the reference's public method, rp_cut is
        accepted but not applied (measure_IA.py:219-258)."""
        self._run("m", dataset_name, corr_type, num_jk, temp_file_path, masks, ellipticity, None)

    # ------------------------------------------------------------------ output
    def _write(self, kind, d, corr_type, num_jk, meas, layout):
        """Datasets in the reference's groups (measure_w_box_jk.py:816-854,
        measure_m_box_jk.py:857-894, measure_IA_base.py:454-668)."""
        f = store_for(self)
        sg = self.snap_group
        a = meas.arrays
        J = meas.J
        top = "w" if kind == "w" else "multipoles"
        rsuf, psuf = ("_rp", "_pi") if kind == "w" else ("_r", "_mu_r")
        rc = _centres(self.r_bins)
        pc = _centres(self.pi_bins if kind == "w" else self.mu_r_bins)
        jkg = f"{d}_jk{num_jk}" if J else ""
        with_sig = J and layout in ("tree", "brute")
        put = lambda grp, name, v: f.write(norm_path(sg, grp), name, v)
        g = f"{top}/xi_g_plus"
        put(g, d, a["xi_gp"]); put(g, d + "_SplusD", a["splusd"]); put(g, d + "_RR_g_plus", a["rr"])
        if with_sig:
            put(g, d + "_sigmasq", a["sigmasq"])
        put(g, d + rsuf, rc); put(g, d + psuf, pc)
        for i in range(J):
            gj = f"{top}/xi_g_plus/{jkg}"
            put(gj, f"{d}_{i}", a["xi_gp_jk"][i]); put(gj, f"{d}_{i}_SplusD", a["splusd_jk"][i])
            put(gj, f"{d}_{i}_RR", a["rr_jk"][i]); put(gj, f"{d}_{i}{rsuf}", rc); put(gj, f"{d}_{i}{psuf}", pc)
        g = f"{top}/xi_g_cross/{jkg}"
        put(g, d + "_ScrossD", a["scrossd"]); put(g, d, a["xi_gx"]); put(g, d + "_RR_g_cross", a["rr"])
        if with_sig:
            put(g, d + "_sigmasq", a["sigmasq"])
        put(g, d + rsuf, rc); put(g, d + psuf, pc)
        g = f"{top}/xi_gg"
        put(g, d, a["xi_gg"]); put(g, d + "_DD", a["DD"]); put(g, d + "_RR_gg", a["rr"])
        if with_sig:
            put(g, d + "_sigmasq", a["sigmasq"])
        put(g, d + rsuf, rc); put(g, d + psuf, pc)
        for i in range(J):
            gj = f"{top}/xi_gg/{jkg}"
            put(gj, f"{d}_{i}", a["xi_gg_jk"][i]); put(gj, f"{d}_{i}_DD", a["dd_jk"][i])
            put(gj, f"{d}_{i}_RR", a["rr_jk"][i]); put(gj, f"{d}_{i}{rsuf}", rc); put(gj, f"{d}_{i}{psuf}", pc)
        types = {"both": [("g_plus", "gp"), ("gg", "gg")], "g+": [("g_plus", "gp")], "gg": [("gg", "gg")]}[corr_type]
        for name, key in types:
            dst = f"w_{name}" if kind == "w" else f"multipoles_{name}"
            put(dst, d + rsuf, rc)
            put(dst, d, a[f"proj_{key}"])
            for i in range(J):
                put(f"{dst}/{jkg}", f"{d}_{i}{rsuf}", rc)
                put(f"{dst}/{jkg}", f"{d}_{i}", a[f"proj_{key}_jk"][i])
            if J:
                put(dst, f"{d}_mean_{J}", a[f"mean_{key}"])
                put(dst, f"{d}_jackknife_{J}", a[f"std_{key}"])
                put(dst, f"{d}_jackknife_cov_{J}", a[f"cov_{key}"])
        f.flush()
