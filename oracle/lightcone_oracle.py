"""CPU oracle for MeasureIA's lightcone pair counts (MeasureIALightcone).

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; only
``tests/`` use it, as the checker.

A numpy restatement of the reference's lightcone path (``src/measureia`` of
MarloesvL/measure_IA):

* the four brute-force pair counters, position by position with the same
  numpy operation sequence per pair (``measure_w_lightcone.py:45-214``,
  ``:216-343``; ``measure_m_lightcone.py:45-219``, ``:221-363``), vectorised
  over blocks of positions -- the elementwise arithmetic, and therefore every
  bin decision, is the reference's; only the order of the histogram sums
  differs;
* the estimator (``measure_IA_base.py:670-743``), the Pi integration and
  multipoles (``measure_IA_base.py:515-668``);
* the whole ``measure_xi_w`` / ``measure_xi_multipoles`` flow of
  ``MeasureIALightcone`` (``measure_IA.py:336-688``, ``:690-1060``) with the
  jackknife realisations of the pooled driver
  (``measure_jackknife.py:265-484``: every patch re-counted with that patch
  masked out) and the covariance (``measure_jackknife.py:172-263``).

Redshifts become distances through a caller-supplied function
``chi(a)``, the role pyccl's ``comoving_radial_distance`` plays in the
reference.

Pinned by ``tests/golden/lc_*.npz``: outputs of the reference itself
(``tests/golden/make_golden.py``).
"""

from __future__ import annotations

import numpy as np

from oracle.ia_oracle import bin_centres

_BLOCK = 64


class LcBinning:
    """Binning of MeasureIABase (measure_IA_base.py:155-167) for lightcone data."""

    def __init__(self, r_min, r_max, num_bins_r, num_bins_pi, pi_max):
        if pi_max is None:
            raise ValueError("Both pi_max and boxsize are None. Provide input on one of them to determine the "
                             "integration limit pi_max.")
        self.r_min, self.r_max = r_min, r_max
        self.num_bins_r, self.num_bins_pi = num_bins_r, num_bins_pi
        self.r_bins = np.logspace(np.log10(r_min), np.log10(r_max), num_bins_r + 1)
        self.pi_bins = np.linspace(-pi_max, pi_max, num_bins_pi + 1)
        self.mu_r_bins = np.linspace(-1, 1, num_bins_pi + 1)


# ----------------------------------------------------------------------------
# input selection (measure_w_lightcone.py:73-107; measure_m_lightcone.py alike)
# ----------------------------------------------------------------------------

def select(data, masks, with_shapes, num_position, num_shape):
    keys = ["Redshift", "Redshift_shape_sample", "RA", "RA_shape_sample", "DEC", "DEC_shape_sample"]
    if with_shapes:
        keys += ["e1", "e2"]
    if masks is None:
        out = {k: data[k] for k in keys}
        out["weight"], out["weight_shape_sample"] = data["weight"], data["weight_shape_sample"]
        return out
    out = {k: data[k][masks[k]] for k in keys}
    if "weight" not in masks:
        masks["weight"] = np.ones(num_position, dtype=bool)
    if "weight_shape_sample" not in masks:
        masks["weight_shape_sample"] = np.ones(num_shape, dtype=bool)
    out["weight"] = data["weight"][masks["weight"]]
    out["weight_shape_sample"] = data["weight_shape_sample"][masks["weight_shape_sample"]]
    return out


# ----------------------------------------------------------------------------
# pair counters
# ----------------------------------------------------------------------------

def _distances(sel, chi, h, over_h):
    los_p = chi(1 / (1 + sel["Redshift"]))
    los_s = chi(1 / (1 + sel["Redshift_shape_sample"]))
    if over_h:
        los_p = los_p * h
        los_s = los_s * h
    return los_p, los_s


def _axis_terms(sel):
    """measure_w_lightcone.py:127-133"""
    e1, e2 = sel["e1"], sel["e2"]
    theta = 1. / 2 * np.arctan2(e2, e1)
    semi = np.array([np.cos(theta), np.sin(theta)])
    length = np.sqrt(np.sum(semi ** 2, axis=0))
    axis = semi / length
    e = np.sqrt(e1 ** 2 + e2 ** 2)
    phi_axis = np.arctan2(axis[1], axis[0])
    return e, phi_axis


def pair_counts(kind, with_shapes, b: LcBinning, sel, chi, h, over_h=False, rp_cut=None, empty_to_one=True):
    """(S+D, SxD, DD) of one brute-force counter, DD with empty bins set to 1
    as the reference leaves them (``empty_to_one=False`` keeps the raw sums);
    S+D and SxD are None when ``with_shapes`` is False.  An index past the
    last bin raises IndexError, as np.add.at does in the reference."""
    RA, DEC = sel["RA"], sel["DEC"]
    RA_s, DEC_s = sel["RA_shape_sample"], sel["DEC_shape_sample"]
    weight, weight_shape = sel["weight"], sel["weight_shape_sample"]
    los_p, los_s = _distances(sel, chi, h, over_h)
    nr, npi = b.num_bins_r, b.num_bins_pi
    dlog = (np.log10(b.r_max) - np.log10(b.r_min)) / nr
    DD = np.zeros((nr, npi))
    SP = np.zeros((nr, npi)) if with_shapes else None
    SX = np.zeros((nr, npi)) if with_shapes else None
    if with_shapes:
        e, phi_axis = _axis_terms(sel)
    if kind == "m":
        rp_cut = 0.0 if rp_cut is None else rp_cut
        dmu = 2.0 / npi
    else:
        dpi = (b.pi_bins[-1] - b.pi_bins[0]) / npi
    for n0 in range(0, len(RA), _BLOCK):
        n = np.arange(n0, min(len(RA), n0 + _BLOCK))[:, None]
        LOS = los_s[None, :] - los_p[n]
        dra = (RA_s[None, :] - RA[n]) / 180 * np.pi
        ddec = (DEC_s[None, :] - DEC[n]) / 180 * np.pi
        dx = dra * los_p[n] * np.cos(DEC[n] / 180 * np.pi)
        dy = ddec * los_p[n]
        projected = np.array([dx, dy])
        if kind == "m":
            separation = np.array([dx, dy, LOS])
        if over_h:
            projected *= h
        with np.errstate(invalid="ignore", divide="ignore"):
            if kind == "w":
                sep_len = np.sqrt(np.sum(projected ** 2, axis=0))
                mask = (sep_len >= b.r_bins[0]) * (sep_len < b.r_bins[-1]) * (LOS >= b.pi_bins[0]) * (
                    LOS < b.pi_bins[-1])
                ind_r = np.floor(np.log10(sep_len[mask]) / dlog - np.log10(b.r_bins[0]) / dlog).astype(int)
                ind_p = np.floor(LOS[mask] / dpi - b.pi_bins[0] / dpi).astype(int)
                if with_shapes:   # only this counter clamps (measure_w_lightcone.py:170-173)
                    ind_r[ind_r == nr] = nr - 1
                    ind_p[ind_p == npi] = npi - 1
                rp_len = sep_len
            else:
                rp_len = np.sqrt(np.sum(projected ** 2, axis=0))
                sep_len = np.sqrt(np.sum(separation ** 2, axis=0))
                mu_r = LOS / sep_len
                mask = (rp_len > rp_cut) * (sep_len >= b.r_bins[0]) * (sep_len < b.r_bins[-1])
                ind_r = np.floor(np.log10(sep_len[mask]) / dlog - np.log10(b.r_bins[0]) / dlog).astype(int)
                ind_p = np.floor(mu_r[mask] / dmu - b.mu_r_bins[0] / dmu).astype(int)
            ww = (weight[n] * np.ones_like(dx))[mask] * np.broadcast_to(weight_shape[None, :], dx.shape)[mask]
            if with_shapes:
                sep_dir = projected / rp_len
                phi_sep = np.arctan2(sep_dir[1], sep_dir[0])
                phi = phi_axis[None, :] - phi_sep
                e_plus, e_cross = -e[None, :] * np.cos(2 * phi), -e[None, :] * np.sin(2 * phi)
                e_plus[np.isnan(e_plus)] = 0.0
                e_cross[np.isnan(e_cross)] = 0.0
        np.add.at(DD, (ind_r, ind_p), ww)
        if with_shapes:
            np.add.at(SP, (ind_r, ind_p), ww * e_plus[mask])
            np.add.at(SX, (ind_r, ind_p), ww * e_cross[mask])
    if empty_to_one:
        DD[np.where(DD == 0)] = 1
    return SP, SX, DD


# ----------------------------------------------------------------------------
# post-processing
# ----------------------------------------------------------------------------

def w_integral(b: LcBinning, xi):
    """measure_IA_base.py:553-562"""
    dpi = b.pi_bins[1:] - b.pi_bins[:-1]
    return np.sum(xi * abs(np.array([dpi] * len(xi[:, 0]))), axis=1)


def multipole(b: LcBinning, xi, l):
    """measure_IA_base.py:628-655 for (l, m) = (2, 2) and (0, 0):
    P_2^2(mu) = 3 (1 - mu^2), P_0^0 = 1 (scipy's lpmn convention)."""
    import math
    mu_c = bin_centres(b.mu_r_bins)
    leg = 3.0 * (1.0 - mu_c ** 2) if l == 2 else np.ones_like(mu_c)
    dmu = b.mu_r_bins[1:] - b.mu_r_bins[:-1]
    fac = (2 * l + 1) / 2.0 * math.factorial(0) / math.factorial(2 * l)
    return np.sum(fac * np.array([leg] * xi.shape[0]) * xi * np.array([dmu] * xi.shape[0]), axis=1)


def covariance(reals):
    """mean, std and covariance with the (n-1)/n factor (measure_jackknife.py:237-250)."""
    reals = np.asarray(reals)
    n, nr = reals.shape
    mean = np.zeros(nr)
    for x in reals:
        mean += x
    mean /= n
    cov = np.zeros((nr, nr))
    std = np.zeros(nr)
    for x in reals:
        std += (x - mean) ** 2
        for i in range(nr):
            cov[:, i] += (x - mean) * (x[i] - mean[i])
    std *= (n - 1) / n
    return mean, np.sqrt(std), cov * ((n - 1) / n)


def estimator(corr_type, IA_estimator, SpD, SpR, DD, SR, RD, RR, ns):
    """measure_IA_base.py:670-743: returns (xi_g+, xi_gg), None where not formed."""
    gp = gg = None
    if IA_estimator == "clusters":
        SR = SR * (ns["D"] / ns["R_D"])
        if corr_type in ("g+", "both"):
            SpR = SpR * (ns["D"] / ns["R_D"])
            gp = SpD / DD - SpR / SR
        if corr_type in ("gg", "both"):
            RD = RD * (ns["S"] / ns["R_S"])
            RR = RR * ((ns["S"] / ns["R_S"]) * (ns["D"] / ns["R_D"]))
            gg = (DD - RD - SR) / RR - 1
    else:
        RR = RR * ((ns["S"] / ns["R_S"]) * (ns["D"] / ns["R_D"]))
        if corr_type in ("g+", "both"):
            SpR = SpR * (ns["D"] / ns["R_D"])
            gp = (SpD - SpR) / RR
        if corr_type in ("gg", "both"):
            RD = RD * (ns["S"] / ns["R_S"])
            SR = SR * (ns["D"] / ns["R_D"])
            gg = (DD - RD - SR) / RR + 1
    return gp, gg


# ----------------------------------------------------------------------------
# the whole measurement
# ----------------------------------------------------------------------------

def _combo(data_dir, randoms, pos_from, shape_from, with_shapes):
    src = {"D": data_dir, "R": randoms}
    p, s = src[pos_from], src[shape_from]
    out = {"Redshift": p["Redshift"], "Redshift_shape_sample": s["Redshift_shape_sample"],
           "RA": p["RA"], "RA_shape_sample": s["RA_shape_sample"], "DEC": p["DEC"],
           "DEC_shape_sample": s["DEC_shape_sample"], "weight": p["weight"],
           "weight_shape_sample": s["weight_shape_sample"]}
    if with_shapes:
        out["e1"], out["e2"] = s["e1"], s["e2"]
    return out


def measure(kind, IA_estimator, dataset_name, corr_type, data, randoms, b: LcBinning, chi, h, jk_patches=None,
            measure_cov=True, masks=None, masks_randoms=None, over_h=False, rp_cut=None):
    """{hdf5 path: array} as ``MeasureIALightcone.measure_xi_w`` (kind 'w')
    or ``measure_xi_multipoles`` (kind 'm') writes them with num_nodes > 1
    (the pooled realisation driver)."""
    if IA_estimator not in ("clusters", "galaxies"):
        raise KeyError("Unknown input for IA_estimator, choose from [clusters, galaxies].")
    if randoms is None:
        raise KeyError("This version does not work yet, add randoms." if IA_estimator == "clusters"
                       else "No randoms given. Please provide input.")
    top = "w" if kind == "w" else "multipoles"
    rs, ps = ("_rp", "_pi") if kind == "w" else ("_r", "_mu_r")
    rc = bin_centres(b.r_bins)
    pc = bin_centres(b.pi_bins if kind == "w" else b.mu_r_bins)
    num_position, num_shape = len(data["RA"]), len(data["RA_shape_sample"])
    one_random = "RA_shape_sample" not in randoms
    if one_random:
        randoms["RA_shape_sample"] = randoms["RA"]
        randoms["DEC_shape_sample"] = randoms["DEC"]
        randoms["Redshift_shape_sample"] = randoms["Redshift"]
    if "weight" not in randoms:
        randoms["weight"] = np.ones(len(randoms["RA"]))
    if "weight_shape_sample" not in randoms:
        randoms["weight_shape_sample"] = randoms["weight"] if one_random else np.ones(len(randoms["RA_shape_sample"]))
    if measure_cov:
        if jk_patches is None:
            raise ValueError("Set calc_errors to False, or provide either jk_patches or num_jk input.")
        if one_random:
            jk_patches["randoms_position"] = jk_patches["randoms"]
            jk_patches["randoms_shape"] = jk_patches["randoms"]
    data.setdefault("weight", np.ones(len(data["RA"])))
    data.setdefault("weight_shape_sample", np.ones(len(data["RA_shape_sample"])))
    ns = {"D": len(data["RA"]) if masks is None else len(data["RA"][masks["RA"]]),
          "S": len(data["RA_shape_sample"]) if masks is None else len(data["RA_shape_sample"][masks["RA_shape_sample"]]),
          "R_D": len(randoms["RA"]) if masks_randoms is None else len(randoms["RA"][masks_randoms["RA"]]),
          "R_S": len(randoms["RA_shape_sample"]) if masks_randoms is None
          else len(randoms["RA_shape_sample"][masks_randoms["RA_shape_sample"]])}
    out = {}

    def put(path, v):
        out[path] = np.asarray(v)

    def counter(pos_from, shape_from, with_shapes, m, name, suffix, group=""):
        sel = select(_combo(data, randoms, pos_from, shape_from, with_shapes), m, with_shapes, num_position,
                     num_shape)
        SP, SX, DD = pair_counts(kind, with_shapes, b, sel, chi, h, over_h, rp_cut)
        g = f"{group}/" if group else ""
        if with_shapes:
            put(f"{top}/xi_g_plus/{g}{name}", SP / DD)
            put(f"{top}/xi_g_plus/{g}{name}_SplusD", SP)
            put(f"{top}/xi_g_cross/{g}{name}_ScrossD", SX)
            put(f"{top}/xi_gg/{g}{name}_DD", DD)
            for grp in ("xi_g_plus", "xi_g_cross", "xi_gg"):
                put(f"{top}/{grp}/{g}{name}{rs}", rc)
                put(f"{top}/{grp}/{g}{name}{ps}", pc)
        else:
            put(f"{top}/xi_gg/{g}{name}{suffix}", DD)
            put(f"{top}/xi_gg/{g}{name}{rs}", rc)
            put(f"{top}/xi_gg/{g}{name}{ps}", pc)
        return SP, DD

    d, dr = dataset_name, f"{dataset_name}_randoms"
    if corr_type in ("g+", "both"):
        counter("D", "D", True, masks, d, "")
        counter("R", "D", True, masks, dr, "")
    if corr_type == "gg":
        counter("D", "D", False, masks, d, "_DD")
        counter("R", "D", False, masks, d, "_SR")
    if corr_type in ("gg", "both"):
        counter("D", "R", False, masks, d, "_RD")
    if IA_estimator == "galaxies" or corr_type in ("gg", "both"):
        counter("R", "R", False, masks, d, "_RR")

    def obs(name, rname, nsi, grp="", grp_r=""):
        g = f"{grp}/" if grp else ""
        gr = f"{grp_r}/" if grp_r else ""
        get = lambda p: out[f"{top}/{p}"]
        SpD = SpR = SR = RD = RR = None
        if corr_type in ("g+", "both"):
            SpD = get(f"xi_g_plus/{g}{name}_SplusD")
            SpR = get(f"xi_g_plus/{gr}{rname}_SplusD")
        DD = get(f"xi_gg/{g}{name}_DD")
        if IA_estimator == "clusters" or corr_type in ("gg", "both"):
            SR = get(f"xi_gg/{g}{name}_SR") if corr_type == "gg" else get(f"xi_gg/{gr}{rname}_DD")
        if corr_type in ("gg", "both"):
            RD = get(f"xi_gg/{g}{name}_RD")
        if IA_estimator == "galaxies" or corr_type in ("gg", "both"):
            RR = get(f"xi_gg/{g}{name}_RR")
        gp, gg = estimator(corr_type, IA_estimator, SpD, SpR, DD, SR, RD, RR, nsi)
        if gp is not None:
            put(f"{top}/xi_g_plus/{g}{name}", gp)
        if gg is not None:
            put(f"{top}/xi_gg/{g}{name}", gg)

    def integrate(name, grp=""):
        g = f"{grp}/" if grp else ""
        todo = {"both": [("g_plus", 2), ("gg", 0)], "g+": [("g_plus", 2)], "gg": [("gg", 0)]}[corr_type]
        for suff, l in todo:
            xi = out[f"{top}/xi_{suff}/{g}{name}"]
            val = w_integral(b, xi) if kind == "w" else multipole(b, xi, l)
            dst = f"w_{suff}" if kind == "w" else f"multipoles_{suff}"
            put(f"{dst}/{g}{name}{rs}", rc)
            put(f"{dst}/{g}{name}", val)

    obs(d, dr, ns)
    integrate(d)
    if not measure_cov:
        return out

    # jackknife realisations (measure_jackknife.py:265-484), then the covariance
    nsj = {}

    def realisations(pos_from, shape_from, patches_pos, patches_shape, count_pairs, name, suffix, names):
        lo, hi = int(min(patches_pos)), int(max(patches_pos))
        n_p = hi - lo + 1
        grp = f"{name}_jk{n_p}"
        for i in range(lo, hi + 1):
            mp = patches_pos != i
            msh = patches_shape != i
            # only the S+D and S+R realisations get the masks (measure_IA.py:562-590 pass
            # masks=masks; the count realisations at :610-680 do not)
            if masks is not None and not count_pairs:
                mp = mp * masks["Redshift"]
                msh = msh * masks["Redshift_shape_sample"]
            nsj.setdefault(f"{i}", {})[names[0]] = sum(msh)
            nsj[f"{i}"][names[1]] = sum(mp)
            mt = {"Redshift": mp, "Redshift_shape_sample": msh, "RA": mp, "RA_shape_sample": msh, "DEC": mp,
                  "DEC_shape_sample": msh, "e1": msh, "e2": msh, "weight": mp, "weight_shape_sample": msh}
            sel = select(_combo(data, randoms, pos_from, shape_from, not count_pairs), mt, not count_pairs,
                         num_position, num_shape)
            SP, _, DD = pair_counts(kind, not count_pairs, b, sel, chi, h, over_h, rp_cut)
            if count_pairs:
                put(f"{top}/xi_gg/{grp}/{name}_{i}{suffix}", DD)
                put(f"{top}/xi_gg/{grp}/{name}_{i}{rs}", rc)
                put(f"{top}/xi_gg/{grp}/{name}_{i}{ps}", pc)
            else:
                for sub, v in (("xi_g_plus", ("SplusD", SP)), ("xi_gg", ("DD", DD))):
                    put(f"{top}/{sub}/{grp}/{name}_{i}_{v[0]}", v[1])
                    put(f"{top}/{sub}/{grp}/{name}_{i}{rs}", rc)
                    put(f"{top}/{sub}/{grp}/{name}_{i}{ps}", pc)

    jp = jk_patches
    if corr_type in ("g+", "both"):
        realisations("D", "D", jp["position"], jp["shape"], False, d, "", ["S", "D"])
        realisations("R", "D", jp["randoms_position"], jp["shape"], False, dr, "", ["S", "R_D"])
    if corr_type == "gg":
        realisations("D", "D", jp["position"], jp["shape"], True, d, "_DD", ["S", "D"])
        realisations("R", "D", jp["randoms_position"], jp["shape"], True, d, "_SR", ["S", "R_D"])
    if corr_type in ("gg", "both"):
        realisations("D", "R", jp["position"], jp["randoms_shape"], True, d, "_RD", ["R_S", "D"])
    if IA_estimator == "galaxies" or corr_type in ("gg", "both"):
        realisations("R", "R", jp["randoms_position"], jp["randoms_shape"], True, d, "_RR", ["R_S", "R_D"])

    lo, hi = int(min(jp["shape"])), int(max(jp["shape"]))
    n_p = hi - lo + 1
    grp, grp_r = f"{d}_jk{n_p}", f"{dr}_jk{n_p}"
    if corr_type == "gg":
        # the estimator opens the randoms realisation group, which only the
        # g+ flow creates (measure_IA_base.py:703): the reference stops here
        raise KeyError(f"Unable to open object '{grp_r}' in '{top}/xi_gg'")
    for i in range(lo, hi + 1):
        obs(f"{d}_{i}", f"{dr}_{i}", nsj[f"{i}"], grp, grp_r)
        integrate(f"{d}_{i}", grp)
    suffs = {"both": ["g_plus", "gg"], "g+": ["g_plus"], "gg": ["gg"]}[corr_type]
    for suff in suffs:
        dst = f"w_{suff}" if kind == "w" else f"multipoles_{suff}"
        reals = [out[f"{dst}/{grp}/{d}_{i}"] for i in range(lo, hi + 1)]
        mean, std, cov = covariance(reals)
        put(f"{dst}/{d}_mean_{n_p}", mean)
        put(f"{dst}/{d}_jackknife_{n_p}", std)
        put(f"{dst}/{d}_jackknife_cov_{n_p}", cov)
    return out
