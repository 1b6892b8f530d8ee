"""Seeded synthetic galaxy catalogues in a periodic box.

The catalogues are the inputs ``MeasureIABox`` expects (``Position``,
``Position_shape_sample``, ``Axis_Direction``, ``q``, ``weight``,
``weight_shape_sample``, ``LOS``).  They stand in for simulation catalogues:

* ``uniform_catalog`` -- uniform positions, shape sample = position sample,
  projected axis angle uniform in [0, pi), axis ratio q uniform in [0.2, 1],
  unit weights (10,000 galaxies in a 205 Mpc/h box is the CPU-sized case).
* ``neyman_scott_catalog`` -- clustered: uniform parent centres, Poisson
  children with Gaussian offsets wrapped into the box, shape sample a random
  subset, axis pointing to the parent in the projected plane plus von Mises
  noise, q ~ Beta(4, 2), lognormal weights.
* ``inject_edge_pairs`` -- adds pairs whose separations sit on bin edges,
  on the neighbour-search radii and on jackknife sub-box faces.

Coordinates are float64 in [0, L); a value that wraps to exactly L is set to 0.
"""

from __future__ import annotations

import numpy as np


def _wrap(x, L):
    x = np.mod(x, L)
    x[x >= L] = 0.0
    return x


def uniform_catalog(n, L, seed, los=2):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0.0, L, (n, 3))
    pos[pos >= L] = 0.0
    ang = rng.uniform(0.0, np.pi, n)
    axis = np.c_[np.cos(ang), np.sin(ang)]
    q = rng.uniform(0.2, 1.0, n)
    return {"Position": pos, "Position_shape_sample": pos.copy(), "Axis_Direction": axis, "LOS": los,
            "q": q, "weight": np.ones(n), "weight_shape_sample": np.ones(n)}


def neyman_scott_catalog(n_centres, L, n_shape, seed, mean_children=50, sigma=1.0, kappa=2.0,
                         weight_sigma=0.3, los=2):
    """Clustered catalogue.  ``n_shape`` galaxies drawn without replacement
    from the positions form the shape sample (their weights go with them)."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.0, L, (n_centres, 3))
    nchild = rng.poisson(mean_children, n_centres)
    parent = np.repeat(np.arange(n_centres), nchild)
    pos = _wrap(centres[parent] + rng.normal(0.0, sigma, (len(parent), 3)), L)
    n = len(pos)
    w = np.exp(rng.normal(0.0, weight_sigma, n))
    n_shape = min(n_shape, n)
    pick = np.sort(rng.choice(n, n_shape, replace=False))
    spos = pos[pick]
    proj = [d for d in range(3) if d != los]
    d = centres[parent[pick]][:, proj] - spos[:, proj]
    d[d > L / 2] -= L
    d[d < -L / 2] += L
    ang = np.arctan2(d[:, 1], d[:, 0]) + rng.vonmises(0.0, kappa, n_shape)
    axis = np.c_[np.cos(ang), np.sin(ang)]
    q = rng.beta(4.0, 2.0, n_shape)
    return {"Position": pos, "Position_shape_sample": spos.copy(), "Axis_Direction": axis, "LOS": los,
            "q": q, "weight": w, "weight_shape_sample": w[pick].copy()}


def inject_edge_pairs(data, L, seed, r_edges, pi_edges, n_sub=3, n_each=6):
    """Return a copy of a catalogue whose shape sample equals its position
    sample, with extra galaxies placed so that some pair separations fall on
    (or within an ulp of) the given r-bin edges, Pi-bin edges, and points lie
    on jackknife sub-box faces or at coordinate 0."""
    rng = np.random.default_rng(seed)
    pts = [data["Position"]]
    L_sub = L / 2.0 * 2.0 / n_sub
    extra = []
    for edge in r_edges:
        for _ in range(n_each):
            s = rng.uniform(30.0, L - 30.0, 3)
            th = rng.uniform(0, 2 * np.pi) if rng.uniform() < 0.5 else 0.0
            p = s - np.array([edge * np.cos(th), edge * np.sin(th), rng.uniform(-5, 5)])
            extra += [s, p]
    for edge in pi_edges:
        for _ in range(n_each):
            s = rng.uniform(30.0, L - 30.0, 3)
            p = s - np.array([rng.uniform(0.5, 5.0), 0.0, edge])
            extra += [s, p]
    for k in range(n_sub + 1):
        for _ in range(n_each):
            s = rng.uniform(0.0, L, 3)
            s[rng.integers(0, 3)] = k * L_sub if k < n_sub else 0.0
            extra.append(s)
    for _ in range(n_each):
        s = rng.uniform(0.0, L, 3)
        s[rng.integers(0, 3)] = 0.0
        extra.append(s)
    extra = _wrap(np.array(extra), L)
    pos = np.concatenate(pts + [extra])
    n_new = len(extra)
    ang = np.concatenate([np.arctan2(data["Axis_Direction"][:, 1], data["Axis_Direction"][:, 0]),
                          rng.uniform(0, np.pi, n_new)])
    # a few axes exactly along x and y so that |cos phi| = 1 occurs
    ang[-n_new::7] = 0.0
    q = np.concatenate([data["q"], rng.uniform(0.2, 1.0, n_new)])
    n = len(pos)
    return {"Position": pos, "Position_shape_sample": pos.copy(), "Axis_Direction": np.c_[np.cos(ang), np.sin(ang)],
            "LOS": data.get("LOS", 2), "q": q, "weight": np.ones(n), "weight_shape_sample": np.ones(n)}


def add_edge_pairs(data, L, seed, r_edges, pi_edges, n_pairs):
    """Append ``n_pairs`` (shape, position) pairs whose projected separation
    equals an r-bin edge, or whose line-of-sight separation equals a Pi-bin
    edge, up to the rounding of the FP64 subtraction.  The new shapes go to
    the shape sample, the new positions to the position sample (LOS = z)."""
    rng = np.random.default_rng(seed)
    edges = [("r", float(x)) for x in r_edges] + [("p", float(x)) for x in pi_edges]
    s_new, p_new = [], []
    for k in range(n_pairs):
        kind, edge = edges[k % len(edges)]
        s = rng.uniform(25.0, L - 25.0, 3)
        if kind == "r":
            th = rng.uniform(0.0, 2 * np.pi)
            off = np.array([edge * np.cos(th), edge * np.sin(th), rng.uniform(-15.0, 15.0)])
        else:
            rp = rng.uniform(0.2, 15.0)
            th = rng.uniform(0.0, 2 * np.pi)
            off = np.array([rp * np.cos(th), rp * np.sin(th), edge])
        s_new.append(s)
        p_new.append(s - off)
    s_new = _wrap(np.array(s_new), L)
    p_new = _wrap(np.array(p_new), L)
    ang = rng.uniform(0.0, np.pi, n_pairs)
    out = dict(data)
    out["Position"] = np.concatenate([data["Position"], p_new])
    out["weight"] = np.concatenate([data["weight"], np.ones(n_pairs)])
    out["Position_shape_sample"] = np.concatenate([data["Position_shape_sample"], s_new])
    out["Axis_Direction"] = np.concatenate([data["Axis_Direction"], np.c_[np.cos(ang), np.sin(ang)]])
    out["q"] = np.concatenate([data["q"], rng.beta(4.0, 2.0, n_pairs)])
    out["weight_shape_sample"] = np.concatenate([data["weight_shape_sample"], np.ones(n_pairs)])
    return out
