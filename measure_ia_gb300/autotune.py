"""Autotuner for the pair-count launch geometry.

Five knobs change speed but never results:

* ``cell_size`` -- shape-cell side in the projected plane.  Narrow cells
  leave fewer positions outside r_p <= r_max among the candidates of a shape;
* ``cell_size_los`` -- shape-cell side along the line of sight (0 = equal to
  ``cell_size``).  Long cells keep many shapes per cell when the projected
  side is small; the line-of-sight window over the staged shapes removes the
  out-of-range ones cheaply;
* ``cell_refine`` / ``cell_refine_los`` -- position cells per shape cell in
  the plane / along the line of sight (0 = equal to ``cell_refine``);
* ``shapes_per_unit`` -- shapes staged per work unit.

``tune`` times candidates on the caller's own device-resident catalogue
(CUDA events, one warm-up and one timed run each) by coordinate descent from
a cubic-cell start, keeps the fastest, and stores the choice in a JSON cache
keyed by the workload shape, so later measurements of the same shape reuse it.
A candidate that fails (workspace too large, edge queue overflow) is skipped.

The cache file is ``$MIA_TUNE_CACHE`` or ``~/.cache/measure_ia_gb300/tune.json``.
"""

from __future__ import annotations

import json
import math
import os

KNOBS = ("cell_size", "cell_refine", "shapes_per_unit", "cell_size_los", "cell_refine_los")
DEFAULT = {"cell_size": 0.0, "cell_refine": 0, "shapes_per_unit": 0, "cell_size_los": 0.0, "cell_refine_los": 0}
_VERSION = "g9"  # short pair path (fixed histogram stride), per-region work units, long-cell family


def cache_path():
    return os.environ.get("MIA_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "measure_ia_gb300",
                                                            "tune.json")


def workload_key(kind, precision, n_pos, n_shape, boxsize, n_r, n_p, range_proj, range_los, l_subboxes, membership,
                 device_name=""):
    """Sizes enter as powers of two (a doubling of the catalogue is a new shape)."""
    lp = int(round(math.log2(max(n_pos, 1))))
    ls = int(round(math.log2(max(n_shape, 1))))
    return "|".join(str(x) for x in (_VERSION, device_name, kind, precision, lp, ls, round(boxsize, 3), n_r, n_p,
                                     round(range_proj, 4), round(range_los, 4), l_subboxes, membership))


def load_cache(path=None):
    path = path or cache_path()
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def store(key, choice, path=None):
    path = path or cache_path()
    data = load_cache(path)
    data[key] = choice
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def candidates(range_proj, range_los=None):
    """Search axes: projected sides, line-of-sight sides, refinements, unit sizes."""
    range_los = range_proj if range_los is None else range_los
    # (cells as wide as the reach or 2/3 of it: a small catalogue with one or
    # two shapes per cell loses more to per-unit work than to extra candidates)
    sides = [range_proj / k for k in (1.0, 1.5, 2.0, 3.0, 4.0, 5.0, 6.0, 8.0)]
    los_sides = [range_los * f for f in (0.5, 1.0, 2.0)]
    return sides, los_sides, (1, 2, 3), (64, 128, 256)


def tune(make_counter, dcat, range_proj, range_los=None, key=None, path=None, log=None, run=None):
    """Return the fastest knob set (a dict over KNOBS, plus its time in 'ms').

    ``make_counter(**knobs)`` builds a PairCounter for the knobs; ``dcat`` is
    the device-resident catalogue.  ``run(**knobs)``, when given, replaces the
    single measurement as the thing timed: it returns a callable that runs
    the whole job once (e.g. a batch of catalogues).  With ``key`` the result
    is cached."""
    import torch

    from ._lib import MiaError

    if key is not None:
        hit = load_cache(path).get(key)
        if hit and all(k in hit for k in KNOBS):
            return hit
    timings = {}
    failures = []

    def norm(knobs):
        return tuple((k, float(knobs[k]) if k.startswith("cell_size") else int(knobs[k])) for k in KNOBS)

    def job(knobs):
        if run is not None:
            return run(**knobs)
        n_pos = dcat["Position"].shape[0]
        n_shape = dcat["Position_shape_sample"].shape[0]
        pc = make_counter(**knobs)
        bufs = pc.allocate(n_pos, n_shape)
        return lambda: pc.run(dcat, bufs)

    def time_one(knobs):
        tkey = norm(knobs)
        if tkey in timings:
            return timings[tkey]
        go = None
        try:
            go = job(knobs)
            go()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            go()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            if log:
                log(f"autotune {dict(tkey)} -> {ms:.3f} ms")
        except (MiaError, torch.cuda.OutOfMemoryError) as exc:
            # a candidate whose workspace does not fit or whose edge queue
            # overflows is not a choice; the others still are
            ms = math.inf
            failures.append(exc)
            if log:
                log(f"autotune {dict(tkey)} -> skipped ({exc})")
        timings[tkey] = ms
        del go
        return ms

    sides, los_sides, refines, units = candidates(range_proj, range_los)
    rl = range_proj if range_los is None else range_los

    def los_refine(ls, depth):
        # position cells about rl / depth deep along the line of sight: the
        # positions a warp holds then span a short stretch of it, so their
        # line-of-sight windows over the staged shapes nearly coincide
        return max(1, int(round(depth * ls / rl)))

    # cubic cells first, then narrow cells one line-of-sight range long, then
    # the line-of-sight geometry, the plane refinement and the unit size
    # around the best so far
    cubic = {"cell_size": range_proj / 3.0, "cell_refine": 2, "shapes_per_unit": 128, "cell_size_los": 0.0,
             "cell_refine_los": 0}
    best = min(({**cubic, "cell_size": s} for s in sides[:5]), key=time_one)
    best = min([best] + [{**best, "cell_size": s, "cell_size_los": rl, "cell_refine_los": los_refine(rl, 6)}
                         for s in sides[3:]], key=time_one)
    # two rounds over the axes: the best side in the plane depends on the
    # line-of-sight geometry, the refinement and the unit size found after it
    for _ in range(2):
        if best["cell_size_los"] > 0.0:
            best = min([best] + [{**best, "cell_size_los": ls, "cell_refine_los": los_refine(ls, d)}
                                 for ls in los_sides for d in (3, 6, 10)], key=time_one)
        best = min([best] + [{**best, "cell_refine": m} for m in refines], key=time_one)
        best = min([best] + [{**best, "shapes_per_unit": u} for u in units], key=time_one)
        best = min([best] + [{**best, "cell_size": s} for s in sides], key=time_one)
    # the long-cell family as a whole (two line-of-sight ranges deep, fine
    # position cells along it, the largest units): coordinate descent changes
    # one axis at a time and can stop short of it
    best = min([best] + [{"cell_size": s, "cell_refine": m, "shapes_per_unit": units[-1], "cell_size_los": 2 * rl,
                          "cell_refine_los": los_refine(2 * rl, 10)} for s in sides[3:7] for m in (1, 2)],
               key=time_one)
    if not math.isfinite(time_one(best)):
        raise failures[-1]
    out = dict(norm(best))
    out["ms"] = time_one(best)
    if key is not None:
        store(key, out, path)
    return out
