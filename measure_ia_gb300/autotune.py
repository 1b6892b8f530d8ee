"""Autotuner for the pair-count launch configuration.

Three knobs change speed but never results: the shape-cell side
(``cell_size``), the number of position cells per shape cell along each
axis (``cell_refine``) and the shapes staged per work unit
(``shapes_per_unit``).  ``tune`` times candidates on the caller's own
device-resident catalogue (CUDA events, one warm-up and one timed run each),
keeps the fastest, and stores the choice in a JSON cache keyed by the
workload shape, so later measurements of the same shape reuse it.

The cache file is ``$MIA_TUNE_CACHE`` or ``~/.cache/measure_ia_gb300/tune.json``.
"""

from __future__ import annotations

import json
import math
import os

DEFAULT = {"cell_size": 0.0, "cell_refine": 0, "shapes_per_unit": 0}


def cache_path():
    return os.environ.get("MIA_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "measure_ia_gb300",
                                                            "tune.json")


def workload_key(kind, precision, n_pos, n_shape, boxsize, n_r, n_p, range_proj, range_los, l_subboxes, membership,
                 device_name=""):
    """Sizes enter as powers of two (a doubling of the catalogue is a new shape)."""
    lp = int(round(math.log2(max(n_pos, 1))))
    ls = int(round(math.log2(max(n_shape, 1))))
    return "|".join(str(x) for x in (device_name, kind, precision, lp, ls, round(boxsize, 3), n_r, n_p,
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


def candidates(range_proj):
    """Shape-cell sides around range/2 first, then refinement and unit size
    around the best side."""
    sides = [range_proj / k for k in (1.5, 1.75, 2.0, 2.5, 3.0)]
    return sides, (2, 3, 4), (64, 128, 256)


def tune(make_counter, dcat, range_proj, key=None, path=None, log=None):
    """Return the fastest {cell_size, cell_refine, shapes_per_unit}.

    ``make_counter(**knobs)`` builds a PairCounter for the knobs; ``dcat`` is
    the device-resident catalogue.  With ``key`` the result is cached."""
    import torch

    from ._lib import MiaError

    if key is not None:
        hit = load_cache(path).get(key)
        if hit:
            return hit
    n_pos = dcat["Position"].shape[0]
    n_shape = dcat["Position_shape_sample"].shape[0]
    timings = {}
    failures = []

    def time_one(knobs):
        tkey = (knobs["cell_size"], knobs["cell_refine"], knobs["shapes_per_unit"])
        if tkey in timings:
            return timings[tkey]
        try:
            pc = make_counter(**knobs)
            bufs = pc.allocate(n_pos, n_shape)
            pc.run(dcat, bufs)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            pc.run(dcat, bufs)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
        except (MiaError, torch.cuda.OutOfMemoryError) as exc:
            # a candidate whose workspace does not fit or whose edge queue
            # overflows is not a choice; the others still are
            ms = math.inf
            bufs = None
            failures.append(exc)
            if log:
                log(f"autotune {knobs} -> skipped ({exc})")
        timings[tkey] = ms
        if log and math.isfinite(ms):
            log(f"autotune {knobs} -> {ms:.3f} ms")
        del bufs
        return ms

    sides, refines, units = candidates(range_proj)
    best = min(({"cell_size": s, "cell_refine": 3, "shapes_per_unit": 128} for s in sides), key=time_one)
    best = min(({**best, "cell_refine": m} for m in refines), key=time_one)
    best = min(({**best, "shapes_per_unit": u} for u in units), key=time_one)
    if not math.isfinite(timings[(best["cell_size"], best["cell_refine"], best["shapes_per_unit"])]):
        raise failures[-1]
    best = {k: (float(v) if k == "cell_size" else int(v)) for k, v in best.items()}
    best["ms"] = timings[(best["cell_size"], best["cell_refine"], best["shapes_per_unit"])]
    if key is not None:
        store(key, best, path)
    return best
