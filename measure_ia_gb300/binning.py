"""Exact bin assignment tables.

The reference assigns bins with floating-point formulas evaluated by numpy
(``measure_w_box_jk.py:603-617``, ``measure_m_box_jk.py:636-653``)::

    r bin : floor(log10(r) / dlog - log10(r_bins[0]) / dlog)   (clamped, numpy index wrap)
    Pi bin: floor(Pi / dpi - pi_bins[0] / dpi)
    mu bin: floor(mu / dmu - mu_r_bins[0] / dmu)

``log10`` is a platform routine (SIMD on x86, libm on aarch64), so a GPU
evaluation could not match it bit for bit.  Instead this module evaluates the
reference's own expression with numpy, on the host that runs the measurement,
and finds every breakpoint: the float64 values at which the assigned bin
changes.  Each breakpoint is located exactly by bisection over the ordered
bit patterns of float64.  The device then only compares the exactly computed
separation against these breakpoints.

For r the table is indexed by q = d^2 (r_p^2 for w, r^2 for multipoles), so
it also carries the KD-tree membership of the reference's tree backends:
scipy's periodic ball query keeps ``d^2 <= r*r`` (``query_ball_tree`` at
r_min and r_max, then their set difference, measure_w_box_jk.py:577-580).
"""

from __future__ import annotations

import functools
from dataclasses import dataclass

import numpy as np

MAX_BREAKS = 96

_SIGN = np.int64(-0x8000000000000000)
_MAG = np.int64(0x7FFFFFFFFFFFFFFF)


def order_key(x):
    """Map float64 values to int64 keys with the same order (-0.0 just below +0.0)."""
    b = np.asarray(x, dtype=np.float64).view(np.int64)
    return np.where(b >= 0, b, -(b & _MAG) - 1)


def from_key(k):
    k = np.asarray(k, dtype=np.int64)
    b = np.where(k >= 0, k, (-(k + 1)) | _SIGN)
    return b.view(np.float64)


@dataclass
class BinTable:
    breaks: np.ndarray   # ascending float64 breakpoints
    bins: np.ndarray     # int32, len(breaks)+1: bin of each interval, -1 = not binned

    def lookup(self, x):
        j = np.searchsorted(self.breaks, np.asarray(x, dtype=np.float64), side="right")
        return self.bins[j]


def _find_breaks(f, lo, hi, seeds, n_samples=40000):
    """All points in (lo, hi] where the integer-valued function f changes.

    f must be vectorised over float64 arrays.  Changes are bracketed on a
    dense sample (log-spaced where lo > 0) plus the seed points and their
    float neighbours, then each bracket is bisected to the exact double."""
    if lo > 0:
        xs = np.geomspace(lo, hi, n_samples)
    else:
        xs = np.linspace(lo, hi, n_samples)
    extra = []
    for s in seeds:
        if not np.isfinite(s):
            continue
        v = np.float64(s)
        for _ in range(4):
            v = np.nextafter(v, -np.inf)
        for _ in range(9):
            extra.append(v)
            v = np.nextafter(v, np.inf)
    xs = np.unique(np.concatenate([xs, np.array(extra, dtype=np.float64), [lo, hi]]))
    xs = xs[(xs >= lo) & (xs <= hi)]
    vals = f(xs)
    breaks = []
    idx = np.nonzero(vals[1:] != vals[:-1])[0]
    todo = [(xs[i], xs[i + 1]) for i in idx]
    while todo:
        a, b = todo.pop()
        ka, kb = int(order_key(a)), int(order_key(b))
        fa, fb = f(np.array([a]))[0], f(np.array([b]))[0]
        if fa == fb:
            continue
        # smallest key in (ka, kb] whose value differs from f(a)
        lo_k, hi_k = ka, kb
        while hi_k - lo_k > 1:
            mid = lo_k + (hi_k - lo_k) // 2
            if f(from_key(np.array([mid])))[0] != fa:
                hi_k = mid
            else:
                lo_k = mid
        t = from_key(np.array([hi_k]))[0]
        breaks.append(t)
        # further changes between t and b (two breakpoints inside one bracket)
        if f(np.array([t]))[0] != fb:
            todo.append((t, b))
    return np.unique(np.array(breaks, dtype=np.float64))


def _table(f, lo, hi, seeds):
    br = _find_breaks(f, lo, hi, seeds)
    if len(br) > MAX_BREAKS:
        raise ValueError(f"too many bin breakpoints ({len(br)} > {MAX_BREAKS})")
    # interval values: f just below the first breakpoint, then at each breakpoint
    pts = np.concatenate([[lo], br])
    bins = f(pts).astype(np.int32)
    tab = BinTable(br, bins)
    _verify(f, tab, lo, hi)
    return tab


def _verify(f, tab, lo, hi, span=1500):
    """Check the table against f on +-span ulps around every breakpoint."""
    for t in tab.breaks:
        k = int(order_key(t))
        keys = np.arange(k - span, k + span + 1, dtype=np.int64)
        xs = from_key(keys)
        xs = xs[(xs >= lo) & (xs <= hi)]
        if len(xs) == 0:
            continue
        got = tab.lookup(xs)
        want = f(xs)
        if not np.array_equal(got, want):
            bad = xs[got != want][:3]
            raise RuntimeError(f"bin table not monotone near {t!r}: {bad!r}")


def _wrap_index(ind, n):
    """Reference clamp 'ind == n -> n-1' and numpy's negative-index wrap."""
    ind = np.where(ind >= n, ind - 1, ind)
    return np.where(ind < 0, ind + n, ind)


_TABLES = {}


def _memo(fn):
    """Tables depend only on their arguments and this host's numpy: build each
    once per process (a table takes ~10 ms of bisection) and share it
    read-only."""

    def key(a):
        if isinstance(a, (np.ndarray, list, tuple)):
            return ("edges",) + tuple(float(x) for x in np.asarray(a, dtype=np.float64).ravel())
        return a

    @functools.wraps(fn)
    def cached(*args, **kw):
        k = (fn.__name__,) + tuple(key(a) for a in args) + tuple(sorted((n, key(v)) for n, v in kw.items()))
        tab = _TABLES.get(k)
        if tab is None:
            tab = fn(*args, **kw)
            tab.breaks.setflags(write=False)
            tab.bins.setflags(write=False)
            _TABLES[k] = tab
        return tab

    return cached


@_memo
def r_table(kind, r_bins, r_min, r_max, num_bins_r, membership="tree", rp_cut=0.0):
    """Bin of q = d^2 (w: r_p^2; multipoles: r^2), -1 if the pair is not binned.

    w:  mask r_p >= r_bins[0] and r_p < r_bins[-1]          (measure_w_box_jk.py:603-604)
    m:  mask r   >= r_bins[0] and r   < r_bins[-1]          (measure_m_box_jk.py:636-640)
    tree membership adds d^2 > r_min*r_min and d^2 <= r_max*r_max."""
    r_bins = np.asarray(r_bins, dtype=np.float64)
    dlog = (np.log10(r_max) - np.log10(r_min)) / num_bins_r
    c0 = np.log10(r_bins[0]) / dlog
    rmin2 = r_min * r_min
    rmax2 = r_max * r_max

    def f(q):
        q = np.asarray(q, dtype=np.float64)
        r = np.sqrt(q)
        ok = (r >= r_bins[0]) & (r < r_bins[-1])
        if membership == "tree":
            ok &= (q > rmin2) & (q <= rmax2)
        with np.errstate(divide="ignore", invalid="ignore"):
            ind = np.floor(np.log10(r) / dlog - c0)
        ind = np.where(ok, ind, 0).astype(np.int64)
        ind = _wrap_index(ind, num_bins_r)
        return np.where(ok, ind, -1)

    top = max(r_bins[-1], r_max) ** 2 * 4.0
    bottom = min(r_bins[0], r_min) ** 2 / 4.0
    seeds = [rmin2, rmax2] + [float(x) ** 2 for x in r_bins]
    return _table(f, bottom, top, seeds)


@_memo
def pi_table(pi_bins, num_bins_pi):
    """Bin of Pi (line-of-sight separation), -1 outside [pi_bins[0], pi_bins[-1])
    (measure_w_box_jk.py:603-617)."""
    pi_bins = np.asarray(pi_bins, dtype=np.float64)
    step = (pi_bins[-1] - pi_bins[0]) / num_bins_pi
    c = pi_bins[0] / step

    def f(x):
        x = np.asarray(x, dtype=np.float64)
        ok = (x >= pi_bins[0]) & (x < pi_bins[-1])
        ind = np.floor(x / step - c)
        ind = np.where(ok, ind, 0).astype(np.int64)
        ind = _wrap_index(ind, num_bins_pi)
        return np.where(ok, ind, -1)

    span = pi_bins[-1] - pi_bins[0]
    return _table(f, pi_bins[0] - span, pi_bins[-1] + span, list(pi_bins))


@_memo
def mu_table(mu_r_bins, num_bins_pi):
    """Bin of mu_r = Pi / r over [-1, 1] (measure_m_box_jk.py:646-653)."""
    mu_r_bins = np.asarray(mu_r_bins, dtype=np.float64)
    step = 2.0 / num_bins_pi
    c = mu_r_bins[0] / step

    def f(x):
        x = np.asarray(x, dtype=np.float64)
        ind = np.floor(x / step - c).astype(np.int64)
        return _wrap_index(ind, num_bins_pi)

    return _table(f, -1.0, 1.0, list(mu_r_bins))


# ---- lightcone counters (measure_w_lightcone.py, measure_m_lightcone.py) ------
#
# Same formulas as above, but the lightcone counters differ in what happens
# past the last bin: only the w counter with shapes clamps 'ind == n -> n-1'
# (measure_w_lightcone.py:170-173); the others hand the index to np.add.at,
# which raises IndexError.  Those intervals carry bin -2.

def _index_or_error(ind, n, clamp):
    ind = np.where(ind < 0, ind + n, ind)          # numpy's negative-index wrap
    if clamp:
        ind = np.where(ind == n, n - 1, ind)
    return np.where(ind >= n, -2, ind)


@_memo
def lc_r_table(kind, r_bins, r_min, r_max, num_bins_r, clamp):
    """Bin of q (w: r_p^2; multipoles: r^2), -1 outside [r_bins[0], r_bins[-1])
    (measure_w_lightcone.py:161-173, measure_m_lightcone.py:167-176)."""
    r_bins = np.asarray(r_bins, dtype=np.float64)
    dlog = (np.log10(r_max) - np.log10(r_min)) / num_bins_r
    c0 = np.log10(r_bins[0]) / dlog

    def f(q):
        q = np.asarray(q, dtype=np.float64)
        r = np.sqrt(q)
        ok = (r >= r_bins[0]) & (r < r_bins[-1])
        with np.errstate(divide="ignore", invalid="ignore"):
            ind = np.floor(np.log10(r) / dlog - c0)
        ind = _index_or_error(np.where(ok, ind, 0).astype(np.int64), num_bins_r, clamp)
        return np.where(ok, ind, -1)

    top = max(r_bins[-1], r_max) ** 2 * 4.0
    bottom = min(r_bins[0], r_min) ** 2 / 4.0
    return _table(f, bottom, top, [float(x) ** 2 for x in r_bins])


@_memo
def lc_pi_table(pi_bins, num_bins_pi, clamp):
    """Bin of Pi, -1 outside [pi_bins[0], pi_bins[-1]) (measure_w_lightcone.py:161-173)."""
    pi_bins = np.asarray(pi_bins, dtype=np.float64)
    step = (pi_bins[-1] - pi_bins[0]) / num_bins_pi
    c = pi_bins[0] / step

    def f(x):
        x = np.asarray(x, dtype=np.float64)
        ok = (x >= pi_bins[0]) & (x < pi_bins[-1])
        ind = _index_or_error(np.where(ok, np.floor(x / step - c), 0).astype(np.int64), num_bins_pi, clamp)
        return np.where(ok, ind, -1)

    span = pi_bins[-1] - pi_bins[0]
    return _table(f, pi_bins[0] - span, pi_bins[-1] + span, list(pi_bins))


@_memo
def lc_mu_table(mu_r_bins, num_bins_pi):
    """Bin of mu_r = Pi / r over [-1, 1], no clamp (measure_m_lightcone.py:172-176)."""
    mu_r_bins = np.asarray(mu_r_bins, dtype=np.float64)
    step = 2.0 / num_bins_pi
    c = mu_r_bins[0] / step

    def f(x):
        x = np.asarray(x, dtype=np.float64)
        return _index_or_error(np.floor(x / step - c).astype(np.int64), num_bins_pi, False)

    return _table(f, -1.0, 1.0, list(mu_r_bins))
