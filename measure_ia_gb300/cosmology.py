"""Comoving radial distances for the lightcone measurements.

The reference converts redshifts with pyccl
(``ccl.comoving_radial_distance(cosmology, 1 / (1 + z))`` in Mpc,
``measure_w_lightcone.py:117-125``) and reads ``cosmology["h"]``.  Any object
with those two capabilities works here:

* a ``pyccl.Cosmology`` when pyccl is importable (used through pyccl itself);
* any object with a ``comoving_radial_distance(a)`` method and ``["h"]``;
* ``None``: :class:`FlatLCDM` with the reference's default parameters
  (Omega_c = 0.225, Omega_b = 0.045, h = 0.7).

:class:`FlatLCDM` is a flat universe of matter, a cosmological constant,
photons at T_CMB = 2.7255 K and three massless neutrino species
(N_eff = 3.044), the ingredients of pyccl's default background.  Its
distance is the integral of c / H(z): tabulated at the nodes z_k = k / 2048
(48-point Gauss-Legendre quadrature per interval, summed outward from
z = 0) and interpolated with cubic Hermite polynomials that use the exact
derivative c / H(z) at the nodes, accurate to ~1e-12 relative.  A redshift
gets the same distance whatever else is in the array (the table's nodes do
not depend on the range asked for).  It is not pyccl's spline integration,
so distances agree with pyccl's only to that method's accuracy.
"""

from __future__ import annotations

import numpy as np

C_KM_S = 299792.458
T_CMB = 2.7255
N_EFF = 3.044

_GL_X, _GL_W = np.polynomial.legendre.leggauss(48)


class FlatLCDM:
    def __init__(self, Omega_c=0.225, Omega_b=0.045, h=0.7, T_CMB=T_CMB, N_eff=N_EFF):
        self.h = float(h)
        self.Omega_m = float(Omega_c) + float(Omega_b)
        # photon density today: rho_gamma = (pi^2/15) (k T)^4 / (hbar c)^3, as Omega_gamma h^2
        og_h2 = 2.4728e-5 * (T_CMB / 2.7255) ** 4
        self.Omega_r = og_h2 / self.h ** 2 * (1.0 + 0.22710731766 * N_eff)
        self.Omega_l = 1.0 - self.Omega_m - self.Omega_r

    def __getitem__(self, key):
        if key == "h":
            return self.h
        raise KeyError(key)

    def E(self, z):
        zp = 1.0 + np.asarray(z, dtype=np.float64)
        return np.sqrt(self.Omega_m * zp ** 3 + self.Omega_r * zp ** 4 + self.Omega_l)

    DZ = 1.0 / 2048.0

    def _integral(self, z0, z1):
        """int_z0^z1 dz / E(z) for arrays of interval ends (48-point Gauss-Legendre)."""
        half = (z1 - z0) / 2.0
        mid = (z1 + z0) / 2.0
        zz = mid[:, None] + half[:, None] * _GL_X[None, :]
        return half * (_GL_W[None, :] / self.E(zz)).sum(axis=1)

    def _table(self, k_lo, k_hi):
        """Distances (units of c/H0) at the nodes k_lo..k_hi (k_lo <= 0 <= k_hi),
        and the Hermite derivatives DZ / E(z_k) there."""
        t = getattr(self, "_tab", None)
        if t is not None and t[0] <= k_lo and t[1] >= k_hi:
            return t
        k_lo = min(k_lo, t[0] if t else 0, 0)
        k_hi = max(k_hi, t[1] if t else 0, 0)
        up = np.arange(0, k_hi + 1, dtype=np.float64) * self.DZ
        down = np.arange(0, k_lo - 1, -1, dtype=np.float64) * self.DZ
        cu = np.concatenate([[0.0], np.cumsum(self._integral(up[:-1], up[1:]))])
        cd = np.concatenate([[0.0], np.cumsum(self._integral(down[:-1], down[1:]))])
        vals = np.concatenate([cd[::-1][:-1], cu])          # nodes k_lo .. k_hi
        # z_k = k * DZ exactly as the query side forms it, so the derivatives
        # are the same doubles as E evaluated per query
        nodes = np.arange(k_lo, k_hi + 1, dtype=np.float64) * self.DZ
        self._tab = (k_lo, k_hi, vals, self.DZ / self.E(nodes))
        return self._tab

    def comoving_radial_distance(self, a):
        """Comoving distance in Mpc to scale factor(s) ``a``."""
        a = np.asarray(a, dtype=np.float64)
        z = (1.0 / a - 1.0).reshape(-1)
        if z.size == 0:
            return np.zeros(a.shape)
        if not np.all(np.isfinite(z)):
            raise ValueError("redshifts must be finite")
        k = np.floor(z / self.DZ)
        k_lo, k_hi, vals, dvals = self._table(int(k.min()) - 1, int(k.max()) + 2)
        i = (k - k_lo).astype(np.int64)
        z0 = k * self.DZ
        t = (z - z0) / self.DZ
        f0, f1 = vals[i], vals[i + 1]
        d0, d1 = dvals[i], dvals[i + 1]
        t2 = t * t
        t3 = t2 * t
        chi = (2 * t3 - 3 * t2 + 1) * f0 + (t3 - 2 * t2 + t) * d0 + (-2 * t3 + 3 * t2) * f1 + (t3 - t2) * d1
        return (chi * (C_KM_S / (100.0 * self.h))).reshape(a.shape)


def comoving_radial_distance(cosmology, a):
    """The reference's distance call for any supported cosmology object."""
    if hasattr(cosmology, "comoving_radial_distance"):
        return np.asarray(cosmology.comoving_radial_distance(a), dtype=np.float64)
    try:
        import pyccl as ccl
    except ImportError as exc:  # pragma: no cover - depends on the host
        raise TypeError("cosmology must provide comoving_radial_distance(a) (pyccl is not installed)") from exc
    return np.asarray(ccl.comoving_radial_distance(cosmology, a), dtype=np.float64)


def default_cosmology():
    return FlatLCDM(Omega_c=0.225, Omega_b=0.045, h=0.7)
