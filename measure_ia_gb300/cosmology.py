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
distance is the integral of c / H(z) by 48-point Gauss-Legendre quadrature,
accurate to ~1e-13 relative for z < 20.  It is not pyccl's spline
integration, so distances agree with pyccl's only to that method's accuracy.
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

    def comoving_radial_distance(self, a):
        """Comoving distance in Mpc to scale factor(s) ``a``."""
        a = np.asarray(a, dtype=np.float64)
        z = 1.0 / a - 1.0
        flat = z.reshape(-1)
        half = flat[:, None] / 2.0
        zz = half * (_GL_X[None, :] + 1.0)
        chi = (half[:, 0] * (_GL_W[None, :] / self.E(zz)).sum(axis=1)) * (C_KM_S / (100.0 * self.h))
        return chi.reshape(z.shape)


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
