"""Public helpers the reference's measurement classes carry, shared by
``MeasureIABox`` and ``MeasureIALightcone``.

* :class:`BaseHelpers` -- the small public methods of ``MeasureIABase``
  (``measure_IA_base.py:186-402, 745-800``): dot products of row pairs, e+/ex
  from |e| and phi, the analytic random-pair counts of an (r_p, Pi) or (r, mu_r)
  bin, spherical-cap volumes, row-wise set differences and the lightcone
  jackknife patches.  Same arguments, results and errors.
* :class:`JackknifeCovariance` -- ``measure_covariance_multiple_datasets`` and
  ``create_full_cov_matrix_projections`` (``measure_jackknife.py:485-652``),
  working on the jackknife realisations a measurement stored in the output.

Not provided: the reference's astropy-based ``get_cosmo_points`` /
``get_pair_coords`` and ``count_pairs_xi_grid_w_update``
(``measure_w_lightcone.py:345-601``), which need astropy and with their
default arguments fail in the reference as well (``cosmology.h`` of ``None``);
the ``ReadData`` methods ``MeasureIABox`` inherits there, which read catalogue
attributes its constructor never sets (use ``ReadData`` itself); and SimInfo's
``get_specs`` / ``get_file_info`` on the lightcone class, which has no named
simulation.
"""

from __future__ import annotations

import numpy as np

from .output import norm_path, store_for


class BaseHelpers:
    @staticmethod
    def calculate_dot_product_arrays(a1, a2):
        """Row-wise dot product: out[i] = a1[i] . a2[i] (measure_IA_base.py:186-207)."""
        out = np.zeros(np.shape(a1)[0])
        for i in range(np.shape(a1)[1]):
            out += a1[:, i] * a2[:, i]
        return out

    @staticmethod
    def get_ellipticity(e, phi):
        """e+ = e cos 2phi, ex = e sin 2phi (measure_IA_base.py:209-228)."""
        return e * np.cos(2 * phi), e * np.sin(2 * phi)

    @staticmethod
    def get_random_pairs(rp_max, rp_min, pi_max, pi_min, L3, corrtype, Num_position, Num_shape):
        """Pairs of a uniform random catalogue in an (r_p, Pi) bin: the
        cylinder shell's volume over the box's (measure_IA_base.py:230-273);
        'auto' counts each pair once."""
        shell = np.pi * (rp_max ** 2 - rp_min ** 2) * abs(pi_max - pi_min) / L3
        if corrtype == "auto":
            return (Num_position - 1.0) * Num_shape / 2.0 * shell
        if corrtype == "cross":
            return Num_position * Num_shape * shell
        raise ValueError("Unknown input for corrtype, choose from auto or cross.")

    @staticmethod
    def get_volume_spherical_cap(mur, r):
        """Volume of the cap of a sphere of radius r above cos(theta) = mur
        (measure_IA_base.py:275-291)."""
        return np.pi / 3.0 * r ** 3 * (2 + mur) * (1 - mur) ** 2

    def get_random_pairs_r_mur(self, r_max, r_min, mur_max, mur_min, L3, corrtype, Num_position, Num_shape):
        """Pairs of a uniform random catalogue in an (r, mu_r) bin, the
        difference of four spherical caps over the box's volume
        (measure_IA_base.py:293-352).  As in the reference, 'cross' keeps the
        (Num_position - 1) factor, and the result is an absolute value."""
        cap = self.get_volume_spherical_cap
        vol = cap(mur_min, r_max) - cap(mur_max, r_max) - (cap(mur_min, r_min) - cap(mur_max, r_min))
        if corrtype == "auto":
            rr = (Num_position - 1.0) / 2.0 * Num_shape * vol / L3
        elif corrtype == "cross":
            rr = (Num_position - 1.0) * Num_shape * vol / L3
        else:
            raise ValueError("Unknown input for corrtype, choose from auto or cross.")
        return abs(rr)

    @staticmethod
    def setdiff2D(a1, a2):
        """Row i: the elements of a1[i] not in a2[i] (measure_IA_base.py:354-376)."""
        assert len(a1) == len(a2), "Lengths of lists where each row is to be compared, are not the same."
        return [np.setdiff1d(a1[i], a2[i]) for i in range(len(a1))]

    @staticmethod
    def setdiff_omit(a1, a2, incl_ind):
        """For the rows of a1 whose index is in incl_ind: the elements not in a2
        (measure_IA_base.py:378-402)."""
        return [np.setdiff1d(a1[i], a2) for i in range(len(a1)) if np.isin(i, incl_ind)]

    def assign_jackknife_patches(self, data, randoms_data, num_jk):
        """Jackknife patches of a lightcone's positions, shapes and randoms by
        k-means on the sky (measure_IA_base.py:745-800)."""
        from .lightcone import assign_jackknife_patches
        return assign_jackknife_patches(data, randoms_data, num_jk)


class JackknifeCovariance:
    """Covariances from the jackknife realisations in ``output_file_name``;
    needs ``output_file_name``, ``snap_group`` and ``device``."""

    def measure_covariance_multiple_datasets(self, corr_type, dataset_names, num_box=27, return_output=False):
        """Jackknife covariance of one dataset with itself or of two datasets
        (e.g. two projections) from the realisations already in the output
        (``MeasureJackknife.measure_covariance_multiple_datasets``,
        measure_jackknife.py:485-571): same checks, same dataset names
        ``<d0>[_<d1>]_jackknife_cov_<n>`` and ``_jackknife_<n>`` under
        ``<snap_group>/<corr_type>``, or (cov, std) with ``return_output``.
        The arithmetic runs on the device (``mia_jackknife_cross_cov``)."""
        from .engine import jackknife_cross_cov
        valid = ["w_g_plus", "multipoles_g_plus", "w_gg", "multipoles_gg"]
        if corr_type not in valid:
            raise ValueError("corr_type must be 'w_g_plus', 'w_gg', 'multipoles_g_plus' or 'multipoles_gg'.")
        store = store_for(self)
        reals = []
        for name in dataset_names:
            grp = norm_path(self.snap_group, corr_type, f"{name}_jk{num_box}")
            try:
                reals.append(np.stack([np.asarray(store.read(norm_path(grp, f"{name}_{b}")), dtype=np.float64)
                                       for b in range(num_box)]))
            except KeyError:
                raise KeyError(f"Unable to open object '{name}_jk{num_box}' in '{self.snap_group}/{corr_type}'")
        if len(dataset_names) not in (1, 2):
            raise KeyError("Too many datasets given, choose either 1 or 2")
        cov_d, std_d = jackknife_cross_cov(reals[0], reals[1] if len(reals) == 2 else None, device=self.device)
        cov, std = cov_d.cpu().numpy(), std_d.cpu().numpy()
        if self.output_file_name is not None and not return_output:
            grp = norm_path(self.snap_group, corr_type)
            tag = "_".join(dataset_names[:2]) if len(dataset_names) == 2 else dataset_names[0]
            store.write(grp, f"{tag}_jackknife_cov_{num_box}", cov)
            store.write(grp, f"{tag}_jackknife_{num_box}", std)
            store.flush()
            return None
        return cov, std

    def create_full_cov_matrix_projections(self, corr_type, dataset_names=["LOS_x", "LOS_y", "LOS_z"], num_box=27,
                                           return_output=False):
        """Combined jackknife covariance of three projections and of each pair
        (``create_full_cov_matrix_projections``, measure_jackknife.py:573-652):
        writes the three pair covariances, then assembles the 3-projection and
        2-projection matrices from the stored ``_jackknife_cov_<n>`` datasets.
        Like the reference, the block it names cov_yz comes from the
        (d0, d2) pair and cov_xz from the (d1, d2) pair."""
        d0, d1, d2 = dataset_names[0], dataset_names[1], dataset_names[2]
        for a, b in ((d0, d1), (d0, d2), (d1, d2)):
            self.measure_covariance_multiple_datasets(corr_type=corr_type, dataset_names=[a, b], num_box=num_box)
        store = store_for(self)
        grp = norm_path(self.snap_group, corr_type)
        rd = lambda name: np.asarray(store.read(norm_path(grp, name)))
        cov_xx = rd(f"{d0}_jackknife_cov_{num_box}")
        cov_yy = rd(f"{d1}_jackknife_cov_{num_box}")
        cov_zz = rd(f"{d2}_jackknife_cov_{num_box}")
        cov_xy = rd(f"{d0}_{d1}_jackknife_cov_{num_box}")
        cov_yz = rd(f"{d0}_{d2}_jackknife_cov_{num_box}")
        cov_xz = rd(f"{d1}_{d2}_jackknife_cov_{num_box}")
        cov3 = np.concatenate((np.concatenate((cov_xx, cov_xy, cov_xz), axis=1),
                               np.concatenate((cov_xy.T, cov_yy, cov_yz), axis=1),
                               np.concatenate((cov_xz.T, cov_yz.T, cov_zz), axis=1)), axis=0)
        cov2xy = np.concatenate((np.concatenate((cov_xx, cov_xy), axis=1),
                                 np.concatenate((cov_xy.T, cov_yy), axis=1)), axis=0)
        cov2xz = np.concatenate((np.concatenate((cov_xx, cov_xz), axis=1),
                                 np.concatenate((cov_xz.T, cov_zz), axis=1)), axis=0)
        cov2yz = np.concatenate((np.concatenate((cov_yy, cov_yz), axis=1),
                                 np.concatenate((cov_yz.T, cov_zz), axis=1)), axis=0)
        if return_output:
            return cov3, cov2xy, cov2xz, cov2yz
        store.write(grp, f"{d0}_{d1}_{d2}_combined_jackknife_cov_{num_box}", cov3)
        store.write(grp, f"{d0}_{d1}_combined_jackknife_cov_{num_box}", cov2xy)
        store.write(grp, f"{d0}_{d2}_combined_jackknife_cov_{num_box}", cov2xz)
        store.write(grp, f"{d1}_{d2}_combined_jackknife_cov_{num_box}", cov2yz)
        store.flush()
        return None
