"""ctypes binding of the C ABI in ``include/measure_ia_gb300.h``.

The library is built in-tree (``measure_ia_gb300/build.py``).  Loading fails
loudly when it is missing: there is no CPU fallback for the pair counts.
"""

from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmeasureia_gb300.so")

MIA_OK, MIA_ERR_ARG, MIA_ERR_CUDA, MIA_ERR_RANGE, MIA_ERR_OVERFLOW, MIA_ERR_WORKSPACE = range(6)
MIA_KIND_W, MIA_KIND_MULTIPOLES = 0, 1
MIA_TREE, MIA_BRUTE = 0, 1
MIA_FP64, MIA_MIXED = 0, 1
MIA_DISTORTION, MIA_ELLIPTICITY = 0, 1
MAX_BINS_R, MAX_BINS_P, MAX_BREAKS = 64, 128, 96

EXPORTED = ("mia_create", "mia_destroy", "mia_last_error", "mia_version", "mia_workspace_size",
            "mia_output_layout", "mia_measure", "mia_measure_static", "mia_batch_workspace_size",
            "mia_batch_prepare", "mia_batch_enqueue", "mia_batch_status", "mia_measure_batch",
            "mia_profile_pairs", "mia_profile_read", "mia_jackknife_cross_cov", "mia_lc_workspace_size",
            "mia_lc_count")
MIA_LC_INDEX_ERROR, MIA_LC_BAD_PATCH = 1, 2
STATIC_SCRATCH_BYTES = 64 * 1024 * 1024


class Catalog(C.Structure):
    _fields_ = [("position", C.c_void_p), ("weight", C.c_void_p), ("position_shape", C.c_void_p),
                ("axis_direction", C.c_void_p), ("q", C.c_void_p), ("weight_shape", C.c_void_p),
                ("n_pos", C.c_int64), ("n_shape", C.c_int64)]


class Config(C.Structure):
    _fields_ = [("kind", C.c_int), ("membership", C.c_int), ("precision", C.c_int), ("los", C.c_int),
                ("l_subboxes", C.c_int), ("ellipticity", C.c_int), ("want_variance", C.c_int),
                ("n_r", C.c_int), ("n_p", C.c_int), ("n_qbreak", C.c_int), ("n_pbreak", C.c_int),
                ("shapes_per_unit", C.c_int), ("cell_refine", C.c_int), ("boxsize", C.c_double), ("volume", C.c_double),
                ("r_min", C.c_double), ("r_max", C.c_double), ("rp_cut", C.c_double), ("cell_size", C.c_double),
                ("r_edges", C.POINTER(C.c_double)), ("p_edges", C.POINTER(C.c_double)),
                ("q_break", C.POINTER(C.c_double)), ("q_bin", C.POINTER(C.c_int)),
                ("p_break", C.POINTER(C.c_double)), ("p_bin", C.POINTER(C.c_int)),
                ("cell_size_los", C.c_double), ("cell_refine_los", C.c_int)]


_LAYOUT_FIELDS = ["total", "dd", "splus", "scross", "variance", "npos_jk", "nshape_jk", "R", "R_jk", "rr", "rr_jk",
                  "xi_gp", "xi_gx", "xi_gg", "splusd", "scrossd", "sigmasq", "xi_gp_jk", "splusd_jk", "xi_gg_jk",
                  "dd_jk", "proj_gp", "proj_gg", "proj_gp_jk", "proj_gg_jk", "mean_gp", "std_gp", "cov_gp",
                  "mean_gg", "std_gg", "cov_gg", "stats"]


class Layout(C.Structure):
    _fields_ = [(f, C.c_int64) for f in _LAYOUT_FIELDS]


class Result(C.Structure):
    _fields_ = [("out", C.c_void_p), ("npairs", C.c_void_p)]


_lib = None


class LcConfig(C.Structure):
    _fields_ = [("kind", C.c_int), ("with_shapes", C.c_int), ("n_r", C.c_int), ("n_p", C.c_int),
                ("n_patch", C.c_int), ("n_qbreak", C.c_int), ("n_pbreak", C.c_int),
                ("q_break", C.POINTER(C.c_double)), ("q_bin", C.POINTER(C.c_int)),
                ("p_break", C.POINTER(C.c_double)), ("p_bin", C.POINTER(C.c_int)),
                ("h_extra", C.c_double), ("rp_cut", C.c_double), ("r_lim", C.c_double), ("pi_lo", C.c_double),
                ("pi_hi", C.c_double), ("ra0", C.c_double), ("ra_cell", C.c_double), ("dec0", C.c_double),
                ("dec_cell", C.c_double), ("chi0", C.c_double), ("chi_cell", C.c_double), ("n_ra", C.c_int),
                ("n_dec", C.c_int), ("n_chi", C.c_int), ("unit_weights", C.c_int),
                ("wide_sums", C.c_int)]


class LcSample(C.Structure):
    _fields_ = [("n", C.c_int64), ("ra", C.c_void_p), ("dec", C.c_void_p), ("chi", C.c_void_p), ("w", C.c_void_p),
                ("cos_dec", C.c_void_p), ("e", C.c_void_p), ("c2a", C.c_void_p), ("s2a", C.c_void_p),
                ("patch", C.c_void_p)]


def load(path=None):
    """The loaded library (built on first use if the sources are present).
    ``MIA_LIB_PATH`` selects another build of the same sources."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("MIA_LIB_PATH") or LIB_PATH
    if not os.path.exists(path):
        from . import build as _build
        try:
            _build.build()
        except Exception as e:  # no nvcc or a failed build: fail loudly
            raise RuntimeError(f"measure_ia_gb300 CUDA library missing at {path} and could not be built: {e}")
    lib = C.CDLL(path)
    lib.mia_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
    lib.mia_create.restype = C.c_int
    lib.mia_destroy.argtypes = [C.c_void_p]
    lib.mia_destroy.restype = C.c_int
    lib.mia_last_error.argtypes = [C.c_void_p]
    lib.mia_last_error.restype = C.c_char_p
    lib.mia_version.argtypes = []
    lib.mia_version.restype = C.c_int
    lib.mia_workspace_size.argtypes = [C.POINTER(Config), C.c_int64, C.c_int64, C.POINTER(C.c_size_t)]
    lib.mia_workspace_size.restype = C.c_int
    lib.mia_output_layout.argtypes = [C.POINTER(Config), C.POINTER(Layout)]
    lib.mia_output_layout.restype = C.c_int
    lib.mia_measure.argtypes = [C.c_void_p, C.POINTER(Config), C.POINTER(Catalog), C.c_void_p, C.c_size_t,
                                C.POINTER(Result), C.c_void_p]
    lib.mia_measure.restype = C.c_int
    lib.mia_measure_static.argtypes = [C.c_void_p, C.POINTER(Config), C.POINTER(Catalog), C.POINTER(Result),
                                       C.c_void_p]
    lib.mia_measure_static.restype = C.c_int
    lib.mia_batch_workspace_size.argtypes = [C.POINTER(Config), C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                             C.POINTER(C.c_size_t)]
    lib.mia_batch_workspace_size.restype = C.c_int
    for name in ("mia_batch_prepare", "mia_batch_enqueue", "mia_measure_batch"):
        f = getattr(lib, name)
        f.argtypes = [C.c_void_p, C.POINTER(Config), C.c_int, C.POINTER(Catalog), C.c_void_p, C.c_size_t,
                      C.POINTER(Result), C.c_void_p]
        f.restype = C.c_int
    lib.mia_batch_status.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    lib.mia_batch_status.restype = C.c_int
    lib.mia_jackknife_cross_cov.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int64, C.c_void_p,
                                            C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.mia_jackknife_cross_cov.restype = C.c_int
    lib.mia_profile_pairs.argtypes = [C.c_void_p, C.c_int]
    lib.mia_profile_pairs.restype = C.c_int
    lib.mia_profile_read.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_int)]
    lib.mia_profile_read.restype = C.c_int
    lib.mia_lc_workspace_size.argtypes = [C.POINTER(LcConfig), C.c_int64, C.c_int64, C.POINTER(C.c_size_t)]
    lib.mia_lc_workspace_size.restype = C.c_int
    lib.mia_lc_count.argtypes = [C.c_void_p, C.POINTER(LcConfig), C.POINTER(LcSample), C.POINTER(LcSample),
                                 C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.mia_lc_count.restype = C.c_int
    _lib = lib
    return lib


class MiaError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[mia error {code}] {msg}")
        self.code = code
