"""mia_measure_static: the entry point for callers that cannot allocate device
memory (a host framework that owns the whole GPU memory budget, or a loop in
which cudaMalloc's implicit device synchronisation is not allowed).  It runs
the same measurement as mia_measure on a scratch array compiled into the
library, so the caller passes only inputs and outputs.

Checked here through the C ABI, in the plain FP64 form and in the mixed form
(whose FP64 edge re-test queue, at least 8 MiB, also lives in the scratch):
two calls in a row give the same counts (bit-exact) and the same products
(1e-10 relative, the FP64 tolerance of the other GPU tests) as the workspace
entry point; a measurement too large for the 64 MiB scratch is refused with
MIA_ERR_WORKSPACE, and an invalid one with mia_measure's own message.  Kept
in its own file, collected last."""

import ctypes as C

import numpy as np
import pytest

from golden_io import assert_close

pytestmark = pytest.mark.gpu


def _catalog(dcat):
    from measure_ia_gb300 import _lib as L
    c = L.Catalog()
    c.position = dcat["Position"].data_ptr()
    c.weight = dcat["weight"].data_ptr()
    c.position_shape = dcat["Position_shape_sample"].data_ptr()
    c.axis_direction = dcat["Axis_Direction"].data_ptr()
    c.q = dcat["q"].data_ptr()
    c.weight_shape = dcat["weight_shape_sample"].data_ptr()
    c.n_pos = dcat["Position"].shape[0]
    c.n_shape = dcat["Position_shape_sample"].shape[0]
    return c


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_static_scratch_entry_point_matches_workspace_entry_point(precision):
    import torch
    from measure_ia_gb300 import _lib as L
    from measure_ia_gb300.catalogs import neyman_scott_catalog
    from measure_ia_gb300.engine import PairCounter, context

    data = neyman_scott_catalog(150, 100.0, 4000, 3, mean_children=30, sigma=1.0)
    keys = ("Position", "weight", "Position_shape_sample", "Axis_Direction", "q", "weight_shape_sample")
    dcat = {k: torch.from_numpy(np.ascontiguousarray(data[k], dtype=np.float64)).cuda() for k in keys}
    pc = PairCounter("w", boxsize=100.0, r_bins=np.logspace(-1, np.log10(20.0), 11), r_min=0.1, r_max=20.0,
                     p_bins=np.linspace(-20.0, 20.0, 9), l_subboxes=3, precision=precision)
    n_pos, n_shape = dcat["Position"].shape[0], dcat["Position_shape_sample"].shape[0]
    assert pc.workspace_bytes(n_pos, n_shape) <= L.STATIC_SCRATCH_BYTES
    if precision == "mixed":  # the edge queue (>= 2^20 entries of 8 bytes) is in the scratch too
        assert pc.workspace_bytes(n_pos, n_shape) > 8 * 2 ** 20

    ref_bufs = pc.allocate(n_pos, n_shape)
    pc.run(dcat, ref_bufs)
    ref = pc.fetch(ref_bufs)

    lib = L.load()
    ctx = context(0)
    cat = _catalog(dcat)
    stream = torch.cuda.current_stream()
    for call in range(2):
        _, out, npairs = pc.allocate(n_pos, n_shape)
        out.fill_(float("nan"))
        npairs.fill_(-1)
        res = L.Result()
        res.out = out.data_ptr()
        res.npairs = npairs.data_ptr()
        rc = lib.mia_measure_static(ctx, C.byref(pc.cfg), C.byref(cat), C.byref(res),
                                    C.c_void_p(stream.cuda_stream))
        assert rc == L.MIA_OK, lib.mia_last_error(ctx).decode()
        got = pc.fetch((None, out, npairs))
        np.testing.assert_array_equal(got.npairs, ref.npairs, err_msg=f"call {call}")
        for k in ("DD_all", "Splus_all", "scross", "rr", "rr_jk", "xi_gp", "xi_gg", "xi_gp_jk", "xi_gg_jk",
                  "proj_gp", "proj_gg", "proj_gp_jk", "cov_gp", "cov_gg", "std_gp"):
            assert_close(got[k], ref[k], 1e-10, f"call {call}: {k}")
        assert got.stats["binned_pairs"] == ref.stats["binned_pairs"]


def test_static_scratch_entry_point_refuses_oversized_measurements():
    import torch
    from measure_ia_gb300 import _lib as L
    from measure_ia_gb300.engine import PairCounter, context

    pc = PairCounter("w", boxsize=100.0, r_bins=np.logspace(-1, np.log10(20.0), 11), r_min=0.1, r_max=20.0,
                     p_bins=np.linspace(-20.0, 20.0, 9), l_subboxes=3, precision="fp64")
    big = 2_000_000
    assert pc.workspace_bytes(big, big) > L.STATIC_SCRATCH_BYTES
    # the size check happens on the host before any device work; the buffers below are never read
    small = torch.zeros(16, dtype=torch.float64, device="cuda")
    out = torch.zeros(pc.layout.total, dtype=torch.float64, device="cuda")
    npairs = torch.zeros((1 + pc.J) * pc.n_r * pc.n_p, dtype=torch.int64, device="cuda")
    cat = L.Catalog()
    for f in ("position", "weight", "position_shape", "axis_direction", "q", "weight_shape"):
        setattr(cat, f, small.data_ptr())
    cat.n_pos = big
    cat.n_shape = big
    res = L.Result()
    res.out = out.data_ptr()
    res.npairs = npairs.data_ptr()
    lib = L.load()
    ctx = context(0)
    rc = lib.mia_measure_static(ctx, C.byref(pc.cfg), C.byref(cat), C.byref(res), None)
    assert rc == L.MIA_ERR_WORKSPACE
    assert "static scratch" in lib.mia_last_error(ctx).decode()


def test_static_scratch_entry_point_reports_invalid_arguments():
    """An empty shape sample gets the same message from both entry points."""
    import torch
    from measure_ia_gb300 import _lib as L
    from measure_ia_gb300.engine import PairCounter, context

    pc = PairCounter("w", boxsize=100.0, r_bins=np.logspace(-1, np.log10(20.0), 11), r_min=0.1, r_max=20.0,
                     p_bins=np.linspace(-20.0, 20.0, 9), l_subboxes=3, precision="mixed")
    small = torch.zeros(16, dtype=torch.float64, device="cuda")
    out = torch.zeros(pc.layout.total, dtype=torch.float64, device="cuda")
    npairs = torch.zeros((1 + pc.J) * pc.n_r * pc.n_p, dtype=torch.int64, device="cuda")
    cat = L.Catalog()
    for f in ("position", "weight", "position_shape", "axis_direction", "q", "weight_shape"):
        setattr(cat, f, small.data_ptr())
    cat.n_pos = 5
    cat.n_shape = 0
    res = L.Result()
    res.out = out.data_ptr()
    res.npairs = npairs.data_ptr()
    lib = L.load()
    ctx = context(0)
    rc = lib.mia_measure_static(ctx, C.byref(pc.cfg), C.byref(cat), C.byref(res), None)
    msg_static = lib.mia_last_error(ctx).decode()
    ws = torch.empty(256, dtype=torch.uint8, device="cuda")
    rc2 = lib.mia_measure(ctx, C.byref(pc.cfg), C.byref(cat), C.c_void_p(ws.data_ptr()), ws.numel(), C.byref(res),
                          None)
    msg = lib.mia_last_error(ctx).decode()
    assert rc == rc2 == L.MIA_ERR_ARG
    assert msg_static == msg == "empty position or shape sample"
