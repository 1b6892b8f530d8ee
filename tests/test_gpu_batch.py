"""Batched catalogues (one persistent pair-kernel launch over many uneven
catalogues, optionally replayed from a CUDA graph) give the same products as
measuring each catalogue alone: integer counts bit-exact, values to 1e-12."""

import numpy as np
import pytest

from golden_io import assert_close

pytestmark = pytest.mark.gpu

KEYS = ("DD_all", "Splus_all", "scross", "rr", "rr_jk", "xi_gp_jk", "xi_gg_jk", "proj_gp", "proj_gg", "proj_gp_jk",
        "cov_gp", "cov_gg")


def _catalogues():
    from measure_ia_gb300.catalogs import neyman_scott_catalog
    sizes = [100, 900, 60, 2500, 300, 1600]  # parents; ~50 children each (5k .. 125k galaxies)
    return [neyman_scott_catalog(n, 205.0, max(1000, n * 12), 40 + i, mean_children=50, sigma=1.0)
            for i, n in enumerate(sizes)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_equals_individual_measurements(precision):
    import torch
    from measure_ia_gb300.engine import BatchCounter, PairCounter
    pc = PairCounter("w", boxsize=205.0, r_bins=np.logspace(-1, np.log10(20.0), 11), r_min=0.1, r_max=20.0,
                     p_bins=np.linspace(-20.0, 20.0, 9), l_subboxes=3, precision=precision)
    dcats = [pc.to_device(c) for c in _catalogues()]
    singles = []
    for d in dcats:
        bufs = pc.allocate(d["Position"].shape[0], d["Position_shape_sample"].shape[0])
        pc.run(d, bufs)
        singles.append(pc.fetch(bufs))
    batch = BatchCounter(pc, dcats)
    batch.prepare()
    batch.run()
    for i, ref in enumerate(singles):
        got = batch.fetch(i)
        np.testing.assert_array_equal(got.npairs, ref.npairs)
        for k in KEYS:
            assert_close(got[k], ref[k], 1e-12, f"catalogue {i}: {k}")
        assert got.stats["binned_pairs"] == ref.stats["binned_pairs"]
    # the same batch recorded in a CUDA graph and replayed twice
    batch.capture()
    for _ in range(2):
        for o in batch.outs:
            o.fill_(float("nan"))
        batch.replay()
        torch.cuda.synchronize()
        for i, ref in enumerate(singles):
            got = batch.fetch(i)
            np.testing.assert_array_equal(got.npairs, ref.npairs)
            assert_close(got["proj_gp"], ref["proj_gp"], 1e-12, f"graph replay {i}")
            assert_close(got["cov_gg"], ref["cov_gg"], 1e-12, f"graph replay {i}")


def test_multipoles_batch():
    from measure_ia_gb300.engine import BatchCounter, PairCounter
    pc = PairCounter("m", boxsize=205.0, r_bins=np.logspace(-1, np.log10(20.0), 11), r_min=0.1, r_max=20.0,
                     p_bins=np.linspace(-1.0, 1.0, 21), l_subboxes=3, precision="mixed")
    dcats = [pc.to_device(c) for c in _catalogues()[:3]]
    batch = BatchCounter(pc, dcats)
    batch.prepare()
    batch.run()
    for i, d in enumerate(dcats):
        bufs = pc.allocate(d["Position"].shape[0], d["Position_shape_sample"].shape[0])
        pc.run(d, bufs)
        ref = pc.fetch(bufs)
        got = batch.fetch(i)
        np.testing.assert_array_equal(got.npairs, ref.npairs)
        assert_close(got["proj_gp"], ref["proj_gp"], 1e-12, "multipole g+")


def test_w_and_multipoles_in_one_graph():
    """w and multipoles of the same uneven catalogues captured in one CUDA
    graph (two batches, one persistent pair-kernel launch each) and replayed
    twice: every catalogue's products equal its single measurements."""
    import torch
    from measure_ia_gb300.engine import BatchCounter, PairCounter, capture_batches
    common = dict(boxsize=205.0, r_bins=np.logspace(-1, np.log10(20.0), 11), r_min=0.1, r_max=20.0, l_subboxes=3,
                  precision="mixed")
    pw = PairCounter("w", p_bins=np.linspace(-20.0, 20.0, 9), **common)
    pm = PairCounter("m", p_bins=np.linspace(-1.0, 1.0, 21), **common)
    dcats = [pw.to_device(c) for c in _catalogues()[:4]]
    refs = {}
    for name, pc in (("w", pw), ("m", pm)):
        for i, d in enumerate(dcats):
            bufs = pc.allocate(d["Position"].shape[0], d["Position_shape_sample"].shape[0])
            pc.run(d, bufs)
            refs[name, i] = pc.fetch(bufs)
    bw, bm = BatchCounter(pw, dcats), BatchCounter(pm, dcats)
    bw.prepare()
    bm.prepare()
    g = capture_batches([bw, bm])
    for _ in range(2):
        for b in (bw, bm):
            for o in b.outs:
                o.fill_(float("nan"))
        g.replay()
        torch.cuda.synchronize()
        bw.status()
        bm.status()
        for name, b in (("w", bw), ("m", bm)):
            for i in range(len(dcats)):
                got, ref = b.fetch(i), refs[name, i]
                np.testing.assert_array_equal(got.npairs, ref.npairs)
                for k in ("proj_gp", "proj_gg", "cov_gp"):
                    assert_close(got[k], ref[k], 1e-12, f"{name} catalogue {i}: {k}")


def test_batch_tuned_on_the_whole_batch(tmp_path, monkeypatch):
    """Launch knobs tuned on a batch as a whole change its speed, never its
    products: the tuned batch's counts equal the single measurements'."""
    from measure_ia_gb300.engine import BatchCounter, PairCounter
    monkeypatch.setenv("MIA_TUNE_CACHE", str(tmp_path / "tune.json"))
    pc = PairCounter("w", boxsize=205.0, r_bins=np.logspace(-1, np.log10(20.0), 11), r_min=0.1, r_max=20.0,
                     p_bins=np.linspace(-20.0, 20.0, 9), l_subboxes=3, precision="mixed")
    dcats = [pc.to_device(c) for c in _catalogues()[:3]]
    tuned = BatchCounter(pc, dcats).tuned()
    import json
    assert len(json.load(open(tmp_path / "tune.json"))) == 1  # the choice is cached per batch shape
    tuned.prepare()
    tuned.run()
    for i, d in enumerate(dcats):
        ref = pc.measure({k: v for k, v in d.items()})
        np.testing.assert_array_equal(tuned.fetch(i).npairs, ref.npairs)
        assert_close(tuned.fetch(i)["proj_gp"], ref["proj_gp"], 1e-12, f"tuned batch {i}")
