"""Opt-in timing of the pair kernel: a ring of CUDA event pairs recorded
around its launch on the caller's stream, read back oldest first."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_pair_kernel_timing_ring():
    import torch
    from measure_ia_gb300 import engine
    from measure_ia_gb300.catalogs import neyman_scott_catalog
    from measure_ia_gb300.engine import PairCounter
    data = neyman_scott_catalog(400, 205.0, 8000, 3, mean_children=40, sigma=1.0)
    pc = PairCounter("w", boxsize=205.0, r_bins=np.logspace(-1, np.log10(20.0), 11), r_min=0.1, r_max=20.0,
                     p_bins=np.linspace(-20.0, 20.0, 9), l_subboxes=3, precision="mixed")
    dcat = pc.to_device(data)
    bufs = pc.allocate(dcat["Position"].shape[0], dcat["Position_shape_sample"].shape[0])
    engine.profile_pairs(pc.device, 3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(4):
        pc.run(dcat, bufs)
    e1.record()
    torch.cuda.synchronize()
    ms = engine.pair_kernel_ms(pc.device, 10)
    assert len(ms) == 3                      # the ring keeps the last three launches
    assert all(m > 0.0 for m in ms)
    assert sum(ms) < e0.elapsed_time(e1)     # inside the four whole measurements
    assert engine.pair_kernel_ms(pc.device, 2) == ms[1:]
    engine.profile_pairs(pc.device, 0)       # off: nothing recorded
    pc.run(dcat, bufs)
    assert engine.pair_kernel_ms(pc.device, 10) == []
