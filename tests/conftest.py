import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built extension")
    config.addinivalue_line("markers", "slow: long-running CPU test")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        have_gpu = torch.cuda.is_available()
    except Exception:
        have_gpu = False
    if have_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


def pytest_terminal_summary(terminalreporter):
    """How many fixture cases had their floats checked against the oracle on
    this host instead of the fixture (whose bins follow the build host's
    numpy log10)."""
    mod = sys.modules.get("test_gpu_parity")
    if mod is None or not getattr(mod, "CHECKED", None):
        return
    fb = mod.FALLBACKS
    terminalreporter.write_line(f"parity: {len(fb)} of {len(mod.CHECKED)} fixture case(s) compared against the "
                                f"host oracle (fixture bins differ on this host){': ' + ', '.join(fb) if fb else ''}")
