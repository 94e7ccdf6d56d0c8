"""Shared fixtures. Tests marked ``gpu`` need a CUDA device and the built libfxe.so; the rest
run on the CPU (oracle, host-side preparation, library loading)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device and the built CUDA library")


def _cuda_ok():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    # the no-allocation entry point's file runs last, after every other test has used the device
    items.sort(key=lambda it: 1 if os.path.basename(str(it.fspath)).startswith("test_zz_") else 0)
    if _cuda_ok():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def small_system():
    """2,000-atom receptor, 8 A cleft, 24-atom ligand with 6 torsions (seed 11)."""
    from flexaidds_gb300 import prepare, system
    inp = system.make_inputs(2000, 8.0, 24, 6, seed=11)
    return inp, prepare.prepare(inp)


@pytest.fixture(scope="session")
def tiny_system():
    """600-atom receptor, 6 A cleft, 12-atom ligand with 3 torsions (seed 5)."""
    from flexaidds_gb300 import prepare, system
    inp = system.make_inputs(600, 6.0, 12, 3, seed=5)
    return inp, prepare.prepare(inp)


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GOLDEN_NAMES = ("c0_2000_24", "curves_900_16", "outside_600_10", "scale_6000_48", "flex_2000_24",
                "flexcurves_900_16", "flexscale_6000_48")


def load_golden(name):
    """(Descriptor, fixture arrays) of tests/golden/<name>.npz (made by make_golden.py)."""
    import numpy as np
    from flexaidds_gb300.system import Descriptor
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return Descriptor.from_arrays(z, "d_"), {k: z[k] for k in z.files if not k.startswith("d_")}


@pytest.fixture(scope="session", params=GOLDEN_NAMES)
def golden(request):
    return (request.param,) + load_golden(request.param)
