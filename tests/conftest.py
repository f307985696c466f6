import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def ref_lib():
    """The reference's own sources compiled on the host (oracle/ref/build_ref.py);
    skipped where the reference tree is absent."""
    from oracle.ref import build_ref

    so = build_ref.build()
    if so is None:
        pytest.skip("reference sources not present on this machine")
    import ctypes as C

    return C.CDLL(so)


@pytest.fixture(scope="session")
def vxl():
    """libvxl through its C ABI on cuda:0 (GPU tests only)."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import voxelengine_gb300 as V

    V.build()
    return V


@pytest.fixture(scope="session")
def ctx(vxl):
    return vxl.Context(0)
