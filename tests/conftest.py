"""Shared test set-up: import paths, the gpu marker, common fixtures."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gpu-out-of-core-volume-data_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the CUDA path")


@pytest.fixture(scope="session")
def gc():
    import gcbuild as pkg_build

    pkg_build.build()
    import gcgb300

    return gcgb300


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle

    return oracle


@pytest.fixture(scope="session")
def torch_cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for gpu-marked tests")
    torch.cuda.init()
    return torch


@pytest.fixture(autouse=True)
def exact_ray_caster():
    """Every test starts and ends with the exact ray-caster build (the FP32
    oracle's operations); tests of the fast build switch it on themselves."""
    yield
    mod = sys.modules.get("gcgb300")
    if mod is not None:
        mod.render_precision(mod.RENDER_EXACT)
