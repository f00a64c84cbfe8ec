import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
CALF20 = os.path.join(GOLDEN, "calf20")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import binding
    binding.build()
    return binding


@pytest.fixture(scope="session")
def fmc_lib():
    """The CUDA library (built in-tree if stale)."""
    from fastmc_gb300 import build
    build.build()
    import fastmc_gb300
    fastmc_gb300.load()
    return fastmc_gb300


@pytest.fixture(scope="session")
def inputs_dir(tmp_path_factory):
    """Factory writing synthetic FIELD/CONFIG/CONTROL for a GcmcSpec."""
    from fastmc_gb300 import synthetic as syn
    base = tmp_path_factory.mktemp("inputs")
    cache = {}

    def make(spec, name):
        if name not in cache:
            d = str(base / name)
            syn.write_inputs(d, spec)
            cache[name] = d
        return cache[name]

    return make
