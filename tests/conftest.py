import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built library")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def model_dir(tmp_path_factory):
    """Write a named synthetic model once per session; returns its directory."""
    from radlite_gb300 import synth
    cache = {}

    def make(name, **over):
        key = (name, tuple(sorted(over.items())))
        if key not in cache:
            d = tmp_path_factory.mktemp(name)
            synth.write_model(synth.config_by_name(name, **over), str(d))
            cache[key] = str(d)
        return cache[key]

    return make


@pytest.fixture(scope="session")
def gpu_lib():
    """The built CUDA library (built here if missing); skips nothing: GPU tests need it."""
    import radlite_gb300
    from radlite_gb300 import build
    if not os.path.exists(radlite_gb300.LIB_PATH):
        build.build()
    return radlite_gb300
