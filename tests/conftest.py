import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "bimsim-cuda_gb300"), os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")


@pytest.fixture(scope="session")
def oracle():
    import oracle_lib
    return oracle_lib.load()


@pytest.fixture(scope="session")
def ref_lib():
    """The reference's own host code (oracle/_ref), where it was built; else skip."""
    import oracle_lib
    lib = oracle_lib.load_ref()
    if lib is None:
        pytest.skip("oracle/_ref not built (needs the reference checkout)")
    return lib


@pytest.fixture(scope="session")
def golden():
    import json
    d = os.path.join(REPO, "tests", "golden")

    def get(name):
        with open(os.path.join(d, name + ".json")) as fh:
            return json.load(fh)
    return get
