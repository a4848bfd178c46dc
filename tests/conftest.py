"""pytest configuration: the `gpu` marker and shared fixtures.

CPU tests (-m "not gpu") cover the oracle against the pinned checks, the
host-side logic and the exported C ABI.  GPU tests (-m gpu) are the parity
tests proper: they call libtsf_gb300 through its C ABI and compare with the
oracle on the same seeded inputs.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "tube-segmentation-framework_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

# The reference source tree (smistad/Tube-Segmentation-Framework), where one is
# checked out; tests that read it skip when it is absent.
REFERENCE = os.environ.get("TSF_REFERENCE_DIR", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def tsf():
    import tsf_gb300
    import build as tsf_build
    tsf_build.build()
    tsf_gb300.load()
    return tsf_gb300


@pytest.fixture(scope="session")
def synth():
    import synthetic
    return synthetic


@pytest.fixture(scope="session")
def reference_dir():
    if not os.path.isdir(REFERENCE):
        pytest.skip("reference source tree not present")
    return REFERENCE
