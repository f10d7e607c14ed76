import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the CUDA library")


@pytest.fixture(scope="session")
def built_lib():
    from specfem3d_geotech_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def ctx(built_lib):
    import specfem3d_geotech_gb300 as sg
    return sg.default_context()
