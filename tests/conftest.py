import importlib
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgbsw.so")


@pytest.fixture(scope="session")
def gbsw():
    return importlib.import_module("gpu-bsw_gb300")


@pytest.fixture(scope="session")
def workloads():
    mod = importlib.import_module("gpu-bsw_gb300.workloads")
    importlib.import_module("gpu-bsw_gb300.build").build_synth()
    return mod


@pytest.fixture(scope="session")
def built(gbsw):
    importlib.import_module("gpu-bsw_gb300.build").build_all()
    return gbsw


@pytest.fixture(scope="session")
def aligner(built):
    a = built.Aligner(0)
    yield a
    a.close()
