import importlib.util
import os
import sys
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (runs the CUDA runtime)")


def _load(name, rel):
    spec = importlib.util.spec_from_file_location(name, os.path.join(ROOT, rel))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def host():
    return _load("gpumpi_host", "dphpc-project_gb300/gpumpi_host.py")


@pytest.fixture(scope="session")
def oracle_built(host):
    r = subprocess.run(["make", "-C", host.ORACLE, f"-j{os.cpu_count() or 1}"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return host


@pytest.fixture(scope="session")
def gpu_built(oracle_built):
    host = oracle_built
    r = subprocess.run(["make", "-C", host.PKG, f"-j{os.cpu_count() or 1}"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-4000:]
    return host
