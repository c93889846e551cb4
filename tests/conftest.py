import importlib.util
import os
import sys
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (runs the CUDA runtime)")


def reference_tree():
    """The reference tree's path as oracle/ref.mk resolves it
    (GPUMPI_REFERENCE_TREE overrides it), or None when it is not present."""
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "-f", "ref.mk", "print-ref"],
                       capture_output=True, text=True)
    path = r.stdout.strip()
    if r.returncode == 0 and path and os.path.isdir(os.path.join(path, "toolchain_tests")):
        return path
    return None


def _load(name, rel):
    spec = importlib.util.spec_from_file_location(name, os.path.join(ROOT, rel))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def host():
    return _load("gpumpi_host", "dphpc-project_gb300/gpumpi_host.py")


def oracle_module():
    return _load("hostmpi_run", "oracle/hostmpi_run.py")


def run_oracle(name, args=None, nranks=2, extra=None, timeout=300.0):
    """A workload program on the host cores through the hostmpi oracle."""
    return oracle_module().run_oracle(name, args, nranks=nranks, extra=extra, timeout=timeout)


@pytest.fixture(scope="session")
def oracle_built():
    mod = oracle_module()
    mod.build(reference=False)
    return mod


@pytest.fixture(scope="session")
def gpu_built(oracle_built, host):
    r = subprocess.run(["make", "-C", host.PKG, f"-j{os.cpu_count() or 1}"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-4000:]
    return host
