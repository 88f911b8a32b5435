"""Shared fixtures: build the oracle and the native library once per session."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) device")


@pytest.fixture(scope="session")
def oracle_bin():
    """The CPU oracle binary (oracle/_build/gsnp_oracle), built from oracle/."""
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "-j8"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return os.path.join(ROOT, "oracle", "_build", "gsnp_oracle")


@pytest.fixture(scope="session")
def native_lib():
    from gsnp_gb300 import build
    return build.build()
