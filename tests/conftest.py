"""Shared fixtures: build the oracle and the native library once per session."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def reference_tree():
    """The reference source tree: $GSNP_REFERENCE, else the tree that
    __graft_entry__.build() compiled oracle/_ref from (recorded in
    oracle/_ref/reference_tree), else None."""
    env = os.environ.get("GSNP_REFERENCE")
    if env:
        return env if os.path.isdir(env) else None
    rec = os.path.join(ROOT, "oracle", "_ref", "reference_tree")
    if os.path.exists(rec):
        with open(rec) as f:
            path = f.read().strip()
        return path if os.path.isdir(path) else None
    return None


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
