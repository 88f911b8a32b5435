"""The C ABI library without a GPU: it loads, exports every function the public
headers declare, builds the host tables, and fails cleanly (no crash) when no
device is present."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from gsnp_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_c_functions():
    text = open(os.path.join(ROOT, "include", "gsnp_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(gsnp_\w+)\(", text, re.M)))


def test_library_exports_header_symbols(native_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", native_lib], capture_output=True, text=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if line.strip())
    names = declared_c_functions()
    assert len(names) >= 15
    missing = [n for n in names if n not in exported]
    assert not missing, missing


BACKEND_SYMBOLS = [
    "GPUInit()", "GSNPKernelInit(", "cuda_init(", "cuda_updateSparse(", "cuda_likelihoodSparse(",
    "cuda_posterior(", "cuda_recycle(", "cuda_quickRecycle(", "gold_pos_match(", "getNumBinWord(",
    "encode(", "decode(", "dictComprStart(", "dictComprEnd()",
    "cuda_dictCompression(unsigned int*, unsigned long*, char*",
    "cuda_dictCompression(unsigned int*, unsigned long*, int*",
    "cuda_dictCompression(unsigned int*, unsigned long*, unsigned int*",
    "cuda_dictCompression(unsigned int*, unsigned long*, double*",
    "RLECompression(int*", "RLECompression(double*", "RLECompression(char*"]


def test_backend_library_exports_reference_symbols(native_lib):
    """The 20 C++ entry points (with overloads) the reference's host objects link against."""
    from gsnp_gb300 import build
    out = subprocess.run(["nm", "-DC", "--defined-only", build.BACKEND_LIB], capture_output=True, text=True).stdout
    exported = [ln.split(" T ", 1)[1] for ln in out.splitlines() if " T " in ln]
    for w in BACKEND_SYMBOLS:
        assert any(e.startswith(w) for e in exported), w
    # the C ABI library does not export the reference's C++ names
    out2 = subprocess.run(["nm", "-DC", "--defined-only", native_lib], capture_output=True, text=True).stdout
    assert "GPUInit()" not in out2


def test_reference_host_objects_link_against_backend(native_lib):
    """The reference's own host objects (compiled in place from its sources)
    link against libgsnp_backend.so with no unresolved symbol."""
    from conftest import reference_tree
    ref = reference_tree()
    if ref is None or not os.path.isdir(os.path.join(ref, "cpp")):
        pytest.skip("reference sources not present")
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref-link", "REF=" + ref],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert os.path.exists(os.path.join(ROOT, "oracle", "_ref", "gsnp_ref_gpu"))


def test_host_tables_without_gpu(native_lib):
    import gsnp_gb300
    lib = gsnp_gb300.native()
    p = api.params_from_flags(["-L", "50", "-t"])
    prior = np.zeros(128)
    assert lib.gsnp_prior_table(ctypes.byref(p), prior.ctypes.data) == 0
    # cpp/prior.cc:3-43 with -t: ref A, genotype AG is a transition het (0.001 * 4)
    assert prior[0 << 4 | 0 << 2 | 3] == 0.004 and prior[0] == 1.0
    assert prior[0 << 4 | 1 << 2 | 1] == 0.0005
    assert prior[4 << 4 | 0] == 0.0625
    rank = np.zeros(64 * 64 * 2048)
    assert lib.gsnp_rank_table(rank.ctypes.data) == 0
    # N = 2, n1 = 1: T1 in {1, 2}, each with probability 1/2 -> two-sided tails 0.5
    assert rank[(2 << 17) | (1 << 11) | 1] == 0.5
    assert rank[(2 << 17) | (1 << 11) | 2] == 0.5
    assert rank[5] == 1.0


def test_context_without_device_fails_cleanly(native_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import gsnp_gb300
    lib = gsnp_gb300.native()
    ctx = ctypes.c_void_p()
    rc = lib.gsnp_context_create(0, ctypes.byref(ctx))
    assert rc == 1 and not ctx
