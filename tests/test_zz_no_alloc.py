"""gsnp_dict_compress_static: the -C dictionary codec over statically reserved
device scratch, for callers that cannot allocate device memory on their path.

Its results are compared with the existing entry point, the reference-
compatible cuda_dictCompression of libgsnp_backend.so, on two calls in a row
for every element type.  The file is named to be collected last, so that it
also runs after every other test in one process; test_fresh_process repeats
the comparison in a new interpreter.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GSNP_OK, GSNP_ERR_CAPACITY = 0, 4
MAX_VALUES = 32 * 8192
# element type -> (GSNP_DICT_* code, numpy dtype, mangled cuda_dictCompression overload)
TYPES = {
    "char": (0, np.int8, "_Z20cuda_dictCompressionPjPmPcS0_S1_m"),
    "int": (1, np.int32, "_Z20cuda_dictCompressionPjPmPiS0_S1_m"),
    "uint32": (2, np.uint32, "_Z20cuda_dictCompressionPjPmS_S0_S_m"),
    "double": (3, np.float64, "_Z20cuda_dictCompressionPjPmPdS0_S1_m"),
}
P = ctypes.c_void_p


def libs():
    from gsnp_gb300 import build
    build.build()
    api = ctypes.CDLL(build.LIB)
    f = api.gsnp_dict_compress_static
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, P, ctypes.c_uint64, P, P, P, P, P]
    backend = ctypes.CDLL(build.BACKEND_LIB)
    return api, backend


def sample(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "double":
        v = np.round(rng.normal(1.0, 0.3, n), 3)
        v[rng.random(n) < 0.05] = 255.0
        return v
    dt = TYPES[kind][1]
    hi = 90 if kind == "char" else 5000
    return rng.integers(0, hi, n).astype(dt)


def static_call(api, kind, values):
    code, dt, _ = TYPES[kind]
    n = values.size
    words = np.zeros(max(n, 1), np.uint32)
    dct = np.zeros(max(n, 1), dt)
    nw, nd = ctypes.c_uint64(words.size), ctypes.c_uint64(dct.size)
    rc = api.gsnp_dict_compress_static(code, values.ctypes.data, n, words.ctypes.data, ctypes.byref(nw),
                                       dct.ctypes.data, ctypes.byref(nd), None)
    return rc, words[:nw.value].copy(), dct[:nd.value].copy()


def reference_call(backend, kind, values):
    _, dt, sym = TYPES[kind]
    n = values.size
    f = getattr(backend, sym)
    f.restype = None
    f.argtypes = [P, P, P, P, P, ctypes.c_ulong]
    words = np.zeros(max(n, 1), np.uint32)
    dct = np.zeros(MAX_VALUES, dt)
    nw, nd = ctypes.c_ulong(words.size), ctypes.c_ulong(dct.size)
    f(words.ctypes.data, ctypes.byref(nw), dct.ctypes.data, ctypes.byref(nd), values.ctypes.data, n)
    return words[:nw.value].copy(), dct[:nd.value].copy()


def compare_all():
    api, backend = libs()
    for kind in TYPES:
        for seed, n in ((1, 20000), (2, MAX_VALUES)):   # two calls in a row, different inputs
            v = sample(kind, n, seed)
            rc, w, d = static_call(api, kind, v)
            assert rc == GSNP_OK, (kind, rc)
            rw, rd = reference_call(backend, kind, v)
            assert np.array_equal(w, rw), kind
            assert np.array_equal(d.view(np.uint8), rd.view(np.uint8)), kind
    return True


def test_rejects_oversize_input():
    """More values than the static scratch holds: GSNP_ERR_CAPACITY, before
    any device work (so this runs without a GPU too)."""
    api, _ = libs()
    v = np.zeros(MAX_VALUES + 1, np.int32)
    rc, _, _ = static_call(api, "int", v)
    assert rc == GSNP_ERR_CAPACITY


@pytest.mark.gpu
def test_matches_existing_entry_point():
    assert compare_all()


@pytest.mark.gpu
def test_fresh_process():
    code = "import sys; sys.path.insert(0, %r); import test_zz_no_alloc as t; t.compare_all(); print('ok')" % (
        os.path.join(ROOT, "tests"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr
