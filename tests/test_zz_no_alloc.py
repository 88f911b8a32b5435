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


def sample(kind, n, seed, wide=False):
    """n values of an element type.  Narrow samples hold a few thousand
    distinct values (the dictionary sorted in shared memory); wide ones span
    the type's range (integers) or hold tens of thousands of distinct doubles
    with both zeros, so that the dictionary is sorted in global memory and the
    indices take up to 18 bits."""
    rng = np.random.default_rng(seed)
    if kind == "double":
        if wide:
            v = rng.normal(0.0, 1e3, n)
            v[rng.random(n) < 0.02] = 0.0
            v[rng.random(n) < 0.02] = -0.0
            return v
        v = np.round(rng.normal(1.0, 0.3, n), 3)
        v[rng.random(n) < 0.05] = 255.0
        return v
    dt = TYPES[kind][1]
    if wide:
        info = np.iinfo(dt)
        return rng.integers(int(info.min), int(info.max), n, endpoint=True, dtype=np.int64).astype(dt)
    hi = 90 if kind == "char" else 5000
    return rng.integers(0, hi, n).astype(dt)


def static_call(api, kind, values, words_cap=None, stream=None):
    code, dt, _ = TYPES[kind]
    n = values.size
    words = np.zeros(max(n, 1), np.uint32)
    dct = np.zeros(max(n, 1), dt)
    nw = ctypes.c_uint64(words.size if words_cap is None else words_cap)
    nd = ctypes.c_uint64(dct.size)
    rc = api.gsnp_dict_compress_static(code, values.ctypes.data if n else None, n, words.ctypes.data,
                                       ctypes.byref(nw), dct.ctypes.data, ctypes.byref(nd), stream)
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


def check_same(api, backend, kind, v, stream=None):
    rc, w, d = static_call(api, kind, v, stream=stream)
    assert rc == GSNP_OK, (kind, rc)
    rw, rd = reference_call(backend, kind, v)
    assert np.array_equal(w, rw), kind
    assert np.array_equal(d.view(np.uint8), rd.view(np.uint8)), kind


def compare_all():
    api, backend = libs()
    for kind in TYPES:
        # two calls in a row with different inputs, then the wide sample
        for seed, n, wide in ((1, 20000, False), (2, MAX_VALUES, False), (3, MAX_VALUES, True)):
            check_same(api, backend, kind, sample(kind, n, seed, wide))
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


@pytest.mark.gpu
def test_word_capacity_error_then_valid_call():
    """Too small a word array: GSNP_ERR_CAPACITY once the distinct count is
    known, with no kernel of the call left running; the next call is right."""
    api, backend = libs()
    v = sample("uint32", 50000, 5, wide=True)
    rc, _, _ = static_call(api, "uint32", v, words_cap=10)
    assert rc == GSNP_ERR_CAPACITY
    check_same(api, backend, "uint32", v)
    check_same(api, backend, "int", sample("int", 30000, 6))


@pytest.mark.gpu
def test_on_a_stream_of_the_caller():
    """The call runs on the cudaStream_t it is given (not the default stream)
    and returns with its outputs in host memory."""
    import torch
    api, backend = libs()
    s = torch.cuda.Stream()
    for seed in (7, 8):
        v = sample("double", 40000, seed, wide=True)
        check_same(api, backend, "double", v, stream=ctypes.c_void_p(s.cuda_stream))


@pytest.mark.gpu
def test_second_call_allocates_nothing():
    """After the first call has reserved the static scratch, a call leaves
    the device's free memory unchanged: it allocates nothing."""
    import torch
    api, backend = libs()
    torch.cuda.init()
    rc, _, _ = static_call(api, "int", np.zeros(0, np.int32))   # set-up only
    assert rc == GSNP_OK
    v1, v2 = sample("int", MAX_VALUES, 9, wide=True), sample("int", MAX_VALUES, 10, wide=True)
    first = static_call(api, "int", v1)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    second = static_call(api, "int", v2)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    for v, (rc, w, d) in ((v1, first), (v2, second)):
        assert rc == GSNP_OK
        rw, rd = reference_call(backend, "int", v)
        assert np.array_equal(w, rw) and np.array_equal(d, rd)
