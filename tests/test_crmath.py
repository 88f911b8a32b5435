"""The correctly rounded exp/log10 of include/gsnp_crmath.h against exact
decimal arithmetic (CPU).  The kernels and the oracle share these functions for
the per-site transcendentals, so their rounding is pinned here."""
import ctypes
import math
import os
import random
import subprocess
from decimal import Decimal, getcontext

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def crlib(tmp_path_factory):
    d = tmp_path_factory.mktemp("crmath")
    src = d / "cr.c"
    src.write_text('#include "gsnp_crmath.h"\n'
                   'double t_exp(double x){return gsnp_cr_exp(x);}\n'
                   'double t_log10(double x){return gsnp_cr_log10(x);}\n')
    so = d / "cr.so"
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(so), "-lm"], check=True)
    lib = ctypes.CDLL(str(so))
    for f in (lib.t_exp, lib.t_log10):
        f.restype = ctypes.c_double
        f.argtypes = [ctypes.c_double]
    return lib


def exact(fn, x):
    getcontext().prec = 60
    return float(fn(Decimal(x)))


def test_exp_correctly_rounded(crlib):
    rnd = random.Random(7)
    xs = [rnd.uniform(-18.0, 0.0) for _ in range(4000)] + [rnd.uniform(-700, 700) for _ in range(1000)]
    xs += [0.0, -0.5, -1.0, 1.0, -17.999]
    for x in xs:
        assert crlib.t_exp(x) == exact(Decimal.exp, x), x


def test_log10_correctly_rounded(crlib):
    rnd = random.Random(11)
    xs = [rnd.random() for _ in range(3000)] + [math.exp(rnd.uniform(-40, 5)) for _ in range(2000)]
    xs += [10.0 ** k for k in range(-18, 4)] + [1.0, 0.5, 0.1, 0.001, 0.0005, 0.004, 2e-4, 1e-300]
    for x in xs:
        assert crlib.t_log10(x) == exact(Decimal.log10, x), x
    assert crlib.t_log10(1.0) == 0.0
