"""The FP32 + FP64-fixup form's claims, on the CPU with the kernels' own
per-site code (site_math.cuh and column.cuh compiled for the host) and the
library's own tables (tables.cpp), in tests/native/posterior_check.cpp:

- the FP32 likelihood sums stay within |S32 - S64| <= |S32| GSNP_FP32_K(num)
  of the FP64 sums in the reference's record order;
- every call decided from FP32 sums (fast_posterior, and site_posterior with
  the error bounds) equals the FP64 posterior's, on realistic sites and on
  adversarial sums placed next to genotype ties and quality boundaries.
"""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def posterior_check(tmp_path_factory):
    from gsnp_gb300 import build
    exe = str(tmp_path_factory.mktemp("posterior") / "posterior_check")
    csrc = os.path.join(ROOT, "gsnp_gb300", "csrc")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-I" + csrc,
                        "-I" + os.path.join(ROOT, "include"), "-I" + build._cuda_include(),
                        os.path.join(ROOT, "tests", "native", "posterior_check.cpp"),
                        os.path.join(csrc, "tables.cpp"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.mark.parametrize("seed", [1, 2])
def test_fp32_decisions_equal_fp64(seed, posterior_check):
    r = subprocess.run([posterior_check, "300000", str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    m = re.search(r"sites (\d+) fp32-decided (\d+) bounded-decided (\d+) max-relerr (\S+) adversarial (\d+) "
                  r"decided (\d+)", r.stdout)
    assert m, r.stdout
    sites, fast, bounded, _, adv, adv_decided = m.groups()
    # not vacuous: most sites and most adversarial sums are decided in FP32
    assert int(fast) > int(sites) // 2 and int(bounded) > int(sites) * 9 // 10
    assert int(adv) > int(sites) and int(adv_decided) > int(adv) // 2
