"""The exact %#.6g formatter of the GPU text emitter (gsnp_gb300/csrc/fmt_g6.h)
against the C library's printf, on every copy ratio of depth <= 1500, random
doubles and values at rounding boundaries (tests/native/fmt_g6_check.cpp)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_fmt_g6_matches_printf(tmp_path):
    exe = str(tmp_path / "fmt_g6_check")
    src = os.path.join(ROOT, "tests", "native", "fmt_g6_check.cpp")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                        "-I" + os.path.join(ROOT, "gsnp_gb300", "csrc"), src, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "checked" in r.stdout
