"""The calling kernels' per-site column passes (gsnp_gb300/csrc/column.cuh),
compiled for the host: the chunked bitonic sort with its merge from the back
against std::sort, and the dependency walk with 1-, 2- and 4-bit saturating
counts against the reference's integer counter per (strand, cycle)
(kernel/likelihood_kernel.cu:200-232), in tests/native/column_check.cpp."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_column_sort_and_walk(tmp_path):
    from gsnp_gb300 import build
    exe = str(tmp_path / "column_check")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                        "-I" + os.path.join(ROOT, "gsnp_gb300", "csrc"), "-I" + os.path.join(ROOT, "include"),
                        "-I" + build._cuda_include(), os.path.join(ROOT, "tests", "native", "column_check.cpp"),
                        "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "checked" in r.stdout
