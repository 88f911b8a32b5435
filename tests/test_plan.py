"""The window replay (gsnp_gb300/csrc/plan.cpp), whose per-alignment pass runs
in parallel chunks, against a walk over the alignments one at a time that
follows the reference's window loop (Call_win::new_soap2cns,
cpp/call_genotype.cc:474-644): calls, host-count and likelihood sources,
deposited alignments and errors (tests/native/plan_check.cpp)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_parallel_replay_matches_sequential_walk(tmp_path):
    from gsnp_gb300 import build
    exe = str(tmp_path / "plan_check")
    csrc = os.path.join(ROOT, "gsnp_gb300", "csrc")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-pthread", "-I" + csrc,
                        "-I" + os.path.join(ROOT, "include"), "-I" + build._cuda_include(),
                        os.path.join(ROOT, "tests", "native", "plan_check.cpp"), os.path.join(csrc, "plan.cpp"),
                        "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "checked" in r.stdout
