"""The restated backend (oracle/backend.cpp, oracle/calling.cpp) against the
reference's own CPU twins of its calling kernels: gold_updateSparse
(kernel/update_kernel.cu:96-195), likelihoodSparse_kernel compiled for the
host (kernel/likelihood_kernel.cu:168-256), gold_posterior and its rank-sum
test (kernel/posterior_kernel.cu:90-426).

`make -C oracle ref-gold` copies those line ranges out of the reference tree
at build time (nothing of them is in this repository) and links them, through
oracle/gold/twins.cpp, with oracle/gold/check.cpp.  The check runs four
windows of 262,144 sites (over a million sites, tens of millions of records)
through both and compares pileups, sorted records, type_likely bit for bit
and every posterior field.  Needs the reference tree ($GSNP_REFERENCE, or the
tree oracle/_ref was built from); skipped elsewhere.
"""
import json
import os
import subprocess

import pytest

from conftest import reference_tree

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CHECK = os.path.join(ROOT, "oracle", "_ref", "gold_check")


@pytest.fixture(scope="module")
def gold_check():
    tree = reference_tree()
    if tree is None:
        pytest.skip("reference tree not mounted ($GSNP_REFERENCE)")
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "-j8", "ref-gold", "REF=" + tree],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return CHECK


def run(exe, seed, windows, plant=False):
    env = dict(os.environ)
    if plant:
        env["GOLD_CHECK_PLANT"] = "1"
    r = subprocess.run([exe, str(seed), str(windows)], capture_output=True, text=True, env=env, timeout=600)
    return r.returncode, json.loads(r.stdout.strip().splitlines()[-1]), r.stderr


def test_backend_matches_reference_twins(gold_check):
    rc, res, err = run(gold_check, 20261, 4)
    assert rc == 0 and res["mismatches"] == 0, err[-2000:]
    assert res["sites_called"] >= 1_000_000
    assert res["records"] >= 20_000_000
    assert res["known_snp_sites"] > 10_000
    assert res["sites_200_records_or_more"] > 1_000     # the 255-record cap and pcr dependency
    assert res["het_calls"] > 1_000 and res["het_calls_normal_path"] > 0   # both rank-sum paths
    print(json.dumps(res))


def test_check_reports_a_planted_difference(gold_check):
    rc, res, err = run(gold_check, 7, 1, plant=True)
    assert rc != 0 and res["mismatches"] == 1, err[-2000:]
    assert "q_cns" in err
