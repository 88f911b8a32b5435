"""gsnp_decompress: the -C reader (gsnp_gb300/csrc/decompress.cpp).

- Its text equals the reference decompressor's (cpp/decompression.cpp) on
  the oracle's -C files.  The golden digests of tests/golden/golden.json pin
  this for c0 and c1 in test_golden.py; here the reference tool itself
  (oracle/_ref/gsnp_ref_decompress, built where the reference tree is
  mounted) is compared directly on c2 (deep hotspots, mixed read lengths) and
  c3 (qualities up to 60).
- Its check mode (the reference's check(), cpp/decompression.cpp:236-401)
  passes a cns text against the -C files of the same run and names the first
  differing row and column when one value is changed.
"""
import os
import subprocess

import pytest

from gsnp_gb300 import build, synth

from oracle_run import flags_for

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_DECOMPRESS = os.path.join(ROOT, "oracle", "_ref", "gsnp_ref_decompress")


def oracle_run(oracle_bin, name, scale, d, compress):
    w = synth.make_workload(name, scale=scale)
    paths = synth.write_inputs(w, str(d))
    flags = [f for f in flags_for(w, paths) if f != "-C"] + (["-C"] if compress else [])
    out = os.path.join(str(d), "cns")
    r = subprocess.run([oracle_bin, "-i", paths["soap"], "-d", paths["ref"], "-o", out] + flags, cwd=str(d),
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


@pytest.mark.parametrize("name,scale", [("c2", 0.01), ("c3", 0.004)])
def test_matches_reference_decompressor(name, scale, tmp_path, oracle_bin, native_lib):
    if not os.path.exists(REF_DECOMPRESS):
        pytest.skip("the reference decompressor is built only where the reference tree is mounted")
    base = oracle_run(oracle_bin, name, scale, tmp_path, True)
    ours, theirs = str(tmp_path / "ours.txt"), str(tmp_path / "ref.txt")
    r = subprocess.run([build.DECOMPRESS, base, ours], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    subprocess.run([REF_DECOMPRESS, base, theirs], check=True, capture_output=True)
    with open(ours, "rb") as a, open(theirs, "rb") as b:
        assert a.read() == b.read()


def test_check_mode(tmp_path, oracle_bin, native_lib):
    (tmp_path / "c").mkdir()
    (tmp_path / "t").mkdir()
    base = oracle_run(oracle_bin, "c1", 0.004, tmp_path / "c", True)
    text = oracle_run(oracle_bin, "c1", 0.004, tmp_path / "t", False)
    r = subprocess.run([build.DECOMPRESS, "--check", text, base], capture_output=True, text=True)
    assert r.returncode == 0 and "rows match" in r.stdout, r.stdout + r.stderr
    # one count changed in the text: the first difference is named
    rows = open(text).read().split("\n")
    f = rows[1234].split("\t")
    f[7] = str(int(f[7]) + 1)
    rows[1234] = "\t".join(f)
    planted = str(tmp_path / "planted.cns")
    with open(planted, "w") as fh:
        fh.write("\n".join(rows))
    r = subprocess.run([build.DECOMPRESS, "--check", planted, base], capture_output=True, text=True)
    assert r.returncode == 1 and "row 1234" in r.stdout and "column 8" in r.stdout, r.stdout
