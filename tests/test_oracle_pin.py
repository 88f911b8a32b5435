"""Pin of the CPU oracle: the restated driver (oracle/driver.cpp) must produce
the same bytes as the reference's own host sources compiled in place
(oracle/_ref/gsnp_ref, built by `make -C oracle ref` where the reference tree is
mounted), both linked to the restated backend.  Skipped where the reference
tree is absent (the GPU machine)."""
import os
import subprocess

import pytest

from conftest import reference_tree
from gsnp_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "gsnp_ref")


@pytest.fixture(scope="module")
def ref_bin():
    tree = reference_tree()
    if tree is None:
        pytest.skip("reference tree not mounted ($GSNP_REFERENCE)")
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "-j8", "ref", "REF=" + tree],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return REF_BIN


def run(exe, paths, flags, out_dir):
    os.makedirs(out_dir, exist_ok=True)
    r = subprocess.run([exe, "-i", paths["soap"], "-d", paths["ref"], "-o", os.path.join(out_dir, "cns")] + flags,
                       cwd=out_dir, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-800:]
    out = {}
    for f in sorted(os.listdir(out_dir)):
        if f.startswith("cns"):
            with open(os.path.join(out_dir, f), "rb") as fh:
                out[f] = fh.read()
    return out


@pytest.mark.parametrize("name,scale,compress", [
    ("c0", 0.05, False), ("c0", 0.05, True), ("c1", 0.002, False), ("c1", 0.002, True),
    ("c2", 0.004, False), ("c3", 0.002, False), ("c4", 0.0101, False), ("c5", 0.004, False)])
def test_restated_driver_matches_reference_host(name, scale, compress, tmp_path, ref_bin, oracle_bin):
    w = synth.make_workload(name, scale=scale)
    paths = synth.write_inputs(w, str(tmp_path))
    flags = [f for f in w.cli_flags(paths.get("dbsnp")) if f != "-C"] + (["-C"] if compress else [])
    a = run(ref_bin, paths, flags, str(tmp_path / "ref"))
    b = run(oracle_bin, paths, flags, str(tmp_path / "oracle"))
    assert sorted(a) == sorted(b)
    for f in a:
        assert a[f] == b[f], f


def test_irregular_reference_files_match_reference_host(tmp_path, ref_bin, oracle_bin):
    """Known-SNP rows that do not parse, blank rows, repeated positions and a
    repeated chromosome name with no sequence (malformed_inputs.py): the
    reference's loader keeps its name, position and SNP fields across rows
    (cpp/chromosome.cc:207-221)."""
    from malformed_inputs import corrupt_workload_inputs
    w = synth.make_workload("c1", scale=0.002)
    paths = synth.write_inputs(w, str(tmp_path))
    corrupt_workload_inputs(paths, w.chr_name, w.genome_len, seed=11)
    flags = [f for f in w.cli_flags(paths.get("dbsnp")) if f != "-C"]
    a = run(ref_bin, paths, flags, str(tmp_path / "ref"))
    b = run(oracle_bin, paths, flags, str(tmp_path / "oracle"))
    assert sorted(a) == sorted(b)
    for f in a:
        assert a[f] == b[f], f


def test_matrix_file_matches_reference_host(tmp_path, ref_bin, oracle_bin):
    w = synth.make_workload("c0", scale=0.03)
    paths = synth.write_inputs(w, str(tmp_path))
    flags = [f for f in w.cli_flags(paths.get("dbsnp")) if f != "-C"]
    outs = []
    for tag, exe in (("ref", ref_bin), ("oracle", oracle_bin)):
        d = tmp_path / tag
        run(exe, paths, flags + ["-M", str(tmp_path / (tag + ".mat"))], str(d))
        outs.append((tmp_path / (tag + ".mat")).read_bytes())
    assert outs[0] == outs[1] and len(outs[0]) > 0
