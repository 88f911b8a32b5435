"""Golden digests of the reference's own host code (tests/golden/golden.json,
made by tests/golden/make_golden.py with oracle/_ref/gsnp_ref).

The inputs are regenerated from the seeded generator and checked against
their recorded digests; then every output file (cns text, -C files, -M
matrix) must have the recorded digest:
  - CPU: the restated oracle, so the oracle stays pinned to the reference on
    machines without the reference tree;
  - GPU: the `gsnp` command.
For the -C cases the files are also decompressed with `gsnp_decompress`,
whose text must have the digest of the reference decompressor's text
(cpp/decompression.cpp) on the reference's files.
"""
import hashlib
import json
import os
import subprocess

import pytest

from gsnp_gb300 import build, synth

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))
CPU_CASES = ["c0_text", "c0_C", "c1_C", "c3_text"]


def sha_file(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def run_case(binary, cid, tmp_path):
    g = GOLDEN[cid]
    w = synth.make_workload(g["config"], scale=g["scale"])
    paths = synth.write_inputs(w, str(tmp_path))
    for k, digest in g["inputs"].items():
        assert sha_file(paths[k]) == digest, f"{cid}: generated {k} differs from the golden input"
    flags = [f for f in w.cli_flags(paths.get("dbsnp")) if f != "-C"]
    if g["compress"]:
        flags.append("-C")
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([binary, "-i", paths["soap"], "-d", paths["ref"], "-o", str(out / "cns"), "-M",
                        str(out / "mat")] + flags, cwd=str(out), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = {f: sha_file(str(out / f)) for f in sorted(os.listdir(str(out))) if f.startswith("cns") or f == "mat"}
    files = {k: v for k, v in g["outputs"].items() if k != "decompressed"}
    assert sorted(got) == sorted(files)
    bad = [f for f in got if got[f] != files[f]]
    assert not bad, f"{cid}: {bad} differ from the reference's output"
    if "decompressed" in g["outputs"]:
        text = str(tmp_path / "decompressed")
        r = subprocess.run([build.DECOMPRESS, str(out / "cns"), text], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        assert sha_file(text) == g["outputs"]["decompressed"], f"{cid}: decompressed text differs from the reference's"


@pytest.mark.parametrize("cid", CPU_CASES)
def test_oracle_matches_golden(cid, tmp_path, oracle_bin, native_lib):
    run_case(oracle_bin, cid, tmp_path)


@pytest.mark.gpu
@pytest.mark.parametrize("cid", sorted(GOLDEN))
def test_gsnp_matches_golden(cid, tmp_path, native_lib):
    run_case(build.CLI, cid, tmp_path)
