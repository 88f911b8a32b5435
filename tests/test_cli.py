"""The `gsnp` command against the oracle: same command line, same files.

The oracle binary restates the reference's command-line program; `gsnp` is
the GB300 program.  Both run on the same seeded input files with the same
flags, and every output file (cns text, the six -C files, the -M matrix) must
be identical byte for byte.
"""
import os
import subprocess

import pytest

from gsnp_gb300 import build, synth

from oracle_run import first_diff, flags_for

CASES = [("c0", 0.1, False), ("c0", 0.1, True), ("c1", 0.004, False), ("c1", 0.004, True), ("c2", 0.01, True),
         ("c3", 0.004, False), ("c4", 0.0101, True)]


def run(binary, paths, flags, out_dir, extra=()):
    os.makedirs(out_dir, exist_ok=True)
    r = subprocess.run([binary, "-i", paths["soap"], "-d", paths["ref"], "-o", os.path.join(out_dir, "cns")]
                       + list(flags) + list(extra), cwd=out_dir, capture_output=True, text=True)
    files = {}
    for f in sorted(os.listdir(out_dir)):
        with open(os.path.join(out_dir, f), "rb") as fh:
            files[f] = fh.read()
    return r, files


def compare(name, got, ref):
    assert sorted(got) == sorted(ref), (sorted(got), sorted(ref))
    for f in ref:
        if got[f] != ref[f]:
            if f == "cns":
                i, x, y = first_diff(got[f], ref[f])
                pytest.fail(f"{name}: {f} row {i}:\n gsnp  : {x!r}\n oracle: {y!r}")
            pytest.fail(f"{name}: {f} differs ({len(got[f])} vs {len(ref[f])} bytes)")


def test_cli_usage_and_no_device(native_lib, tmp_path):
    """Without -i/-d/-o the program prints its usage and exits 1; on a machine
    without a GPU it stops with an error instead of computing on the CPU."""
    r = subprocess.run([build.CLI], capture_output=True, text=True)
    assert r.returncode == 1 and "Compulsory" in r.stderr
    import torch
    if torch.cuda.is_available():
        return
    w = synth.make_workload("c0", scale=0.01)
    paths = synth.write_inputs(w, str(tmp_path))
    r, _ = run(build.CLI, paths, flags_for(w, paths), str(tmp_path / "out"))
    assert r.returncode != 0 and "CUDA" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name,scale,compress", CASES)
def test_cli_matches_oracle(name, scale, compress, tmp_path, oracle_bin, native_lib):
    w = synth.make_workload(name, scale=scale)
    paths = synth.write_inputs(w, str(tmp_path))
    flags = flags_for(w, paths, compress=compress)
    r0, ref = run(oracle_bin, paths, flags + ["-M", "mat"], str(tmp_path / "oracle"))
    assert r0.returncode == 0, r0.stderr
    r1, got = run(build.CLI, paths, flags + ["-M", "mat"], str(tmp_path / "gsnp"))
    assert r1.returncode == 0, r1.stderr
    compare(name, got, ref)


@pytest.mark.gpu
def test_cli_matrix_input_and_fp64_form(tmp_path, oracle_bin, native_lib):
    """-I reads a matrix written by -M; -P fp64 gives the same bytes."""
    w = synth.make_workload("c1", scale=0.004)
    paths = synth.write_inputs(w, str(tmp_path))
    flags = flags_for(w, paths)
    r0, ref = run(oracle_bin, paths, flags + ["-M", "mat"], str(tmp_path / "a"))
    assert r0.returncode == 0, r0.stderr
    mat = str(tmp_path / "a" / "mat")
    r1, got = run(build.CLI, paths, flags + ["-I", mat, "-P", "fp64"], str(tmp_path / "b"))
    assert r1.returncode == 0, r1.stderr
    del ref["mat"]
    compare("c1 -I", got, ref)


@pytest.mark.gpu
def test_cli_irregular_reference_files(tmp_path, oracle_bin, native_lib):
    """Known-SNP rows that do not parse, blank rows, repeated positions and a
    repeated chromosome name with no sequence (malformed_inputs.py), read as
    the reference reads them (cpp/chromosome.cc:172-221)."""
    from malformed_inputs import corrupt_workload_inputs
    w = synth.make_workload("c1", scale=0.004)
    paths = synth.write_inputs(w, str(tmp_path))
    corrupt_workload_inputs(paths, w.chr_name, w.genome_len, seed=11)
    flags = flags_for(w, paths)
    r0, ref = run(oracle_bin, paths, flags, str(tmp_path / "oracle"))
    assert r0.returncode == 0, r0.stderr
    r1, got = run(build.CLI, paths, flags, str(tmp_path / "gsnp"))
    assert r1.returncode == 0, r1.stderr
    compare("c1 irregular reference files", got, ref)
