"""The `gsnp` command's reference-sequence and known-SNP loaders
(load_fasta, load_dbsnp in gsnp_gb300/csrc/cli.cpp) against the oracle's
restatement of the reference's (load_genome in oracle/driver.cpp,
cpp/chromosome.cc:172-221) on files of irregular rows (malformed_inputs.py):
the same site codes, SNP marks and SNP rows, printed by
tests/native/genome_check.cpp built once over each."""
import os
import subprocess

import pytest

from malformed_inputs import write_loader_inputs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_check(out, oracle, native_lib):
    from gsnp_gb300 import build
    src = os.path.join(ROOT, "tests", "native", "genome_check.cpp")
    if oracle:
        objs = [os.path.join(ROOT, "oracle", "_build", o) for o in ("backend.o", "calling.o")]
        cmd = ["g++", "-O2", "-std=c++17", "-fno-fast-math", "-ffp-contract=off", "-DGENOME_ORACLE",
               "-I" + os.path.join(ROOT, "oracle"), "-I" + os.path.join(ROOT, "include"), src] + objs + \
              ["-o", out, "-lm"]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-pthread",
               "-I" + os.path.join(ROOT, "gsnp_gb300", "csrc"), "-I" + os.path.join(ROOT, "include"),
               "-I" + build._cuda_include(), src, "-o", out, "-L" + build.LIBDIR, "-lgsnp_gb300",
               "-Wl,-rpath," + build.LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


@pytest.fixture(scope="module")
def checkers(tmp_path_factory, oracle_bin, native_lib):
    d = tmp_path_factory.mktemp("genome")
    return (build_check(str(d / "genome_oracle"), True, native_lib),
            build_check(str(d / "genome_cli"), False, native_lib))


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_loaders_match_oracle(seed, tmp_path, checkers):
    fasta, dbsnp = write_loader_inputs(str(tmp_path), seed)
    outs = []
    for exe in checkers:
        r = subprocess.run([exe, fasta, dbsnp], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stderr
        outs.append(r.stdout.split("\n"))
    want, got = outs
    # chr1: its second copy; chr2: its first copy (the repeat at the end has
    # no sequence), a CR kept as a base on each of three lines
    assert [x for x in want if x.startswith("chr ")] == ["chr chr1 4000", "chr chr2 3003", "chr chr3 1000"]
    assert sum(x.startswith("snp ") for x in want) > 1000
    # the inputs lead to no position past its chromosome (the reference
    # would write its SNP mark out of bounds there)
    length = 0
    for x in want:
        if x.startswith("chr "):
            length = int(x.split()[2])
        elif x.startswith("snp "):
            assert int(x.split()[1]) < length, x
    assert len(got) == len(want)
    for i, (a, b) in enumerate(zip(got, want)):
        assert a == b, (i, a[:200], b[:200])
