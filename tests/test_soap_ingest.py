"""The `gsnp` command's SOAP loader (load_soap in gsnp_gb300/csrc/cli.cpp) on
files of edge cases, against a restatement of the reference's record parse
(Soap_format::operator>>, cpp/soap_snp.h:132-169): whitespace-separated
fields, 1-based positions made 0-based, an N insertion of mismatch - 200
bases (mismatch > 200) or a deletion of mismatch - 100 bases (mismatch > 100)
at the indel position; lines whose fields do not parse are skipped.  Files
with and without a final newline, with empty and blank lines, tabs or
spaces, and more than one chromosome name, with the lines shared among 1, 3
and 64 threads (GSNP_HOST_THREADS)."""
import os
import random
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_parse(lines, L):
    """rows of (pos, len, hit, strand, chr, seq, qual) and the first error"""
    rows, bad = [], ""
    for line in lines:
        f = line.replace("\r", " ").split()
        if len(f) < 10:
            continue
        try:
            hit, read_len, position, mismatch = int(f[3]), int(f[5]), int(f[8]), int(f[9])
        except ValueError:
            continue
        read, qual = f[1], f[2]
        if mismatch > 100:
            if len(f) < 11:
                continue
            p = int(f[10])
            if mismatch > 200:
                ns = "N" * (mismatch - 200)
                read = read[:p] + ns + read[p:read_len]
                qual = qual[:p] + ns + qual[p:read_len]
            else:
                n = mismatch - 100
                read = read[:p] + read[p + n:read_len]
                qual = qual[:p] + qual[p + n:read_len]
        if read_len < 0 or read_len > L or len(read) < read_len or len(qual) < read_len:
            bad = bad or "alignment longer than -L or than its sequence field"
            continue
        rows.append((position - 1, read_len, hit, f[6][0], f[7], read[:read_len],
                     ",".join(str(ord(c)) for c in qual[:read_len])))
    return rows, bad


def make_lines(rng, n, L, with_bad):
    lines = []
    for i in range(n):
        ln = rng.randint(max(1, L // 2), L)
        seq = "".join(rng.choice("ACGT") for _ in range(ln))
        qual = "".join(chr(rng.randint(33, 80)) for _ in range(ln))
        fields = [f"r{i}", seq, qual, str(rng.choice([1, 1, 1, 2, 3])), "a", str(ln), rng.choice("+-"),
                  rng.choice(["chr1"] * 9 + ["chrX"]), str(rng.randint(1, 10 ** 6)), str(rng.randint(0, 3))]
        k = rng.random()
        if k < 0.08:     # deletion of 1..3 bases
            d = rng.randint(1, 3)
            fields[9] = str(100 + d)
            fields.append(str(rng.randint(0, ln - d)))
        elif k < 0.16:   # N insertion of 1..3 bases
            fields[9] = str(200 + rng.randint(1, 3))
            fields.append(str(rng.randint(0, ln)))
        elif k < 0.19:
            lines.append("")
            continue
        elif k < 0.21:
            lines.append("   \t ")
            continue
        elif k < 0.23:   # too few fields
            lines.append("\t".join(fields[:7]))
            continue
        elif k < 0.25:   # a field that does not parse as a number
            fields[8] = "x" + fields[8]
        elif k < 0.26:   # mismatch above 100 without the indel position
            fields[9] = "150"
        elif k < 0.27 and with_bad:
            fields[5] = str(L + 1)
        sep = " " if rng.random() < 0.1 else "\t"
        lines.append(sep.join(fields))
    return lines


@pytest.fixture(scope="module")
def soap_check(tmp_path_factory, native_lib):
    from gsnp_gb300 import build
    exe = str(tmp_path_factory.mktemp("soap") / "soap_check")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-pthread",
                        "-I" + os.path.join(ROOT, "gsnp_gb300", "csrc"), "-I" + os.path.join(ROOT, "include"),
                        "-I" + build._cuda_include(), os.path.join(ROOT, "tests", "native", "soap_check.cpp"),
                        "-o", exe, "-L" + build.LIBDIR, "-lgsnp_gb300", "-Wl,-rpath," + build.LIBDIR],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run_loader(exe, path, L, threads=None):
    env = dict(os.environ)
    if threads:
        env["GSNP_HOST_THREADS"] = str(threads)
    r = subprocess.run([exe, path, str(L)], capture_output=True, text=True, timeout=120, env=env)
    assert r.returncode == 0, r.stderr
    out = r.stdout.split("\n")
    assert out[-1] == "" and out[-2].startswith("bad ") and out[-3].startswith("padding ")
    rows = []
    for line in out[:-3]:
        f = line.split(" ")
        rows.append((int(f[0]), int(f[1]), int(f[2]), f[3], f[4], f[5], f[6]))
    return rows, out[-3].split(" ", 1)[1], out[-2].split(" ", 1)[1]


@pytest.mark.parametrize("seed,n,L,ending,with_bad", [(1, 4000, 50, "\n", False), (2, 4000, 100, "", False),
                                                     (3, 3000, 100, "\n\n\n", True), (4, 1, 35, "", False),
                                                     (5, 7, 100, "\n", False)])
@pytest.mark.parametrize("threads", [1, 3, 64])
def test_soap_loader_matches_reference_parse(seed, n, L, ending, with_bad, threads, tmp_path, soap_check):
    rng = random.Random(seed)
    lines = make_lines(rng, n, L, with_bad)
    path = str(tmp_path / "in.soap")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + ending)
    rows, padding, bad = run_loader(soap_check, path, L, threads)
    want_rows, want_bad = reference_parse(lines, L)
    assert padding == "ok"
    assert bad == want_bad
    assert len(rows) == len(want_rows)
    for i, (a, b) in enumerate(zip(rows, want_rows)):
        assert a == b, (i, a, b)


def test_soap_loader_empty_file(tmp_path, soap_check):
    path = str(tmp_path / "empty.soap")
    open(path, "w").close()
    rows, padding, bad = run_loader(soap_check, path, 100)
    assert rows == [] and padding == "ok" and bad == ""


@pytest.mark.parametrize("threads", [1, 3, 64])
def test_soap_loader_many_chromosome_names(threads, tmp_path, soap_check):
    """Names are looked up through a table, not a scan: 2,000 names keep
    their alignments apart; more than 65,536 (the ids are 16-bit) are an
    input error."""
    rng = random.Random(7)
    for n_names, want_bad in ((2000, ""), (65537, "more than 65536 chromosome names")):
        lines = []
        for i in range(n_names):
            seq = "".join(rng.choice("ACGT") for _ in range(20))
            lines.append("\t".join([f"r{i}", seq, "I" * 20, "1", "a", "20", "+", f"contig{i}", str(1 + i), "0"]))
        path = str(tmp_path / f"names{n_names}.soap")
        with open(path, "w") as fh:
            fh.write("\n".join(lines) + "\n")
        rows, padding, bad = run_loader(soap_check, path, 20, threads)
        assert bad == want_bad
        if not want_bad:
            assert [(r[0], r[4]) for r in rows] == [(i, f"contig{i}") for i in range(n_names)]
