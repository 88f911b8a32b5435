#!/usr/bin/env python
"""Generate tests/golden/golden.json: SHA-256 digests of the reference's own
outputs on seeded inputs.

Each case writes a seeded synthetic workload (gsnp_gb300.synth) as the
reference's input files and runs oracle/_ref/gsnp_ref on them.  That binary is
the reference's own host code (cpp/main.cc, call_genotype.cc, matrix.cc,
prior.cc, rank_sum.cc, chromosome.cc, normal_dis.cc, compiled in place from
the reference tree by `make -C oracle ref`) over the restated backend. The
digests of the inputs and of every output file (cns text, the -C files, the
-M matrix) are recorded.  For the -C cases the reference's own decompressor
(cpp/decompression.cpp, built in place by `make -C oracle ref-decompress`)
turns the files back into text, and that text's digest is recorded too.  The reference tree is needed to run this script;
the tests that read golden.json are not.

With --full it makes tests/golden/golden_full.json instead: the full-size
30x workloads (c1 with its -C files, and c3), each recorded by the digest of
the generator's arrays (synth.workload_digest) rather than of the
multi-gigabyte text files, so that a GPU test can check its own regenerated
input without writing them.

    python tests/golden/make_golden.py [--ref /path/to/reference] [--full]

The reference tree is taken from --ref, else from $GSNP_REFERENCE.
"""
import argparse
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

# (case id, config, scale, -C)
CASES = [
    ("c0_text", "c0", 0.1, False),
    ("c0_C", "c0", 0.1, True),
    ("c1_text", "c1", 0.004, False),
    ("c1_C", "c1", 0.004, True),
    ("c2_text", "c2", 0.01, False),
    ("c3_text", "c3", 0.004, False),
    ("c4_text", "c4", 0.0101, False),   # -C aborts in the reference here (empty dictionary assert)
]


def sha(data: bytes) -> str:
    return hashlib.sha256(data).hexdigest()


def sha_path(path: str) -> str:
    h = hashlib.sha256()
    with open(path, "rb") as fh:
        for block in iter(lambda: fh.read(1 << 24), b""):
            h.update(block)
    return h.hexdigest()


def case_flags(w, paths, compress):
    flags = [f for f in w.cli_flags(paths.get("dbsnp")) if f != "-C"]
    if compress:
        flags.append("-C")
    return flags


def inputs(name, scale, directory):
    from gsnp_gb300 import synth
    w = synth.make_workload(name, scale=scale)
    paths = synth.write_inputs(w, directory)
    digests = {}
    for k, p in sorted(paths.items()):
        with open(p, "rb") as f:
            digests[k] = sha(f.read())
    return w, paths, digests


def run_and_digest(binary, paths, flags, out_dir):
    os.makedirs(out_dir, exist_ok=True)
    r = subprocess.run([binary, "-i", paths["soap"], "-d", paths["ref"], "-o", os.path.join(out_dir, "cns"),
                        "-M", os.path.join(out_dir, "mat")] + flags, cwd=out_dir, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    out = {}
    for f in sorted(os.listdir(out_dir)):
        if f.startswith("cns") or f == "mat":
            out[f] = sha_path(os.path.join(out_dir, f))
    return out


# full-size cases: (case id, config, -C)
FULL_CASES = [
    ("c1_full_text", "c1", False),
    ("c1_full_C", "c1", True),
    ("c3_full_text", "c3", False),
]

# The full-size workloads hold 15,000,000 alignments.  The reference's pass-1
# spill (SoapData, cpp/soap_snp.h:325-416) writes an empty block when the
# number of parsed lines is a multiple of its 1,000,000-line buffer, and its
# pass 2 then fails.  Its input therefore gets one extra first line: an
# alignment at 1-based position 0, which the reference parses but skips in
# calibration (cpp/matrix.cc:62-64) and in calling (cpp/call_genotype.cc:495),
# before any other use.  The restated driver runs on the file without it, and
# the two must write identical files.
PAD_LINE = b"pad\t" + b"A" * 10 + b"\t" + b"h" * 10 + b"\t1\ta\t10\t+\tchr1\t0\t0\n"


def padded_copy(src, dst):
    with open(dst, "wb") as out, open(src, "rb") as f:
        out.write(PAD_LINE)
        shutil.copyfileobj(f, out, 1 << 24)


def run_full(ref_bin, ref_decompress, oracle_bin):
    """Full-size cases: the inputs are written once per config; each case
    runs the reference's host code (on the padded file) and the restated
    driver (on the file itself) in processes of their own, side by side."""
    import concurrent.futures as cf
    from gsnp_gb300 import synth
    golden = {}
    for name in sorted({c[1] for c in FULL_CASES}):
        cases = [c for c in FULL_CASES if c[1] == name]
        with tempfile.TemporaryDirectory() as d:
            w = synth.make_workload(name, scale=1.0)
            wd = synth.workload_digest(w)
            paths = synth.write_inputs(w, d)
            padded = dict(paths, soap=os.path.join(d, "reads_padded.soap"))
            padded_copy(paths["soap"], padded["soap"])
            runs = {}
            with cf.ThreadPoolExecutor(2 * len(cases)) as ex:
                for cid, _, compress in cases:
                    flags = case_flags(w, paths, compress)
                    runs[cid] = (flags,
                                 ex.submit(run_and_digest, ref_bin, padded, flags, os.path.join(d, cid + "_ref")),
                                 ex.submit(run_and_digest, oracle_bin, paths, flags, os.path.join(d, cid + "_oracle")))
                for cid, _, compress in cases:
                    flags, fut_ref, fut_oracle = runs[cid]
                    outs, outs_oracle = fut_ref.result(), fut_oracle.result()
                    if outs != outs_oracle:
                        sys.exit("%s: the restated driver's files differ from the reference host code's: %s" % (
                            cid, sorted(k for k in outs if outs[k] != outs_oracle.get(k))))
                    if compress:
                        text = os.path.join(d, cid + ".decompressed")
                        subprocess.run([ref_decompress, os.path.join(d, cid + "_ref", "cns"), text], check=True,
                                       capture_output=True)
                        outs["decompressed"] = sha_path(text)
                        os.unlink(text)
                    golden[cid] = {"config": name, "scale": 1.0, "compress": compress,
                                   "flags": [f if not os.path.isabs(f) else os.path.basename(f) for f in flags],
                                   "workload_sha256": wd, "sites": w.genome_len, "reads": w.num_reads,
                                   "reference_input": "the alignments with one extra first line at 1-based "
                                                      "position 0, which the reference skips (its pass-1 spill "
                                                      "fails on a multiple of 1,000,000 lines)",
                                   "restated_driver_identical": True,
                                   "outputs": outs}
                    print(cid, len(outs), "files", flush=True)
            del w
    with open(os.path.join(HERE, "golden_full.json"), "w") as f:
        json.dump(golden, f, indent=1, sort_keys=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("GSNP_REFERENCE"))
    ap.add_argument("--full", action="store_true")
    args = ap.parse_args()
    if not args.ref:
        sys.exit("give the reference tree with --ref or $GSNP_REFERENCE")
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "ref-decompress", "REF=" + args.ref])
    if r.returncode:
        sys.exit("cannot build the reference host code")
    ref_bin = os.path.join(ROOT, "oracle", "_ref", "gsnp_ref")
    ref_decompress = os.path.join(ROOT, "oracle", "_ref", "gsnp_ref_decompress")
    if args.full:
        r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"])
        if r.returncode:
            sys.exit("cannot build the oracle")
        run_full(ref_bin, ref_decompress, os.path.join(ROOT, "oracle", "_build", "gsnp_oracle"))
        return
    golden = {}
    for cid, name, scale, compress in CASES:
        with tempfile.TemporaryDirectory(dir=HERE) as d:
            w, paths, in_digests = inputs(name, scale, d)
            flags = case_flags(w, paths, compress)
            outs = run_and_digest(ref_bin, paths, flags, os.path.join(d, "out"))
            if compress:
                text = os.path.join(d, "decompressed")
                subprocess.run([ref_decompress, os.path.join(d, "out", "cns"), text], check=True,
                               capture_output=True)
                with open(text, "rb") as fh:
                    outs["decompressed"] = sha(fh.read())
        golden[cid] = {"config": name, "scale": scale, "compress": compress,
                       "flags": [f if not os.path.isabs(f) else os.path.basename(f) for f in flags],
                       "inputs": in_digests, "outputs": outs}
        print(cid, len(outs), "files")
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
