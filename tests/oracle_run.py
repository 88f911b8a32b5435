"""Run the CPU oracle binary on a synthetic workload (test helper)."""
import os
import subprocess

from gsnp_gb300 import synth


def oracle_outputs(oracle_bin, w, flags, directory):
    """Write the workload's input files, run the oracle and return {suffix: bytes}."""
    paths = synth.write_inputs(w, directory)
    out_dir = os.path.join(directory, "oracle_out")
    os.makedirs(out_dir, exist_ok=True)
    cns = os.path.join(out_dir, "cns")
    cmd = [oracle_bin, "-i", paths["soap"], "-d", paths["ref"], "-o", cns] + list(flags)
    r = subprocess.run(cmd, cwd=out_dir, capture_output=True, text=True)
    res = {"rc": r.returncode, "stderr": r.stderr, "paths": paths}
    for f in os.listdir(out_dir):
        if f.startswith("cns"):
            with open(os.path.join(out_dir, f), "rb") as fh:
                res[f[3:] or "cns"] = fh.read()
    return res


def flags_for(w, paths, compress=False):
    flags = w.cli_flags(paths.get("dbsnp"))
    flags = [f for f in flags if f != "-C"]
    if compress:
        flags.append("-C")
    return flags


def first_diff(a: bytes, b: bytes):
    la, lb = a.split(b"\n"), b.split(b"\n")
    for i, (x, y) in enumerate(zip(la, lb)):
        if x != y:
            return i, x, y
    return min(len(la), len(lb)), None, None
