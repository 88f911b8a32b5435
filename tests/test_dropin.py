"""Drop-in parity of the GPU backend (libgsnp_backend.so, the reference's C++
backend functions on sm_103a).

The oracle's restatement of the reference's host driver (window loop, cns
text, -C files) is linked once against its CPU backend (gsnp_oracle) and once
against the GPU backend (gsnp_dropin).  Every output file must be identical
byte for byte: the window state, the stale-host-array quirks and the codecs
of the GPU backend then behave exactly as the reference's do, call for call.
"""
import os
import subprocess

import pytest

from gsnp_gb300 import synth

from oracle_run import first_diff, flags_for

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = [("c0", 0.1, False), ("c0", 0.1, True), ("c1", 0.004, True), ("c2", 0.01, False), ("c3", 0.004, False),
         ("c4", 0.0101, True)]


@pytest.fixture(scope="module")
def dropin_bin(oracle_bin, native_lib):
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return os.path.join(ROOT, "oracle", "_build", "gsnp_dropin")


def run_driver(binary, paths, flags, out_dir):
    os.makedirs(out_dir, exist_ok=True)
    r = subprocess.run([binary, "-i", paths["soap"], "-d", paths["ref"], "-o", os.path.join(out_dir, "cns")]
                       + flags, cwd=out_dir, capture_output=True, text=True)
    files = {}
    for f in sorted(os.listdir(out_dir)):
        if f.startswith("cns"):
            with open(os.path.join(out_dir, f), "rb") as fh:
                files[f] = fh.read()
    return r, files


@pytest.mark.gpu
@pytest.mark.parametrize("name,scale,compress", CASES)
def test_gpu_backend_is_a_drop_in(name, scale, compress, tmp_path, oracle_bin, dropin_bin):
    w = synth.make_workload(name, scale=scale)
    paths = synth.write_inputs(w, str(tmp_path))
    flags = flags_for(w, paths, compress=compress)
    r0, ref = run_driver(oracle_bin, paths, flags, str(tmp_path / "cpu"))
    assert r0.returncode == 0, r0.stderr
    r1, got = run_driver(dropin_bin, paths, flags, str(tmp_path / "gpu"))
    assert r1.returncode == 0, r1.stderr
    assert sorted(got) == sorted(ref)
    for f in ref:
        if got[f] != ref[f]:
            if f == "cns":
                i, x, y = first_diff(got[f], ref[f])
                pytest.fail(f"{name}: {f} row {i}:\n gpu   : {x!r}\n oracle: {y!r}")
            pytest.fail(f"{name}: {f} differs ({len(got[f])} vs {len(ref[f])} bytes)")
