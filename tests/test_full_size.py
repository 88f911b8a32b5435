"""Parity at the headline size: the full 50 Mbp, 30x workloads (15 M
alignments) against the reference's own host code.

tests/golden/golden_full.json holds, for c1 (with its -C files) and c3 (Phred
qualities to 60), the digest of the generator's arrays and the digests of
every file that oracle/_ref/gsnp_ref - the reference's host sources compiled
in place, over the restated backend - wrote for them (made by
`tests/golden/make_golden.py --full`).  Here the same workload is generated on
the GPU, its arrays must have the recorded digest, and it is called through
the C ABI in both numeric forms: the cns text, and for c1 the six -C files,
must have the reference's digests.  Zero differing rows is then a
measurement at the size the throughput is quoted on.
"""
import hashlib
import json
import os

import pytest

from gsnp_gb300 import api, synth

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN_PATH = os.path.join(HERE, "golden", "golden_full.json")
GOLDEN = json.load(open(GOLDEN_PATH)) if os.path.exists(GOLDEN_PATH) else {}
FORMS = {"fp32_fixup": api.PRECISION_FP32_FIXUP, "fp64": api.PRECISION_FP64}


def sha(data: bytes) -> str:
    return hashlib.sha256(data).hexdigest()


def sha_file(path: str) -> str:
    h = hashlib.sha256()
    with open(path, "rb") as f:
        for block in iter(lambda: f.read(1 << 24), b""):
            h.update(block)
    return h.hexdigest()


_workloads = {}


def workload(name):
    """One GPU-generated full-size workload per config, checked against the
    recorded digest of the arrays the reference's inputs were written from."""
    if name not in _workloads:
        _workloads.clear()
        w = synth.make_workload(name, scale=1.0, backend="torch")
        want = next(g["workload_sha256"] for g in GOLDEN.values() if g["config"] == name)
        assert synth.workload_digest(w) == want, f"{name}: generated workload differs from the golden one"
        _workloads[name] = w
    return _workloads[name]


@pytest.mark.gpu
@pytest.mark.parametrize("form", sorted(FORMS))
@pytest.mark.parametrize("cid", sorted(GOLDEN))
def test_full_size_matches_reference(cid, form, tmp_path, native_lib):
    g = GOLDEN[cid]
    w = workload(g["config"])
    flags = list(g["flags"])
    c, _, _ = api.run_workload(w, flags, precision=FORMS[form])
    try:
        if g["compress"]:
            base = str(tmp_path / "cns")
            rc = c.lib.gsnp_write_columns(c.ctx, w.chr_name.encode(), base.encode())
            assert rc == 0, c.lib.gsnp_context_error(c.ctx)
            want = {k: v for k, v in g["outputs"].items() if k.startswith("cns.")}
            got = {k: sha_file(str(tmp_path / k)) for k in want}
            bad = sorted(k for k in want if got[k] != want[k])
            assert not bad, f"{cid} ({form}): {bad} differ from the reference's files"
        else:
            text = c.format_cns(w.chr_name)
            assert text.count(b"\n") == w.genome_len
            assert sha(text) == g["outputs"]["cns"], f"{cid} ({form}): cns text differs from the reference's"
        if form == "fp32_fixup":
            st = c.stats()
            assert st["sample_mismatches"] == 0
    finally:
        c.close()
