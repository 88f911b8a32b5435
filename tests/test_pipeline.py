"""The call in window-aligned segments (uploads, calling and downloads
overlapped): byte-identical to the oracle and to the one-segment call.

GSNP_SEGMENTS forces the number of segments, so that the small cases the
oracle can check are cut at several places: segment boundaries that fall in
gap windows (c4's N block), next to deep hotspots (c2), and inside dbSNP-
flagged stretches (c1).
"""
import numpy as np
import pytest

from gsnp_gb300 import api, synth

from oracle_run import first_diff, flags_for, oracle_outputs


@pytest.mark.gpu
@pytest.mark.parametrize("name,scale,segs", [("c4", 0.0101, 3), ("c4", 0.0101, 7), ("c2", 0.02, 2),
                                             ("c1", 0.02, 3), ("c0", 1.0, 4)])
def test_segmented_call_matches_oracle(name, scale, segs, tmp_path, oracle_bin, native_lib, monkeypatch):
    monkeypatch.setenv("GSNP_SEGMENTS", str(segs))
    w = synth.make_workload(name, scale=scale)
    paths = synth.write_inputs(w, str(tmp_path))
    flags = flags_for(w, paths)
    ref = oracle_outputs(oracle_bin, w, flags, str(tmp_path))
    assert ref["rc"] == 0, ref["stderr"]
    c, reads, pm = api.run_workload(w, flags, precision=api.PRECISION_FP32_FIXUP)
    try:
        got = c.format_cns(w.chr_name)
        stats = c.stats()
    finally:
        c.close()
    if got != ref["cns"]:
        i, x, y = first_diff(got, ref["cns"])
        pytest.fail(f"{name}, {segs} segments: first differing row {i}:\n gpu   : {x!r}\n oracle: {y!r}")
    assert stats["sample_mismatches"] == 0, stats


@pytest.mark.gpu
@pytest.mark.parametrize("segs", [1, 4, 9])
def test_call_into_equals_call_and_fetch(segs, native_lib, monkeypatch):
    """gsnp_call_chromosome_into downloads the same calls as
    gsnp_call_chromosome + gsnp_fetch_sites, at any segment count; the calls
    stay on the device for fetch and text output afterwards."""
    w = synth.make_workload("c1", scale=0.05)
    flags = flags_for(w, {"ref": "ref.fa", "soap": "in.soap", "dbsnp": "db.txt"})
    c, reads, pm = api.run_workload(w, flags, precision=api.PRECISION_FP32_FIXUP)
    try:
        want = c.fetch(0, w.genome_len).copy()
        monkeypatch.setenv("GSNP_SEGMENTS", str(segs))
        got = np.zeros(w.genome_len, dtype=api.SITE_DTYPE)
        c.call_into(reads, got.ctypes.data)
        again = c.fetch(0, w.genome_len)
    finally:
        c.close()
    assert got.tobytes() == want.tobytes()
    assert again.tobytes() == want.tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("up_streams,segs", [(2, 5), (4, 9)])
def test_upload_over_several_copy_streams(up_streams, segs, native_lib, monkeypatch):
    """The upload's pieces spread over several copy streams finish in any
    order; every segment's gather waits for all the pieces it reads, and the
    calls equal those of a one-stream, one-segment call."""
    w = synth.make_workload("c2", scale=0.02)
    flags = [f for f in w.cli_flags() if f != "-C"]
    c, reads, pm = api.run_workload(w, flags, precision=api.PRECISION_FP32_FIXUP)
    try:
        want = c.fetch(0, w.genome_len).copy()
    finally:
        c.close()
    monkeypatch.setenv("GSNP_OPTIONS", "upload_streams=%d" % up_streams)
    monkeypatch.setenv("GSNP_SEGMENTS", str(segs))
    c, reads, pm = api.run_workload(w, flags, precision=api.PRECISION_FP32_FIXUP)
    try:
        got = np.zeros(w.genome_len, dtype=api.SITE_DTYPE)
        c.call_into(reads, got.ctypes.data)
    finally:
        c.close()
    assert got.tobytes() == want.tobytes()
