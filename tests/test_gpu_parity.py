"""GPU parity: the sm_103a caller against the CPU oracle, byte for byte.

Each case generates a seeded workload, runs the oracle binary on its text
files, runs the same alignments through the C ABI (calibration, tables, whole
chromosome call) and compares the cns text.  The shapes cover the window
quirks: c4 has an N block longer than a window (gap windows, stale host
counts), c2 has deep hotspots (record cap, deep tile bins) and mixed read
lengths, c1/c3 carry dbSNP priors and c3 qualities up to 60, c5 has reads of
150-250 bp under -L 250 (the widest read rows and dependency state).
"""
import os

import numpy as np
import pytest

from gsnp_gb300 import api, synth

from oracle_run import first_diff, flags_for, oracle_outputs

CASES = [("c0", 0.1), ("c1", 0.004), ("c2", 0.01), ("c3", 0.004), ("c4", 0.0101), ("c5", 0.004)]


@pytest.mark.gpu
@pytest.mark.parametrize("name,scale", CASES)
def test_cns_text_matches_oracle(name, scale, tmp_path, oracle_bin, native_lib):
    w = synth.make_workload(name, scale=scale)
    paths = synth.write_inputs(w, str(tmp_path))
    flags = flags_for(w, paths)
    ref = oracle_outputs(oracle_bin, w, flags, str(tmp_path))
    assert ref["rc"] == 0, ref["stderr"]
    c, reads, pm = api.run_workload(w, flags)
    try:
        got = c.format_cns(w.chr_name)
    finally:
        c.close()
    if got != ref["cns"]:
        i, x, y = first_diff(got, ref["cns"])
        pytest.fail(f"{name}: first differing row {i}:\n gpu   : {x!r}\n oracle: {y!r}")


@pytest.mark.gpu
@pytest.mark.parametrize("name,scale", [("c0", 0.1), ("c1", 0.004), ("c2", 0.01), ("c3", 0.004), ("c4", 0.0101),
                                        ("c5", 0.004)])
def test_fp32_fixup_form_matches_oracle(name, scale, tmp_path, oracle_bin, native_lib):
    """FP32 compensated sums with FP64 recomputation near decision boundaries
    must give the same cns bytes as the FP64 form and the oracle."""
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
        pytest.fail(f"{name}: first differing row {i}:\n gpu   : {x!r}\n oracle: {y!r}")
    assert stats["sample_mismatches"] == 0, stats
    assert stats["sampled_sites"] > 0, stats
    assert stats["max_abs_err"] < 1e-2, stats
    assert stats["fixup_sites"] < w.genome_len // 100, stats


@pytest.mark.gpu
@pytest.mark.parametrize("name,scale", [("c1", 0.05), ("c2", 0.05), ("c3", 0.05)])
def test_fp32_form_equals_fp64_form(name, scale, native_lib):
    """At sizes beyond the oracle's: every site call of the FP32 form equals
    the FP64 form's, field for field."""
    w = synth.make_workload(name, scale=scale)
    flags = flags_for(w, {"ref": "ref.fa", "soap": "in.soap", "dbsnp": "db.txt"})
    out = {}
    for prec in (api.PRECISION_FP64, api.PRECISION_FP32_FIXUP):
        c, reads, pm = api.run_workload(w, flags, precision=prec)
        try:
            calls = c.fetch(0, w.genome_len)
            out[prec] = (calls, c.stats())
        finally:
            c.close()
    a, b = out[api.PRECISION_FP64][0].copy(), out[api.PRECISION_FP32_FIXUP][0].copy()
    a["flags"] = 0
    b["flags"] = 0
    bad = np.nonzero(a != b)[0]
    assert bad.size == 0, f"{bad.size} sites differ, first {bad[:5]}"
    st = out[api.PRECISION_FP32_FIXUP][1]
    assert st["sample_mismatches"] == 0, st
    assert st["deferred_sites"] < w.genome_len // 10, st


@pytest.mark.gpu
def test_calibration_matrix_matches_oracle(tmp_path, oracle_bin, native_lib):
    w = synth.make_workload("c0", scale=0.05)
    paths = synth.write_inputs(w, str(tmp_path))
    flags = flags_for(w, paths)
    mat = os.path.join(str(tmp_path), "mat.txt")
    ref = oracle_outputs(oracle_bin, w, flags + ["-M", mat], str(tmp_path))
    assert ref["rc"] == 0, ref["stderr"]
    c, reads, pm = api.run_workload(w, flags)
    c.close()
    L = int(flags[flags.index("-L") + 1])
    rows = 0
    with open(mat) as f:
        for line in f:
            parts = line.split()
            q, coord = int(parts[0]), int(parts[1])
            vals = np.array([float(x) for x in parts[2:]])
            base = (q << 12) | (coord << 4)
            np.testing.assert_array_equal(pm[base:base + 16], vals)
            rows += 1
    assert rows == 41 * L


@pytest.mark.gpu
@pytest.mark.parametrize("pcr", ["0.9", "0.25"])
def test_deep_sites_pcr_dependency(pcr, tmp_path, oracle_bin, native_lib):
    """Deep hotspots (c2) under a pcr dependency whose adjusted-quality table
    is longer than the deep bins' 4-bit occurrence counts reach (-p 0.9: tmax
    47, the walk falls back to the bit set and the scan) or shorter (-p 0.25:
    tmax 5, the counts), both forms against the oracle."""
    w = synth.make_workload("c2", scale=0.01)
    paths = synth.write_inputs(w, str(tmp_path))
    flags = flags_for(w, paths) + ["-p", pcr]
    ref = oracle_outputs(oracle_bin, w, flags, str(tmp_path))
    assert ref["rc"] == 0, ref["stderr"]
    for prec in (api.PRECISION_FP64, api.PRECISION_FP32_FIXUP):
        c, reads, pm = api.run_workload(w, flags, precision=prec)
        try:
            got = c.format_cns(w.chr_name)
        finally:
            c.close()
        if got != ref["cns"]:
            i, x, y = first_diff(got, ref["cns"])
            pytest.fail(f"-p {pcr}, precision {prec}: first differing row {i}:\n gpu   : {x!r}\n oracle: {y!r}")


@pytest.mark.gpu
@pytest.mark.parametrize("name,scale", [("c1", 0.02), ("c2", 0.02), ("c4", 0.0101)])
def test_persistent_and_binned_paths_agree(name, scale, native_lib, monkeypatch):
    """The FP32 form's persistent kernel (tiles in genome order, leftover
    tiles to the binned kernels) gives the same site calls, byte for byte, as
    the depth-binned kernels alone: with 48 and 64 record slots, and with its
    reads loaded from global memory, prefetched into L2 by the bulk-copy unit,
    or staged in shared memory by bulk copies."""
    w = synth.make_workload(name, scale=scale)
    flags = [f for f in w.cli_flags("dbsnp") if f != "-C"]
    calls = {}
    for path, slots, mode in (("binned", "48", "0"), ("persistent", "48", "0"), ("persistent", "64", "0"),
                              ("persistent", "48", "1"), ("persistent", "48", "2"), ("persistent", "64", "2"),
                              ("binned-host", "48", "0"), ("persistent-host", "64", "1")):
        monkeypatch.setenv("GSNP_OPTIONS", "persistent=%d,persistent_slots=%s,persistent_mode=%s,device_driven=%d" % (
            path.startswith("persistent"), slots, mode, not path.endswith("-host")))
        c, _, _ = api.run_workload(w, flags, precision=api.PRECISION_FP32_FIXUP)
        try:
            calls[(path, slots, mode)] = c.fetch()
            kinds = {li["kind"] for li in c.last_launches()}
        finally:
            c.close()
        assert (4 in kinds) == path.startswith("persistent")
    base = calls[("binned", "48", "0")].tobytes()
    for key, v in calls.items():
        assert v.tobytes() == base, f"{name}: {key} differs from the binned path"



@pytest.mark.gpu
def test_graph_replay_and_tuning_keep_the_calls(tmp_path, native_lib, monkeypatch):
    """The resident recall replayed as a CUDA graph, the autotuner's sample
    passes and its chosen settings, and a new context loading them from the
    tuning file, all give the calls of the first pass."""
    tune_file = str(tmp_path / "tune.txt")
    monkeypatch.setenv("GSNP_TUNE_FILE", tune_file)
    w = synth.make_workload("c1", scale=0.05)
    flags = [f for f in w.cli_flags("dbsnp") if f != "-C"]
    c, reads, pm = api.run_workload(w, flags, precision=api.PRECISION_FP32_FIXUP)
    try:
        want = c.fetch().tobytes()
        for _ in range(3):
            c.recall_resident()
            assert [li["kind"] for li in c.last_launches()] == [5]
        assert c.fetch().tobytes() == want
        c.set_stream(0)   # the legacy default stream: captured on the library's own stream, replayed here
        for _ in range(2):
            c.recall_resident()
        assert c.fetch().tobytes() == want
        report = c.tune(sample_windows=4)
        assert "persistent " in report and "fast_carveout_40 " in report
        c.recall_resident()
        assert c.fetch().tobytes() == want
    finally:
        c.close()
    lines = open(tune_file).read().split("\n")
    assert any(x.startswith("persistent ") for x in lines)
    c, reads, pm = api.run_workload(w, flags, precision=api.PRECISION_FP32_FIXUP)
    try:
        assert c.fetch().tobytes() == want
    finally:
        c.close()
