"""The streamed call (gsnp_call_streamed): the chromosome in chunks of whole
windows, with two chunks' alignments and calls on the device at a time.  Its
calls, cns text and -C files must equal, byte for byte, those of the
resident call on the same inputs (which the parity tests pin to the oracle
and to the reference's own files).

Chunks of 1, 2 and 3 windows cut the small cases at many places: inside
c4's N block, whose gap windows show the counts of, and use the likelihood
of, a window before them that can lie one or more chunks back (the carried
window); next to c2's deep hotspots; inside c1's dbSNP-flagged stretches;
and at the shorter last window of every chromosome."""
import os

import numpy as np
import pytest

from gsnp_gb300 import api, synth

FILES = [".1_2", ".3_4_6", ".5_7_8_9_14_16", ".10", ".11_12_13", ".15_17"]


def resident_outputs(c, w, reads, out_dir):
    """calls, cns text and -C files of the resident call already made"""
    calls = c.fetch(0, w.genome_len).copy()
    text = c.format_cns(w.chr_name)
    base = os.path.join(out_dir, "resident", "cns")
    os.makedirs(os.path.dirname(base))
    rc = c.lib.gsnp_write_columns(c.ctx, w.chr_name.encode(), base.encode())
    assert rc == 0, c.lib.gsnp_context_error(c.ctx)
    return calls, text, {f: open(base + f, "rb").read() for f in FILES}


def streamed_outputs(c, w, reads, out_dir, windows):
    c.set_option("stream_windows", windows)
    d = os.path.join(out_dir, f"streamed{windows}")
    os.makedirs(d)
    calls = np.zeros(w.genome_len, dtype=api.SITE_DTYPE)
    c.call_streamed(reads, w.chr_name, calls.ctypes.data, os.path.join(d, "cns.txt"), os.path.join(d, "cns"))
    text = open(os.path.join(d, "cns.txt"), "rb").read()
    return calls, text, {f: open(os.path.join(d, "cns") + f, "rb").read() for f in FILES}


@pytest.mark.gpu
@pytest.mark.parametrize("name,scale", [("c4", 0.0101), ("c2", 0.02), ("c1", 0.02), ("c0", 1.0), ("c5", 0.01)])
def test_streamed_call_equals_resident(name, scale, tmp_path, native_lib):
    w = synth.make_workload(name, scale=scale)
    flags = [f for f in w.cli_flags("dbsnp") if f != "-C"]
    c, reads, _ = api.run_workload(w, flags, precision=api.PRECISION_FP32_FIXUP)
    try:
        want = resident_outputs(c, w, reads, str(tmp_path))
        stats_resident = c.stats()
        for windows in (1, 2, 3):
            got = streamed_outputs(c, w, reads, str(tmp_path), windows)
            assert got[0].tobytes() == want[0].tobytes(), f"{name}, {windows}-window chunks: calls differ"
            assert got[1] == want[1], f"{name}, {windows}-window chunks: cns text differs"
            for f in FILES:
                assert got[2][f] == want[2][f], f"{name}, {windows}-window chunks: {f} differs"
            st = c.stats()
            assert st["sites"] == stats_resident["sites"]
            assert st["sample_mismatches"] == 0
    finally:
        c.close()


@pytest.mark.gpu
def test_streamed_fp64_form_and_no_resident_calls(tmp_path, native_lib):
    """The plain FP64 form streams the same way; after a streamed call no
    call is resident, and a resident call afterwards works again."""
    w = synth.make_workload("c4", scale=0.0101)
    flags = [f for f in w.cli_flags("dbsnp") if f != "-C"]
    c, reads, _ = api.run_workload(w, flags, precision=api.PRECISION_FP64)
    try:
        want = resident_outputs(c, w, reads, str(tmp_path))
        got = streamed_outputs(c, w, reads, str(tmp_path), 2)
        assert got[0].tobytes() == want[0].tobytes()
        assert got[1] == want[1]
        assert c.lib.gsnp_write_cns(c.ctx, w.chr_name.encode(), str(tmp_path / "x").encode()) != 0
        # outputs may be left out: only the calls
        calls = np.zeros(w.genome_len, dtype=api.SITE_DTYPE)
        c.call_streamed(reads, None, calls.ctypes.data)
        assert calls.tobytes() == want[0].tobytes()
        c.call(reads)
        assert c.fetch(0, w.genome_len).tobytes() == want[0].tobytes()
    finally:
        c.close()
