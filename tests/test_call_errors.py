"""Input errors of a whole-chromosome call, through gsnp_call_chromosome and
the segmented gsnp_call_chromosome_into: the status code and message, and a
context that stays usable (a valid call afterwards gives the same calls as
before the failed one).

The reference exits on these inputs: unsorted alignments with "Errors in
sorting:<pos><<previous pos>" (cpp/call_genotype.cc:516-523), a read longer
than -L and a base other than ACGT/acgt through its asserts
(kernel/compress_kernel.cu:121-123).  A site covered by more than 65535
alignments is this build's capacity limit (its per-site counts are 16-bit):
the kernels raise the device error word and the call returns
GSNP_ERR_CAPACITY.
"""
import numpy as np
import pytest

from gsnp_gb300 import api, synth

from oracle_run import flags_for

GSNP_ERR_CAPACITY, GSNP_ERR_UNSORTED, GSNP_ERR_INPUT = 4, 5, 6


def bad_reads(w, kind):
    """copies of the workload's alignment arrays with one defect"""
    pos, length, hit, strand = w.pos.copy(), w.length.copy(), w.hit.copy(), w.strand.copy()
    seq, qual = w.seq.copy(), w.qual.copy()
    i = len(pos) // 2
    if kind == "unsorted":
        pos[i] = pos[i - 1] - 7
    elif kind == "too_long":
        length[i] = seq.shape[1] + 1
    elif kind == "bad_base":
        seq[i, 3] = ord("X")
    elif kind == "no_position":
        pos[:] = -1
    elif kind == "too_deep":
        # 70,000 copies of one alignment, next to it in file order
        rep = np.ones(len(pos), dtype=np.int64)
        rep[i] = 70_000
        pos, length, hit, strand = (np.repeat(x, rep) for x in (pos, length, hit, strand))
        seq, qual = np.repeat(seq, rep, axis=0), np.repeat(qual, rep, axis=0)
    return pos, length, hit, strand, seq, qual


@pytest.mark.gpu
@pytest.mark.parametrize("kind,code,text", [("unsorted", GSNP_ERR_UNSORTED, "Errors in sorting:"),
                                            ("too_long", GSNP_ERR_INPUT, "longer than -L"),
                                            ("bad_base", GSNP_ERR_INPUT, "unknown base"),
                                            ("no_position", GSNP_ERR_INPUT, "non-negative position"),
                                            ("too_deep", GSNP_ERR_CAPACITY, "more than 65535 alignments")])
@pytest.mark.parametrize("into", [False, True])
def test_input_error_then_valid_call(kind, code, text, into, native_lib, monkeypatch):
    monkeypatch.setenv("GSNP_SEGMENTS", "4")
    w = synth.make_workload("c1", scale=0.02)
    flags = flags_for(w, {"ref": "ref.fa", "soap": "in.soap", "dbsnp": "db.txt"})
    c, reads, pm = api.run_workload(w, flags, precision=api.PRECISION_FP32_FIXUP)
    try:
        want = c.fetch(0, w.genome_len).copy()
        arrs = [np.ascontiguousarray(x) for x in bad_reads(w, kind)]
        c._keep += arrs
        bad = api.Caller.reads_struct(*arrs)
        out = np.zeros(w.genome_len, dtype=api.SITE_DTYPE)
        with pytest.raises(RuntimeError) as e:
            if into:
                c.call_into(bad, out.ctypes.data)
            else:
                c.call(bad)
        assert f"({code})" in str(e.value) and text in str(e.value), str(e.value)
        # the context is still usable and gives the same calls
        c.call_into(reads, out.ctypes.data)
        assert out.tobytes() == want.tobytes()
    finally:
        c.close()
