"""Packed reads (gsnp_pack_reads, gsnp_reads.packed): base and quality in one
byte per position, which halves what a call uploads.

CPU: the packer's bytes against the layout written out here (base A C T G as
0-3 in bits 7:6, quality - q_min in bits 5:0, 63 for a quality below q_min,
zeros past a read's end), and its refusals.
GPU: a call, a segmented call, a streamed call and the calibration from packed
reads equal those from the same reads as bases and qualities."""
import numpy as np
import pytest

from gsnp_gb300 import api, synth

CODE = {ord("A"): 0, ord("C"): 1, ord("T"): 2, ord("G"): 3, ord("a"): 0, ord("c"): 1, ord("t"): 2, ord("g"): 3}


def layout(seq, qual, length, q_min):
    out = np.zeros(seq.shape, dtype=np.uint8)
    for i in range(seq.shape[0]):
        for c in range(int(length[i])):
            q = int(np.int8(qual[i, c])) - q_min
            out[i, c] = (CODE[int(seq[i, c])] << 6) | (63 if q < 0 else q)
    return out


def test_pack_reads_layout(native_lib):
    rng = np.random.default_rng(7)
    n, pitch, q_min = 300, 40, 64
    seq = rng.choice(np.frombuffer(b"ACGTacgt", dtype=np.uint8), size=(n, pitch))
    qual = rng.integers(q_min - 5, q_min + 63, size=(n, pitch)).astype(np.uint8)
    length = rng.integers(0, pitch + 1, size=n).astype(np.int32)
    for threads in (1, 3, 0):
        got = api.pack_reads(seq, qual, length, q_min, threads=threads)
        assert np.array_equal(got, layout(seq, qual, length, q_min))


@pytest.mark.parametrize("q_min", [-127, -5, 0, 33, 64, 65, 100, 127])
def test_pack_reads_every_byte_pair(q_min, native_lib):
    """every (base byte, quality byte) pair: the valid ones packed as the
    layout says, a sample of the others refused one read at a time"""
    b = np.repeat(np.arange(256, dtype=np.uint8), 256).reshape(-1, 1)
    q = np.tile(np.arange(256, dtype=np.uint8), 256).reshape(-1, 1)
    ones = np.ones(len(b), dtype=np.int32)
    qq = q[:, 0].view(np.int8).astype(int) - q_min
    good = np.isin(b[:, 0], np.frombuffer(b"ACGTacgt", dtype=np.uint8)) & (qq <= 62)
    got = api.pack_reads(b[good], q[good], ones[good], q_min)
    want = [(CODE[int(x)] << 6) | (63 if y < 0 else y) for x, y in zip(b[good, 0], qq[good])]
    assert np.array_equal(got[:, 0], np.array(want, dtype=np.uint8))
    for i in np.flatnonzero(~good)[::97]:
        with pytest.raises(RuntimeError):
            api.pack_reads(b[i:i + 1], q[i:i + 1], ones[i:i + 1], q_min)


def test_pack_reads_refusals(native_lib):
    seq = np.frombuffer(b"ACGN", dtype=np.uint8).reshape(1, 4).copy()
    qual = np.full((1, 4), 70, dtype=np.uint8)
    length = np.array([4], dtype=np.int32)
    with pytest.raises(RuntimeError):            # N is refused, as the calls refuse it
        api.pack_reads(seq, qual, length, 64)
    assert api.pack_reads(seq, qual, np.array([3], dtype=np.int32), 64)[0, 3] == 0   # past the read's end
    seq[0, 3] = ord("T")
    qual[0, 2] = 64 + 63                         # no code for q_min + 63
    with pytest.raises(RuntimeError):
        api.pack_reads(seq, qual, length, 64)
    qual[0, 2] = 64 + 62
    assert api.pack_reads(seq, qual, length, 64)[0, 2] == (3 << 6) | 62


@pytest.mark.gpu
@pytest.mark.parametrize("name,scale", [("c1", 0.02), ("c4", 0.0101), ("c2", 0.02), ("c3", 0.02), ("c5", 0.01)])
def test_packed_calls_equal_unpacked(name, scale, native_lib, monkeypatch):
    w = synth.make_workload(name, scale=scale)
    flags = [f for f in w.cli_flags("dbsnp") if f != "-C"]
    c, reads, pm = api.run_workload(w, flags, precision=api.PRECISION_FP32_FIXUP)
    try:
        want = c.fetch(0, w.genome_len).copy()
        q_min = api.params_from_flags(flags).q_min
        packed = api.pack_reads(w.seq, w.qual, w.length, q_min)
        arrs = [np.ascontiguousarray(x) for x in (w.pos, w.length, w.hit, w.strand)]
        pr = api.Caller.reads_struct(*arrs, None, None, packed=packed, packed_qmin=q_min)
        c._keep += arrs + [packed]
        p = api.params_from_flags(flags, api.PRECISION_FP32_FIXUP)
        assert np.array_equal(c.calibrate(p, pr), pm)
        for segs in (1, 3):
            monkeypatch.setenv("GSNP_SEGMENTS", str(segs))
            got = np.zeros(w.genome_len, dtype=api.SITE_DTYPE)
            c.call_into(pr, got.ctypes.data)
            assert got.tobytes() == want.tobytes(), f"{name}: {segs} segments"
        c.set_option("stream_windows", 2)
        got = np.zeros(w.genome_len, dtype=api.SITE_DTYPE)
        c.call_streamed(pr, None, got.ctypes.data)
        assert got.tobytes() == want.tobytes(), f"{name}: streamed"
        bad = api.Caller.reads_struct(*arrs, None, None, packed=packed, packed_qmin=q_min + 1)
        assert c.lib.gsnp_call_chromosome(c.ctx, bad) != 0       # packed with another q_min
    finally:
        c.close()
