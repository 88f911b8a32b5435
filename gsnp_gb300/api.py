"""ctypes declarations of include/gsnp_gb300.h and a small caller object.

`Caller` mirrors the reference's calling sequence (cpp/main.cc:363-403):
reference and dbSNP load, pass-1 calibration, prior and rank tables, then the
call of every site; each step is one C-ABI call into libgsnp_gb300.so.
"""
from __future__ import annotations

import ctypes
import math
from typing import List, Optional, Sequence

import numpy as np

GSNP_OK = 0
PRECISION_FP64 = 0
PRECISION_FP32_FIXUP = 1


class Params(ctypes.Structure):
    _fields_ = [
        ("read_length", ctypes.c_int),
        ("q_min", ctypes.c_int),
        ("q_max", ctypes.c_int),
        ("pcr_dependency", ctypes.c_double),
        ("global_dependency", ctypes.c_double),
        ("het_val", ctypes.c_double),
        ("het_unval", ctypes.c_double),
        ("althom_val", ctypes.c_double),
        ("althom_unval", ctypes.c_double),
        ("rank_sum", ctypes.c_int),
        ("monoploid", ctypes.c_int),
        ("refine", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("het_novel", ctypes.c_double),
        ("althom_novel", ctypes.c_double),
        ("transition_dominant", ctypes.c_int),
    ]


class Reads(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64),
        ("pos", ctypes.c_void_p),
        ("len", ctypes.c_void_p),
        ("hit", ctypes.c_void_p),
        ("strand", ctypes.c_void_p),
        ("seq", ctypes.c_void_p),
        ("qual", ctypes.c_void_p),
        ("pitch", ctypes.c_int32),
        ("packed", ctypes.c_void_p),
        ("packed_qmin", ctypes.c_int32),
    ]


class LaunchInfo(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("slots", ctypes.c_int), ("tiles", ctypes.c_int64),
                ("sites", ctypes.c_int64), ("ms", ctypes.c_float)]


SNP_DTYPE = np.dtype([("pos", "<u4"), ("validated", "u1"), ("hapmap", "u1"), ("indel", "u1"), ("pad", "u1"),
                      ("freq", "<f8", (4,))])
SITE_DTYPE = np.dtype([("type1", "u1"), ("base1", "u1"), ("base2", "u1"), ("q_cns", "u1"),
                       ("avg_q1", "u1"), ("avg_q2", "u1"), ("flags", "u1"), ("pad", "u1"),
                       ("cu1", "<u2"), ("ca1", "<u2"), ("cu2", "<u2"), ("ca2", "<u2"),
                       ("depth", "<u4"), ("repeat_time", "<u4"), ("rank_sum", "<f8")])
assert SNP_DTYPE.itemsize == 40 and SITE_DTYPE.itemsize == 32

_P = ctypes.c_void_p
_I64 = ctypes.c_int64


def declare(lib: ctypes.CDLL) -> None:
    sigs = {
        "gsnp_context_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_P)]),
        "gsnp_context_destroy": (None, [_P]),
        "gsnp_context_error": (ctypes.c_char_p, [_P]),
        "gsnp_set_stream": (ctypes.c_int, [_P, _P]),
        "gsnp_load_tables": (ctypes.c_int, [_P, ctypes.POINTER(Params), _P, _P, _P]),
        "gsnp_load_reference": (ctypes.c_int, [_P, _P, _I64, _P, _I64]),
        "gsnp_calibrate": (ctypes.c_int, [_P, ctypes.POINTER(Params), ctypes.POINTER(Reads), _P]),
        "gsnp_prior_table": (ctypes.c_int, [ctypes.POINTER(Params), _P]),
        "gsnp_rank_table": (ctypes.c_int, [_P]),
        "gsnp_call_chromosome": (ctypes.c_int, [_P, ctypes.POINTER(Reads)]),
        "gsnp_call_chromosome_into": (ctypes.c_int, [_P, ctypes.POINTER(Reads), _P]),
        "gsnp_call_streamed": (ctypes.c_int, [_P, ctypes.POINTER(Reads), ctypes.c_char_p, _P, ctypes.c_char_p,
                                              ctypes.c_char_p]),
        "gsnp_stream_footprint": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
        "gsnp_pack_reads": (ctypes.c_int, [_P, _P, _P, _I64, ctypes.c_int32, ctypes.c_int, _P, ctypes.c_int]),
        "gsnp_write_cns": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_char_p]),
        "gsnp_write_columns": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_char_p]),
        "gsnp_recall_resident": (ctypes.c_int, [_P]),
        "gsnp_fetch_sites": (ctypes.c_int, [_P, _I64, _I64, _P]),
        "gsnp_format_cns": (ctypes.c_int, [_P, ctypes.c_char_p, _P, ctypes.POINTER(_I64)]),
        "gsnp_get_stats": (ctypes.c_int, [_P, _P, ctypes.c_int]),
        "gsnp_last_launches": (ctypes.c_int, [_P, _P, ctypes.POINTER(ctypes.c_int)]),
        "gsnp_transfer_bytes": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
        "gsnp_set_option": (ctypes.c_int, [_P, ctypes.c_char_p, _I64]),
        "gsnp_tune": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t]),
    }
    for name, (res, args) in sigs.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args


def pack_reads(seq: np.ndarray, qual: np.ndarray, length: np.ndarray, q_min: int, out: Optional[np.ndarray] = None,
               threads: int = 0) -> np.ndarray:
    """gsnp_pack_reads: bases and qualities in one byte per position (out, or a
    new [n][pitch] uint8 array); raises on a base other than ACGT/acgt or a
    quality above q_min + 62."""
    from . import native
    seq = np.ascontiguousarray(seq, dtype=np.uint8)
    qual = np.ascontiguousarray(qual, dtype=np.uint8)
    length = np.ascontiguousarray(length, dtype=np.int32)
    if out is None:
        out = np.empty(seq.shape, dtype=np.uint8)
    rc = native().gsnp_pack_reads(seq.ctypes.data, qual.ctypes.data, length.ctypes.data, int(seq.shape[0]),
                                  int(seq.shape[1]), int(q_min), out.ctypes.data, int(threads))
    if rc != 0:
        raise RuntimeError("gsnp_pack_reads failed (%d)" % rc)
    return out


def params_from_flags(flags: Sequence[str], precision: int = PRECISION_FP64) -> Params:
    """SOAPsnp option semantics of cpp/main.cc:104-316 for the calling options.

    -a/-b and -j/-k are assigned crosswise to their usage text, as the
    reference does; -z resets q_max to q_min + 40, so option order matters.
    """
    p = Params()
    p.read_length = 45
    p.q_min = 64
    p.q_max = 64 + 40
    p.pcr_dependency = math.log10(0.5)
    p.global_dependency = math.log10(0.9)
    p.het_val, p.het_unval, p.althom_val, p.althom_unval = 0.10, 0.02, 0.05, 0.01
    p.het_novel, p.althom_novel = 0.0010, 0.0005
    p.rank_sum = p.monoploid = p.refine = p.transition_dominant = 0
    p.precision = precision
    args = list(flags)
    i = 0
    while i < len(args):
        a = args[i]
        val = args[i + 1] if i + 1 < len(args) else None
        takes = a in ("-z", "-g", "-p", "-r", "-e", "-s", "-a", "-b", "-j", "-k", "-M", "-I", "-L", "-Q", "-S",
                      "-F", "-E", "-T", "-i", "-d", "-o")
        if a == "-z":
            c = ord(val[0])
            p.q_min = c - 256 if c > 127 else c
            p.q_max = p.q_min + 40
        elif a == "-g":
            p.global_dependency = math.log10(float(val))
        elif a == "-p":
            p.pcr_dependency = math.log10(float(val))
        elif a == "-r":
            p.althom_novel = float(val)
        elif a == "-e":
            p.het_novel = float(val)
        elif a == "-t":
            p.transition_dominant = 1
        elif a == "-2":
            p.refine = 1
        elif a == "-a":
            p.althom_val = float(val)
        elif a == "-b":
            p.het_val = float(val)
        elif a == "-j":
            p.althom_unval = float(val)
        elif a == "-k":
            p.het_unval = float(val)
        elif a == "-u":
            p.rank_sum = 1
        elif a == "-m":
            p.monoploid = 1
        elif a == "-L":
            p.read_length = int(val) & 0xFF
        elif a == "-Q":
            c = ord(val[0])
            p.q_max = c - 256 if c > 127 else c
        i += 2 if takes else 1
    return p


def site_codes(ref_ascii: np.ndarray, dbsnp_pos: Optional[np.ndarray] = None) -> np.ndarray:
    """4-bit site codes of cpp/chromosome.cc:28-64: (char >> 1) & 7, bit 3 = dbSNP."""
    codes = ((ref_ascii.astype(np.uint8) >> 1) & 7).astype(np.uint8)
    if dbsnp_pos is not None and len(dbsnp_pos):
        codes[np.asarray(dbsnp_pos, dtype=np.int64)] |= 8
    return codes


class Caller:
    """One device context calling one chromosome."""

    def __init__(self, device: int = 0):
        from . import native
        self.lib = native()
        self.ctx = _P()
        rc = self.lib.gsnp_context_create(device, ctypes.byref(self.ctx))
        if rc != GSNP_OK:
            raise RuntimeError(f"gsnp_context_create failed ({rc})")
        self._keep: List[object] = []

    def close(self) -> None:
        if self.ctx:
            self.lib.gsnp_context_destroy(self.ctx)
            self.ctx = _P()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int, what: str) -> None:
        if rc != GSNP_OK:
            msg = self.lib.gsnp_context_error(self.ctx)
            raise RuntimeError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")

    def set_option(self, name: str, value: int) -> None:
        """A launch option of the context (gsnp_set_option)."""
        self._check(self.lib.gsnp_set_option(self.ctx, name.encode(), int(value)), "gsnp_set_option")

    def tune(self, sample_windows: int = 16) -> str:
        """Run the launch autotuner on the resident reads of the last call
        (gsnp_tune); returns its report."""
        buf = ctypes.create_string_buffer(1 << 16)
        self._check(self.lib.gsnp_tune(self.ctx, int(sample_windows), buf, len(buf)), "gsnp_tune")
        return buf.value.decode()

    def set_stream(self, stream_ptr: int) -> None:
        self._check(self.lib.gsnp_set_stream(self.ctx, _P(stream_ptr)), "gsnp_set_stream")

    @staticmethod
    def reads_struct(pos, length, hit, strand, seq, qual, packed=None, packed_qmin: int = 0) -> Reads:
        """The C ABI's read arrays; with packed (gsnp_pack_reads's bytes),
        seq and qual may be None and are not read."""
        r = Reads()
        r.n = int(pos.shape[0])
        r.pos = pos.ctypes.data
        r.len = length.ctypes.data
        r.hit = hit.ctypes.data
        r.strand = strand.ctypes.data
        r.seq = seq.ctypes.data if seq is not None else None
        r.qual = qual.ctypes.data if qual is not None else None
        r.pitch = int((packed if packed is not None else seq).shape[1])
        r.packed = packed.ctypes.data if packed is not None else None
        r.packed_qmin = int(packed_qmin)
        return r

    def load_reference(self, codes: np.ndarray, snp: Optional[np.ndarray] = None) -> None:
        codes = np.ascontiguousarray(codes, dtype=np.uint8)
        snp = np.zeros(0, dtype=SNP_DTYPE) if snp is None else np.ascontiguousarray(snp, dtype=SNP_DTYPE)
        self._keep += [codes, snp]
        self._check(self.lib.gsnp_load_reference(self.ctx, codes.ctypes.data, codes.shape[0],
                                                 snp.ctypes.data if snp.size else None, snp.shape[0]),
                    "gsnp_load_reference")
        self.length = int(codes.shape[0])

    def calibrate(self, params: Params, reads: Reads) -> np.ndarray:
        pm = np.empty(256 * 256 * 16, dtype=np.float64)
        self._check(self.lib.gsnp_calibrate(self.ctx, ctypes.byref(params), ctypes.byref(reads), pm.ctypes.data),
                    "gsnp_calibrate")
        return pm

    def prior_table(self, params: Params) -> np.ndarray:
        out = np.empty(128, dtype=np.float64)
        self._check(self.lib.gsnp_prior_table(ctypes.byref(params), out.ctypes.data), "gsnp_prior_table")
        return out

    def rank_table(self) -> np.ndarray:
        out = np.empty(64 * 64 * 2048, dtype=np.float64)
        self._check(self.lib.gsnp_rank_table(out.ctypes.data), "gsnp_rank_table")
        return out

    def load_tables(self, params: Params, p_matrix: np.ndarray, p_prior: np.ndarray, p_rank: np.ndarray) -> None:
        self._keep += [p_matrix, p_prior, p_rank]
        self._check(self.lib.gsnp_load_tables(self.ctx, ctypes.byref(params), p_matrix.ctypes.data,
                                              p_prior.ctypes.data, p_rank.ctypes.data), "gsnp_load_tables")

    def call(self, reads: Reads) -> None:
        self._check(self.lib.gsnp_call_chromosome(self.ctx, ctypes.byref(reads)), "gsnp_call_chromosome")

    def call_into(self, reads: Reads, out_ptr: int) -> None:
        """Call the chromosome and download every site's call to out_ptr (host
        memory of length * 32 bytes, pinned for the downloads to overlap)."""
        self._check(self.lib.gsnp_call_chromosome_into(self.ctx, ctypes.byref(reads), out_ptr),
                    "gsnp_call_chromosome_into")

    def call_streamed(self, reads: Reads, chr_name: Optional[str] = None, out_ptr: Optional[int] = None,
                      cns_path: Optional[str] = None, columns_base: Optional[str] = None) -> None:
        """Call the chromosome in chunks of the "stream_windows" option's
        windows with bounded device memory, writing each chunk's calls to
        out_ptr and its cns text and -C windows to the files given."""
        enc = lambda s: s.encode() if s is not None else None
        self._check(self.lib.gsnp_call_streamed(self.ctx, ctypes.byref(reads), enc(chr_name), out_ptr,
                                                enc(cns_path), enc(columns_base)), "gsnp_call_streamed")

    def stream_footprint(self) -> tuple:
        """(ring bytes, -C writer bytes) a streamed call holds on the device"""
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        self._check(self.lib.gsnp_stream_footprint(self.ctx, ctypes.byref(a), ctypes.byref(b)), "gsnp_stream_footprint")
        return int(a.value), int(b.value)

    def recall_resident(self) -> None:
        self._check(self.lib.gsnp_recall_resident(self.ctx), "gsnp_recall_resident")

    def fetch(self, first: int = 0, count: Optional[int] = None) -> np.ndarray:
        if count is None:
            count = self.length - first
        out = np.empty(count, dtype=SITE_DTYPE)
        self._check(self.lib.gsnp_fetch_sites(self.ctx, first, count, out.ctypes.data), "gsnp_fetch_sites")
        return out

    def format_cns(self, chr_name: str) -> bytes:
        size = _I64(0)
        self._check(self.lib.gsnp_format_cns(self.ctx, chr_name.encode(), None, ctypes.byref(size)),
                    "gsnp_format_cns")
        buf = ctypes.create_string_buffer(size.value)
        self._check(self.lib.gsnp_format_cns(self.ctx, chr_name.encode(), buf, ctypes.byref(size)),
                    "gsnp_format_cns")
        return buf.raw[:size.value]

    def last_launches(self) -> List[dict]:
        n = ctypes.c_int(32)
        arr = (LaunchInfo * 32)()
        self._check(self.lib.gsnp_last_launches(self.ctx, arr, ctypes.byref(n)), "gsnp_last_launches")
        return [dict(kind=arr[i].kind, slots=arr[i].slots, tiles=arr[i].tiles, sites=arr[i].sites, ms=arr[i].ms)
                for i in range(min(n.value, len(arr)))]

    def transfer_bytes(self):
        h, d = ctypes.c_uint64(), ctypes.c_uint64()
        self._check(self.lib.gsnp_transfer_bytes(self.ctx, ctypes.byref(h), ctypes.byref(d)), "gsnp_transfer_bytes")
        return h.value, d.value

    def stats(self) -> dict:
        """Diagnostics of the last call (gsnp_get_stats)."""
        out = np.zeros(8, dtype=np.uint64)
        self._check(self.lib.gsnp_get_stats(self.ctx, out.ctypes.data, 8), "gsnp_get_stats")
        return {
            "sites": int(out[0]),
            "fixup_sites": int(out[1]),
            "sampled_sites": int(out[2]),
            "max_abs_err": float(np.frombuffer(out[3].tobytes(), dtype=np.float64)[0]),
            "deferred_sites": int(out[4]),
            "sample_mismatches": int(out[5]),
        }


def snp_table(w) -> np.ndarray:
    """dbSNP rows of a synthetic workload as the C ABI's gsnp_snp array."""
    t = np.zeros(w.db_pos.size, dtype=SNP_DTYPE)
    t["pos"] = w.db_pos
    t["validated"] = w.db_validated
    t["hapmap"] = w.db_hapmap
    t["freq"] = w.db_freq
    return t


def run_workload(w, flags: Sequence[str], precision: int = PRECISION_FP64, device: int = 0):
    """Call a synthetic workload end to end; returns (Caller, reads struct, p_matrix)."""
    p = params_from_flags(flags, precision)
    refine_db = "-s" in flags
    codes = site_codes(w.ref, w.db_pos if refine_db else None)
    snp = snp_table(w) if refine_db else None
    c = Caller(device)
    c.load_reference(codes, snp)
    arrs = [np.ascontiguousarray(x) for x in (w.pos, w.length, w.hit, w.strand, w.seq, w.qual)]
    c._keep += arrs
    reads = Caller.reads_struct(*arrs)
    pm = c.calibrate(p, reads)
    pr = c.prior_table(p)
    rk = c.rank_table()
    c.load_tables(p, pm, pr, rk)
    c.call(reads)
    return c, reads, pm
