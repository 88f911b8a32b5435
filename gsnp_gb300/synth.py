"""Seeded synthetic SOAPsnp workloads (reference genome, dbSNP table, SOAP alignments).

The reference project ships no data, so every test and benchmark runs on
inputs generated here.  The five workload shapes follow the configurations the
caller is measured on:

  c0  1 Mbp genome, one 2 kbp N run, 50 bp single-end reads at 10x
  c1  50 Mbp genome, 100 bp reads at 30x, dbSNP table on 1% of sites
  c2  50 Mbp genome, copy-number segments (0/0.5/1/2/8 x 30x), deep hotspot
      clusters, read lengths mixed 35/50/75/100 bp
  c3  c1 with Phred qualities on [2, 60]
  c4  250 Mbp genome, one 3 Mbp N block, 100 bp reads at 40x, rare runs of
      5 low-quality cycles

and one more shape for parity tests only:

  c5  c1 with long reads, 150/200/250 bp under -L 250: the widest read rows
      and per-site dependency state the record layout allows

Every random quantity is drawn from a counter-based SplitMix64 stream keyed by
(seed, stream id, element index).  The draws therefore do not depend on numpy's
Generator implementation or on how the work is chunked, and the same seed gives
byte-identical inputs on x86-64 and aarch64.  The per-base stage (qualities,
sequencing errors) uses integer arithmetic only - inverse-CDF tables of 2^16
entries per read cycle and 32-bit error thresholds - so it can also run on the
GPU through torch (backend="torch") and produce the same bytes.

Base codes follow the caller's ACTG order (A=0, C=1, T=2, G=3).  Positions are
0-based in memory and written 1-based in the SOAP and dbSNP text formats.
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import Dict, List, Optional

import numpy as np

ACTG = np.frombuffer(b"ACTG", dtype=np.uint8)
_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)

# stream ids
S_REF, S_NRUN, S_SNP, S_SNPTYPE, S_START, S_HAP, S_STRAND, S_HIT, S_QUAL, \
    S_ERR, S_ERRBASE, S_DBSNP, S_DBFLAG, S_CN, S_HOT, S_LEN, S_LOWQ = range(17)


def _mix(z: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


class Stream:
    """Counter-based generator: value(i) = splitmix64(key + i*gamma)."""

    def __init__(self, seed: int, stream: int):
        k = np.array([(seed * 1000003 + stream * 7919 + 12345) & 0xFFFFFFFFFFFFFFFF],
                     dtype=np.uint64)
        with np.errstate(over="ignore"):
            self.key = _mix(k + _GAMMA)[0]

    def u64(self, start: int, n: int) -> np.ndarray:
        idx = np.arange(start, start + n, dtype=np.uint64)
        with np.errstate(over="ignore"):
            return _mix(self.key + (idx + np.uint64(1)) * _GAMMA)

    def uniform(self, start: int, n: int) -> np.ndarray:
        """Doubles in [0, 1) with 53 random bits."""
        return (self.u64(start, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)

    def below(self, start: int, n: int, bound) -> np.ndarray:
        """Integers in [0, bound) (bound scalar or array), multiply-shift on 32 bits."""
        hi = (self.u64(start, n) >> np.uint64(32)).astype(np.uint64)
        return ((hi * np.asarray(bound, dtype=np.uint64)) >> np.uint64(32)).astype(np.int64)

    def normal(self, start: int, n: int) -> np.ndarray:
        """Standard normal deviates (Box-Muller on two uniforms per draw)."""
        u = self.u64(start * 2, n * 2)
        u1 = ((u[0::2] >> np.uint64(11)).astype(np.float64) + 1.0) * (1.0 / 9007199254740993.0)
        u2 = (u[1::2] >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


@dataclasses.dataclass
class Config:
    name: str
    genome_len: int
    depth: float
    read_lens: List[int]
    q_mu0: float = 38.0
    q_mu1: float = 22.0
    q_sd: float = 5.0
    q_lo: int = 2
    q_hi: int = 40
    n_runs: List[int] = dataclasses.field(default_factory=lambda: [2000])
    snp_rate: float = 1e-3
    multi_hit_frac: float = 0.05
    dbsnp_frac: float = 0.0
    cn_segments: bool = False
    hotspots: bool = False
    lowq_clusters: float = 0.0
    flags: List[str] = dataclasses.field(default_factory=list)
    q_max_char: Optional[str] = None


CONFIGS: Dict[str, Config] = {
    "c0": Config("c0", 1_000_000, 10.0, [50], flags=["-L", "50", "-t", "-u"]),
    "c1": Config("c1", 50_000_000, 30.0, [100], dbsnp_frac=0.01,
                 flags=["-L", "100", "-t", "-u", "-2"]),
    "c2": Config("c2", 50_000_000, 30.0, [35, 50, 75, 100], n_runs=[], cn_segments=True,
                 hotspots=True, flags=["-L", "100", "-t", "-u"]),
    "c3": Config("c3", 50_000_000, 30.0, [100], q_mu0=45.0, q_mu1=25.0, q_sd=8.0, q_hi=60,
                 dbsnp_frac=0.01, flags=["-L", "100", "-Q", "|", "-t", "-u", "-2"],
                 q_max_char="|"),
    "c4": Config("c4", 250_000_000, 40.0, [100], n_runs=[3_000_000], lowq_clusters=1e-4,
                 flags=["-L", "100", "-t", "-u", "-C"]),
    "c5": Config("c5", 50_000_000, 30.0, [150, 200, 250], dbsnp_frac=0.01,
                 flags=["-L", "250", "-t", "-u", "-2"]),
}


@dataclasses.dataclass
class Workload:
    config: Config
    seed: int
    chr_name: str
    ref: np.ndarray            # uint8 ASCII, length G
    read_length: int           # -L value (max read length)
    pos: np.ndarray            # int32, 0-based start, sorted ascending
    length: np.ndarray         # int32
    hit: np.ndarray            # int32
    strand: np.ndarray         # uint8 ASCII '+' / '-'
    seq: np.ndarray            # uint8 [R, L] ASCII bases (forward reference orientation)
    qual: np.ndarray           # uint8 [R, L] ASCII quality chars (Phred+64)
    mismatch: np.ndarray       # int32
    db_pos: np.ndarray         # int64 0-based positions of dbSNP rows (sorted)
    db_hapmap: np.ndarray      # uint8 0/1
    db_validated: np.ndarray   # uint8 0/1
    db_freq: np.ndarray        # float64 [K, 4] in ACTG order

    @property
    def num_reads(self) -> int:
        return int(self.pos.shape[0])

    @property
    def num_bases(self) -> int:
        return int(self.length.sum())

    @property
    def genome_len(self) -> int:
        return int(self.ref.shape[0])

    def cli_flags(self, dbsnp_path: Optional[str] = None) -> List[str]:
        f = list(self.config.flags)
        if dbsnp_path is not None and self.db_pos.size:
            f += ["-s", dbsnp_path]
        elif "-2" in f:
            f.remove("-2")
        return f


def _transition(b: np.ndarray) -> np.ndarray:
    # ACTG codes: A(0)<->G(3), C(1)<->T(2): transition partner is b ^ 3
    return b ^ 3


def _alt_base(ref_code: np.ndarray, u: np.ndarray, pick: np.ndarray) -> np.ndarray:
    """Transition with probability 2/3, else one of the two transversions."""
    tv = np.where(pick == 0, ref_code ^ 1, ref_code ^ 2)
    return np.where(u < 2.0 / 3.0, _transition(ref_code), tv).astype(np.int64)


def make_workload(name: str, scale: float = 1.0, seed: Optional[int] = None,
                  genome_len: Optional[int] = None, backend: str = "numpy", device: str = "cuda") -> Workload:
    """Build workload `name` ("c0".."c4").

    scale shrinks the genome (and with it the read count) while keeping depth,
    read lengths and quality model.  seed defaults to 20260000 + config index.
    backend "torch" runs the per-base stage on `device` and returns seq/qual in
    pinned host memory; the bytes equal the numpy backend's.
    """
    cfg = CONFIGS[name]
    if seed is None:
        seed = 20260000 + int(name[1:])
    G = genome_len if genome_len is not None else max(20_000, int(round(cfg.genome_len * scale)))
    Lmax = max(cfg.read_lens)

    # ---- reference: i.i.d. bases, GC 41% ----
    u = Stream(seed, S_REF).uniform(0, G)
    code = np.where(u < 0.295, 0, np.where(u < 0.5, 1, np.where(u < 0.795, 2, 3))).astype(np.int64)
    isn = np.zeros(G, dtype=bool)
    ns = Stream(seed, S_NRUN)
    for k, run in enumerate(cfg.n_runs):
        run = min(run, G // 4)
        # keep N runs away from the first window and from the chromosome end
        lo = min(G // 3, 262_144 + 1000) if G > 262_144 * 2 else G // 3
        hi = max(lo + 1, G - run - G // 5)
        start = lo + int(ns.below(k, 1, hi - lo)[0])
        isn[start:start + run] = True
    ref = ACTG[code].copy()
    ref[isn] = ord("N")

    # ---- diploid sample: SNPs at rate snp_rate on non-N sites ----
    su = Stream(seed, S_SNP).uniform(0, G)
    snp = (su < cfg.snp_rate) & ~isn
    snp_pos = np.nonzero(snp)[0]
    st = Stream(seed, S_SNPTYPE)
    t_u = st.uniform(0, snp_pos.size)          # het (2/3) / hom (1/3)
    a_u = st.uniform(snp_pos.size, snp_pos.size)
    a_p = st.below(2 * snp_pos.size, snp_pos.size, 2)
    h_p = st.below(3 * snp_pos.size, snp_pos.size, 2)
    alt = _alt_base(code[snp_pos], a_u, a_p)
    hap = np.stack([code.astype(np.uint8), code.astype(np.uint8)])
    is_het = t_u < 2.0 / 3.0
    hap[h_p[is_het], snp_pos[is_het]] = alt[is_het]
    hap[0, snp_pos[~is_het]] = alt[~is_het]
    hap[1, snp_pos[~is_het]] = alt[~is_het]
    true_alt = np.full(G, -1, dtype=np.int64)
    true_alt[snp_pos] = alt

    # ---- read starts ----
    n_prefix = np.concatenate([[0], np.cumsum(isn, dtype=np.int64)])
    weight = np.ones(G, dtype=np.float64)
    if cfg.cn_segments:
        cs = Stream(seed, S_CN)
        mult_vals = np.array([0.0, 0.5, 1.0, 2.0, 8.0])
        mult_cdf = np.cumsum([0.05, 0.15, 0.6, 0.15, 0.05])
        p = 0
        k = 0
        while p < G:
            uu = cs.uniform(2 * k, 2)
            seg = 1 + int(-math.log(1.0 - uu[0]) * 100_000)
            m = mult_vals[min(4, int(np.searchsorted(mult_cdf, uu[1], side="right")))]
            weight[p:p + seg] = m
            p += seg
            k += 1
    mean_len = float(np.mean(cfg.read_lens))
    R = int(round(cfg.depth * float(weight.sum()) / mean_len))
    starts = np.empty(0, dtype=np.int64)
    lens = np.empty(0, dtype=np.int64)
    ss = Stream(seed, S_START)
    ls = Stream(seed, S_LEN)
    cw = np.cumsum(weight) if cfg.cn_segments else None
    total_w = cw[-1] if cfg.cn_segments else float(G)
    drawn = 0
    while starts.size < R:
        need = int((R - starts.size) * 1.1) + 64
        ln = np.asarray(cfg.read_lens, dtype=np.int64)[ls.below(drawn, need, len(cfg.read_lens))]
        if cfg.cn_segments:
            uu = ss.uniform(drawn, need)
            cand = np.searchsorted(cw, uu * total_w, side="right").astype(np.int64)
        else:
            cand = ss.below(drawn, need, G)
        drawn += need
        ok = (cand + ln < G) & (n_prefix[np.minimum(cand + ln, G)] - n_prefix[np.minimum(cand, G)] == 0)
        starts = np.concatenate([starts, cand[ok]])
        lens = np.concatenate([lens, ln[ok]])
    starts = starts[:R]
    lens = lens[:R]

    if cfg.hotspots:
        # clusters of reads starting within +-10 bp of a centre, so that about
        # 0.5% of sites sit under a pileup of 300-1000x
        hs = Stream(seed, S_HOT)
        n_clusters = max(1, int(0.005 * G / 80))
        centres = 200 + hs.below(0, n_clusters, G - 400)
        extra_s, extra_l = [], []
        for c in range(n_clusters):
            d = 300 + int(hs.below(n_clusters + c, 1, 701)[0])
            base_depth = int(weight[centres[c]] * cfg.depth)
            n_extra = max(0, d - base_depth)
            if n_extra == 0:
                continue
            off = hs.below(10_000_000 + c * 4096, n_extra, 21) - 10
            lnx = np.asarray(cfg.read_lens, dtype=np.int64)[
                hs.below(20_000_000 + c * 4096, n_extra, len(cfg.read_lens))]
            st_x = np.clip(centres[c] + off - lnx // 2, 0, None)
            okx = (st_x + lnx < G) & (n_prefix[np.minimum(st_x + lnx, G)] - n_prefix[st_x] == 0)
            extra_s.append(st_x[okx])
            extra_l.append(lnx[okx])
        if extra_s:
            starts = np.concatenate([starts] + extra_s)
            lens = np.concatenate([lens] + extra_l)

    order = np.argsort(starts, kind="stable")
    starts = starts[order]
    lens = lens[order]
    R = int(starts.size)
    if name == "c2":
        win = starts // 262_144
        assert np.bincount(win).max() <= 4 * 262_144 + 100, "per-window read cap exceeded"

    # ---- per-read attributes ----
    hap_id = Stream(seed, S_HAP).below(0, R, 2)
    strand_minus = Stream(seed, S_STRAND).below(0, R, 2) == 1
    hu = Stream(seed, S_HIT)
    multi = hu.uniform(0, R) < cfg.multi_hit_frac
    hit = np.where(multi, 2 + hu.below(R, R, 4), 1).astype(np.int32)

    # ---- bases and qualities ----
    if backend == "torch":
        seq, qual, mism = _bases_torch(cfg, seed, G, Lmax, starts, lens, hap, hap_id, strand_minus, code, device)
    else:
        seq, qual, mism = _bases_numpy(cfg, seed, G, Lmax, starts, lens, hap, hap_id, strand_minus, code)

    strand = np.where(strand_minus, ord("-"), ord("+")).astype(np.uint8)

    # ---- dbSNP table ----
    if cfg.dbsnp_frac > 0:
        nonN = np.nonzero(~isn)[0]
        du = Stream(seed, S_DBSNP).uniform(0, nonN.size)
        db_pos = nonN[du < cfg.dbsnp_frac]
        K = db_pos.size
        df = Stream(seed, S_DBFLAG)
        hapmap = (df.uniform(0, K) < 0.5).astype(np.uint8)
        validated = (df.uniform(K, K) < 0.8).astype(np.uint8)
        f = 0.01 + 0.49 * df.uniform(2 * K, K)
        f = np.round(f, 4)
        second = true_alt[db_pos]
        fallback = _alt_base(code[db_pos], df.uniform(3 * K, K), df.below(4 * K, K, 2))
        second = np.where(second >= 0, second, fallback)
        freq = np.zeros((K, 4), dtype=np.float64)
        freq[np.arange(K), code[db_pos]] = np.round(1.0 - f, 4)
        freq[np.arange(K), second] = f
    else:
        db_pos = np.zeros(0, dtype=np.int64)
        hapmap = np.zeros(0, dtype=np.uint8)
        validated = np.zeros(0, dtype=np.uint8)
        freq = np.zeros((0, 4), dtype=np.float64)

    return Workload(config=cfg, seed=seed, chr_name="chr1", ref=ref, read_length=Lmax,
                    pos=starts.astype(np.int32), length=lens.astype(np.int32), hit=hit,
                    strand=strand, seq=seq, qual=qual, mismatch=mism,
                    db_pos=db_pos.astype(np.int64), db_hapmap=hapmap, db_validated=validated,
                    db_freq=freq)


# ---------------------------------------------------------------------------
# per-base stage: integer-only draws
# ---------------------------------------------------------------------------

_U64 = (1 << 64) - 1


def _signed(x: int) -> int:
    x &= _U64
    return x - (1 << 64) if x >= (1 << 63) else x


def quality_tables(cfg: Config, read_len: int) -> np.ndarray:
    """[read_len][65536] uint8: inverse CDF of the Phred quality at each cycle.

    q = round(N(mu(c), sd)) clipped to [q_lo, q_hi], mu falling linearly from
    q_mu0 at the first cycle to q_mu1 at the last; the CDF is resolved to
    1/65536.
    """
    out = np.empty((read_len, 65536), dtype=np.uint8)
    ks = np.arange(cfg.q_lo, cfg.q_hi + 1)
    grid = np.arange(65536, dtype=np.int64)
    for c in range(read_len):
        mu = cfg.q_mu0 + (cfg.q_mu1 - cfg.q_mu0) * (c / max(read_len - 1, 1))
        cdf = [0.5 * (1.0 + math.erf((k + 0.5 - mu) / (cfg.q_sd * math.sqrt(2.0)))) for k in ks[:-1]]
        thr = np.array([int(round(x * 65536.0)) for x in cdf] + [65536], dtype=np.int64)
        out[c] = ks[np.searchsorted(thr, grid, side="right")]
    return out


def error_thresholds() -> np.ndarray:
    """floor(10^(-q/10) * 2^32) for q in [0, 128): a base is miscalled when the
    high 32 bits of its draw fall below the threshold of its quality."""
    return np.array([min(int(math.floor((10.0 ** (-q / 10.0)) * 4294967296.0)), (1 << 32) - 1)
                     for q in range(128)], dtype=np.uint64)


def _bases_numpy(cfg, seed, G, Lmax, starts, lens, hap, hap_id, strand_minus, code):
    R = starts.size
    seq = np.zeros((R, Lmax), dtype=np.uint8)
    qual = np.zeros((R, Lmax), dtype=np.uint8)
    mism = np.zeros(R, dtype=np.int32)
    qs, es, lq = Stream(seed, S_QUAL), Stream(seed, S_ERR), Stream(seed, S_LOWQ)
    lens_set = sorted(set(int(x) for x in cfg.read_lens))
    tables = np.stack([np.vstack([quality_tables(cfg, Lr), np.zeros((Lmax - Lr, 65536), np.uint8)])
                       for Lr in lens_set])
    len_index = np.zeros(Lmax + 1, dtype=np.int64)
    for i, Lr in enumerate(lens_set):
        len_index[Lr] = i
    thr = error_thresholds()
    low_thr = np.uint64(int(cfg.lowq_clusters * 4294967296.0))
    coord = np.arange(Lmax, dtype=np.int64)
    CH = 1 << 16
    m32 = np.uint64(0xFFFFFFFF)
    for r0 in range(0, R, CH):
        r1 = min(R, r0 + CH)
        n = r1 - r0
        st_ = starts[r0:r1]
        ln_ = lens[r0:r1]
        valid = coord[None, :] < ln_[:, None]
        gpos = np.minimum(st_[:, None] + coord[None, :], G - 1)
        truth = hap[hap_id[r0:r1][:, None], gpos].astype(np.int64)
        minus = strand_minus[r0:r1][:, None]
        cycle = np.where(minus, ln_[:, None] - 1 - coord[None, :], coord[None, :])
        cycle = np.where(valid, cycle, 0)
        uq = qs.u64(r0 * Lmax, n * Lmax).reshape(n, Lmax)
        q = tables[len_index[ln_][:, None], cycle, (uq >> np.uint64(48)).astype(np.int64)].astype(np.int64)
        if cfg.lowq_clusters > 0:
            ul = lq.u64(r0 * Lmax, n * Lmax).reshape(n, Lmax)
            startc = ((ul >> np.uint64(32)) < low_thr) & (cycle + 5 <= ln_[:, None]) & valid
            lowv = (2 + (((ul & m32) * np.uint64(7)) >> np.uint64(32))).astype(np.int64)
            forced = np.zeros((n, Lmax + 5), dtype=np.int64)
            rows, cols = np.nonzero(startc)
            cst = cycle[rows, cols]
            for d in range(5):
                forced[rows, cst + d] = lowv[rows, cols]
            fq = np.take_along_axis(forced, cycle, axis=1)
            q = np.where(fq > 0, fq, q)
        ue = es.u64(r0 * Lmax, n * Lmax).reshape(n, Lmax)
        err = (ue >> np.uint64(32)) < thr[q]
        shift = (1 + (((ue & m32) * np.uint64(3)) >> np.uint64(32))).astype(np.int64)
        obs = np.where(err, (truth + shift) & 3, truth)
        s_ascii = ACTG[obs]
        q_ascii = (64 + q).astype(np.uint8)
        s_ascii[~valid] = 0
        q_ascii[~valid] = 0
        seq[r0:r1] = s_ascii
        qual[r0:r1] = q_ascii
        refc = np.where(valid, code[gpos], -1)
        mism[r0:r1] = np.sum((obs != refc) & valid, axis=1)
    return seq, qual, mism


def _bases_torch(cfg, seed, G, Lmax, starts, lens, hap, hap_id, strand_minus, code, device):
    import torch
    dev = torch.device(device)
    R = starts.size
    pin = dev.type == "cuda"
    seq = torch.empty((R, Lmax), dtype=torch.uint8, pin_memory=pin)
    qual = torch.empty((R, Lmax), dtype=torch.uint8, pin_memory=pin)
    mism = torch.empty(R, dtype=torch.int32, pin_memory=pin)
    M1 = torch.tensor(_signed(0xBF58476D1CE4E5B9), dtype=torch.int64, device=dev)
    M2 = torch.tensor(_signed(0x94D049BB133111EB), dtype=torch.int64, device=dev)
    GAM = torch.tensor(_signed(0x9E3779B97F4A7C15), dtype=torch.int64, device=dev)

    def lsr(z, k):
        return (z >> k) & ((1 << (64 - k)) - 1)

    def mix(z):
        z = (z ^ lsr(z, 30)) * M1
        z = (z ^ lsr(z, 27)) * M2
        return z ^ lsr(z, 31)

    def u64(stream: Stream, start: int, n: int):
        key = torch.tensor(_signed(int(stream.key)), dtype=torch.int64, device=dev)
        idx = torch.arange(start + 1, start + 1 + n, dtype=torch.int64, device=dev)
        return mix(key + idx * GAM)

    qs, es, lq = Stream(seed, S_QUAL), Stream(seed, S_ERR), Stream(seed, S_LOWQ)
    lens_set = sorted(set(int(x) for x in cfg.read_lens))
    tables = np.stack([np.vstack([quality_tables(cfg, Lr), np.zeros((Lmax - Lr, 65536), np.uint8)])
                       for Lr in lens_set])
    len_index = np.zeros(Lmax + 1, dtype=np.int64)
    for i, Lr in enumerate(lens_set):
        len_index[Lr] = i
    t_tab = torch.from_numpy(tables).to(dev).to(torch.int64)
    t_len_index = torch.from_numpy(len_index).to(dev)
    t_thr = torch.from_numpy(error_thresholds().astype(np.int64)).to(dev)
    t_hap = torch.from_numpy(hap).to(dev)
    t_code = torch.from_numpy(code.astype(np.uint8)).to(dev).to(torch.int64)
    t_starts = torch.from_numpy(starts.astype(np.int64)).to(dev)
    t_lens = torch.from_numpy(lens.astype(np.int64)).to(dev)
    t_hapid = torch.from_numpy(hap_id.astype(np.int64)).to(dev)
    t_minus = torch.from_numpy(strand_minus).to(dev)
    t_actg = torch.tensor([65, 67, 84, 71], dtype=torch.uint8, device=dev)
    low_thr = int(cfg.lowq_clusters * 4294967296.0)
    coord = torch.arange(Lmax, dtype=torch.int64, device=dev)
    m32 = 0xFFFFFFFF
    CH = 1 << 20
    for r0 in range(0, R, CH):
        r1 = min(R, r0 + CH)
        n = r1 - r0
        st_ = t_starts[r0:r1]
        ln_ = t_lens[r0:r1]
        valid = coord[None, :] < ln_[:, None]
        gpos = torch.clamp(st_[:, None] + coord[None, :], max=G - 1)
        truth = t_hap[t_hapid[r0:r1][:, None], gpos].to(torch.int64)
        minus = t_minus[r0:r1][:, None]
        cycle = torch.where(minus, ln_[:, None] - 1 - coord[None, :], coord[None, :])
        cycle = torch.where(valid, cycle, torch.zeros_like(cycle))
        uq = u64(qs, r0 * Lmax, n * Lmax).reshape(n, Lmax)
        q = t_tab[t_len_index[ln_][:, None], cycle, lsr(uq, 48)]
        if cfg.lowq_clusters > 0:
            ul = u64(lq, r0 * Lmax, n * Lmax).reshape(n, Lmax)
            startc = (lsr(ul, 32) < low_thr) & (cycle + 5 <= ln_[:, None]) & valid
            lowv = 2 + (((ul & m32) * 7) >> 32)
            forced = torch.zeros((n, Lmax + 5), dtype=torch.int64, device=dev)
            rows, cols = torch.nonzero(startc, as_tuple=True)
            cst = cycle[rows, cols]
            for d in range(5):
                forced[rows, cst + d] = lowv[rows, cols]
            fq = torch.gather(forced, 1, cycle)
            q = torch.where(fq > 0, fq, q)
        ue = u64(es, r0 * Lmax, n * Lmax).reshape(n, Lmax)
        err = lsr(ue, 32) < t_thr[q]
        shift = 1 + (((ue & m32) * 3) >> 32)
        obs = torch.where(err, (truth + shift) & 3, truth)
        s_ascii = t_actg[obs]
        q_ascii = (64 + q).to(torch.uint8)
        s_ascii[~valid] = 0
        q_ascii[~valid] = 0
        seq[r0:r1].copy_(s_ascii, non_blocking=True)
        qual[r0:r1].copy_(q_ascii, non_blocking=True)
        refc = torch.where(valid, t_code[gpos], torch.full_like(gpos, -1))
        mism[r0:r1].copy_(((obs != refc) & valid).sum(dim=1).to(torch.int32), non_blocking=True)
    if pin:
        torch.cuda.synchronize(dev)
    return seq.numpy(), qual.numpy(), mism.numpy()


# ---------------------------------------------------------------------------
# text writers (the reference's input formats)
# ---------------------------------------------------------------------------

def write_fasta(w: Workload, path: str, width: int = 60) -> None:
    with open(path, "wb") as f:
        f.write(b">" + w.chr_name.encode() + b"\n")
        ref = w.ref.tobytes()
        for i in range(0, len(ref), width):
            f.write(ref[i:i + width] + b"\n")


def write_dbsnp(w: Workload, path: str) -> None:
    """Rows: chr pos(1-based) hapmap validated indel fA fC fT fG rsID."""
    with open(path, "w") as f:
        for k in range(w.db_pos.size):
            fr = w.db_freq[k]
            f.write("%s\t%d\t%d\t%d\t0\t%.4f\t%.4f\t%.4f\t%.4f\trs%d\n" % (
                w.chr_name, int(w.db_pos[k]) + 1, int(w.db_hapmap[k]), int(w.db_validated[k]),
                fr[0], fr[1], fr[2], fr[3], k + 1))


def soap_lines(w: Workload, r0: int = 0, r1: Optional[int] = None) -> bytes:
    """SOAP alignment text: id seq qual hit a/b len strand chr pos(1-based) mismatch."""
    if r1 is None:
        r1 = w.num_reads
    out = []
    chrb = w.chr_name.encode()
    for r in range(r0, r1):
        n = int(w.length[r])
        out.append(b"r%d\t%s\t%s\t%d\ta\t%d\t%c\t%s\t%d\t%d\n" % (
            r, w.seq[r, :n].tobytes(), w.qual[r, :n].tobytes(), int(w.hit[r]), n,
            int(w.strand[r]), chrb, int(w.pos[r]) + 1, int(w.mismatch[r])))
    return b"".join(out)


def write_soap(w: Workload, path: str) -> None:
    with open(path, "wb") as f:
        CH = 1 << 16
        for r0 in range(0, w.num_reads, CH):
            f.write(soap_lines(w, r0, min(w.num_reads, r0 + CH)))


def workload_digest(w: Workload) -> str:
    """SHA-256 over every array of the workload, in a fixed order and layout.

    The text files of write_inputs are a function of these arrays, so equal
    digests mean the same input files; the digest is cheap to take where the
    multi-gigabyte text files are not written (the GPU generator).
    """
    import hashlib
    h = hashlib.sha256()
    h.update(w.chr_name.encode() + b"\0")
    for a, dt in ((w.ref, "u1"), (w.pos, "<i4"), (w.length, "<i4"), (w.hit, "<i4"), (w.strand, "u1"),
                  (w.seq, "u1"), (w.qual, "u1"), (w.mismatch, "<i4"), (w.db_pos, "<i8"), (w.db_hapmap, "u1"),
                  (w.db_validated, "u1"), (w.db_freq, "<f8")):
        b = np.ascontiguousarray(a, dtype=dt)
        h.update(np.asarray(b.shape, dtype="<i8").tobytes())
        h.update(memoryview(b).cast("B"))
    return h.hexdigest()


def write_inputs(w: Workload, directory: str) -> Dict[str, str]:
    """Write ref.fa, reads.soap and (when present) dbsnp.txt under `directory`."""
    os.makedirs(directory, exist_ok=True)
    paths = {"ref": os.path.join(directory, "ref.fa"),
             "soap": os.path.join(directory, "reads.soap")}
    write_fasta(w, paths["ref"])
    write_soap(w, paths["soap"])
    if w.db_pos.size:
        paths["dbsnp"] = os.path.join(directory, "dbsnp.txt")
        write_dbsnp(w, paths["dbsnp"])
    return paths
