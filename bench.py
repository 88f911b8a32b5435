#!/usr/bin/env python
"""Benchmark of the GB300 consensus caller on the 30x workload (c1 shape).

Workload: 50 Mbp reference (GC 41%, one 2 kbp N run), 100 bp single-end reads
at 30x (15 M alignments, 1.5e9 bases), dbSNP rows on 1% of sites, flags
-L 100 -t -u -2 -s.  The inputs are seeded synthetic data of that shape
(gsnp_gb300.synth), generated on the GPU; there is no public dataset.

A step is one calling pass over the whole chromosome.  The headline form is
the FP32 compensated likelihood with FP64 fixup; the plain FP64 form is timed
beside it in the same run (the "compare" object).
  value : sites/s with the alignments resident in HBM (tile classification and
          the binned calling kernels, CUDA events on the launching stream);
          the alignments (3 GB) exceed L2, so no flush is needed between steps.
  e2e   : sites/s through the C ABI (gsnp_call_chromosome_into) from pinned
          host buffers: upload of the alignments, window replay, gather,
          calling, and the download of every site's 32-byte call, all inside
          the timed step (the library overlaps them segment by segment).  The
          reads are uploaded packed, base and quality in one byte per
          position (gsnp_pack_reads, untimed, its time given as pack_ms);
          e2e_unpacked is the same call with two bytes per position.
The calling kernels' roofline is the HBM bandwidth; the algorithmic bytes of a
site are 2*D + 9*D/Lbar + 0.5 + 32 (bases and qualities of the covering reads,
per-read start/length/strand, the 4-bit reference code, a 32-byte call).

--impl reference times the reference's calling algorithm on the host cores:
the CPU oracle (oracle/, a restatement of the reference's single-threaded
calling code) on a bounded sample of the same workload, one process per core.
The cpu_baseline object of the GPU line is the same code on one core.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIG = "c1"
WORKLOADS = {
    "c0": "c0: 1 Mbp reference, 50 bp reads at 10x (200 k alignments), -L 50 -t -u",
    "c1": "c1: 50 Mbp reference, 100 bp reads at 30x (15 M alignments), dbSNP 1%, -L 100 -t -u -2 -s",
    "c2": "c2: 50 Mbp, copy-number segments and 300-1000x hotspots, 35/50/75/100 bp reads, -L 100 -t -u",
    "c3": "c3: c1 with Phred 2-60 qualities, -L 100 -Q '|' -t -u -2 -s",
    "c4": "c4: 250 Mbp, 3 Mbp N block, 100 bp reads at 40x (100 M alignments), -L 100 -t -u",
}
METRIC = "sites/s at 30x (bases/s = sites/s x mean depth)"
UNIT = "sites/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gsnp", "reference"], default="gsnp")
    ap.add_argument("--precision", choices=["fp64", "fp32"], default="fp32",
                    help="headline form: fp32 = FP32 compensated sums with FP64 fixup, fp64 = plain FP64")
    ap.add_argument("--no-compare", action="store_true", help="do not also time the other form")
    ap.add_argument("--scale", type=float, default=1.0, help="genome scale (1.0 = the named workload's full size)")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=CONFIG,
                    help="synthetic workload shape (the headline is c1, the 30x configuration)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch settings (no autotuner)")
    ap.add_argument("--tune-windows", type=int, default=32, help="windows of 262,144 sites the autotuner samples")
    ap.add_argument("--stream-windows", type=int, default=16,
                    help="windows per chunk of the streamed (bounded device memory) e2e call")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_max(dist, x, device="cuda"):
    """The largest x over the ranks (x itself without a process group): each
    rank times its own replica, and the job's step takes the slowest."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world, units_per_rank, seconds):
    """Whole-job rate of replicas: every rank's units over the slowest rank's
    time (per-rank work fixed as ranks are added: weak scaling)."""
    return world * units_per_rank / seconds


class ClockSampler:
    """nvidia-smi clock and throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.first = 0

    def __enter__(self):
        if self.device < 0:
            return self
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
            return self
        # nvidia-smi takes a while to start: wait for its first sample, so that
        # the timed region that follows is sampled from its beginning
        t0 = time.time()
        while not self.lines and self.proc.poll() is None and time.time() - t0 < 20:
            time.sleep(0.02)
        self.first = len(self.lines)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        """samples taken after the first one (which precedes the timed region)"""
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[self.first:] or self.lines[-1:]:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# DRAM traffic per site of the dominant calling kernel (dram__bytes_read.sum +
# dram__bytes_write.sum of one ncu capture of that kernel on a 10%-scale case
# of the workload, divided by the sites of the captured launch).  The traffic
# of a full-size launch is that figure times its sites: a launch reads its
# tiles' reads once and writes one call per site, so traffic grows with the
# sites.  Keyed by (workload, kernel kind, record slots); other kernels report
# no traffic.
# file outputs of the timed e2e steps go to a RAM-backed directory where the
# host has one, so that a disk's write-back does not time the caller
RAM_DIR = "/dev/shm" if os.path.isdir("/dev/shm") and os.access("/dev/shm", os.W_OK) else None

NCU_BYTES_PER_SITE = {
    ("c1", 2, 40): 150.6,   # call_fast_kernel<40>: 324.6 MB (dram__bytes.sum) over 2,154,656 sites
    ("c1", 4, 48): 95.0,    # call_stream_kernel<48>: 325.2 MB read + 150.1 MB written over 5,000,000 sites
}


def site_bytes(w):
    """Algorithmic bytes of one called site."""
    sites = w.genome_len
    D = w.num_bases / sites
    reads_per_site = w.num_reads / sites
    return 2.0 * D + 9.0 * reads_per_site + 0.5 + 32.0


class OracleSample:
    """A bounded sample of the workload's shape written as the reference's
    input files, timed through the CPU oracle (a port of the reference's
    single-threaded calling code, run on one core)."""

    def __init__(self, sample_len: int, workload: str = CONFIG):
        from gsnp_gb300 import synth
        self.oracle = os.path.join(ROOT, "oracle", "_build", "gsnp_oracle")
        if not os.path.exists(self.oracle):
            subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "-j8"], check=True)
        self.w = synth.make_workload(workload, genome_len=sample_len)
        self.dir = tempfile.TemporaryDirectory()
        self.paths = synth.write_inputs(self.w, self.dir.name)
        self.flags = [f for f in self.w.cli_flags(self.paths.get("dbsnp")) if f != "-C"]
        self.sample = "%d-site %s-shaped sample (%d reads), calling pass (window loop + cns text), 1 thread" % (
            self.w.genome_len, workload, self.w.num_reads)

    def start(self, out_dir: str) -> subprocess.Popen:
        env = dict(os.environ, GSNP_ORACLE_TIMING="1")
        return subprocess.Popen([self.oracle, "-i", self.paths["soap"], "-d", self.paths["ref"], "-o",
                                 os.path.join(out_dir, "cns")] + self.flags, cwd=out_dir, env=env,
                                stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True)

    @staticmethod
    def seconds(proc: subprocess.Popen) -> float:
        _, err = proc.communicate()
        if proc.returncode != 0:
            raise RuntimeError("oracle failed: " + err[-500:])
        for line in err.splitlines():
            if line.startswith("pass2_seconds="):
                return float(line.split("=")[1])
        raise RuntimeError("oracle printed no timing")

    def run(self) -> float:
        """sites/s of one process (one core)."""
        return self.w.genome_len / self.seconds(self.start(self.dir.name))

    def run_parallel(self, procs: int) -> float:
        """Aggregate sites/s of `procs` concurrent processes on the sample,
        counted against the slowest one."""
        dirs = [tempfile.mkdtemp(dir=self.dir.name) for _ in range(procs)]
        running = [self.start(d) for d in dirs]
        secs = [self.seconds(p) for p in running]
        return procs * self.w.genome_len / max(secs)


def cpu_baseline(sample_len: int, workload: str = CONFIG):
    s = OracleSample(sample_len, workload)
    return s.run(), s.sample


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args, rank, world):
    """The reference's calling code (single-threaded per chromosome) on every
    host core: one process per core, each calling its own copy of the sample."""
    if rank != 0:
        return
    sample_len = 600_000 if args.scale >= 1.0 else max(40_000, int(600_000 * args.scale))
    smp = OracleSample(sample_len, args.workload)
    cores = host_cores()
    vals = []
    for i in range(args.warmup + args.steps):
        v = smp.run_parallel(cores)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.mean(vals)
    sample = "%s; %d concurrent processes, one per host core" % (smp.sample.replace(", 1 thread", ""), cores)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * cores * sample_len / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload], "sample_sites": sample_len, "processes": cores},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    rank, world, local = dist_info()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import numpy as np
    import torch
    from gsnp_gb300 import api, synth

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        dist = None

    precision = api.PRECISION_FP64 if args.precision == "fp64" else api.PRECISION_FP32_FIXUP
    other = api.PRECISION_FP32_FIXUP if precision == api.PRECISION_FP64 else api.PRECISION_FP64
    t0 = time.time()
    w = synth.make_workload(args.workload, scale=args.scale, backend="torch", device="cuda:%d" % local)
    t_gen = time.time() - t0
    flags = w.cli_flags("dbsnp")   # the dbSNP rows are passed in memory
    codes = api.site_codes(w.ref, w.db_pos)
    caller = api.Caller(local)
    caller.load_reference(codes, api.snp_table(w))
    def pinned(x):
        """x in page-locked host memory (the e2e copies read the inputs from pinned memory)"""
        x = np.ascontiguousarray(x)
        t = torch.empty(x.shape, dtype=getattr(torch, x.dtype.name), pin_memory=True)
        t.numpy()[...] = x
        return t.numpy()

    arrs = [pinned(x) for x in (w.pos, w.length, w.hit, w.strand, w.seq, w.qual)]
    # pinned destination of the e2e steps' site calls, allocated with the inputs
    out_pinned = torch.empty(w.genome_len * 32, dtype=torch.uint8, pin_memory=True)
    reads = api.Caller.reads_struct(*arrs)
    p = api.params_from_flags(flags, precision)
    # the same reads with base and quality in one byte per position, the form
    # the e2e steps upload (gsnp_pack_reads on all host threads, untimed; its
    # time is reported beside the e2e figure)
    packed = torch.empty(tuple(w.seq.shape), dtype=torch.uint8, pin_memory=True).numpy()
    t1 = time.perf_counter()
    api.pack_reads(arrs[4], arrs[5], arrs[1], p.q_min, out=packed)
    pack_ms = (time.perf_counter() - t1) * 1e3
    reads_packed = api.Caller.reads_struct(*arrs[:4], None, None, packed=packed, packed_qmin=p.q_min)
    pm = caller.calibrate(p, reads)
    prior, rank_tab = caller.prior_table(p), caller.rank_table()
    caller.load_tables(p, pm, prior, rank_tab)
    stream = torch.cuda.current_stream()
    caller.set_stream(stream.cuda_stream)
    caller.call(reads)                       # uploads the alignments, first pass
    sites = w.genome_len
    # the launch autotuner on a sample of the resident workload (untimed): the
    # chosen settings are those of every timed pass below
    tuning = None
    if not args.no_tune:
        t1 = time.time()
        report = caller.tune(sample_windows=args.tune_windows)
        tuning = {"options": dict(ln.split() for ln in report.splitlines() if ln and not ln.startswith("#")
                                  and len(ln.split()) == 2 and not ln.split()[1].endswith("ms")),
                  "summary": next((ln[2:] for ln in report.splitlines() if ln.startswith("# ")), ""),
                  "seconds": round(time.time() - t1, 2)}

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x):
        return replica_max(dist, x)

    def time_form(prec):
        """Per-kernel times from passes launched one kernel at a time (each
        timed by events, untimed region), then, after the warm-up, exactly
        args.steps device-resident calling passes replayed as a CUDA graph."""
        caller.load_tables(api.params_from_flags(flags, prec), pm, prior, rank_tab)
        caller.set_option("graphs", 0)
        kernel_ms = {}
        for i in range(3):
            caller.recall_resident()
            if i == 0:
                continue
            for li in caller.last_launches():
                key = (li["kind"], li["slots"])
                kernel_ms.setdefault(key, []).append((li["ms"], li["sites"], li["tiles"]))
        n_launch = len(caller.last_launches())
        caller.set_option("graphs", 1)
        for _ in range(args.warmup):
            caller.recall_resident()
        barrier()
        torch.cuda.synchronize()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(args.steps):
            caller.recall_resident()
        end.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms_step = max_over_ranks(start.elapsed_time(end)) / args.steps
        return {"ms_step": ms_step, "value": replica_rate(world, sites, ms_step / 1000.0), "launches": n_launch,
                "kernel_ms": kernel_ms, "stats": caller.stats()}

    compare = time_form(other) if not args.no_compare else None
    # clocks are sampled through the headline's timed steps and the e2e steps
    sampler = ClockSampler(local)
    sampler.__enter__()
    head = time_form(precision)
    value, ms_step, kernel_ms = head["value"], head["ms_step"], head["kernel_ms"]
    stats = head["stats"]

    # ---- end to end through the C ABI from pinned host buffers ----
    e2e_steps = args.e2e_steps if args.e2e_steps is not None else min(args.steps, 5)

    def e2e_run(rd):
        times = []
        for i in range(1 + e2e_steps):       # the first pass warms the pinned result buffer, untimed
            barrier()
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            caller.call_into(rd, out_pinned.data_ptr())
            torch.cuda.synchronize()
            if i > 0:
                times.append(time.perf_counter() - t1)
        # median step: the host link is shared with the other GPUs of the
        # machine, and a step that meets their traffic is reported in step_ms,
        # not averaged in
        return times, caller.transfer_bytes(), max_over_ranks(max(statistics.median(times), 1e-9))

    e2e_times, (h2d, d2h), e2e_s = e2e_run(reads_packed)
    e2e_value = replica_rate(world, sites, e2e_s)
    un_times, (h2d_u, d2h_u), un_s = e2e_run(reads)
    e2e_unpacked = {"value": replica_rate(world, sites, un_s), "unit": UNIT, "h2d_bytes_per_step": int(h2d_u),
                    "d2h_bytes_per_step": int(d2h_u), "step_ms": [round(t * 1e3, 2) for t in un_times],
                    "note": "the same call with bases and qualities as two bytes per position"}

    # ---- end to end with the cns text, the output the reference's pass writes ----
    # each step: upload and call (gsnp_call_chromosome), then the text of every
    # site formatted on the GPU, downloaded and written (gsnp_write_cns, to the
    # null device)
    text_times = []
    for i in range(1 + e2e_steps):
        barrier()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        caller.call(reads_packed)
        rc = caller.lib.gsnp_write_cns(caller.ctx, w.chr_name.encode(), os.devnull.encode())
        torch.cuda.synchronize()
        if rc != 0:
            text_times = []
            break
        if i > 0:
            text_times.append(time.perf_counter() - t1)
    e2e_text = None
    if text_times:
        h2d_t, d2h_t = caller.transfer_bytes()
        ts = max_over_ranks(statistics.median(text_times))
        e2e_text = {"value": world * sites / ts, "unit": UNIT, "h2d_bytes_per_step": int(h2d_t),
                    "d2h_bytes_per_step": int(d2h_t), "steps": e2e_steps, "stat": "median step",
                    "step_ms": [round(t * 1e3, 2) for t in text_times],
                    "note": "gsnp_call_chromosome + gsnp_write_cns (cns text of every site to the null device)"}
    sampler.__exit__(None, None, None)

    # ---- parity of the headline form at full size: the cns text of the last
    # call against the digest of the reference host code's text for the same
    # workload (tests/golden/golden_full.json), after the timed region ----
    parity = None
    try:
        gpath = os.path.join(ROOT, "tests", "golden", "golden_full.json")
        golden = json.load(open(gpath)) if os.path.exists(gpath) else {}
        cid = next((k for k, g in golden.items() if g["config"] == args.workload and not g["compress"]
                    and args.scale == g["scale"]), None)
        if cid is not None:
            import hashlib
            wd = synth.workload_digest(w) == golden[cid]["workload_sha256"]
            text = caller.format_cns(w.chr_name)
            match = hashlib.sha256(text).hexdigest() == golden[cid]["outputs"]["cns"]
            parity = {"golden": cid, "workload_digest_match": wd, "cns_digest_match": match,
                      "rows": text.count(b"\n"), "cns_rows_differing": 0 if (wd and match) else None,
                      "form": args.precision}
            del text
    except Exception as e:   # informational: never costs the bench line
        parity = {"error": repr(e)[:200]}

    # ---- the cns text of the last call (what the reference's pass writes), informational ----
    text_ms = []
    for _ in range(2):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        rc = caller.lib.gsnp_write_cns(caller.ctx, w.chr_name.encode(), os.devnull.encode())
        text_ms.append((time.perf_counter() - t1) * 1e3)
        if rc != 0:
            text_ms = []
            break

    # ---- the -C files of the last call, informational ----
    columns = None
    cdir = None
    try:
        cdir = tempfile.mkdtemp(prefix="gsnp_bench_columns_", dir=RAM_DIR)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        rc = caller.lib.gsnp_write_columns(caller.ctx, w.chr_name.encode(), os.path.join(cdir, "cns").encode())
        ms = (time.perf_counter() - t1) * 1e3
        files = [os.path.join(cdir, f) for f in os.listdir(cdir)]
        columns = ({"ms": round(ms, 2), "bytes": sum(os.path.getsize(f) for f in files), "files": len(files),
                    "note": "gsnp_write_columns of the last call: windows encoded on the GPU (the host encoder takes "
                            "any window that overflows its buffers), downloaded, the five binary files written by a "
                            "thread each, to a temporary directory (%s)" % (RAM_DIR or "the default")}
                   if rc == 0 else {"error": "gsnp_write_columns returned %d" % rc})
    except Exception as e:   # informational only: never costs the bench line
        columns = {"error": repr(e)[:200]}
    finally:
        if cdir:
            shutil.rmtree(cdir, ignore_errors=True)

    # ---- end to end in bounded device memory (gsnp_call_streamed), both forms:
    # each step uploads the alignments chunk by chunk, calls them and writes
    # every call to pinned host memory and the -C files to a temporary
    # directory; measured last, since no call stays resident after it ----
    streamed = None
    sdir = None
    try:
        sdir = tempfile.mkdtemp(prefix="gsnp_bench_streamed_", dir=RAM_DIR)
        caller.set_option("stream_windows", args.stream_windows)
        forms = {}
        for prec in (precision, other):
            caller.load_tables(api.params_from_flags(flags, prec), pm, prior, rank_tab)
            ts = []
            for i in range(1 + e2e_steps):
                barrier()
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                caller.call_streamed(reads_packed, w.chr_name, out_pinned.data_ptr(), None, os.path.join(sdir, "cns"))
                torch.cuda.synchronize()
                if i > 0:
                    ts.append(time.perf_counter() - t1)
            forms[prec] = ts
        h2d_s, d2h_s = caller.transfer_bytes()
        ring, writer = caller.stream_footprint()
        ts = max_over_ranks(statistics.median(forms[precision]))
        ts_other = max_over_ranks(statistics.median(forms[other]))
        streamed = {"value": world * sites / ts, "unit": UNIT, "h2d_bytes_per_step": int(h2d_s),
                    "d2h_bytes_per_step": int(d2h_s), "steps": e2e_steps, "stat": "median step",
                    "step_ms": [round(t * 1e3, 2) for t in forms[precision]],
                    "other_form": {"form": "fp64 plain" if other == api.PRECISION_FP64 else "fp32+fp64 fixup",
                                   "value": world * sites / ts_other,
                                   "step_ms": [round(t * 1e3, 2) for t in forms[other]]},
                    "stream_windows": args.stream_windows,
                    "device_ring_bytes": ring, "columns_writer_bytes": writer,
                    "per_site_resident_bytes": 1 + 4 / 32,
                    "note": "gsnp_call_streamed: chunks of stream_windows windows through a two-slot device ring "
                            "(alignments of the chunk being uploaded and of the one being called, its calls); "
                            "outputs: every call to pinned host memory and the six -C files"}
    except Exception as e:   # informational: never costs the bench line
        streamed = {"error": repr(e)[:200]}
    finally:
        if sdir:
            shutil.rmtree(sdir, ignore_errors=True)

    # ---- roofline of the dominant kernel (the calling launch with most device time) ----
    peaks, peak_kind = load_peaks()
    bsite = site_bytes(w)
    names = {1: "call_tiles_kernel", 2: "call_fast_kernel", 3: "deferred_sites_kernel", 4: "call_stream_kernel",
             5: "graph", 6: "call_deep_kernel"}
    dom_key = max((k for k in kernel_ms if k[0] in (1, 2, 4, 6)), key=lambda k: sum(x[0] for x in kernel_ms[k]))
    dom = kernel_ms[dom_key]
    dom_ms = statistics.mean(x[0] for x in dom)
    dom_sites = dom[0][1]
    achieved = bsite * dom_sites / (dom_ms / 1000.0) / 1e9
    peak = float(peaks.get("hbm_gbs", 6800.0))

    def kernel_table(km):
        def name(k):
            if k[0] == 0:
                return "classify"
            return names[k[0]] if k[0] == 3 else "%s<%d>" % (names[k[0]], k[1])
        return {name(k): round(statistics.mean(x[0] for x in v), 4) for k, v in sorted(km.items())}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cv, sample = cpu_baseline(1_200_000 if args.scale >= 1.0 else max(40_000, int(1_200_000 * args.scale)),
                                      args.workload)
            cpu = {"value": cv, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample}
        except Exception as exc:  # the baseline is reported, not required
            cpu = {"value": None, "unit": UNIT, "cores": 1, "kind": "port", "sample": "failed: %s" % exc}

    if rank == 0:
        depth = w.num_bases / sites
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if precision == api.PRECISION_FP64 else "f32+f64",
            "data": "synthetic (seeded generator of the %s shape, generated on the GPU in %.1f s)" % (args.workload, t_gen),
            "config": {"workload": WORKLOADS[args.workload] + "; scale %.3g" % args.scale,
                       "sites": sites, "reads": w.num_reads, "bases": w.num_bases, "mean_depth": depth,
                       "precision": args.precision, "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs (3 GB of alignments) exceed the 129 MB L2; no flush"},
            "bases_per_s": value * depth,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "steps": e2e_steps, "stat": "median step",
                    "step_ms": [round(t * 1e3, 2) for t in e2e_times],
                    "input": "packed reads (base and quality in one byte per position)",
                    "pack_ms": round(pack_ms, 1)},
            "e2e_unpacked": e2e_unpacked,
            "e2e_text": e2e_text,
            "e2e_streamed": streamed,
            "cns_parity": parity,
            "cns_text": ({"ms": round(min(text_ms), 2), "rows": sites,
                          "note": "gsnp_write_cns of the last call to the null device: GPU formatting, download, write"}
                         if text_ms else None),
            "cns_columns": columns,
            "gpu_launches": head["launches"] * args.steps,
            "kernels_ms": kernel_table(kernel_ms),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": (round(NCU_BYTES_PER_SITE[(args.workload,) + dom_key] * dom_sites)
                                     if (args.workload,) + dom_key in NCU_BYTES_PER_SITE else None),
                         "kernel": "%s<%d>" % (names[dom_key[0]], dom_key[1]), "sites_per_launch": dom_sites,
                         "bytes_per_site": bsite, "peak_source": peak_kind},
            "tuning": tuning,
            "cpu_baseline": cpu,
            "clocks": sampler.summary(),
            "stats": stats,
        }
        if compare is not None:
            line["compare"] = {
                "form": "fp64 plain" if other == api.PRECISION_FP64 else "fp32+fp64 fixup",
                "value": compare["value"], "ms_per_step": compare["ms_step"],
                "bases_per_s": compare["value"] * depth, "kernels_ms": kernel_table(compare["kernel_ms"]),
                "speedup_of_headline": value / compare["value"]}
        print(json.dumps(line), flush=True)
    caller.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
