#!/usr/bin/env python3
"""Aligned reads/s of strobealign's mapping path on GB300, with bit-exact SAM.

Default workload (--workload human): a 3.1 Gbp synthetic genome in 24 contigs (GC 41%,
50% interspersed repeats from 300 bp-6 kbp families at 10-20% divergence, 3% tandem
repeats of period 2-50) and 10M read pairs of 2x150 bp, insert N(400, 50), 1%
substitutions, 0.1% indels.  Other shapes: pe50m (50 Mbp, 10% segmental copies, 1M
pairs with mate rescue), se5m (5 Mbp, 100k single-end 150 bp), uneven200m (200 Mbp,
20% repeats, 2M single-end reads of 50-500 bp).  Seeded generators
(strobealign_gb300.synthetic) stand in for the reference's read sets.

One step maps the whole batch: NAM finding, SSW-exact (paired-end / --ssw) or piecewise
(single-end) extension waves and SAM record formatting, chunked as the reference chunks
its input.
  value   the batched engine (continuous batching, overlapped NAM parts) with the reads
          resident in device memory (sa_map_uploaded)
  e2e     the served form: the same reads as a stream of requests (log-uniform 1..100k
          pairs) through sa_session submit/wait from host buffers
  plain   the plain, stage-synchronous GPU form (sa_mapper_set_schedule overlap = 0)
          from host buffers, beside the batched engine from host buffers
An open-loop pass at 70% of the served capacity gives p50/p99 request latency.

Parity leg (--parity full, the default): after the timed passes the batch is mapped once
more and its SAM bytes are compared with the oracle's (the CPU restatement of the
reference path) on the whole batch, and the GPU-built index with the oracle's; the
oracle's run is also the CPU baseline (all host threads).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload W]

Under torchrun each rank maps its own replica of the workload (no data exchange:
chunks are independent), and rank 0 prints one JSON line with the aggregate rate
over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "aligned reads/s on 1 GB300 (bit-exact SAM), served vs plain; p50/p99 latency"

# Synthetic stand-ins for the reference's benchmark shapes (seeded generators in
# strobealign_gb300/synthetic.py; genome seeds 1..4, read seeds 101..104).
WORKLOADS = {
    "human": "human scale: 3.1 Gbp / 24 contigs (GC 41%, 50% interspersed repeats from 300 bp-6 kbp families at "
             "10-20% divergence, 3% tandem repeats of period 2-50), 10M pairs 2x150 bp, insert N(400,50), 1% sub, "
             "0.1% indel",
    "pe50m": "paired-end repetitive: 50 Mbp / 20 contigs (GC 41%, 10% 2 kbp segmental copies at 2%), "
             "1M pairs 2x150 bp, insert N(300,30), 1% sub, 0.1% indel, 2% of pairs need mate rescue",
    "se5m": "plain small: 5 Mbp uniform / 1 contig, 100k single-end 150 bp, 1% sub, 0.1% indel",
    "uneven200m": "uneven lengths: 200 Mbp / 8 contigs (GC 41%, 20% repeats from 300 bp-6 kbp families at "
                  "10-20% divergence), 2M single-end reads U[50,500] bp, 1.5% sub, 0.2% indel",
}
DEFAULT_WORKLOAD = "human"


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of the workload (1.0 = full)")
    ap.add_argument("--pairs", type=int, default=0, help="override the read (pair) count")
    ap.add_argument("--ssw", action="store_true", help="single-end extension by SSW (--ssw) instead of piecewise")
    ap.add_argument("--parity", default="full", choices=["full", "off"],
                    help="compare the whole batch's SAM (and the index) with the oracle's")
    ap.add_argument("--cpu-sample-pairs", type=int, default=0,
                    help="reference arm: records per step (0 = four 1 Mnt chunks per host thread)")
    ap.add_argument("--aux-steps", type=int, default=3, help="steps of the plain and batched host-buffer passes")
    ap.add_argument("--no-served", action="store_true", help="skip the served and latency passes (profiling runs)")
    ap.add_argument("--stream-pairs", type=int, default=2_000_000,
                    help="records of the file-to-file leg (FASTQ and FASTQ.gz through sa_map_files); 0: skip")
    ap.add_argument("--tune", type=int, default=1, help="1: autotune the mapper on a calibration sample first")
    ap.add_argument("--tune-records", type=int, default=0,
                    help="records in the calibration sample (0: the whole batch; the best knobs depend on its size)")
    return ap.parse_args(argv)


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload(scale: float, name: str = DEFAULT_WORKLOAD, pairs: int = 0):
    """(genome, reads 1, reads 2 or None, read length for the seeding preset)"""
    from strobealign_gb300 import synthetic as syn
    if name == "se5m":
        g = syn.make_genome(1, int(5_000_000 * scale), 1, gc=0.5)
        r = syn.make_single_end(101, g, pairs or int(100_000 * scale), 150, 0.01, 0.001)
        return g, r, None, 150
    if name == "uneven200m":
        g = syn.make_genome(3, int(200_000_000 * scale), 8, gc=0.41, repeat_fraction=0.20, family_len=(300, 6000),
                            family_div=(0.10, 0.20))
        r = syn.make_single_end(103, g, pairs or int(2_000_000 * scale), (50, 500), 0.015, 0.002)
        n = min(500, len(r))
        return g, r, None, int(r.offsets[n] // n) if n else 150  # read length estimated like the reference
    if name == "human":
        g = syn.make_genome(4, int(3_100_000_000 * scale), 24, gc=0.41, repeat_fraction=0.50, family_len=(300, 6000),
                            family_div=(0.10, 0.20), tandem_fraction=0.03)
        r1, r2 = syn.make_paired_end(104, g, pairs or int(10_000_000 * scale), 150, 400, 50, 0.01, 0.001)
        return g, r1, r2, 150
    g = syn.make_genome(2, int(50_000_000 * scale), 20, gc=0.41, segdup_fraction=0.10, segdup_len=2000,
                        segdup_div=0.02)
    r1, r2 = syn.make_paired_end(102, g, pairs or int(1_000_000 * scale), 150, 300, 30, 0.01, 0.001,
                                 rescue_fraction=0.02)
    return g, r1, r2, 150


def host_cpu() -> dict:
    """Host cores as nproc and lscpu report them."""
    info = {"nproc": os.cpu_count(), "machine": platform.machine()}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            k, _, v = line.partition(":")
            if k.strip() in ("Model name", "CPU(s)", "Thread(s) per core"):
                info[k.strip()] = v.strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return info


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.f = None

    def __enter__(self):
        try:
            self.f = tempfile.TemporaryFile(mode="w+")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if not self.f:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _prefix(rs, n: int):
    """The first n records of a ReadSet (views, no copy of the bases)."""
    from strobealign_gb300 import synthetic as syn
    o, no = rs.offsets, rs.name_offsets
    return syn.ReadSet(rs.seq[:int(o[n])], o[:n + 1], rs.names[:int(no[n])], no[:n + 1],
                       rs.qual[:int(o[n])] if rs.qual is not None else None)


def _slice(rs, a: int, b: int):
    """Records [a, b) of a ReadSet with offsets starting at 0."""
    from strobealign_gb300 import synthetic as syn
    o, no = rs.offsets, rs.name_offsets
    return syn.ReadSet(rs.seq[int(o[a]):int(o[b])], o[a:b + 1] - o[a], rs.names[int(no[a]):int(no[b])],
                       no[a:b + 1] - no[a], rs.qual[int(o[a]):int(o[b])] if rs.qual is not None else None)


def _calib(rs, n: int):
    """Reads.from_arrays arguments for the first n records of a ReadSet."""
    p = _prefix(rs, n)
    return p.seq, p.offsets, p.names, p.name_offsets, p.qual


def oracle_index(g, read_length: int, threads: int):
    """The oracle's make_index over the workload's genome (all host threads)."""
    from oracle.binding import OracleIndex
    return OracleIndex(g.names, g.seqs, read_length, threads=threads)


def chunk_records(rs, rs2, chunks: int, chunk_size: int = 1_000_000) -> int:
    """Records that make `chunks` of the reference's chunks (src/main.rs:591-604)."""
    import numpy as np
    lens = np.diff(rs.offsets).astype(np.int64)
    if rs2 is not None:
        lens = lens + np.diff(rs2.offsets).astype(np.int64)
    n, i = len(lens), 0
    c = np.cumsum(lens)
    for _ in range(chunks):
        if i >= n:
            break
        base = c[i - 1] if i else 0
        j = int(np.searchsorted(c, base + chunk_size, side="right"))  # first record past the limit
        i = min(n, j + 1)
    return i


def run_reference(args, ws, rank):
    """The reference arm: the oracle (the CPU restatement of the reference's path; the
    Rust crate cannot be built here) on the host cores, index built once, each step a
    bounded sample of the same workload of at least four 1 Mnt chunks per thread."""
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    g, r1, r2, rl = workload(args.scale, args.workload, args.pairs)
    idx = oracle_index(g, rl, threads)
    n = len(r1)
    per = args.cpu_sample_pairs or chunk_records(r1, r2, 4 * threads)
    per = max(1, min(per, n))
    use_ssw = bool(args.ssw)

    def step(i: int, m: int, th: int):
        a = (i * m) % max(1, n - m + 1)
        x1 = _slice(r1, a, a + m)
        x2 = _slice(r2, a, a + m) if r2 is not None else None
        _, sec = idx.map_batch(x1, x2, threads=th, use_ssw=use_ssw)
        return sec

    for w in range(args.warmup):
        step(w, min(per, 2000), threads)
    secs = [step(i, per, threads) for i in range(args.steps)]
    reads = per * (2 if r2 is not None else 1)
    value = reads / statistics.median(secs)
    # one chunk's worth on a single thread (the per-core rate)
    one = chunk_records(r1, r2, 1)
    t1 = reads_1 = None
    if one:
        t1 = step(0, one, 1)
        reads_1 = one * (2 if r2 is not None else 1)
    cpu = host_cpu()
    out = {"metric": METRIC, "value": value, "unit": "reads/s", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1000 * statistics.median(secs), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
           "impl": "reference",
           "config": {"workload": WORKLOADS[args.workload], "scale": args.scale, "pairs_per_step": per,
                      "ssw": use_ssw},
           "cpu_baseline": {"value": value, "unit": "reads/s", "cores": threads, "kind": "port",
                            "sample": f"{per} {'pairs' if r2 is not None else 'reads'} per step (at least four "
                                      f"1 Mnt chunks per thread), records rotating through the batch; index built "
                                      f"once ({idx.build_seconds:.1f} s); the Rust reference cannot be built here "
                                      f"(no cargo), the oracle restates its CPU path",
                            "single_thread": None if t1 is None else
                            {"value": reads_1 / t1, "unit": "reads/s", "cores": 1,
                             "sample": f"one 1 Mnt chunk ({one} records)"},
                            "host": cpu},
           "e2e": {"value": value, "unit": "reads/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    return out


def parity_leg(g, r1, r2, rl, idx, gpu_sam: bytes, use_ssw: bool, threads: int) -> tuple[dict, dict]:
    """The whole batch through the oracle: SAM bytes and the index compared with the
    GPU's; the oracle's mapping time is the CPU baseline on all host threads."""
    import numpy as np
    t0 = time.perf_counter()
    o = oracle_index(g, rl, threads)
    n, bits, cutoff = o.info()
    ot, od = o.arrays()
    gt, gd = idx.to_host()
    index_same = (bits == idx.bits and cutoff == idx.filter_cutoff and n == len(gt) and
                  bool(np.array_equal(gd, od)) and bool(np.array_equal(gt.view(np.uint8), ot.view(np.uint8))))
    del gt, gd
    want, sec = o.map_batch(r1, r2, threads=threads, use_ssw=use_ssw, eqx=False)
    same = want == gpu_sam
    first = None
    if not same:
        a = np.frombuffer(gpu_sam, np.uint8)
        b = np.frombuffer(want, np.uint8)
        m = min(len(a), len(b))
        k = int(np.argmax(a[:m] != b[:m])) if m and (a[:m] != b[:m]).any() else m
        line = int(np.count_nonzero(a[:k] == 10))
        lo = gpu_sam.rfind(b"\n", 0, k) + 1
        first = {"byte": k, "line": line, "gpu": gpu_sam[lo:gpu_sam.find(b"\n", k)][:300].decode(errors="replace"),
                 "oracle": want[lo:want.find(b"\n", k)][:300].decode(errors="replace")}
    reads = len(r1) * (2 if r2 is not None else 1)
    # the lookup roofline's algorithmic bytes: distinct 32-byte index sectors the
    # reference's lookups read per read, counted by the oracle on a sample
    m = min(len(r1), 20000)
    cnt = [o.lookup_sectors(_prefix(x, m)) for x in (r1, r2) if x is not None]
    sectors = {"sample_reads": sum(x["reads"] for x in cnt), "dir_sectors": sum(x["dir_sectors"] for x in cnt),
               "table_sectors": sum(x["table_sectors"] for x in cnt),
               "randstrobes": sum(x["randstrobes"] for x in cnt)}
    parity = {"reads": reads, "records": len(r1), "sam_bytes": len(gpu_sam), "identical": same, "first_diff": first,
              "lookup_sectors": sectors,
              "index_identical": index_same, "index": {"bits": bits, "filter_cutoff": cutoff, "randstrobes": n},
              "oracle_index_s": round(o.build_seconds, 2), "oracle_map_s": round(sec, 2),
              "leg_s": round(time.perf_counter() - t0, 1)}
    cpu = {"value": reads / sec, "unit": "reads/s", "cores": threads, "kind": "port",
           "sample": f"the whole batch ({len(r1)} {'pairs' if r2 is not None else 'reads'}), index build excluded "
                     f"({o.build_seconds:.1f} s on {threads} threads); the oracle restates the reference's CPU path",
           "seconds": sec, "host": host_cpu()}
    # one chunk on one thread
    one = chunk_records(r1, r2, 1)
    if one:
        x1 = _prefix(r1, one)
        x2 = _prefix(r2, one) if r2 is not None else None
        _, s1 = o.map_batch(x1, x2, threads=1, use_ssw=use_ssw)
        cpu["single_thread"] = {"value": one * (2 if r2 is not None else 1) / s1, "unit": "reads/s", "cores": 1,
                                "sample": f"one 1 Mnt chunk ({one} records)"}
    return parity, cpu


def stream_leg(sa, mapper, refs, r1, r2, pairs: int) -> dict:
    """File to file: the first `pairs` records written as FASTQ (and gzip level 1), then
    mapped into a SAM file by sa_map_files (parsing, mapping and writing overlapped);
    the file's bytes are checked against the SAM header plus sa_map_batch's output for
    the same records."""
    import gzip
    import hashlib
    import shutil
    import threading
    n = min(pairs, len(r1))
    d = tempfile.mkdtemp(prefix="sa_stream_")
    try:
        files = [os.path.join(d, "r1.fq")] + ([os.path.join(d, "r2.fq")] if r2 is not None else [])
        sets = [_prefix(r1, n)] + ([_prefix(r2, n)] if r2 is not None else [])
        t = time.time()
        for f, rs in zip(files, sets):
            rs.write_fastq(f)

        def gz(src):
            with open(src, "rb") as fi, gzip.open(src + ".gz", "wb", compresslevel=1) as fo:
                shutil.copyfileobj(fi, fo, 16 << 20)
        ths = [threading.Thread(target=gz, args=(f,)) for f in files]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        write_s = time.time() - t
        c1 = sa.Reads.from_arrays(*_calib(r1, n))
        c2 = sa.Reads.from_arrays(*_calib(r2, n)) if r2 is not None else None
        hdr = sa.sam_header(refs)
        want = hashlib.sha256(hdr + mapper.map(c1, c2)).hexdigest()
        del c1, c2
        out = {"records": n, "input_bytes": {"plain": sum(os.path.getsize(f) for f in files),
                                             "gzip": sum(os.path.getsize(f + ".gz") for f in files)},
               "write_inputs_s": round(write_s, 1), "unit": "reads/s"}
        for kind, ext in (("plain", ""), ("gzip", ".gz")):
            o = os.path.join(d, "out.sam")
            t = time.time()
            st = mapper.map_files(files[0] + ext, files[1] + ext if len(files) > 1 else None, o, header=hdr)
            sec = time.time() - t
            h = hashlib.sha256()
            with open(o, "rb") as f:
                for blk in iter(lambda: f.read(64 << 20), b""):
                    h.update(blk)
            os.remove(o)
            out[kind] = {"reads_per_s": st["n_reads"] / sec, "seconds": round(sec, 3),
                         "seconds_map": round(st["seconds_map"], 3),
                         "seconds_wait_input": round(st["seconds_wait_input"], 3), "batches": st["n_batches"],
                         "sam_bytes": st["bytes_out"], "identical": h.hexdigest() == want}
        return out
    finally:
        shutil.rmtree(d, ignore_errors=True)


def slowest_rank(pg, seconds: float, device: str = "cpu") -> float:
    """Max over ranks of a rank's wall time (the job's time); identity without a process group."""
    if pg is None:
        return seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def request_sizes(n_pairs: int, seed: int = 105, lo: int = 1, hi: int = 100_000) -> list[int]:
    """Request sizes in pairs, log-uniform in [lo, hi], covering the workload's pairs in order."""
    import numpy as np
    rng = np.random.default_rng(seed)
    sizes, total = [], 0
    while total < n_pairs:
        s = int(np.exp(rng.uniform(np.log(lo), np.log(hi + 1))))
        s = max(lo, min(s, n_pairs - total))
        sizes.append(s)
        total += s
    return sizes


def slice_reads(sa, rs, a: int, b: int):
    o, no = rs.offsets, rs.name_offsets
    return sa.Reads.from_arrays(rs.seq[o[a]:o[b]], o[a:b + 1] - o[a], rs.names[no[a]:no[b]], no[a:b + 1] - no[a],
                                rs.qual[o[a]:o[b]] if rs.qual is not None else None)


def served_pass(session, reqs) -> tuple[float, list[dict]]:
    """Submit every request at once (saturating load) and wait for all."""
    t0 = time.perf_counter()
    tickets = [session.submit(a, b) for a, b in reqs]
    stats = [session.wait(t, copy=False)[1] for t in tickets]
    return time.perf_counter() - t0, stats


def latency_pass(session, reqs, rate: float, n: int, seed: int = 5) -> dict:
    """Open loop: n requests with Poisson arrivals at `rate` per second."""
    import queue
    import threading

    import numpy as np
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
    q: queue.Queue = queue.Queue()
    t0 = time.perf_counter()

    def submitter():
        for i, a in enumerate(arrivals):
            d = t0 + a - time.perf_counter()
            if d > 0:
                time.sleep(d)
            x, y = reqs[i % len(reqs)]
            q.put((session.submit(x, y), i))

    th = threading.Thread(target=submitter)
    th.start()
    lat, reads = [], 0
    for _ in range(n):
        t, i = q.get()
        _, st = session.wait(t, copy=False)
        lat.append(st["seconds_total"])
        reads += st["n_reads"]
    th.join()
    wall = time.perf_counter() - t0
    lat = np.array(lat)
    return {"requests": n, "offered_requests_per_s": rate, "p50_ms": 1000 * float(np.percentile(lat, 50)),
            "p99_ms": 1000 * float(np.percentile(lat, 99)), "mean_ms": 1000 * float(lat.mean()),
            "reads_per_s": reads / wall}


def main():
    args = parse()
    ws, rank, local = dist_info()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    import torch
    torch.cuda.set_device(local)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist
    import strobealign_gb300 as sa

    # the device's integer instruction rate: the Smith-Waterman rooflines' denominator
    alu = sa.measure_int_alu()
    t = time.time()
    g, r1, r2, read_length = workload(args.scale, args.workload, args.pairs)
    gen_s = time.time() - t
    single_end = r2 is None
    use_ssw = bool(args.ssw) and single_end
    refs = sa.References.from_sequences(g.names, [s.tobytes() for s in g.seqs])
    params = sa.SeedingParameters.from_read_length(read_length)
    t = time.time()
    index = sa.StrobemerIndex.build(refs, params)
    torch.cuda.synchronize()
    index_s = time.time() - t
    R1 = sa.Reads.from_arrays(r1.seq, r1.offsets, r1.names, r1.name_offsets, r1.qual)
    R2 = sa.Reads.from_arrays(r2.seq, r2.offsets, r2.names, r2.name_offsets, r2.qual) if r2 is not None else None
    n_reads = (2 if r2 is not None else 1) * len(R1)
    mapper = sa.Mapper(index, refs, use_ssw=1 if use_ssw else 0)
    # the autotuner on a calibration sample of the workload (output-invariant knobs);
    # its choice stays in the mapper for the timed passes
    tune = None
    if args.tune:
        m = min(len(R1), args.tune_records or len(R1))
        c1 = sa.Reads.from_arrays(*_calib(r1, m)) if m < len(R1) else R1
        c2 = (sa.Reads.from_arrays(*_calib(r2, m)) if m < len(R1) else R2) if r2 is not None else None
        t0 = time.time()
        tune = mapper.autotune(c1, c2, rounds=1 if m == len(R1) else 2)
        calib_reads = m * (2 if r2 is not None else 1)
        tune.update(sample_records=m, tune_s=round(time.time() - t0, 1),
                    default_reads_per_s=calib_reads / tune["seconds_default"],
                    tuned_reads_per_s=calib_reads / tune["seconds_tuned"])
    mapper.upload(R1, R2)

    def barrier():
        torch.cuda.synchronize()
        if pg:
            pg.barrier()

    for _ in range(max(3, args.warmup)):
        mapper.map_uploaded(copy=False)
    # timed region: the batched engine, reads resident in device memory
    # timed region: the stage timers stay off (their events would perturb the overlap of
    # the two streams); the same maps run again with them on below for the rooflines
    kern = {}
    cells = {}
    phases = {}
    launches = 0
    waves = []
    barrier()
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        ev0.record(stream)
        for _ in range(args.steps):
            out = mapper.map_uploaded(copy=False)
            st = mapper.stats()
            launches += int(st["n_launches"])
            waves.append(int(st["n_waves"]))
            for k in ("seconds_nams", "seconds_extension", "seconds_policy"):
                phases[k] = phases.get(k, 0.0) + st[k] / args.steps
            for k, v in st["sw_cells"].items():
                cells[k] = cells.get(k, 0) + int(v)
        ev1.record(stream)
        barrier()
        wall = time.perf_counter() - t0
        # the stage timers (CUDA events on each stage's stream) over the same maps
        mapper.set_profiling(True)
        barrier()
        tp = time.perf_counter()
        for _ in range(args.steps):
            mapper.map_uploaded(copy=False)
            st = mapper.stats()
            for k, v in st["kernel_ms"].items():
                kern.setdefault(k, [0.0, 0])
                kern[k][0] += v
                kern[k][1] += int(st["kernel_launches"][k])
        barrier()
        profiled_s = time.perf_counter() - tp
        mapper.set_profiling(False)
    ev_ms = ev0.elapsed_time(ev1)
    elapsed = max(wall, ev_ms / 1000.0)
    elapsed = slowest_rank(pg, elapsed, "cuda")
    value = ws * n_reads * args.steps / elapsed
    sam_bytes = int(out)
    aux = max(1, min(args.steps, args.aux_steps))

    def host_pass(steps: int):
        """Whole batch from host buffers through sa_map_batch: (rate, h2d, d2h)."""
        h2d = d2h = 0
        barrier()
        t0 = time.perf_counter()
        for _ in range(steps):
            mapper.map(R1, R2, copy=False)
            st = mapper.stats()
            h2d, d2h = int(st["h2d_bytes"]), int(st["d2h_bytes"])
        barrier()
        sec = slowest_rank(pg, time.perf_counter() - t0, "cuda")
        return ws * n_reads * steps / sec, h2d, d2h, int(st["n_waves"]), int(st["n_launches"])

    # the batched engine from host buffers, then the plain stage-synchronous form
    batched_e2e, b_h2d, b_d2h, _, _ = host_pass(aux)
    mapper.set_schedule(overlap=False)
    mapper.map(R1, R2, copy=False)  # warm-up of the plain form
    plain_e2e, plain_h2d, plain_d2h, plain_waves, plain_launches = host_pass(aux)
    # one more plain map with the stage timers on: in the plain form no NAM part runs
    # beside the extension waves, so these are each kernel's times alone on the GPU
    mapper.set_profiling(True)
    mapper.map(R1, R2, copy=False)
    st_iso = mapper.stats()
    mapper.set_profiling(False)
    kern_iso = {k: [v, int(st_iso["kernel_launches"][k])] for k, v in st_iso["kernel_ms"].items()}
    cells_iso = {k: int(v) for k, v in st_iso["sw_cells"].items()}
    counts_iso = {k: int(st_iso[k]) for k in ("n_bases", "n_randstrobes", "n_anchor_total")}
    mapper.set_schedule()
    # served: the same records as a stream of requests (log-uniform 1..100k pairs), each
    # its own chunk stream, through one session with continuous batching
    reqs, lat = [], None
    served = s_h2d = s_d2h = None
    if not args.no_served:
        sizes = request_sizes(len(R1))
        a = 0
        for n in sizes:
            reqs.append((slice_reads(sa, r1, a, a + n), slice_reads(sa, r2, a, a + n) if r2 is not None else None))
            a += n
        session = sa.Session(index, refs, use_ssw=1 if use_ssw else 0)
        served_pass(session, reqs)  # warm-up: arena, workspaces
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            _, sst = served_pass(session, reqs)
            s_h2d = sum(int(x["h2d_bytes"]) for x in sst)
            s_d2h = sum(int(x["d2h_bytes"]) for x in sst)
        barrier()
        served_s = time.perf_counter() - t0
        served_s = slowest_rank(pg, served_s, "cuda")
        served = ws * n_reads * args.steps / served_s
        cap_rps = len(reqs) * args.steps / served_s
        lat = latency_pass(session, reqs, 0.7 * cap_rps, max(60, min(400, int(3 * 0.7 * cap_rps))))
        session.close()
    e2e = served if served is not None else batched_e2e
    if served is None:
        s_h2d, s_d2h = b_h2d, b_d2h
    # parity: the batch once more, its bytes against the oracle's (rank 0 only)
    parity = cpu = None
    if rank == 0 and args.parity == "full":
        try:
            gpu_sam = mapper.map_uploaded(copy=True)
            parity, cpu = parity_leg(g, r1, r2, read_length, index, gpu_sam, use_ssw, os.cpu_count() or 1)
            del gpu_sam
        except Exception as e:  # reported, never fatal for the GPU line
            parity = {"identical": None, "error": f"{type(e).__name__}: {str(e)[:300]}"}
    stream = None
    if rank == 0 and args.stream_pairs:
        try:
            stream = stream_leg(sa, mapper, refs, r1, r2, args.stream_pairs)
        except Exception as e:  # reported, never fatal for the GPU line
            stream = {"error": f"{type(e).__name__}: {str(e)[:300]}"}
    if rank != 0:
        pg.destroy_process_group()
        return
    # roofline of the dominant stage, from the CUDA-event times of the timed steps
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    total_ms = sum(v[0] for v in kern.values())
    # the headline roofline: the slowest of the stages with a roofline model (seeding:
    # bytes, lookups: random sectors, extension: SW cells); chaining, sorting and the
    # anchor walk are reported as rates (their bound is issue / latency, not HBM)
    modelled = {k: v for k, v in kern.items() if k in ("seed", "hits", "sw_byte")}
    dom = max(modelled, key=lambda k: modelled[k][0]) if modelled else None
    shares = {k: round(v[0] / total_ms, 4) for k, v in kern.items() if total_ms and v[0] > 0}
    counts = {k: int(st[k]) for k in ("n_bases", "n_randstrobes", "n_anchor_total")}
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    lookup = (parity or {}).get("lookup_sectors")
    roofline, rooflines = roofline_for(dom, kern, cells, peaks, clk.summary(), counts, args.steps, sms, n_reads,
                                       lookup, alu) if dom else (None, {})
    _, rooflines_iso = roofline_for(dom, kern_iso, cells_iso, peaks, clk.summary(), counts_iso, 1, sms, n_reads,
                                    lookup, alu) if dom else (None, {})
    reads_gb = int(R1.seq_offsets[-1]) * (2 if R2 is not None else 1) / 1e9
    out = {
        "metric": METRIC, "value": value, "unit": "reads/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": 1000 * elapsed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload], "scale": args.scale, "reads_per_step": n_reads,
                   "extension": "ssw" if (use_ssw or not single_end) else "piecewise",
                   "l2": f"no flush: index {index.info.device_bytes / 1e6:.0f} MB + reads {reads_gb * 1e3:.0f} MB "
                         f"exceed the 129 MB L2",
                   "value_form": "batched engine: the whole batch through sa_map_uploaded, reads resident on the "
                                 "device, NAM parts overlapped with the policy and extension waves",
                   "e2e_form": "served: the same records as requests of log-uniform 1..100k pairs through "
                               "sa_session submit/wait from host buffers, continuous batching",
                   "stream_form": "file to file: the first stream-pairs records as FASTQ and as FASTQ.gz (level 1) "
                                  "mapped into a SAM file by sa_map_files (reader, mapper and writer threads "
                                  "overlapped), bytes checked against sa_map_batch",
                   "plain_form": "stage-synchronous: sa_map_batch from host buffers with overlap = 0 (NAM parts "
                                 "one after another, then policy and extension waves taking turns)",
                   "aux_steps": aux, "requests_per_step": len(reqs), "sam_bytes_per_step": sam_bytes,
                   "index_build_s": round(index_s, 3), "generate_s": round(gen_s, 1),
                   "waves_per_step": waves},
        "e2e": {"value": e2e, "unit": "reads/s", "h2d_bytes_per_step": s_h2d, "d2h_bytes_per_step": s_d2h},
        "parity": parity,
        "plain": {"e2e": plain_e2e, "unit": "reads/s", "h2d_bytes_per_step": plain_h2d,
                  "d2h_bytes_per_step": plain_d2h, "waves": plain_waves, "launches": plain_launches},
        "batched": {"value_resident": value, "e2e": batched_e2e, "unit": "reads/s", "h2d_bytes_per_step": b_h2d,
                    "d2h_bytes_per_step": b_d2h},
        "served": None if served is None else {"value": served, "unit": "reads/s",
                                               "vs_plain_e2e": served / plain_e2e,
                                               "vs_batched_e2e": served / batched_e2e,
                                               "latency_open_loop": lat},
        "gpu_launches": launches,
        "profiled_ms_per_step": 1000 * profiled_s / args.steps,
        "stream": stream,
        "tuning": tune,
        "stage_share": shares,
        # wall seconds per step: NAM pipeline (GPU), extension waves (GPU, incl. job
        # upload and result download), host policy between and after waves
        "phases_s": {k.replace("seconds_", ""): round(v, 4) for k, v in phases.items()},
        "roofline": roofline,
        "rooflines": rooflines,
        # the same stages timed in one plain (stage-synchronous) map, each kernel alone on
        # the GPU: the kernels' own rates, without the NAM stream sharing the SMs
        "rooflines_isolated": rooflines_iso,
        "int_alu": alu,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
    }
    print(json.dumps(out), flush=True)
    if pg:
        pg.destroy_process_group()


# Algorithmic (compulsory) bytes per unit of the NAM stages: what the reference's
# algorithm must read or write at least once, whatever the implementation.
ALGO_BYTES = {
    # read bases in; per randstrobe out: hash, reverse-complement hash, start, end
    "seed": lambda c: c["n_bases"] + 24 * c["n_randstrobes"],
}
# DRAM bytes (read + write) the kernels moved in one ncu capture of the human-shaped
# workload at 1/10 scale (profiles/dram_traffic_nam_and_extension_kernels_human_scale0.1.md),
# per unit of work; a full-scale launch's traffic is this times the units it processes
# (the kernels touch the index at random, so the bytes grow with the reads).
NCU_DRAM = {
    "lookup": (24.8e3, "read"),     # k_probe 11.8 KB + k_anchors (two passes) 11.2 KB + k_hits 1.7 KB
    "seed": (2.46e3, "read"),       # k_seed: 349 MB read + 882 MB written per 500k reads
    "sw": (0.012, "canonical cell"),  # k_ssw_wave: 8.9 MB per launch of 7.4e8 canonical cells
}
NCU_DRAM_SOURCE = "ncu dram__bytes_read.sum + dram__bytes_write.sum, 1/10-scale capture, scaled by units per launch"
# stages reported as anchors per second (no HBM or ALU roofline model)
ANCHOR_RATE = ("sort", "chain")


def roofline_for(dom, kern, cells, peaks, clocks, counts, steps, sms, n_reads, lookup=None, alu=None) -> dict:
    """Roofline of every timed stage, and of the dominant one.

    Seeding is framed against HBM bandwidth with its algorithmic bytes per launch
    (ALGO_BYTES, from the batch's counts).  The index lookups (the probe, hit and anchor
    kernels) are framed against HBM random 32-byte sectors: their algorithmic bytes are
    the distinct index sectors the reference's lookups read per read (the oracle counts
    them on a sample of the batch, `lookup`), 32 bytes each; without the sample, 64
    bytes per randstrobe.  The anchor sort and chaining are reported as anchors per
    second.  Extension (the SSW kernels: byte pass, word passes of the byte overflows,
    reverse passes) is integer-ALU bound: its unit is one SSW call of |query| x
    |reference window| canonical cells, against SMs x 128 INT32 lanes x SM clock / 11
    ops per cell; the cells the passes actually computed are reported beside it."""
    hbm = peaks.get("hbm_gbs", 6800.0)
    out = {}
    lk = [kern.get(k, [0.0, 0]) for k in ("hits", "anchors")]
    if lk[0][1]:
        ms = lk[0][0] + lk[1][0]
        if lookup and lookup.get("sample_reads"):
            per_read = 32.0 * (lookup["dir_sectors"] + lookup["table_sectors"]) / lookup["sample_reads"]
            model = (f"{per_read / 32:.1f} distinct 32-byte index sectors per read (oracle count over "
                     f"{lookup['sample_reads']} reads of the batch) x 32 B")
        else:
            per_read = 64.0 * counts["n_randstrobes"] / max(1, n_reads)
            model = "64 B per randstrobe probe (no oracle sample)"
        total = per_read * n_reads * steps
        achieved = total / (ms / 1000.0) / 1e9 if ms else 0.0
        out["lookup"] = {"kernel": "k_probe + k_hits + k_anchors", "bound": "hbm (random 32-byte sectors)",
                         "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": NCU_DRAM["lookup"][0] * n_reads * steps / max(1, lk[0][1]),
                         "traffic_source": NCU_DRAM_SOURCE,
                         "avg_launch_ms": ms / max(1, lk[0][1]), "launches": lk[0][1] + lk[1][1],
                         "algorithmic_bytes_per_read": per_read, "model": model}
    for st, f in ALGO_BYTES.items():
        if st not in kern or not kern[st][1]:
            continue
        ms, n = kern[st]
        sec = ms / 1000.0
        per_launch = f(counts) * steps / n
        achieved = per_launch * n / sec / 1e9
        traffic = NCU_DRAM[st][0] * n_reads * steps / n if st in NCU_DRAM else None
        out[st] = {"kernel": st, "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                   "frac": achieved / hbm, "traffic": traffic, "traffic_source": NCU_DRAM_SOURCE,
                   "avg_launch_ms": ms / n, "launches": n,
                   "algorithmic_bytes_per_launch": per_launch}
    for st in ANCHOR_RATE:
        if st in kern and kern[st][1]:
            ms, n = kern[st]
            out[st] = {"kernel": st, "bound": "issue/latency", "achieved": counts["n_anchor_total"] * steps / (ms / 1e3),
                       "peak": None, "unit": "anchors/s", "frac": None, "traffic": None, "avg_launch_ms": ms / n,
                       "launches": n}
    # the integer-ALU denominator: the device's measured add-then-max rate / 11
    # instructions per cell when measured, else SMs x 128 lanes x clock / 11
    clock = (clocks.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)) * 1e6
    model_gcups = sms * 128 * clock / 11 / 1e9
    if alu and alu.get("viaddmax_per_s"):
        peak_gcups = alu["viaddmax_per_s"] / 11 / 1e9
        peak_source = ("measured add-then-max instruction rate (sa_measure_int_alu, all SMs) / 11 instructions "
                       "per cell")
    else:
        peak_gcups = model_gcups
        peak_source = f"{sms} SMs x 128 INT32 lanes x median SM clock under load / 11 ops per cell"
    if kern.get("sw_byte", [0, 0])[1]:
        ms = kern.get("sw_byte", [0.0, 0])[0] + kern.get("sw_word", [0.0, 0])[0]
        n = kern.get("sw_byte", [0.0, 0])[1] + kern.get("sw_word", [0.0, 0])[1]
        sec = ms / 1000.0
        achieved = cells.get("canonical", 0) / sec / 1e9 if sec else 0.0
        computed = sum(cells.get(k, 0) for k in ("forward_byte", "forward_word", "reverse_byte", "reverse_word"))
        sw_cells = {k: v for k, v in cells.items() if not k.startswith("band_")}
        out["sw"] = {"kernel": "k_ssw (byte, word, reverse passes)", "bound": "int32", "achieved": achieved,
                     "peak": peak_gcups, "unit": "GCUPS", "frac": achieved / peak_gcups,
                     "traffic": NCU_DRAM["sw"][0] * cells.get("canonical", 0) / max(n, 1),
                     "traffic_source": NCU_DRAM_SOURCE,
                     "avg_launch_ms": ms / max(n, 1), "launches": n,
                     "computed_gcups": computed / sec / 1e9 if sec else 0.0, "cells": sw_cells,
                     "peak_source": peak_source, "model_peak_gcups": model_gcups}
    if kern.get("banded_traceback", [0, 0])[1] and cells.get("band_canonical"):
        # banded_sw (ext/ssw/ssw.c:598-769): the final pass's band cells per second, the
        # same integer-ALU model as SSW; the doubling passes' cells beside it
        ms, n = kern["banded_traceback"]
        sec = ms / 1000.0
        achieved = cells["band_canonical"] / sec / 1e9 if sec else 0.0
        out["band"] = {"kernel": "k_band_small + k_band_warp + k_band_width_wide + k_band_trace_wide", "bound": "int32",
                       "achieved": achieved, "peak": peak_gcups, "unit": "GCUPS", "frac": achieved / peak_gcups,
                       "traffic": None, "avg_launch_ms": ms / max(n, 1), "launches": n,
                       "computed_gcups": cells.get("band_computed", 0) / sec / 1e9 if sec else 0.0,
                       "cells": {"canonical": cells["band_canonical"], "computed": cells.get("band_computed", 0)},
                       "peak_source": peak_source}
    key = "sw" if dom in ("sw_byte", "sw_word") else "lookup" if dom == "hits" else dom
    head = dict(out.get(key) or {"kernel": dom, "bound": "hbm", "achieved": None, "peak": hbm, "unit": "GB/s",
                                 "frac": None, "traffic": None})
    head["stage"] = dom
    return head, out


if __name__ == "__main__":
    main()
