#!/usr/bin/env python3
"""Aligned reads/s of strobealign's mapping path on GB300.

Default workload (--workload pe50m): 50 Mbp synthetic reference in 20 contigs (GC 41%,
10% of it 2 kbp segmental copies at 2% divergence), 1M read pairs 2x150 bp, insert
N(300, 30), 1% substitutions, 0.1% indels, 2% of pairs with one mate too mutated to
seed (mate rescue).  Other shapes: se5m (5 Mbp, 100k single-end), uneven200m (200 Mbp
with repeat families, 2M single-end reads of 50-500 bp), human (3.1 Gbp with 50%
repeats; --pairs sets the pair count).  Seeded generators (strobealign_gb300.synthetic)
stand in for the reference's read sets.

One step maps the whole batch: NAM finding, SSW-exact (paired-end / --ssw) or piecewise
(single-end) extension waves and SAM record formatting, chunked as the reference chunks
its input.  `value` is the plain form with the reads already resident in device memory
(sa_map_uploaded); `plain.e2e` maps from host buffers through sa_map_batch; `e2e` is the
served form: the same reads as a stream of requests (log-uniform 1..100k pairs) through
sa_session submit/wait from host buffers, with continuous batching.  An open-loop pass
at 70% of the served capacity gives p50/p99 request latency.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload W]

Under torchrun each rank maps its own replica of the workload (no data exchange:
chunks are independent), and rank 0 prints one JSON line with the aggregate rate
over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
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
    "pe50m": "paired-end repetitive: 50 Mbp / 20 contigs (GC 41%, 10% 2 kbp segmental copies at 2%), "
             "1M pairs 2x150 bp, insert N(300,30), 1% sub, 0.1% indel, 2% of pairs need mate rescue",
    "se5m": "plain small: 5 Mbp uniform / 1 contig, 100k single-end 150 bp, 1% sub, 0.1% indel",
    "uneven200m": "uneven lengths: 200 Mbp / 8 contigs (GC 41%, 20% repeats from 300 bp-6 kbp families at "
                  "10-20% divergence), 2M single-end reads U[50,500] bp, 1.5% sub, 0.2% indel",
    "human": "human scale: 3.1 Gbp / 24 contigs (GC 41%, 50% interspersed repeats, 3% tandem), "
             "pairs 2x150 bp, insert N(400,50), 1% sub, 0.1% indel",
}
WORKLOAD = WORKLOADS["pe50m"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="pe50m", choices=sorted(WORKLOADS))
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of the workload (1.0 = full)")
    ap.add_argument("--pairs", type=int, default=0, help="override the read (pair) count")
    ap.add_argument("--cpu-sample-pairs", type=int, default=20000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-served", action="store_true", help="skip the served and latency passes (profiling runs)")
    return ap.parse_args()


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload(scale: float, name: str = "pe50m", pairs: int = 0):
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


def cpu_baseline(g, r1, r2, pairs: int, threads: int) -> dict:
    """The oracle (C++ restatement of the reference's CPU path) on a bounded sample,
    all host threads; index build excluded from the rate."""
    from oracle import build as oracle_build
    from strobealign_gb300 import synthetic as syn
    oracle_build.build()
    pairs = min(pairs, len(r1))
    with tempfile.TemporaryDirectory() as d:
        fa = os.path.join(d, "ref.fa")
        g.write_fasta(fa)
        files = []
        for i, rs in enumerate(x for x in (r1, r2) if x is not None):
            f = os.path.join(d, f"r{i + 1}.fq")
            syn.ReadSet(rs.seq[:int(rs.offsets[pairs])], rs.offsets[:pairs + 1], rs.names,
                        rs.name_offsets[:pairs + 1], rs.qual).write_fastq(f)
            files.append(f)
        r = subprocess.run([str(oracle_build.cli_path()), "-t", str(threads), "--timing", "-o", os.path.join(d, "o.sam"),
                            fa] + files, capture_output=True, text=True, check=True)
    line = [l for l in r.stderr.splitlines() if l.startswith("oracle_timing")][-1]
    kv = dict(x.split("=") for x in line.split()[1:])
    map_s = float(kv["map_s"])
    reads = pairs * len(files)
    return {"value": reads / map_s, "unit": "reads/s", "cores": threads, "kind": "port",
            "sample": f"{pairs} {'pairs' if len(files) == 2 else 'reads'} of the same workload, index build excluded "
                      f"({float(kv['index_s']):.1f} s)", "seconds": map_s}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    g, r1, r2, _ = workload(args.scale, args.workload, args.pairs)
    for _ in range(args.warmup):
        cpu_baseline(g, r1, r2, min(2000, args.cpu_sample_pairs), threads)
    vals, secs = [], []
    for _ in range(args.steps):
        b = cpu_baseline(g, r1, r2, args.cpu_sample_pairs, threads)
        vals.append(b["value"])
        secs.append(b["seconds"])
    value = statistics.median(vals)
    out = {"metric": METRIC, "value": value, "unit": "reads/s", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1000 * statistics.median(secs), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
           "impl": "reference",
           "config": {"workload": WORKLOADS[args.workload], "scale": args.scale,
                      "sample_pairs": args.cpu_sample_pairs},
           "cpu_baseline": {"value": value, "unit": "reads/s", "cores": threads, "kind": "port",
                            "sample": f"{args.cpu_sample_pairs} pairs per step; the Rust reference cannot be built "
                                      "(no cargo); the oracle restates its CPU path"},
           "e2e": {"value": value, "unit": "reads/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


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

    g, r1, r2, read_length = workload(args.scale, args.workload, args.pairs)
    refs = sa.References.from_sequences(g.names, [s.tobytes() for s in g.seqs])
    params = sa.SeedingParameters.from_read_length(read_length)
    t = time.time()
    index = sa.StrobemerIndex.build(refs, params)
    torch.cuda.synchronize()
    index_s = time.time() - t
    R1 = sa.Reads.from_arrays(r1.seq, r1.offsets, r1.names, r1.name_offsets, r1.qual)
    R2 = sa.Reads.from_arrays(r2.seq, r2.offsets, r2.names, r2.name_offsets, r2.qual) if r2 is not None else None
    n_reads = (2 if r2 is not None else 1) * len(R1)
    mapper = sa.Mapper(index, refs)
    mapper.upload(R1, R2)

    def barrier():
        torch.cuda.synchronize()
        if pg:
            pg.barrier()

    for _ in range(max(3, args.warmup)):
        mapper.map_uploaded(copy=False)
    # timed region: reads resident in device memory
    mapper.set_profiling(True)
    kern = {}
    cells = {}
    phases = {}
    launches = 0
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
            for k in ("seconds_nams", "seconds_extension", "seconds_policy"):
                phases[k] = phases.get(k, 0.0) + st[k] / args.steps
            for k, v in st["sw_cells"].items():
                cells[k] = cells.get(k, 0) + int(v)
            for k, v in st["kernel_ms"].items():
                kern.setdefault(k, [0.0, 0])
                kern[k][0] += v
                kern[k][1] += int(st["kernel_launches"][k])
        ev1.record(stream)
        barrier()
        wall = time.perf_counter() - t0
    mapper.set_profiling(False)
    ev_ms = ev0.elapsed_time(ev1)
    elapsed = max(wall, ev_ms / 1000.0)
    elapsed = slowest_rank(pg, elapsed, "cuda")
    value = ws * n_reads * args.steps / elapsed
    sam_bytes = int(out)
    # end to end: host buffers in, SAM bytes out, every step
    h2d = d2h = 0
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        mapper.map(R1, R2, copy=False)
        st = mapper.stats()
        h2d, d2h = int(st["h2d_bytes"]), int(st["d2h_bytes"])
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_s = slowest_rank(pg, e2e_s, "cuda")
    plain_e2e = ws * n_reads * args.steps / e2e_s
    plain_h2d, plain_d2h = h2d, d2h
    # served: the same pairs as a stream of requests (log-uniform 1..100k pairs), each
    # its own chunk stream, through one session with continuous batching
    reqs, lat = [], None
    served = s_h2d = s_d2h = None
    if not args.no_served:
        sizes = request_sizes(len(R1))
        a = 0
        for n in sizes:
            reqs.append((slice_reads(sa, r1, a, a + n), slice_reads(sa, r2, a, a + n) if r2 is not None else None))
            a += n
        session = sa.Session(index, refs)
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
    e2e = served if served is not None else plain_e2e
    if served is None:
        s_h2d, s_d2h = plain_h2d, plain_d2h
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
    roofline, rooflines = roofline_for(dom, kern, cells, peaks, clk.summary(), counts, args.steps) if dom else (None, {})
    cpu = None
    if not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(g, r1, r2, args.cpu_sample_pairs, os.cpu_count() or 1)
        except Exception as e:  # reported, never fatal for the GPU line
            cpu = {"value": None, "error": str(e)[:200]}
    out = {
        "metric": METRIC, "value": value, "unit": "reads/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": 1000 * elapsed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload], "scale": args.scale, "reads_per_step": n_reads,
                   "l2": f"no flush: index {index.info.device_bytes / 1e6:.0f} MB + reads "
                         f"{int(R1.seq_offsets[-1]) * (2 if R2 is not None else 1) / 1e6:.0f} MB "
                         f"({'exceed' if index.info.device_bytes > 129e6 else 'with the reads exceed'} the 129 MB L2)",
                   "value_form": "plain: the whole batch through sa_map_uploaded, reads resident on the device",
                   "e2e_form": "served: the same pairs as requests of log-uniform 1..100k pairs through "
                               "sa_session submit/wait from host buffers, continuous batching",
                   "requests_per_step": len(reqs), "sam_bytes_per_step": sam_bytes,
                   "index_build_s": round(index_s, 3)},
        "e2e": {"value": e2e, "unit": "reads/s", "h2d_bytes_per_step": s_h2d, "d2h_bytes_per_step": s_d2h},
        "plain": {"value_resident": value, "e2e": plain_e2e, "unit": "reads/s", "h2d_bytes_per_step": plain_h2d,
                  "d2h_bytes_per_step": plain_d2h},
        "served": None if served is None else {"value": served, "unit": "reads/s",
                                               "vs_plain_e2e": served / plain_e2e, "latency_open_loop": lat},
        "gpu_launches": launches,
        "stage_share": shares,
        # wall seconds per step: NAM pipeline (GPU), extension waves (GPU, incl. job
        # upload and result download), host policy between and after waves
        "phases_s": {k.replace("seconds_", ""): round(v, 4) for k, v in phases.items()},
        "roofline": roofline,
        "rooflines": rooflines,
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
    # per randstrobe probe: the bucket-directory pair (16 B) and one 32-byte table sector,
    # and the hit record out (position, info, count: 16 B)
    "hits": lambda c: 64 * c["n_randstrobes"],
}
# stages reported as anchors per second (no HBM or ALU roofline model)
ANCHOR_RATE = ("anchors", "sort", "chain")


def roofline_for(dom, kern, cells, peaks, clocks, counts, steps) -> dict:
    """Roofline of every timed stage, and of the dominant one.

    Seeding and the index lookups are framed against HBM bandwidth with their
    algorithmic bytes per launch (ALGO_BYTES, from the batch's counts); the anchor walk,
    the anchor sort and chaining as anchors per second.  Extension (the SSW kernel k_sw:
    byte pass, word reruns of the byte overflows, reverse passes) is integer-ALU bound:
    its unit is one SSW call of |query| x |reference window| canonical cells, against
    152 SMs x 128 INT32 lanes x SM clock / 11 ops per cell; the cells the passes
    actually computed are reported beside it."""
    hbm = peaks.get("hbm_gbs", 6800.0)
    out = {}
    for st, f in ALGO_BYTES.items():
        if st not in kern or not kern[st][1]:
            continue
        ms, n = kern[st]
        sec = ms / 1000.0
        per_launch = f(counts) * steps / n
        achieved = per_launch * n / sec / 1e9
        out[st] = {"kernel": st, "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                   "frac": achieved / hbm, "traffic": None, "avg_launch_ms": ms / n, "launches": n,
                   "algorithmic_bytes_per_launch": per_launch}
    for st in ANCHOR_RATE:
        if st in kern and kern[st][1]:
            ms, n = kern[st]
            out[st] = {"kernel": st, "bound": "issue/latency", "achieved": counts["n_anchor_total"] * steps / (ms / 1e3),
                       "peak": None, "unit": "anchors/s", "frac": None, "traffic": None, "avg_launch_ms": ms / n,
                       "launches": n}
    if kern.get("sw_byte", [0, 0])[1]:
        ms = kern.get("sw_byte", [0.0, 0])[0] + kern.get("sw_word", [0.0, 0])[0]
        n = kern.get("sw_byte", [0.0, 0])[1] + kern.get("sw_word", [0.0, 0])[1]
        sec = ms / 1000.0
        clock = (clocks.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)) * 1e6
        peak_gcups = 152 * 128 * clock / 11 / 1e9
        achieved = cells.get("canonical", 0) / sec / 1e9 if sec else 0.0
        computed = sum(v for k, v in cells.items() if k != "canonical")
        out["sw"] = {"kernel": "k_ssw (byte, word, reverse passes)", "bound": "int32", "achieved": achieved,
                     "peak": peak_gcups, "unit": "GCUPS", "frac": achieved / peak_gcups, "traffic": None,
                     "avg_launch_ms": ms / max(n, 1), "launches": n,
                     "computed_gcups": computed / sec / 1e9 if sec else 0.0, "cells": cells,
                     "peak_source": "152 SMs x 128 INT32 lanes x median SM clock under load / 11 ops per cell"}
    key = "sw" if dom in ("sw_byte", "sw_word") else dom
    head = dict(out.get(key) or {"kernel": dom, "bound": "hbm", "achieved": None, "peak": hbm, "unit": "GB/s",
                                 "frac": None, "traffic": None})
    head["stage"] = dom
    return head, out


if __name__ == "__main__":
    main()
