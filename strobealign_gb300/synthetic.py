"""Seeded synthetic genomes and reads with the shapes of the benchmark workloads.

The reference measures on public read sets; these generators stand in for them
with the same sizes and error/length/insert distributions (fixed seeds), so runs are
reproducible and need no data download.  The generation itself is native
(synth.cpp, multithreaded; its output does not depend on the thread count).
"""
from __future__ import annotations

import ctypes as C
import functools
import os
from dataclasses import dataclass

import numpy as np

ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)
COMP = np.zeros(256, dtype=np.uint8)
COMP[:] = ord("N")
for a, b in zip(b"ACGT", b"TGCA"):
    COMP[a] = b


def revcomp(a: np.ndarray) -> np.ndarray:
    return COMP[a[::-1]]


@dataclass
class Genome:
    names: list[str]
    seqs: list[np.ndarray]  # uint8 ASCII

    @property
    def total(self) -> int:
        return sum(len(s) for s in self.seqs)

    def write_fasta(self, path: str, width: int = 80) -> None:
        with open(path, "wb") as f:
            for n, s in zip(self.names, self.seqs):
                f.write(b">" + n.encode() + b"\n")
                b = s.tobytes()
                for i in range(0, len(b), width):
                    f.write(b[i:i + width] + b"\n")


@functools.lru_cache(None)
def _native() -> C.CDLL:
    from . import build as _build
    lib = C.CDLL(str(_build.build_synth()))
    lib.syn_genome.restype = C.c_int32
    lib.syn_genome.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_double, C.c_double, C.c_uint32, C.c_double,
                               C.c_double, C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_void_p,
                               C.c_int32]
    lib.syn_reads.restype = C.c_int32
    lib.syn_reads.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32,
                              C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_char, C.c_void_p,
                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]
    lib.syn_write_fastq.restype = C.c_int32
    lib.syn_write_fastq.argtypes = [C.c_char_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_char_p, C.c_void_p,
                                    C.c_char_p]
    return lib


def _threads() -> int:
    return max(1, min(32, os.cpu_count() or 1))


def make_genome(seed: int, total: int, n_contigs: int = 1, gc: float = 0.5, segdup_fraction: float = 0.0,
                segdup_len: int = 2000, segdup_div: float = 0.02, repeat_fraction: float = 0.0,
                family_len: tuple[int, int] = (300, 6000), family_div: tuple[float, float] = (0.10, 0.20),
                tandem_fraction: float = 0.0) -> Genome:
    """Uniform or GC-biased random contigs with optional segmental duplications,
    interspersed repeat families and tandem repeats (synth.cpp syn_genome)."""
    buf = np.empty(total, dtype=np.uint8)
    r = _native().syn_genome(seed, total, n_contigs, gc, segdup_fraction, segdup_len, segdup_div, repeat_fraction,
                             family_len[0], family_len[1], family_div[0], family_div[1], tandem_fraction,
                             buf.ctypes.data, _threads())
    if r != 0:
        raise ValueError("syn_genome: bad arguments")
    lens = np.full(n_contigs, total // n_contigs, dtype=np.int64)
    lens[: total % n_contigs] += 1
    starts = np.concatenate([[0], np.cumsum(lens)])
    seqs = [buf[int(starts[i]):int(starts[i + 1])] for i in range(n_contigs)]
    names = [f"chr{i + 1}" if n_contigs > 1 else "contig1" for i in range(n_contigs)]
    g = Genome(names, seqs)
    g.buffer = buf
    return g


@dataclass
class ReadSet:
    seq: np.ndarray          # uint8 concatenated
    offsets: np.ndarray      # uint64 n + 1
    names: bytes
    name_offsets: np.ndarray
    qual: bytes

    def __len__(self):
        return len(self.offsets) - 1

    def record(self, i: int) -> tuple[str, bytes]:
        s = self.seq[self.offsets[i]:self.offsets[i + 1]].tobytes()
        n = self.names[self.name_offsets[i]:self.name_offsets[i + 1]].decode()
        return n, s

    def write_fastq(self, path: str) -> None:
        """FASTQ with 'I' for every quality (synth.cpp syn_write_fastq)."""
        seq = np.ascontiguousarray(self.seq, dtype=np.uint8)
        off = np.ascontiguousarray(self.offsets, dtype=np.uint64)
        no = np.ascontiguousarray(self.name_offsets, dtype=np.uint64)
        if _native().syn_write_fastq(os.fsencode(path), len(self), seq.ctypes.data, off.ctypes.data, bytes(self.names),
                                     no.ctypes.data, None) != 0:
            raise OSError(f"cannot write {path}")


def _genome_arrays(genome: Genome):
    buf = getattr(genome, "buffer", None)
    if buf is None:
        buf = np.concatenate(genome.seqs) if genome.seqs else np.zeros(0, np.uint8)
    starts = np.zeros(len(genome.seqs) + 1, dtype=np.uint64)
    starts[1:] = np.cumsum([len(x) for x in genome.seqs])
    return np.ascontiguousarray(buf, dtype=np.uint8), starts


def _reads(seed, genome, n, lo, hi, insert_mean, insert_sd, sub, indel, rescue_fraction, paired):
    g, starts = _genome_arrays(genome)
    cap = max(1, n * hi)
    s1 = np.empty(cap, dtype=np.uint8)
    o1 = np.empty(n + 1, dtype=np.uint64)
    s2 = np.empty(cap, dtype=np.uint8) if paired else None
    o2 = np.empty(n + 1, dtype=np.uint64) if paired else None
    names = np.empty(max(1, n * (2 + len(str(n)))), dtype=np.uint8)
    no = np.empty(n + 1, dtype=np.uint64)
    prefix = b"p" if paired else b"r"
    r = _native().syn_reads(seed, g.ctypes.data, starts.ctypes.data, len(genome.seqs), n, lo, hi, insert_mean,
                            insert_sd, sub, indel, rescue_fraction, prefix, s1.ctypes.data, o1.ctypes.data,
                            s2.ctypes.data if paired else None, o2.ctypes.data if paired else None,
                            names.ctypes.data, no.ctypes.data, _threads())
    if r != 0:
        raise ValueError("syn_reads: bad arguments")
    nb = names[:int(no[-1])].tobytes()

    def rs(s, o):
        t = int(o[-1])
        return ReadSet(s[:t], o, nb, no, b"I" * t)
    return (rs(s1, o1), rs(s2, o2)) if paired else rs(s1, o1)


def make_single_end(seed: int, genome: Genome, n: int, length: int | tuple[int, int] = 150, sub: float = 0.01,
                    indel: float = 0.001, block: int = 0) -> ReadSet:
    """Reads of `length` (or a length uniform in [lo, hi]) from uniform positions on both
    strands (synth.cpp syn_reads)."""
    lo, hi = (length, length) if isinstance(length, int) else length
    return _reads(seed, genome, n, lo, hi, 0.0, 0.0, sub, indel, 0.0, False)


def make_paired_end(seed: int, genome: Genome, n: int, length: int = 150, insert_mean: float = 300,
                    insert_sd: float = 30, sub: float = 0.01, indel: float = 0.001,
                    rescue_fraction: float = 0.0, block: int = 0) -> tuple[ReadSet, ReadSet]:
    """Pairs in FR orientation; `rescue_fraction` of pairs get one mate mutated
    heavily so that it finds few or no seeds and has to be rescued from its mate
    (synth.cpp syn_reads)."""
    return _reads(seed, genome, n, length, length, insert_mean, insert_sd, sub, indel, rescue_fraction, True)


# Workload shapes (benchmark configurations)
def workload_paired_repetitive(scale: float = 1.0):
    """50 Mbp in 20 contigs, GC 41%, 10% 2 kbp segmental copies at 2%; 1M pairs
    2x150, insert N(300, 30), 1% substitutions, 0.1% indels, mate rescue."""
    g = make_genome(2, int(50_000_000 * scale), 20, gc=0.41, segdup_fraction=0.10, segdup_len=2000, segdup_div=0.02)
    r1, r2 = make_paired_end(102, g, int(1_000_000 * scale), 150, 300, 30, 0.01, 0.001, rescue_fraction=0.02)
    return g, r1, r2


def workload_single_small(scale: float = 1.0):
    """5 Mbp uniform in one contig; 100k single-end 150 bp, 1% substitutions, 0.1% indels."""
    g = make_genome(1, int(5_000_000 * scale), 1, gc=0.5)
    r = make_single_end(101, g, int(100_000 * scale), 150, 0.01, 0.001)
    return g, r
