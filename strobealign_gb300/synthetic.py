"""Seeded synthetic genomes and reads with the shapes of the benchmark workloads.

The reference measures on public read sets; these generators stand in for them
with the same sizes and error/length/insert distributions (numpy PCG64, fixed
seeds), so runs are reproducible and need no data download.
"""
from __future__ import annotations

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


def random_bases(rng: np.random.Generator, n: int, gc: float = 0.5) -> np.ndarray:
    p = [(1 - gc) / 2, gc / 2, gc / 2, (1 - gc) / 2]
    return ACGT[rng.choice(4, size=n, p=p)]


def mutate_subs(rng: np.random.Generator, a: np.ndarray, rate: float) -> np.ndarray:
    a = a.copy()
    m = rng.random(a.size) < rate
    k = int(m.sum())
    if k:
        cur = a[m]
        shift = rng.integers(1, 4, size=k)
        idx = (np.searchsorted(ACGT, cur) + shift) % 4
        a[m] = ACGT[idx]
    return a


def make_genome(seed: int, total: int, n_contigs: int = 1, gc: float = 0.5, segdup_fraction: float = 0.0,
                segdup_len: int = 2000, segdup_div: float = 0.02, repeat_fraction: float = 0.0,
                family_len: tuple[int, int] = (300, 6000), family_div: tuple[float, float] = (0.10, 0.20),
                tandem_fraction: float = 0.0) -> Genome:
    """Uniform or GC-biased random contigs with optional segmental duplications,
    interspersed repeat families and tandem repeats."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lens = np.full(n_contigs, total // n_contigs, dtype=np.int64)
    lens[: total % n_contigs] += 1
    seqs = [random_bases(rng, int(L), gc) for L in lens]
    # segmental duplications: copy 2 kbp segments elsewhere at small divergence
    n_dup = int(total * segdup_fraction / max(segdup_len, 1))
    for _ in range(n_dup):
        a, b = rng.integers(0, n_contigs, size=2)
        if lens[a] <= segdup_len or lens[b] <= segdup_len:
            continue
        src = int(rng.integers(0, lens[a] - segdup_len))
        dst = int(rng.integers(0, lens[b] - segdup_len))
        seqs[b][dst:dst + segdup_len] = mutate_subs(rng, seqs[a][src:src + segdup_len], segdup_div)
    # interspersed repeat families
    if repeat_fraction > 0:
        n_fam = 50
        fams = [random_bases(rng, int(rng.integers(family_len[0], family_len[1] + 1)), gc) for _ in range(n_fam)]
        budget = int(total * repeat_fraction)
        while budget > 0:
            f = fams[int(rng.integers(0, n_fam))]
            c = int(rng.integers(0, n_contigs))
            if lens[c] <= len(f):
                continue
            d = int(rng.integers(0, lens[c] - len(f)))
            div = float(rng.uniform(*family_div))
            seqs[c][d:d + len(f)] = mutate_subs(rng, f, div)
            budget -= len(f)
    if tandem_fraction > 0:
        budget = int(total * tandem_fraction)
        while budget > 0:
            period = int(rng.integers(2, 51))
            unit = random_bases(rng, period, gc)
            length = int(rng.integers(100, 3000))
            c = int(rng.integers(0, n_contigs))
            if lens[c] <= length:
                continue
            d = int(rng.integers(0, lens[c] - length))
            rep = np.resize(unit, length)
            seqs[c][d:d + length] = mutate_subs(rng, rep, 0.02)
            budget -= length
    names = [f"chr{i + 1}" if n_contigs > 1 else "contig1" for i in range(n_contigs)]
    return Genome(names, seqs)


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
        with open(path, "wb") as f:
            for i in range(len(self)):
                n, s = self.record(i)
                f.write(b"@" + n.encode() + b"\n" + s + b"\n+\n" + b"I" * len(s) + b"\n")


def _indels(rng: np.random.Generator, a: np.ndarray, rate: float) -> np.ndarray:
    """Insertions/deletions of length 1-3 (geometric p=0.5, truncated) at `rate` per base."""
    n_ev = rng.poisson(rate * a.size)
    if n_ev == 0:
        return a
    pos = np.sort(rng.integers(0, a.size, size=n_ev))
    out = []
    last = 0
    for p in pos:
        L = int(min(rng.geometric(0.5), 3))
        out.append(a[last:p])
        if rng.random() < 0.5:
            out.append(ACGT[rng.integers(0, 4, size=L)])
            last = p
        else:
            last = min(a.size, p + L)
    out.append(a[last:])
    return np.concatenate(out)


def _pack(reads: list[np.ndarray], names: list[str]) -> ReadSet:
    lens = np.array([len(r) for r in reads], dtype=np.uint64)
    off = np.zeros(len(reads) + 1, dtype=np.uint64)
    off[1:] = np.cumsum(lens)
    bn = [n.encode() for n in names]
    no = np.zeros(len(bn) + 1, dtype=np.uint64)
    no[1:] = np.cumsum([len(x) for x in bn])
    seq = np.concatenate(reads) if reads else np.zeros(0, np.uint8)
    return ReadSet(seq, off, b"".join(bn), no, b"I" * int(off[-1]))


def _concat(genome: Genome):
    lens = np.array([len(x) for x in genome.seqs], dtype=np.int64)
    starts = np.zeros(len(lens) + 1, dtype=np.int64)
    starts[1:] = np.cumsum(lens)
    return np.concatenate(genome.seqs), lens, starts


def _positions(rng, lens, starts, frag: np.ndarray):
    """Global start of a fragment of length frag[i] drawn uniformly over the genome."""
    n = frag.size
    c = rng.choice(lens.size, size=n, p=lens / lens.sum())
    room = np.maximum(lens[c] - frag, 1)
    p = (rng.random(n) * room).astype(np.int64)
    return starts[c] + p, np.minimum(frag, lens[c])


def _finish(rng, mat: np.ndarray, lens: np.ndarray, sub: float, indel: float, heavy: np.ndarray | None = None):
    """Substitutions over the whole batch, indels per affected read; returns a list of reads."""
    mat = mutate_subs(rng, mat.reshape(-1), sub).reshape(mat.shape)
    if heavy is not None and heavy.any():
        idx = np.nonzero(heavy)[0]
        mat[idx] = mutate_subs(rng, mat[idx].reshape(-1), 0.15).reshape(len(idx), -1)
    n_ev = rng.poisson(indel * lens.astype(np.float64))
    reads = []
    for i in range(mat.shape[0]):
        r = mat[i, : lens[i]]
        if n_ev[i]:
            r = _indels(rng, r, indel)[: lens[i]]
        reads.append(r)
    return reads


def _blocks(n: int, block: int):
    return [(a, min(n, a + block)) for a in range(0, n, block)] or [(0, 0)]


def _join(sets: list[ReadSet]) -> ReadSet:
    if len(sets) == 1:
        return sets[0]
    seq = np.concatenate([x.seq for x in sets])
    off = np.zeros(sum(len(x) for x in sets) + 1, dtype=np.uint64)
    no = np.zeros_like(off)
    i, so, nb = 0, 0, 0
    for x in sets:
        k = len(x)
        off[i + 1:i + k + 1] = x.offsets[1:] + so
        no[i + 1:i + k + 1] = x.name_offsets[1:] + nb
        i += k
        so += int(x.offsets[-1])
        nb += int(x.name_offsets[-1])
    return ReadSet(seq, off, b"".join(x.names for x in sets), no, b"".join(x.qual for x in sets))


def make_single_end(seed: int, genome: Genome, n: int, length: int | tuple[int, int] = 150, sub: float = 0.01,
                    indel: float = 0.001, block: int = 1_000_000) -> ReadSet:
    """Reads from uniform positions on both strands; generated in blocks of `block`
    reads (one RNG stream) to bound memory."""
    rng = np.random.Generator(np.random.PCG64(seed))
    g, lens, starts = _concat(genome)
    return _join([_single_block(rng, g, lens, starts, a, b, length, sub, indel) for a, b in _blocks(n, block)])


def _single_block(rng, g, lens, starts, first, last, length, sub, indel) -> ReadSet:
    n = last - first
    if isinstance(length, int):
        L = np.full(n, length, dtype=np.int64)
    else:
        L = rng.integers(length[0], length[1] + 1, size=n).astype(np.int64)
    pos, L = _positions(rng, lens, starts, L)
    flip = rng.random(n) < 0.5
    W = int(L.max()) if n else 0
    j = np.arange(W)
    fwd_idx = pos[:, None] + np.minimum(j[None, :], L[:, None] - 1)
    rev_idx = pos[:, None] + np.maximum(L[:, None] - 1 - j[None, :], 0)
    mat = np.where(flip[:, None], COMP[g[rev_idx]], g[fwd_idx])
    reads = _finish(rng, mat, L, sub, indel)
    return _pack(reads, [f"r{i}" for i in range(first, last)])


def make_paired_end(seed: int, genome: Genome, n: int, length: int = 150, insert_mean: float = 300,
                    insert_sd: float = 30, sub: float = 0.01, indel: float = 0.001,
                    rescue_fraction: float = 0.0, block: int = 1_000_000) -> tuple[ReadSet, ReadSet]:
    """Pairs in FR orientation; `rescue_fraction` of pairs get one mate mutated
    heavily so that it finds few or no seeds and has to be rescued from its mate.
    Generated in blocks of `block` pairs (one RNG stream) to bound memory."""
    rng = np.random.Generator(np.random.PCG64(seed))
    g, lens, starts = _concat(genome)
    parts = [_paired_block(rng, g, lens, starts, a, b, length, insert_mean, insert_sd, sub, indel, rescue_fraction)
             for a, b in _blocks(n, block)]
    return _join([p[0] for p in parts]), _join([p[1] for p in parts])


def _paired_block(rng, g, lens, starts, first, last, length, insert_mean, insert_sd, sub, indel, rescue_fraction):
    n = last - first
    ins = np.maximum(np.rint(rng.normal(insert_mean, insert_sd, size=n)).astype(np.int64), length)
    pos, ins = _positions(rng, lens, starts, ins)
    flip = rng.random(n) < 0.5
    L = np.minimum(ins, length)
    j = np.arange(length)
    head = pos[:, None] + np.minimum(j[None, :], ins[:, None] - 1)
    tail = pos[:, None] + np.maximum(ins[:, None] - 1 - j[None, :], 0)
    a = np.where(flip[:, None], COMP[g[tail]], g[head])
    b = np.where(flip[:, None], g[head], COMP[g[tail]])
    heavy = rng.random(n) < rescue_fraction if rescue_fraction else None
    which = rng.random(n) < 0.5
    ha = None if heavy is None else (heavy & which)
    hb = None if heavy is None else (heavy & ~which)
    names = [f"p{i}" for i in range(first, last)]
    return _pack(_finish(rng, a, L, sub, indel, ha), names), _pack(_finish(rng, b, L, sub, indel, hb), names)


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
