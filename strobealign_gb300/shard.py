"""One input split across ranks by contiguous runs of whole chunks, gathered in order.

The reference cuts its input into chunks (records until the chunk's nucleotides, both
mates, exceed chunk_size; src/main.rs:591-604), maps chunks independently -- each with a
fresh RNG and insert-size estimate -- and writes them in chunk order
(src/main.rs:653-667).  So a rank that maps a run of whole chunks writes exactly those
chunks' bytes, and the concatenation of the ranks' outputs in rank order is the
single-process output.  shard_ranges cuts the records at chunk starts with the bases
balanced over the ranks; gather_in_order brings the ranks' bytes to rank 0 (the only data
exchange: the output, on the host).  Each rank keeps its own copy of the index
(replicas): nothing else is exchanged.
"""
from __future__ import annotations

import numpy as np


def record_lengths(offsets1: np.ndarray, offsets2: np.ndarray | None = None) -> np.ndarray:
    """Nucleotides per record (both mates for paired-end) from read offset arrays."""
    n = np.diff(np.asarray(offsets1, dtype=np.int64))
    if offsets2 is not None:
        n = n + np.diff(np.asarray(offsets2, dtype=np.int64))
    return n


def interleaved_record_lengths(seq_offsets: np.ndarray, first_read: np.ndarray) -> np.ndarray:
    """Nucleotides per record of interleaved input (a single read or a pair), from the
    reads' offsets and each record's first read (Reads.interleaved_records: record r is
    reads first_read[r] .. first_read[r + 1]); a record range [a, b) is then the reads
    [first_read[a], first_read[b])."""
    o = np.asarray(seq_offsets, dtype=np.int64)
    f = np.asarray(first_read, dtype=np.int64)
    return o[f[1:]] - o[f[:-1]]


def chunk_starts(lengths: np.ndarray, chunk_size: int = 1_000_000) -> np.ndarray:
    """Record index of every chunk start, then the record count: a chunk takes records
    until its nucleotides exceed chunk_size (the record that crosses is its last)."""
    lengths = np.asarray(lengths, dtype=np.int64)
    n = len(lengths)
    cum = np.concatenate([[0], np.cumsum(lengths)])
    starts = [0]
    i = 0
    while i < n:
        # the first j > i with cum[j] - cum[i] > chunk_size; the chunk is [i, j)
        j = int(np.searchsorted(cum, cum[i] + chunk_size, side="right"))
        j = min(max(j, i + 1), n)
        starts.append(j)
        i = j
    return np.asarray(starts, dtype=np.int64)


def shard_ranges(lengths: np.ndarray, world: int, chunk_size: int = 1_000_000) -> list[tuple[int, int]]:
    """Contiguous record ranges, one per rank, each a run of whole chunks, cut where the
    cumulative bases cross k / world of the total (empty ranges when there are fewer
    chunks than ranks)."""
    lengths = np.asarray(lengths, dtype=np.int64)
    starts = chunk_starts(lengths, chunk_size)
    cum = np.concatenate([[0], np.cumsum(lengths)])
    at = cum[starts]  # bases before each chunk start (and the total at the end)
    total = int(cum[-1])
    cuts = [0]
    for k in range(1, world):
        c = int(np.searchsorted(at, total * k / world, side="left"))
        cuts.append(max(cuts[-1], min(c, len(starts) - 1)))
    cuts.append(len(starts) - 1)
    return [(int(starts[cuts[r]]), int(starts[cuts[r + 1]])) for r in range(world)]


def gather_in_order(data: bytes, rank: int, world: int, dist) -> bytes | None:
    """The ranks' bytes concatenated in rank order on rank 0 (None on the others), over
    torch.distributed (gloo or nccl)."""
    if world == 1:
        return data
    got = [None] * world if rank == 0 else None
    dist.gather_object(data, got, dst=0)
    return b"".join(got) if rank == 0 else None
