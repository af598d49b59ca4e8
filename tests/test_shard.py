"""Sharding one input over ranks (strobealign_gb300/shard.py), on CPU: the ranks map
contiguous runs of whole chunks and rank 0 gathers their bytes in rank order; the
result is the single-process output (src/main.rs:591-604 cuts the chunks, :653-667
writes them in order).  Two gloo ranks map their ranges with the oracle (the CPU
restatement of the reference path) and compare with the oracle over the whole input."""
import os
import socket
import sys

import numpy as np
import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

sys.path.insert(0, str(ROOT))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _slice(rs, a, b):
    from strobealign_gb300 import synthetic as syn
    o, no = rs.offsets, rs.name_offsets
    return syn.ReadSet(rs.seq[int(o[a]):int(o[b])], o[a:b + 1] - o[a], rs.names[int(no[a]):int(no[b])],
                       no[a:b + 1] - no[a], rs.qual[int(o[a]):int(o[b])] if rs.qual is not None else None)


def _data():
    from strobealign_gb300 import synthetic as syn
    g = syn.make_genome(71, 300_000, 2, gc=0.42, segdup_fraction=0.05)
    r1, r2 = syn.make_paired_end(72, g, 1500, 150, 300, 30, 0.01, 0.002, rescue_fraction=0.03)
    return g, r1, r2


CHUNK = 20_000


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle.binding import OracleIndex
    from strobealign_gb300 import shard
    g, r1, r2 = _data()
    idx = OracleIndex(g.names, g.seqs, 150, threads=1)
    a, b = shard.shard_ranges(shard.record_lengths(r1.offsets, r2.offsets), world, CHUNK)[rank]
    mine = idx.map_batch(_slice(r1, a, b), _slice(r2, a, b), chunk_size=CHUNK, threads=1)[0] if b > a else b""
    out = shard.gather_in_order(mine, rank, world, dist)
    q.put((rank, (a, b), out))
    dist.destroy_process_group()


def test_chunk_starts_follow_the_reference_rule():
    from strobealign_gb300 import shard
    lens = np.array([300] * 10 + [5000] + [300] * 5, dtype=np.int64)
    st = shard.chunk_starts(lens, 1000)
    # records until the sum exceeds 1000: 4 records (1200), 4 (1200), 2 + the long one...
    want, i = [0], 0
    while i < len(lens):
        s = 0
        while i < len(lens):
            s += lens[i]
            i += 1
            if s > 1000:
                break
        want.append(i)
    assert list(st) == want
    r = shard.shard_ranges(lens, 3, 1000)
    assert r[0][0] == 0 and r[-1][1] == len(lens)
    assert all(x[1] == y[0] for x, y in zip(r, r[1:]))
    assert all(a in want and b in want for a, b in r)
    # more ranks than chunks: some ranges are empty, the cover is still whole
    r = shard.shard_ranges(lens[:3], 4, 1000)
    assert r[0][0] == 0 and r[-1][1] == 3 and all(x[1] == y[0] for x, y in zip(r, r[1:]))


def test_two_gloo_ranks_reproduce_the_single_process_bytes():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, rng0, got), (r1_, rng1, none) = out
    assert none is None and rng0[1] == rng1[0] and rng0[0] == 0 and rng1[0] > 0
    from oracle.binding import OracleIndex
    g, r1, r2 = _data()
    want = OracleIndex(g.names, g.seqs, 150, threads=1).map_batch(r1, r2, chunk_size=CHUNK, threads=1)[0]
    assert got == want


def _interleaved_data():
    # a mixed file's reads in order: pairs (mates with one name) and single reads
    from strobealign_gb300 import synthetic as syn
    g, r1, r2 = _data()
    se = syn.make_single_end(73, g, 700, (60, 300), 0.01, 0.002)
    seqs, names = [], []
    rnd = np.random.default_rng(74)
    i = j = 0
    while i < len(r1) or j < len(se):
        if j == len(se) or (i < len(r1) and rnd.random() < 0.6):
            for rs in (r1, r2):
                n, s = rs.record(i)
                names.append(n)
                seqs.append(s)
            i += 1
        else:
            n, s = se.record(j)
            names.append(n)
            seqs.append(s)
            j += 1
    return g, names, seqs


def _read_set(names, seqs):
    from strobealign_gb300 import synthetic as syn
    off = np.zeros(len(seqs) + 1, dtype=np.uint64)
    off[1:] = np.cumsum([len(s) for s in seqs])
    no = np.zeros(len(names) + 1, dtype=np.uint64)
    no[1:] = np.cumsum([len(n) for n in names])
    seq = np.frombuffer(b"".join(seqs), dtype=np.uint8)
    return syn.ReadSet(seq, off, "".join(names).encode(), no, b"I" * int(off[-1]))


def _rank_interleaved(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle.binding import OracleIndex
    from strobealign_gb300 import Reads, shard
    g, names, seqs = _interleaved_data()
    first = Reads.from_lists(names, seqs).interleaved_records()
    off = np.concatenate([[0], np.cumsum([len(s) for s in seqs])])
    a, b = shard.shard_ranges(shard.interleaved_record_lengths(off, first), world, CHUNK)[rank]
    ra, rb = int(first[a]), int(first[b])
    idx = OracleIndex(g.names, g.seqs, 150, threads=1)
    mine = idx.map_interleaved(_read_set(names[ra:rb], seqs[ra:rb]), chunk_size=CHUNK, threads=1)[0] \
        if rb > ra else b""
    out = shard.gather_in_order(mine, rank, world, dist)
    q.put((rank, (a, b), out))
    dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_the_single_process_bytes_interleaved():
    # mixed single-end and paired records: ranges of whole records, pairs never split
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_interleaved, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, rng0, got), (_, rng1, none) = out
    assert none is None and rng0[1] == rng1[0] > 0
    from oracle.binding import OracleIndex
    g, names, seqs = _interleaved_data()
    want = OracleIndex(g.names, g.seqs, 150, threads=1).map_interleaved(_read_set(names, seqs), chunk_size=CHUNK,
                                                                        threads=1)[0]
    assert got == want
