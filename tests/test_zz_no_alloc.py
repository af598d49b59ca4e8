"""Allocation-free seeding (sa_randstrobes_device_noalloc) through the C ABI,
checked against sa_randstrobes_batch on the same reads.

The entry point takes device buffers owned by the caller (allocated here with
torch) and keeps its syncmer scratch in a static device array, so two calls in a
row must not see each other's data, and a call must not change the device's free
memory.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SA_OK = 0
SA_ERR_INVALID = -1
MAX_BASES = 1048576
U32_MAX = 0xFFFFFFFF


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import strobealign_gb300 as sa
    from strobealign_gb300 import synthetic as syn
    from strobealign_gb300._lib import load

    g = syn.make_genome(11, 200_000, 2)
    refs = sa.References.from_sequences(g.names, [s.tobytes() for s in g.seqs])
    idx = sa.StrobemerIndex.build(refs, sa.SeedingParameters.from_read_length(150))
    return torch, sa, idx, load()


def _reads(seed, n):
    rng = np.random.default_rng(seed)
    seqs = []
    for i in range(n):
        L = int(rng.integers(100, 400))
        s = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, L)].copy()
        if i % 7 == 3:
            s[L // 3:L // 3 + 5] = ord("N")
        if i % 11 == 5:
            s = np.frombuffer(s.tobytes().lower(), np.uint8).copy()
        seqs.append(s.tobytes())
    # edge cases: empty, shorter than k, shorter than w_max syncmers, all N
    seqs += [b"", b"ACGTACGTAC", b"ACGT" * 8, b"N" * 200, b"ACGTTGCA" * 40]
    return seqs


def _device_call(torch, lib, idx, seqs, stream, total_override=None, offsets=None):
    lens = [len(s) for s in seqs]
    offs = np.zeros(len(seqs) + 1, np.int64) if offsets is None else offsets
    if offsets is None:
        offs[1:] = np.cumsum(lens)
    total = int(offs[-1]) if total_override is None else total_override
    flat = np.frombuffer(b"".join(seqs) or b"\0", np.uint8)
    d_seq = torch.from_numpy(flat.copy()).cuda()
    d_off = torch.from_numpy(offs).cuda()
    cap = max(1, 2 * total)
    # outputs start with garbage: the entry point must not rely on zeroed buffers
    d_hash = torch.full((cap,), 0x5A5A5A5A5A5A5A5A, dtype=torch.int64, device="cuda")
    d_hash_rc = torch.full((cap,), 0x3C3C3C3C3C3C3C3C, dtype=torch.int64, device="cuda")
    d_start = torch.full((cap,), 0x12345678, dtype=torch.int32, device="cuda")
    d_end = torch.full((cap,), 0x12345678, dtype=torch.int32, device="cuda")
    d_cnt = torch.full((2 * len(seqs),), 0x12345678, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    rc = lib.sa_randstrobes_device_noalloc(idx.h, d_seq.data_ptr(), d_off.data_ptr(), len(seqs), total,
                                           d_hash.data_ptr(), d_hash_rc.data_ptr(), d_start.data_ptr(),
                                           d_end.data_ptr(), d_cnt.data_ptr(), C.c_void_p(stream.cuda_stream))
    stream.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert rc == SA_OK, lib.sa_last_error()
    out = dict(hash=d_hash.cpu().numpy().view(np.uint64), hash_revcomp=d_hash_rc.cpu().numpy().view(np.uint64),
               start=d_start.cpu().numpy().view(np.uint32), end=d_end.cpu().numpy().view(np.uint32),
               counts=d_cnt.cpu().numpy().view(np.uint32), offs=offs, total=total)
    return out, free0 - free1


def _check_against_batch(sa, idx, seqs, out):
    want = sa.randstrobes_batch(idx, sa.Reads.from_lists([f"r{i}" for i in range(len(seqs))], seqs))
    offs, total, cnt = out["offs"], out["total"], out["counts"]
    for r, (fw, rc) in enumerate(want):
        assert cnt[2 * r] == len(fw) and cnt[2 * r + 1] == len(rc), r
        for base, arr in ((int(offs[r]), fw), (total + int(offs[r]), rc)):
            sl = slice(base, base + len(arr))
            for f in ("hash", "hash_revcomp", "start", "end"):
                assert (out[f][sl] == arr[f]).all(), (r, f)


def test_noalloc_matches_batch_entry_point_two_calls_in_a_row(env):
    torch, sa, idx, lib = env
    stream = torch.cuda.Stream()
    a, b = _reads(1, 300), _reads(2, 170)
    out_a, _ = _device_call(torch, lib, idx, a, stream)
    out_b, grew_b = _device_call(torch, lib, idx, b, stream)
    _check_against_batch(sa, idx, a, out_a)
    _check_against_batch(sa, idx, b, out_b)
    # the same batch again after a different one gives the same result
    out_a2, grew_a2 = _device_call(torch, lib, idx, a, stream)
    for f in ("hash", "hash_revcomp", "start", "end", "counts"):
        n = 2 * out_a["total"] if f != "counts" else 2 * len(a)
        used = np.zeros(n, bool)
        if f == "counts":
            used[:] = True
        else:
            for r in range(len(a)):
                o = int(out_a["offs"][r])
                used[o:o + out_a["counts"][2 * r]] = True
                used[out_a["total"] + o:out_a["total"] + o + out_a["counts"][2 * r + 1]] = True
        assert (out_a2[f][:n][used] == out_a[f][:n][used]).all(), f
    # after the first call on the device, calls allocate nothing
    assert grew_b == 0 and grew_a2 == 0


def test_noalloc_default_stream_and_setup_call(env):
    torch, sa, idx, lib = env
    # n_reads = 0 only performs the per-device setup
    assert lib.sa_randstrobes_device_noalloc(idx.h, None, None, 0, 0, None, None, None, None, None, None) == SA_OK
    seqs = _reads(3, 64)
    out, grew = _device_call(torch, lib, idx, seqs, torch.cuda.default_stream())
    _check_against_batch(sa, idx, seqs, out)
    assert grew == 0
    out2, grew2 = _device_call(torch, lib, idx, seqs, torch.cuda.default_stream())
    _check_against_batch(sa, idx, seqs, out2)
    assert grew2 == 0


def test_noalloc_rejects_oversized_batch(env):
    torch, sa, idx, lib = env
    rc = lib.sa_randstrobes_device_noalloc(idx.h, None, None, 1, MAX_BASES + 1, None, None, None, None, None, None)
    assert rc == SA_ERR_INVALID
    assert b"at most" in lib.sa_last_error()


def test_noalloc_marks_reads_outside_the_batch(env):
    torch, sa, idx, lib = env
    stream = torch.cuda.Stream()
    seqs = _reads(4, 20)
    # a read longer than 2048 bases and a read ending past total_bases are marked, the rest are seeded
    long_read = b"ACGT" * 600
    seqs2 = seqs[:5] + [long_read] + seqs[5:]
    out, _ = _device_call(torch, lib, idx, seqs2, stream)
    assert out["counts"][10] == U32_MAX and out["counts"][11] == U32_MAX
    ok = [i for i in range(len(seqs2)) if i != 5]
    want = sa.randstrobes_batch(idx, sa.Reads.from_lists([f"r{i}" for i in ok], [seqs2[i] for i in ok]))
    for j, i in enumerate(ok):
        assert out["counts"][2 * i] == len(want[j][0]) and out["counts"][2 * i + 1] == len(want[j][1])
    lens = [len(s) for s in seqs]
    offs = np.zeros(len(seqs) + 1, np.int64)
    offs[1:] = np.cumsum(lens)
    short_total = int(offs[-2])  # the last read ends past total_bases
    out2, _ = _device_call(torch, lib, idx, seqs, stream, total_override=short_total, offsets=offs)
    last = len(seqs) - 1
    assert lens[last] > 0
    assert out2["counts"][2 * last] == U32_MAX and out2["counts"][2 * last + 1] == U32_MAX
    _check_against_batch(sa, idx, seqs[:last], dict(out2, counts=out2["counts"][:2 * last]))
