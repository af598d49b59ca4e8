"""Serving sessions: each request's output is identical to mapping the same records
alone with a Mapper, whatever else is in flight, in whatever order requests are
submitted, and under tight admission limits."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import strobealign_gb300 as sa
    from strobealign_gb300 import synthetic as syn

    g = syn.make_genome(21, 3_000_000, 6, gc=0.41, segdup_fraction=0.10, segdup_len=2000, segdup_div=0.02)
    r1, r2 = syn.make_paired_end(121, g, 24_000, 150, 300, 30, 0.01, 0.001, rescue_fraction=0.02)
    refs = sa.References.from_sequences(g.names, [s.tobytes() for s in g.seqs])
    idx = sa.StrobemerIndex.build(refs, sa.SeedingParameters.from_read_length(150))
    return sa, refs, idx, r1, r2


def _slice(sa, rs, a, b):
    o = rs.offsets
    no = rs.name_offsets
    seq = rs.seq[o[a]:o[b]]
    qual = rs.qual[o[a]:o[b]] if rs.qual is not None else None
    return sa.Reads.from_arrays(seq, o[a:b + 1] - o[a], rs.names[no[a]:no[b]], no[a:b + 1] - no[a], qual)


# (first pair, pairs, paired)
REQUESTS = [(0, 1, True), (1, 7, True), (8, 300, True), (308, 2500, True), (2808, 9000, True), (11808, 40, False),
            (11848, 3000, False), (14848, 6000, True), (20848, 3152, True)]


def _requests(sa, r1, r2):
    out = []
    for a, n, paired in REQUESTS:
        out.append((_slice(sa, r1, a, a + n), _slice(sa, r2, a, a + n) if paired else None))
    return out


def _alone(sa, refs, idx, reqs, **kw):
    m = sa.Mapper(idx, refs, **kw)
    return [m.map(x, y) for x, y in reqs]


@pytest.mark.parametrize("kw", [dict(use_ssw=1, eqx=1), dict(use_ssw=1, chunk_size=60_000), dict(eqx=1)])
def test_session_requests_identical_alone_and_in_the_mix(setup, kw):
    sa, refs, idx, r1, r2 = setup
    reqs = _requests(sa, r1, r2)
    want = _alone(sa, refs, idx, reqs, **kw)
    s = sa.Session(idx, refs, **kw)
    tickets = [s.submit(x, y) for x, y in reqs]
    got = [s.wait(t)[0] for t in tickets]
    for i, (g, w) in enumerate(zip(got, want)):
        assert g == w, f"request {i} differs"
    # reversed submission order, waited in a different order
    tickets = [s.submit(x, y) for x, y in reversed(reqs)]
    got = {}
    for t, i in sorted(zip(tickets, reversed(range(len(reqs)))), key=lambda p: p[1] % 3):
        got[i] = s.wait(t)[0]
    for i, w in enumerate(want):
        assert got[i] == w, f"request {i} differs (reversed order)"
    s.close()


def test_session_admission_limits(setup):
    sa, refs, idx, r1, r2 = setup
    reqs = _requests(sa, r1, r2)
    want = _alone(sa, refs, idx, reqs, use_ssw=1)
    # an arena of 4 Mbases admits only a few requests at a time; one request in flight at most
    for kw in (dict(max_inflight_bases=4_000_000), dict(max_inflight_requests=1, policy_threads=3),
               dict(admission_streams=1), dict(admission_streams=4, max_inflight_bases=8_000_000),
               dict(borrow_inputs=True), dict(borrow_inputs=True, max_inflight_bases=4_000_000)):
        s = sa.Session(idx, refs, use_ssw=1, **kw)
        tickets = [s.submit(x, y) for x, y in reqs]
        for i, t in enumerate(tickets):
            data, st = s.wait(t)
            assert data == want[i], f"request {i} differs with {kw}"
            assert st["seconds_total"] >= st["seconds_service"] >= 0
            assert st["n_reads"] == (2 if reqs[i][1] is not None else 1) * REQUESTS[i][1]
        s.close()


def test_session_admission_by_free_device_memory(setup):
    # admission is bounded by the device memory free beyond the reserve: with a reserve
    # that leaves 2 GiB, requests are admitted in small groups and map to the
    # same bytes; with a reserve above the free memory, nothing can ever be admitted and
    # the request is refused (SA_ERR_BUSY) instead of waiting forever
    import torch
    sa, refs, idx, r1, r2 = setup
    reqs = _requests(sa, r1, r2)
    want = _alone(sa, refs, idx, reqs, use_ssw=1)
    free, _ = torch.cuda.mem_get_info()
    s = sa.Session(idx, refs, use_ssw=1, device_reserve_bytes=max(1, free - (2 << 30)))
    info = s.info
    assert info["device_reserve_bytes"] == max(1, free - (2 << 30))
    assert (1 << 24) <= info["arena_bases"] <= (1 << 33)
    tickets = [s.submit(x, y) for x, y in reqs]
    for i, t in enumerate(tickets):
        assert s.wait(t)[0] == want[i], f"request {i} differs under a reduced reserve"
    assert s.info["refused_requests"] == 0
    s.close()
    s = sa.Session(idx, refs, use_ssw=1, device_reserve_bytes=free + (64 << 30))
    t = s.submit(*reqs[0])
    with pytest.raises(sa.SaError) as e:
        s.wait(t)
    assert e.value.code == -9  # SA_ERR_BUSY
    assert s.info["refused_requests"] == 1
    s.close()
    # the default: the arena from free memory, and the reserve at least 2 GiB
    s = sa.Session(idx, refs)
    assert s.info["device_reserve_bytes"] >= (2 << 30) and s.info["arena_bases"] >= (1 << 24)
    s.close()


def test_session_rejects_oversized_and_unknown(setup):
    sa, refs, idx, r1, r2 = setup
    s = sa.Session(idx, refs, use_ssw=1, max_inflight_bases=100_000)
    big = _slice(sa, r1, 0, 1000)  # 150 kbases
    with pytest.raises(sa.SaError):
        s.submit(big, None)
    with pytest.raises(sa.SaError):
        s.poll(12345)
    t = s.submit(_slice(sa, r1, 0, 10), _slice(sa, r2, 0, 10))
    data, st = s.wait(t)
    assert data.count(b"\n") >= 20
    with pytest.raises(sa.SaError):
        s.wait(t)  # a ticket is released by the wait that returned its output
    s.close()


def test_session_abundance_mode_matches_mapper(setup):
    sa, refs, idx, r1, r2 = setup
    reqs = _requests(sa, r1, r2)[:5]
    m = sa.Mapper(idx, refs, mode=sa.MODE_ABUNDANCE)
    s = sa.Session(idx, refs, mode=sa.MODE_ABUNDANCE)
    tickets = [s.submit(x, y) for x, y in reqs]
    total = np.zeros(len(refs))
    for t, (x, y) in zip(tickets, reqs):
        _, _, ab = s.wait(t, abundances=True)
        total += ab
    for x, y in reqs:
        m.map(x, y)
    np.testing.assert_allclose(total, m.abundances(), rtol=1e-12, atol=0)
    s.close()


def test_session_comments_and_missing_qualities(setup):
    # FASTQ comments (--fastq-comments) and reads without qualities go through a
    # session's record copies as through the mapper
    sa, refs, idx, r1, r2 = setup
    n = 500
    seqs1 = [bytes(r1.seq[r1.offsets[i]:r1.offsets[i + 1]]) for i in range(n)]
    seqs2 = [bytes(r2.seq[r2.offsets[i]:r2.offsets[i + 1]]) for i in range(n)]
    names = [f"q{i}" for i in range(n)]
    comments = [f"BX:Z:{i % 7}" if i % 3 else "" for i in range(n)]
    a1 = sa.Reads.from_lists(names, seqs1, comments=comments)
    a2 = sa.Reads.from_lists(names, seqs2, comments=comments)
    for kw, skw in ((dict(fastq_comments=1), {}), (dict(), {}), (dict(fastq_comments=1), dict(borrow_inputs=True))):
        want = sa.Mapper(idx, refs, **kw).map(a1, a2)
        s = sa.Session(idx, refs, **skw, **kw)
        t = [s.submit(a1, a2), s.submit(a1, None)]
        got = [s.wait(x)[0] for x in t]
        assert got[0] == want
        assert got[1] == sa.Mapper(idx, refs, **kw).map(a1, None)
        s.close()
