"""The reference's own unit-test vectors (tests/golden/unit_vectors.json, extracted from
its Rust unit tests by tests/golden/extract_unit_vectors.py): exact scores, spans,
CIGARs and edit distances of the Hamming path, the piecewise-extension pieces, the
anchor pruning and extend_piecewise, plus the chaining, xxh64, pick_bits and
shared-substring known answers.

The CPU tests pin the oracle to them; the GPU tests run the same vectors through the
library's stage entry points (sa_hamming_batch, sa_piecewise_pieces,
sa_remove_spurious_anchors, sa_piecewise_batch, sa_align_batch), i.e. through the
device functions of the mapping path's extension kernels."""
import ctypes as C
import json

import numpy as np
import pytest

from conftest import GOLDEN
from oracle_lib import oracle

V = json.loads((GOLDEN / "unit_vectors.json").read_text())
PIECE_KIND = {"global": 0, "xdrop_GlobalStartLocalEnd": 1, "xdrop_LocalStartGlobalEnd": 2}
OPS = "MIDNSHP=X"


class OraStage(C.Structure):
    _fields_ = [("valid", C.c_int32), ("score", C.c_int32)] + [
        (n, C.c_uint32) for n in ("query_start", "query_end", "ref_start", "ref_end", "edit_distance", "cigar_len")]


def _lib():
    lib = oracle()
    lib.ora_xxh64.restype = C.c_uint64
    lib.ora_xxh64.argtypes = [C.c_uint64]
    lib.ora_pick_bits.restype = C.c_uint32
    lib.ora_pick_bits.argtypes = [C.c_char_p, C.c_uint32, C.c_uint32]
    lib.ora_hamming.argtypes = [C.c_int32, C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t, C.c_uint8, C.c_uint8,
                                C.c_uint32, C.POINTER(OraStage), C.POINTER(C.c_uint32), C.c_size_t]
    lib.ora_piece.argtypes = [C.c_int32, C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t, C.c_uint8, C.c_uint8,
                              C.c_uint8, C.c_uint8, C.c_uint32, C.POINTER(OraStage), C.POINTER(C.c_uint32),
                              C.c_size_t]
    lib.ora_remove_spurious_anchors.restype = C.c_uint32
    lib.ora_remove_spurious_anchors.argtypes = [C.POINTER(C.c_int32), C.c_uint32]
    lib.ora_extend_piecewise.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t, C.POINTER(C.c_uint32),
                                         C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint8, C.c_uint8, C.c_uint8,
                                         C.c_uint8, C.c_uint32, C.c_int32, C.c_int32, C.POINTER(OraStage),
                                         C.POINTER(C.c_uint32), C.c_size_t]
    lib.ora_chain_best_score.restype = C.c_float
    lib.ora_chain_best_score.argtypes = [C.POINTER(C.c_uint64), C.c_size_t, C.c_uint32, C.c_uint64]
    lib.ora_has_shared_substring.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t, C.c_uint32]
    return lib


def _result(o: OraStage, cig) -> dict | None:
    if not o.valid:
        return None
    return dict(score=o.score, query_start=o.query_start, query_end=o.query_end, ref_start=o.ref_start,
                ref_end=o.ref_end, edit_distance=o.edit_distance,
                cigar="".join(f"{cig[i] >> 4}{OPS[cig[i] & 15]}" for i in range(o.cigar_len)))


def _check(got: dict | None, expected: dict | None, name: str) -> None:
    if expected is None:
        assert got is None, f"{name}: expected None, got {got}"
        return
    assert got is not None, f"{name}: got None"
    for k, v in expected.items():
        g = got["ref_end"] - got["ref_start"] if k == "ref_span" else got[k]
        assert g == v, f"{name}: {k} = {g}, expected {v} ({got})"


def _pairs(case_anchors):
    """(query_start, ref_start) pairs in the given order (last to first)."""
    return [(a["query_start"], a["ref_start"]) for a in case_anchors]


# ------------------------------------------------------------------ oracle (CPU)

def test_oracle_xxh64_known_answer():
    for kat in V["xxh64"]:
        assert _lib().ora_xxh64(int(kat["input"], 16)) == int(kat["expected"], 16)


def test_pick_bits_phix():
    # the oracle and the library's host-side pick_bits (no device work)
    import strobealign_gb300 as sa
    for c in V["pick_bits"]:
        fa = str(GOLDEN / c["fasta"])
        assert _lib().ora_pick_bits(fa.encode(), c["k"], c["s"]) == c["expected"]
        p = sa.SeedingParameters.from_read_length(150)
        assert (p.k, p.s) == (c["k"], c["s"])
        assert sa.References.from_fasta(fa).pick_bits(p) == c["expected"]


def _ora_hamming(kind, c):
    cig = (C.c_uint32 * (len(c["query"]) + 8))()
    o = OraStage()
    q, r = c["query"].encode(), c["ref"].encode()
    assert _lib().ora_hamming(kind, q, len(q), r, len(r), c["match"], c["mismatch"], c.get("end_bonus", 0),
                              C.byref(o), cig, len(cig)) == 0
    return _result(o, cig)


def test_oracle_highest_scoring_segment():
    for c in V["highest_scoring_segment"]:
        got = _ora_hamming(0, c)
        s, e, sc = c["expected"]
        assert (got["query_start"], got["query_end"]) == (s, e), c
        if sc is not None:
            assert got["score"] == sc, c


def test_oracle_hamming_align():
    for c in V["hamming_align"]:
        _check(_ora_hamming(0, c), c["expected"], c["name"])
    for c in V["hamming_align_global"]:
        _check(_ora_hamming(1, c), c["expected"], c["name"])


def _ora_piece(c):
    s = c["scores"]
    q, r = c["query"].encode(), c["ref"].encode()
    cig = (C.c_uint32 * (len(q) + len(r) + 8))()
    o = OraStage()
    assert _lib().ora_piece(PIECE_KIND[c["kind"]], q, len(q), r, len(r), s["match"], s["mismatch"], s["gap_open"],
                            s["gap_extend"], s["end_bonus"], C.byref(o), cig, len(cig)) == 0
    return _result(o, cig)


def _ora_extend(c, prune):
    s = c["scores"]
    q, r = c["query"].encode(), c["ref"].encode()
    pairs = np.array(_pairs(c["anchors"]), dtype=np.uint32).reshape(-1)
    cig = (C.c_uint32 * (2 * len(q) + len(r) + 8))()
    o = OraStage()
    assert _lib().ora_extend_piecewise(q, len(q), r, len(r), pairs.ctypes.data_as(C.POINTER(C.c_uint32)),
                                       len(c["anchors"]), c["k"], c["padding"], s["match"], s["mismatch"],
                                       s["gap_open"], s["gap_extend"], s["end_bonus"], c["xdrop"], prune, C.byref(o),
                                       cig, len(cig)) == 0
    return _result(o, cig)


def _ora_prune(anchors):
    a = np.array(_pairs(anchors), dtype=np.int32).reshape(-1)
    n = _lib().ora_remove_spurious_anchors(a.ctypes.data_as(C.POINTER(C.c_int32)), len(anchors))
    return [(int(a[2 * i]), int(a[2 * i + 1])) for i in range(n)]


@pytest.mark.parametrize("case", V["piecewise"], ids=lambda c: c["name"])
def test_oracle_piecewise(case):
    if case["kind"] == "remove_spurious_anchors":
        assert _ora_prune(case["anchors"]) == _pairs(case["expected"])
    elif case["kind"] == "extend_piecewise":
        _check(_ora_extend(case, 0), case["expected"], case["name"])
        # the mapper prunes the chain first; these chains are unchanged by it
        assert _ora_extend(case, 1) == _ora_extend(case, 0)
    else:
        _check(_ora_piece(case), case["expected"], case["name"])


def _chain_best(c, n=None):
    an = c["anchors"][: n or len(c["anchors"])]
    t = np.array([[a["ref_id"], a["ref_start"], a["query_start"]] for a in an], dtype=np.uint64).reshape(-1)
    return _lib().ora_chain_best_score(t.ctypes.data_as(C.POINTER(C.c_uint64)), len(an), c["k"], c["max_ref_gap"])


def test_oracle_chaining():
    for c in V["chaining"]:
        if "best_score_above" in c:
            assert _chain_best(c) > c["best_score_above"], c["name"]
        if c.get("best_score_equals_k"):
            assert _chain_best(c) == np.float32(c["k"]), c["name"]
        if "linear_prefixes" in c:
            s1 = _chain_best(c, 1)
            for m in c["linear_prefixes"]:
                assert _chain_best(c, m) == np.float32(s1 * m), c["name"]


def test_oracle_has_shared_substring():
    for c in V["has_shared_substring"]:
        a, b = c["read"].encode(), c["ref"].encode()
        assert bool(_lib().ora_has_shared_substring(a, len(a), b, len(b), c["k"])) == c["expected"], c["name"]


def test_oracle_aligner_some_none():
    from oracle_lib import aligner_oracle
    for c in V["align"]:
        got = aligner_oracle(c["query"].encode(), c["ref"].encode())
        assert (got is not None) == c["some"], c["name"]


def test_fixture_counts():
    # every vector of the reference's test modules was extracted
    assert len(V["piecewise"]) == 30
    assert len(V["hamming_align"]) >= 8 and len(V["hamming_align_global"]) == 5
    assert len(V["highest_scoring_segment"]) >= 10 and len(V["chaining"]) == 3


# ------------------------------------------------------------------ GPU stage entry points

@pytest.fixture(scope="module")
def sa():
    import strobealign_gb300 as sa
    return sa


def _mp(sa, s: dict):
    return sa.mapping_defaults(match=s["match"], mismatch=s["mismatch"], gap_open=s.get("gap_open", 12),
                               gap_extend=s.get("gap_extend", 1), end_bonus=s.get("end_bonus", 0))


@pytest.mark.gpu
def test_gpu_hamming_vectors(sa):
    cases = [(0, c) for c in V["highest_scoring_segment"] + V["hamming_align"]] + \
            [(1, c) for c in V["hamming_align_global"]]
    for kind, c in cases:
        got = sa.hamming_batch([c["query"]], [c["ref"]], [kind], _mp(sa, c))[0]
        assert got == _ora_hamming(kind, c), c["name"]
        if "expected" in c and isinstance(c["expected"], dict):
            _check(got, c["expected"], c["name"])
        elif "expected" in c:
            s, e, sc = c["expected"]
            assert (got["query_start"], got["query_end"]) == (s, e) and (sc is None or got["score"] == sc), c


@pytest.mark.gpu
def test_gpu_hamming_batch_many(sa):
    # all cases in one launch, and random pairs against the oracle
    rng = np.random.default_rng(7)
    qs, rs, kinds, sc = [], [], [], []
    for _ in range(300):
        L = int(rng.integers(0, 300))
        q = "".join(rng.choice(list("ACGTN"), L))
        r = "".join(c if rng.random() > 0.1 else rng.choice(list("ACGT")) for c in q)
        qs.append(q)
        rs.append(r)
        kinds.append(int(rng.integers(0, 2)))
    got = sa.hamming_batch(qs, rs, kinds, sa.mapping_defaults(match=2, mismatch=8, end_bonus=10))
    for q, r, k, g in zip(qs, rs, kinds, got):
        assert g == _ora_hamming(k, dict(query=q, ref=r, match=2, mismatch=8, end_bonus=10))


@pytest.mark.gpu
@pytest.mark.parametrize("case", V["piecewise"], ids=lambda c: c["name"])
def test_gpu_piecewise_vectors(sa, case):
    if case["kind"] == "remove_spurious_anchors":
        got = sa.remove_spurious_anchors([_pairs(case["anchors"])])[0]
        assert got == _pairs(case["expected"])
        return
    mp = _mp(sa, case["scores"])
    if case["kind"] == "extend_piecewise":
        # the stage runs with the mapper's padding rule, |query| / 10
        assert case["padding"] == len(case["query"]) // 10
        got = sa.piecewise_batch([case["query"]], [case["ref"]], [_pairs(case["anchors"])], case["k"], mp)[0]
        _check(got, case["expected"], case["name"])
        assert got == _ora_extend(case, 1)
    else:
        got = sa.piecewise_pieces([case["query"]], [case["ref"]], [PIECE_KIND[case["kind"]]], mp)[0]
        _check(got, case["expected"], case["name"])
        assert got == _ora_piece(case)


@pytest.mark.gpu
def test_gpu_piecewise_random_against_oracle(sa):
    # random pieces and whole piecewise extensions (chains cut from a noisy copy of the
    # query) against the oracle's restatement, in single launches
    rng = np.random.default_rng(11)
    sc = {"match": 2, "mismatch": 8, "gap_open": 12, "gap_extend": 1, "end_bonus": 10}
    qs, rs, kinds = [], [], []
    for _ in range(200):
        q = "".join(rng.choice(list("ACGT"), int(rng.integers(1, 120))))
        r = list(q)
        for _ in range(int(rng.integers(0, 6))):
            p = int(rng.integers(0, max(1, len(r))))
            op = rng.integers(0, 3)
            if op == 0 and r:
                r[min(p, len(r) - 1)] = rng.choice(list("ACGT"))
            elif op == 1:
                r.insert(p, rng.choice(list("ACGT")))
            elif r:
                del r[min(p, len(r) - 1)]
        r = "".join(r) or "A"
        qs.append(q)
        rs.append(r)
        kinds.append(int(rng.integers(0, 3)))
    got = sa.piecewise_pieces(qs, rs, kinds, _mp(sa, sc))
    for q, r, k, g in zip(qs, rs, kinds, got):
        want = _ora_piece(dict(query=q, ref=r, kind={0: "global", 1: "xdrop_GlobalStartLocalEnd",
                                                      2: "xdrop_LocalStartGlobalEnd"}[k], scores=sc))
        assert g == want, (q, r, k)
    k = 15
    Q, R, A = [], [], []
    cases = []
    for _ in range(150):
        L = int(rng.integers(60, 300))
        q = "".join(rng.choice(list("ACGT"), L))
        lead = "".join(rng.choice(list("ACGT"), int(rng.integers(0, 30))))
        body = list(q)
        for _ in range(int(rng.integers(0, 4))):
            p = int(rng.integers(0, len(body)))
            body[p] = rng.choice(list("ACGT"))
        cut = int(rng.integers(20, L - 20))
        ins = int(rng.integers(0, 4))
        ref = lead + "".join(body[:cut]) + "".join(rng.choice(list("ACGT"), ins)) + "".join(body[cut:]) + \
            "".join(rng.choice(list("ACGT"), int(rng.integers(0, 30))))
        # exact k-mer anchors along the diagonal(s), last to first
        anchors = []
        for qs_ in range(0, L - k + 1, int(rng.integers(8, 30))):
            rs_ = len(lead) + qs_ + (ins if qs_ >= cut else 0)
            if q[qs_:qs_ + k] == ref[rs_:rs_ + k] and (qs_ + k <= cut or qs_ >= cut):
                anchors.append((qs_, rs_))
        if not anchors:
            continue
        anchors.reverse()
        Q.append(q)
        R.append(ref)
        A.append(anchors)
        cases.append(dict(query=q, ref=ref, anchors=[dict(ref_id=0, ref_start=b, query_start=a) for a, b in anchors],
                          k=k, padding=L // 10, xdrop=500, scores=sc))
    got = sa.piecewise_batch(Q, R, A, k, _mp(sa, sc))
    for c, g in zip(cases, got):
        assert g == _ora_extend(c, 1), c


@pytest.mark.gpu
def test_gpu_aligner_some_none(sa):
    got = sa.align_batch([c["query"] for c in V["align"]], [c["ref"] for c in V["align"]])
    for c, g in zip(V["align"], got):
        assert (g is not None) == c["some"], c["name"]


def test_stage_entry_points_reject_bad_input(sa):
    # argument errors are reported before any device work
    with pytest.raises(sa.SaError):
        sa.piecewise_batch(["ACGTACGTAC"], ["ACGTACGTAC"], [[(8, 0)]], 5)  # anchor past the query end
    with pytest.raises(sa.SaError):
        sa.piecewise_batch(["ACGTACGTAC"], ["ACGTACGTAC"], [[]], 5)  # no anchors
    with pytest.raises(sa.SaError):
        sa.hamming_batch(["ACGT"], ["ACGT"], [2])


def test_oracle_pair_helpers():
    # src/mapper.rs tests: is_proper_pair_within_distance, _rev_within_distance,
    # _incompatible, _too_far (mu 300, sigma 50), deduplicate_scored_pairs_works,
    # count_best_alignment_pairs_works
    lib = oracle()
    lib.ora_is_proper_pair.restype = C.c_int32
    lib.ora_is_proper_pair.argtypes = [C.c_uint64, C.c_uint64, C.c_int32, C.c_uint64, C.c_uint64, C.c_int32,
                                       C.c_float, C.c_float]
    proper = lambda a, b: lib.ora_is_proper_pair(a[0], a[1], a[2], b[0], b[1], b[2], 300.0, 50.0) == 1
    assert proper((0, 100, False), (0, 350, True))
    assert proper((0, 350, True), (0, 100, False))
    assert not proper((0, 100, False), (0, 350, False))
    assert not proper((0, 100, False), (0, 10_000, True))
    d = C.POINTER(C.c_double)
    i64 = C.POINTER(C.c_int64)
    lib.ora_deduplicate_scored_pairs.restype = C.c_size_t
    lib.ora_deduplicate_scored_pairs.argtypes = [C.c_size_t, d, i64, i64, i64, i64, d]

    def dedup(rows):
        n = len(rows)
        arr = lambda k, t: (t * n)(*[r[k] for r in rows])
        out = (C.c_double * max(n, 1))()
        m = lib.ora_deduplicate_scored_pairs(n, arr(0, C.c_double), arr(1, C.c_int64), arr(2, C.c_int64),
                                             arr(3, C.c_int64), arr(4, C.c_int64), out)
        return list(out[:m])

    assert dedup([(733.0, 0, 1906, 0, 123), (724.0, 0, 1906, 0, 123)]) == [733.0]
    # consecutive duplicates only, compared with the last kept pair; an absent mate
    # matches only an absent mate
    assert dedup([(9.0, 0, 5, 0, 9), (8.0, 0, 5, 0, 9), (7.0, 0, 6, 0, 9), (6.0, 0, 5, 0, 9),
                  (5.0, 0, 5, -1, -1), (4.0, 0, 5, -1, -1)]) == [9.0, 7.0, 6.0, 5.0]
    lib.ora_count_best_alignment_pairs.restype = C.c_size_t
    lib.ora_count_best_alignment_pairs.argtypes = [C.c_size_t, d]
    best = lambda s: lib.ora_count_best_alignment_pairs(len(s), (C.c_double * max(len(s), 1))(*s))
    assert [best([]), best([10.0]), best([10.0, 10.0]), best([10.0, 10.0, 5.0]), best([10.0, 5.0, 5.0])] == \
        [0, 1, 2, 2, 1]
