"""GPU parity: each stage of the CUDA path against the oracle, and whole-run SAM /
PAF / abundance bytes against the reference's goldens and the oracle."""
import os
import random
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN
from oracle_lib import OracleIndex, aligner_oracle, randstrobes_oracle, run_oracle_cli

pytestmark = pytest.mark.gpu

RG = ["--rg-id=1", "--rg=SM:sample", "--rg=LB:library"]


@pytest.fixture(scope="module")
def sa():
    import strobealign_gb300 as sa
    return sa


@pytest.fixture(scope="module")
def synth(tmp_path_factory):
    from strobealign_gb300 import synthetic as syn
    d = tmp_path_factory.mktemp("synth")
    g = syn.make_genome(21, 400_000, 3, gc=0.41, segdup_fraction=0.10, segdup_div=0.02)
    fa = str(d / "ref.fa")
    g.write_fasta(fa)
    r1, r2 = syn.make_paired_end(22, g, 3000, 150, 300, 30, 0.01, 0.002, rescue_fraction=0.03)
    f1, f2 = str(d / "r1.fq"), str(d / "r2.fq")
    r1.write_fastq(f1)
    r2.write_fastq(f2)
    se = syn.make_single_end(23, g, 2000, (50, 500), 0.015, 0.002)
    fse = str(d / "se.fq")
    se.write_fastq(fse)
    return dict(dir=d, fa=fa, f1=f1, f2=f2, fse=fse, genome=g)


@pytest.fixture(scope="module")
def repeats(tmp_path_factory):
    # many-copy families and tandem arrays: hashes above the repeat cutoff, buckets of
    # hundreds of entries, local and global seed rescue, long rescue chains
    from strobealign_gb300 import synthetic as syn
    d = tmp_path_factory.mktemp("repeats")
    g = syn.make_genome(31, 300_000, 2, gc=0.41, repeat_fraction=0.5, family_len=(300, 500),
                        family_div=(0.0, 0.02), tandem_fraction=0.05)
    fa = str(d / "ref.fa")
    g.write_fasta(fa)
    r1, r2 = syn.make_paired_end(32, g, 3000, 150, 300, 30, 0.01, 0.002, rescue_fraction=0.05)
    f1, f2 = str(d / "r1.fq"), str(d / "r2.fq")
    r1.write_fastq(f1)
    r2.write_fastq(f2)
    return dict(dir=d, fa=fa, f1=f1, f2=f2, genome=g)


def _index(sa, fa, read_length=150):
    refs = sa.References.from_fasta(fa)
    p = sa.SeedingParameters.from_read_length(read_length)
    return refs, sa.StrobemerIndex.build(refs, p)


@pytest.mark.parametrize("which,read_length", [("phix", 150), ("phix", 300), ("synth", 150), ("synth", 250)])
def test_index_identical_to_oracle(sa, synth, which, read_length):
    fa = str(GOLDEN / "phix.fasta") if which == "phix" else synth["fa"]
    refs, idx = _index(sa, fa, read_length)
    rs, bs = idx.to_host()
    o = OracleIndex(fa, read_length)
    ors, obs = o.arrays()
    n, bits, cutoff = o.info()
    assert idx.bits == bits and idx.filter_cutoff == cutoff and len(rs) == n
    assert (rs["hash_offset"] == ors["hash_offset"]).all()
    assert (rs["position"] == ors["position"]).all() and (rs["ref_index"] == ors["ref_index"]).all()
    assert (bs == obs).all()


def test_index_lookups(sa, synth):
    # get_full_forward / get_count (src/index.rs:159-197, 272-295) restated over the
    # host copy of the table and its bucket directory
    refs, idx = _index(sa, synth["fa"])
    rs, bs = idx.to_host()
    h = rs["hash_offset"] & np.uint64(0xFFFFFFFFFFFFFF00)
    bits = idx.bits
    rng = np.random.default_rng(5)
    q = np.concatenate([h[rng.integers(0, len(h), 2000)], rng.integers(0, 2**63, 2000, dtype=np.uint64)])
    pos, cnt = idx.lookup(q, kind=0, counts=True)
    for x, p, c in zip(q, pos, cnt):
        top = int(x) >> (64 - bits)
        ps, pe = int(bs[top]), int(bs[top + 1])
        seg = h[ps:pe]
        i = int(np.searchsorted(seg, x, side="left"))
        if i < len(seg) and seg[i] == x:
            assert p == ps + i
            top2 = int(h[p]) >> (64 - bits)
            end = int(bs[top2 + 1])
            assert c == int(np.searchsorted(h[p:end], x, side="right"))
        else:
            assert p == -1


def _reads_with_edge_cases(synth):
    rnd = random.Random(3)
    g = synth["genome"].seqs[0].tobytes()
    names, seqs = [], []
    for i in range(300):
        L = rnd.choice([0, 5, 10, 15, 20, 21, 30, 50, 100, 150, 151, 250, 500, 1000])
        p = rnd.randint(0, len(g) - L - 1)
        s = bytearray(g[p:p + L])
        if rnd.random() < 0.3 and L > 4:
            for _ in range(rnd.randint(1, 3)):
                s[rnd.randrange(L)] = ord("N")
        if rnd.random() < 0.1 and L:
            s = bytearray(b"A" * L)  # homopolymer: every window is a syncmer
        names.append(f"e{i}")
        seqs.append(bytes(s))
    return names, seqs


@pytest.mark.parametrize("read_length", [150, 250])
def test_randstrobes_identical_to_oracle(sa, synth, read_length):
    refs, idx = _index(sa, synth["fa"], read_length)
    names, seqs = _reads_with_edge_cases(synth)
    got = sa.randstrobes_batch(idx, sa.Reads.from_lists(names, seqs))
    for s, (f, r) in zip(seqs, got):
        of, orc = randstrobes_oracle(s, read_length)
        for a, b in ((f, of), (r, orc)):
            assert len(a) == len(b), s
            if len(a):
                assert (a["hash"] == b[:, 0]).all() and (a["hash_revcomp"] == b[:, 1]).all()
                assert (a["start"] == b[:, 2]).all() and (a["end"] == b[:, 3]).all()


def _nam_rows(arr):
    return [(int(x["nam_id"]), int(x["ref_id"]), int(x["ref_start"]), int(x["ref_end"]), int(x["query_start"]),
             int(x["query_end"]), int(x["matching_bases"]), int(x["n_anchors"]),
             np.float32(x["score"]).view(np.uint32), int(x["is_revcomp"])) for x in arr]


@pytest.mark.parametrize("genome", ["synth", "repeats"])
@pytest.mark.parametrize("mcs", ["always", "rescue", "off", "first-strobe"])
def test_nams_identical_to_oracle(sa, synth, repeats, mcs, genome):
    src = synth if genome == "synth" else repeats
    refs, idx = _index(sa, src["fa"])
    reads = sa.Reads.from_file(src["f1"])
    names, seqs = _reads_with_edge_cases(src)
    batch_seqs = [reads.seq[reads.seq_offsets[i]:reads.seq_offsets[i + 1]] for i in range(600)] + seqs
    rb = sa.Reads.from_lists([f"n{i}" for i in range(len(batch_seqs))], batch_seqs)
    nams, det = sa.nams_batch(idx, rb, mapping=sa.mapping_defaults(mcs_strategy=mcs))
    o = OracleIndex(src["fa"], 150)
    mcs_i = sa.MCS[mcs]
    for i, s in enumerate(batch_seqs):
        rows, od = o.nams(bytes(s), mcs_i)
        want = [r[:8] + (np.float32(r[8]).view(np.uint32), r[9]) for r in rows]
        assert _nam_rows(nams[i]) == want, (i, s)
        for k, v in od.items():
            assert det[i][k] == v, (i, k)


# the longest query of a batch picks the striped kernel variant (rows per lane); the
# scores cover the defaults, equal gap penalties (the library's lazy-F loop then stops
# after each lane's first row) and a larger gap extension
@pytest.mark.parametrize("max_len,scores", [(64, None), (160, None), (192, None), (256, None), (500, None),
                                            (160, (2, 4, 2, 2)), (500, (2, 4, 2, 2)), (160, (3, 5, 6, 2))])
def test_align_batch_identical_to_oracle(sa, max_len, scores):
    rnd = random.Random(11 + max_len)
    qs, rs = [], []
    lengths = [x for x in (1, 10, 17, 50, 64, 100, 127, 150, 160, 191, 192, 200, 256, 300, 500) if x <= max_len]
    for _ in range(1500):
        L = rnd.choice(lengths)
        q = bytes(rnd.choice(b"ACGT") for _ in range(L))
        if rnd.random() < 0.1 and L > 3:
            q = q[:L // 2] + b"N" + q[L // 2 + 1:]
        core = bytearray()
        for c in q:
            x = rnd.random()
            if x < 0.03:
                core.append(rnd.choice(b"ACGT"))
            elif x < 0.04:
                pass
            elif x < 0.05:
                core += bytes([c, rnd.choice(b"ACGT")])
            else:
                core.append(c)
        # wide flanks make windows like mate rescue's (read + 450 nt)
        fl = 300 if rnd.random() < 0.2 else 30
        r = bytes(rnd.choice(b"ACGT") for _ in range(rnd.randint(0, fl))) + bytes(core) + \
            bytes(rnd.choice(b"ACGT") for _ in range(rnd.randint(0, fl)))
        if rnd.random() < 0.05:
            r = bytes(rnd.choice(b"ACGT") for _ in range(rnd.randint(1, 80)))
        qs.append(q)
        rs.append(r)
    mp = None
    kw = {}
    if scores is not None:
        mp = sa.mapping_defaults()
        mp.match, mp.mismatch, mp.gap_open, mp.gap_extend = scores
        kw = dict(match=scores[0], mismatch=scores[1], go=scores[2], ge=scores[3])
    got = sa.align_batch(qs, rs, mp)
    for q, r, g in zip(qs, rs, got):
        assert g == aligner_oracle(q, r, **kw), (q, r)


def _map_files(sa, fa, files, read_length=None, header=True, **kw):
    refs = sa.References.from_fasta(fa)
    r1 = sa.Reads.from_file(files[0])
    if read_length is None:
        n = min(500, len(r1))
        read_length = int(r1.seq_offsets[n] // n) if n else 0
    idx = sa.StrobemerIndex.build(refs, sa.SeedingParameters.from_read_length(read_length))
    rg = kw.pop("rg", None)
    m = sa.Mapper(idx, refs, **kw)
    r2 = sa.Reads.from_file(files[1]) if len(files) > 1 else None
    body = m.map(r1, r2)
    if kw.get("mode", 0) == sa.MODE_ABUNDANCE:
        ab = m.abundances()
        return "".join(f"{n}\t{a:.6f}\n" for n, a in zip(_fasta_names(fa), ab)).encode()
    if header and kw.get("mode", 0) == sa.MODE_SAM:
        return sa.sam_header(refs, rg_id=rg[0] if rg else None, rg_fields=rg[1] if rg else ()) + body
    return body


def _fasta_names(fa):
    return [l[1:].split()[0].decode() for l in open(fa, "rb") if l.startswith(b">")]


def _fasta_lengths(fa):
    seqs, cur = [], None
    for l in open(fa, "rb"):
        if l.startswith(b">"):
            cur = []
            seqs.append(cur)
        else:
            cur.append(l.strip())
    return [b"".join(c) for c in seqs]


def test_phix_paired_end_golden(sa):
    got = _map_files(sa, str(GOLDEN / "phix.fasta"), [str(GOLDEN / "phix.1.fastq"), str(GOLDEN / "phix.2.fastq")],
                     eqx=1, rg_id="1", rg=("1", ["SM:sample", "LB:library"]))
    assert got == (GOLDEN / "phix.pe.sam").read_bytes()


def test_phix_tags_golden(sa):
    got = _map_files(sa, str(GOLDEN / "phix.fasta"), [str(GOLDEN / "phix.tags.fastq")], use_ssw=1,
                     fastq_comments=1, rg_id="1", rg=("1", ["SM:sample", "LB:library"]))
    assert got == (GOLDEN / "phix.tags.sam").read_bytes()


def test_phix_single_end_ssw_matches_oracle(sa):
    want = run_oracle_cli(["--chunk-size=3", "--no-PG", "--eqx", "--ssw", "phix.fasta", "phix.1.fastq"], cwd=GOLDEN)
    got = _map_files(sa, str(GOLDEN / "phix.fasta"), [str(GOLDEN / "phix.1.fastq")], eqx=1, use_ssw=1, chunk_size=3)
    assert got == want


def test_phix_single_end_golden(sa):
    # single-end without --ssw: piecewise extension on the NAM's anchors
    got = _map_files(sa, str(GOLDEN / "phix.fasta"), [str(GOLDEN / "phix.1.fastq")], eqx=1, chunk_size=3, rg_id="1",
                     rg=("1", ["SM:sample", "LB:library"]))
    assert got == (GOLDEN / "phix.se.sam").read_bytes()


def test_phix_paf_and_abundance_goldens(sa):
    got = _map_files(sa, str(GOLDEN / "phix.fasta"), [str(GOLDEN / "phix.1.fastq")], mode=sa.MODE_PAF)
    assert b"".join(got.splitlines(keepends=True)[-11:]) == (GOLDEN / "phix.se.paf").read_bytes()
    got = _map_files(sa, str(GOLDEN / "phix.fasta"), [str(GOLDEN / "phix.1.fastq")], mode=sa.MODE_PAF,
                     mcs_strategy="rescue")
    assert b"".join(got.splitlines(keepends=True)[-11:]) == (GOLDEN / "phix.mcsrescue.se.paf").read_bytes()
    got = _map_files(sa, str(GOLDEN / "phix.fasta"), [str(GOLDEN / "phix.1.fastq")], mode=sa.MODE_ABUNDANCE)
    assert got == (GOLDEN / "phix.abun.se.txt").read_bytes()
    got = _map_files(sa, str(GOLDEN / "phix.fasta"), [str(GOLDEN / "phix.1.fastq"), str(GOLDEN / "phix.2.fastq")],
                     mode=sa.MODE_ABUNDANCE)
    assert got == (GOLDEN / "phix.abun.pe.txt").read_bytes()


def _first_diff(a: bytes, b: bytes) -> str:
    la, lb = a.splitlines(), b.splitlines()
    for i in range(min(len(la), len(lb))):
        if la[i] != lb[i]:
            return f"line {i}:\n gpu    {la[i][:300]!r}\n oracle {lb[i][:300]!r}"
    return f"lengths {len(la)} vs {len(lb)}"


def test_synthetic_paired_end_sam_matches_oracle(sa, synth):
    want = run_oracle_cli(["--no-PG", "--eqx", synth["fa"], synth["f1"], synth["f2"]])
    got = _map_files(sa, synth["fa"], [synth["f1"], synth["f2"]], eqx=1)
    assert got == want, _first_diff(got, want)


def test_repetitive_paired_end_sam_matches_oracle(sa, repeats):
    want = run_oracle_cli(["--no-PG", "--eqx", repeats["fa"], repeats["f1"], repeats["f2"]])
    got = _map_files(sa, repeats["fa"], [repeats["f1"], repeats["f2"]], eqx=1)
    assert got == want, _first_diff(got, want)


def test_mapping_is_independent_of_parts(sa, synth):
    # a batch cut into NAM-pipeline parts (runs of whole chunks) maps to the same bytes
    # as the whole batch in one part, and an empty batch maps to nothing
    refs, idx = _index(sa, synth["fa"])
    r1 = sa.Reads.from_file(synth["f1"])
    r2 = sa.Reads.from_file(synth["f2"])
    outs = []
    for parts in (1, 2, 5):
        m = sa.Mapper(idx, refs, chunk_size=20000, eqx=1)
        m.set_parts(parts)
        outs.append(m.map(r1, r2))
    assert outs[0] == outs[1] == outs[2] and len(outs[0]) > 0
    empty = sa.Reads.from_lists([], [])
    assert sa.Mapper(idx, refs).map(empty, empty) == b""


def test_plain_schedule_matches_batched_engine(sa, synth):
    # the stage-synchronous form (overlap = 0: NAM parts one after another, then policy
    # and waves taking turns, small waves) maps to the same bytes as the batched engine
    # and the oracle, paired-end and single-end
    refs, idx = _index(sa, synth["fa"])
    r1 = sa.Reads.from_file(synth["f1"])
    r2 = sa.Reads.from_file(synth["f2"])
    se = sa.Reads.from_file(synth["fse"])
    want = run_oracle_cli(["--no-PG", "--chunk-size=20000", synth["fa"], synth["f1"], synth["f2"]])
    want = want[len(sa.sam_header(refs)):]
    for r in ((r1, r2), (se, None)):
        outs = []
        for overlap, parts, max_wave in ((True, 4, 0), (False, 1, 0), (False, 3, 500)):
            m = sa.Mapper(idx, refs, chunk_size=20000)
            m.set_schedule(parts=parts, overlap=overlap, max_wave_jobs=max_wave)
            outs.append(m.map(*r))
            outs.append(m.map(*r))  # the same mapper again (pooled buffers)
        assert all(o == outs[0] for o in outs) and outs[0]
        if r[1] is not None:
            assert outs[0] == want, _first_diff(outs[0], want)


def test_tuning_knobs_do_not_change_output(sa, synth, repeats):
    # every tuning knob at an extreme: all clusters of long read orientations chained a
    # warp each (or a thread each), SSW tasks of reads over 64 nt a warp each, one part,
    # tiny waves; and the autotuner's choice -- all write the oracle's bytes
    for d in (synth, repeats):
        refs, idx = _index(sa, d["fa"])
        r1 = sa.Reads.from_file(d["f1"])
        r2 = sa.Reads.from_file(d["f2"])
        want = run_oracle_cli(["--no-PG", d["fa"], d["f1"], d["f2"]])[len(sa.sam_header(refs)):]
        for kw in (dict(chain_lane_cluster_max=1), dict(chain_lane_cluster_max=4096),
                   dict(ssw_wave_max_qlen=64, parts=1, max_wave_jobs=300, wave_min_jobs=1),
                   dict(l2_fetch_bytes=32), dict(l2_fetch_bytes=128)):
            m = sa.Mapper(idx, refs)
            m.set_tuning(**kw)
            got = m.map(r1, r2)
            assert got == want, (kw, _first_diff(got, want))
        m = sa.Mapper(idx, refs)
        rep = m.autotune(r1, r2, rounds=1)
        assert rep["trials"] >= 5 and rep["seconds_tuned"] <= rep["seconds_default"] * 1.0001
        assert m.tuning() == rep["chosen"]
        assert m.map_uploaded() == want
    with pytest.raises(sa.SaError):
        sa.Mapper(idx, refs).set_tuning(ssw_wave_max_qlen=500)
    with pytest.raises(sa.SaError):
        sa.Mapper(idx, refs).set_tuning(l2_fetch_bytes=48)
    # a mapper gives the context's fetch granularity back when it is set to 0
    m = sa.Mapper(idx, refs)
    m.set_tuning(l2_fetch_bytes=32)
    assert m.tuning()["l2_fetch_bytes"] == 32
    m.set_tuning(l2_fetch_bytes=0)
    assert m.tuning()["l2_fetch_bytes"] == 0


def test_synthetic_paired_end_small_chunks_matches_oracle(sa, synth):
    # many chunks: the per-chunk RNG and insert-size restarts are exercised
    want = run_oracle_cli(["--no-PG", "--chunk-size=20000", synth["fa"], synth["f1"], synth["f2"]])
    got = _map_files(sa, synth["fa"], [synth["f1"], synth["f2"]], chunk_size=20000)
    assert got == want, _first_diff(got, want)


def test_synthetic_single_end_ssw_matches_oracle(sa, synth):
    want = run_oracle_cli(["--no-PG", "--eqx", "--ssw", synth["fa"], synth["fse"]])
    got = _map_files(sa, synth["fa"], [synth["fse"]], eqx=1, use_ssw=1)
    assert got == want, _first_diff(got, want)


def test_synthetic_single_end_piecewise_matches_oracle(sa, synth):
    # piecewise extension (block-aligner in the reference) restated as full affine DPs:
    # parity with the oracle's restatement, unpinned beyond the reference's goldens
    want = run_oracle_cli(["--no-PG", "--eqx", synth["fa"], synth["fse"]])
    got = _map_files(sa, synth["fa"], [synth["fse"]], eqx=1)
    assert got == want, _first_diff(got, want)


def test_synthetic_paf_matches_oracle(sa, synth):
    want = run_oracle_cli(["-x", synth["fa"], synth["f1"], synth["f2"]])
    got = _map_files(sa, synth["fa"], [synth["f1"], synth["f2"]], mode=sa.MODE_PAF)
    assert got == want, _first_diff(got, want)
