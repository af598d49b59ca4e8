"""Interleaved input on the GPU: sa_map_batch_interleaved and sa_map_files with
interleaved input map mixed single-end and paired-end records (paired by name as
src/io/reads.rs:68-113 pairs them) to the oracle's --interleaved bytes; phiX mates
interleaved in one file give the reference's paired-end golden; a streamed mixed file
gives the bytes of one batch; a serving session's mixed requests give the mapper's
bytes."""
import gzip
import random

import pytest

from conftest import GOLDEN
from oracle_lib import run_oracle_cli

pytestmark = pytest.mark.gpu


def _records(path):
    lines = open(path, "rb").read().splitlines(keepends=True)
    return [b"".join(lines[i:i + 4]) for i in range(0, len(lines), 4)]


def _first_diff(a: bytes, b: bytes) -> str:
    la, lb = a.splitlines(), b.splitlines()
    for i in range(min(len(la), len(lb))):
        if la[i] != lb[i]:
            return f"line {i}:\n gpu    {la[i][:300]!r}\n oracle {lb[i][:300]!r}"
    return f"lengths {len(la)} vs {len(lb)}"


@pytest.fixture(scope="module")
def mixed(tmp_path_factory):
    import strobealign_gb300 as sa
    from strobealign_gb300 import synthetic as syn
    d = tmp_path_factory.mktemp("interleaved")
    g = syn.make_genome(71, 400_000, 3, gc=0.41, segdup_fraction=0.10, repeat_fraction=0.1)
    fa = str(d / "ref.fa")
    g.write_fasta(fa)
    r1, r2 = syn.make_paired_end(72, g, 2500, 150, 300, 30, 0.01, 0.002, rescue_fraction=0.03)
    se = syn.make_single_end(73, g, 1500, (50, 400), 0.015, 0.002)
    r1.write_fastq(str(d / "r1.fq"))
    r2.write_fastq(str(d / "r2.fq"))
    se.write_fastq(str(d / "se.fq"))
    p1, p2, s1 = _records(d / "r1.fq"), _records(d / "r2.fq"), _records(d / "se.fq")
    rnd = random.Random(74)
    out, i, j = [], 0, 0
    while i < len(p1) or j < len(s1):
        if j == len(s1) or (i < len(p1) and rnd.random() < 0.62):
            out += [p1[i], p2[i]]
            i += 1
        else:
            out.append(s1[j])
            j += 1
    f = str(d / "mixed.fq")
    open(f, "wb").write(b"".join(out))
    data = b"".join(out)
    cut = len(data) // 2
    open(f + ".gz", "wb").write(gzip.compress(data[:cut], 1) + gzip.compress(data[cut:], 6))
    refs = sa.References.from_fasta(fa)
    idx = sa.StrobemerIndex.build(refs, sa.SeedingParameters.from_read_length(150))
    return dict(sa=sa, refs=refs, idx=idx, fa=fa, f=f, dir=d, records=len(p1) + len(s1), reads=len(out))


def _map(s, **kw):
    sa = s["sa"]
    m = sa.Mapper(s["idx"], s["refs"], **kw)
    return m.map_interleaved(sa.Reads.from_file(s["f"])), m


@pytest.mark.parametrize("chunk_size", [1_000_000, 20_000])
@pytest.mark.parametrize("ssw", [False, True])
def test_mixed_sam_matches_oracle(mixed, chunk_size, ssw):
    s, sa = mixed, mixed["sa"]
    args = ["--no-PG", "--eqx", "--interleaved", "-r", "150", f"--chunk-size={chunk_size}"]
    want = run_oracle_cli([*args, *(["--ssw"] if ssw else []), s["fa"], s["f"]])
    body, m = _map(s, eqx=1, use_ssw=int(ssw), chunk_size=chunk_size)
    got = sa.sam_header(s["refs"]) + body
    assert m.last["n_reads"] == s["reads"]
    assert got == want, _first_diff(got, want)


def test_mixed_paf_and_abundances_match_oracle(mixed):
    s, sa = mixed, mixed["sa"]
    want = run_oracle_cli(["-x", "--interleaved", "-r", "150", s["fa"], s["f"]])
    got, _ = _map(s, mode=sa.MODE_PAF)
    assert got == want, _first_diff(got, want)
    want = run_oracle_cli(["--aemb", "--interleaved", "-r", "150", s["fa"], s["f"]])
    _, m = _map(s, mode=sa.MODE_ABUNDANCE)
    names = [l[1:].split()[0].decode() for l in open(s["fa"], "rb") if l.startswith(b">")]
    assert "".join(f"{n}\t{a:.6f}\n" for n, a in zip(names, m.abundances())).encode() == want


def test_phix_mates_interleaved_give_paired_end_golden(tmp_path):
    import strobealign_gb300 as sa
    r1, r2 = _records(GOLDEN / "phix.1.fastq"), _records(GOLDEN / "phix.2.fastq")
    f = tmp_path / "il.fq"
    f.write_bytes(b"".join(a + b for a, b in zip(r1, r2)))
    refs = sa.References.from_fasta(str(GOLDEN / "phix.fasta"))
    first = sa.Reads.from_file(str(GOLDEN / "phix.1.fastq"))
    n = min(500, len(first))
    idx = sa.StrobemerIndex.build(refs, sa.SeedingParameters.from_read_length(int(first.seq_offsets[n] // n)))
    m = sa.Mapper(idx, refs, eqx=1, rg_id="1")
    got = sa.sam_header(refs, rg_id="1", rg_fields=["SM:sample", "LB:library"]) + \
        m.map_interleaved(sa.Reads.from_file(str(f)))
    assert got == (GOLDEN / "phix.pe.sam").read_bytes()


@pytest.mark.parametrize("gz", [False, True])
def test_map_files_interleaved_matches_one_batch(mixed, gz):
    s, sa = mixed, mixed["sa"]
    want, _ = _map(s, chunk_size=40_000)
    head = sa.sam_header(s["refs"])
    for batch_bases in (1, 150_000, 0):
        m = sa.Mapper(s["idx"], s["refs"], chunk_size=40_000)
        out = str(s["dir"] / f"out_{gz}_{batch_bases}.sam")
        st = m.map_files(s["f"] + (".gz" if gz else ""), None, out, header=head, batch_bases=batch_bases,
                         interleaved=True)
        got = open(out, "rb").read()
        assert got == head + want, _first_diff(got, head + want)
        assert st["n_records"] == s["records"] and st["n_reads"] == s["reads"]
        if batch_bases == 1:
            assert st["n_batches"] > 10
        if batch_bases == 0:
            assert st["n_batches"] == 1


def test_map_files_interleaved_takes_one_file(mixed):
    s, sa = mixed, mixed["sa"]
    m = sa.Mapper(s["idx"], s["refs"])
    with pytest.raises(sa.SaError, match="one reads file"):
        m.map_files(s["f"], s["f"], str(s["dir"] / "x.sam"), interleaved=True)


@pytest.mark.parametrize("kw", [dict(eqx=1), dict(use_ssw=1, chunk_size=30_000, borrow_inputs=True)])
def test_session_interleaved_requests(mixed, kw):
    # mixed requests beside paired-end and single-end ones: each request's bytes equal
    # the mapper's on the same records alone
    s, sa = mixed, mixed["sa"]
    kw = dict(kw)
    borrow = kw.pop("borrow_inputs", False)
    reads = sa.Reads.from_file(s["f"])
    r1 = sa.Reads.from_file(str(s["dir"] / "r1.fq"))
    r2 = sa.Reads.from_file(str(s["dir"] / "r2.fq"))
    se = sa.Reads.from_file(str(s["dir"] / "se.fq"))
    m = sa.Mapper(s["idx"], s["refs"], **kw)
    want = [m.map_interleaved(reads), m.map(r1, r2), m.map(se), m.map_interleaved(reads)]
    sess = sa.Session(s["idx"], s["refs"], borrow_inputs=borrow, **kw)
    tickets = [sess.submit_interleaved(reads), sess.submit(r1, r2), sess.submit(se), sess.submit_interleaved(reads)]
    got = [sess.wait(t)[0] for t in tickets]
    for i, (g, w) in enumerate(zip(got, want)):
        assert g == w, f"request {i} differs: " + _first_diff(g, w)
