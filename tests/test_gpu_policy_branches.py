"""GPU parity for the policy and format branches the default runs do not reach:
secondary alignments (-N), the --details SAM tags, reference FASTAs with wildcard and
IUPAC bases and lower case, and the index at the size where pick_bits gives 24 bits.
Each compares the library's output with the oracle's on the same input, byte for
byte; the secondary-alignment checks also restate the reference's own run.sh checks
(tests/run.sh:80-99)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle_lib import OracleIndex, run_oracle_cli

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sa():
    import strobealign_gb300 as sa
    return sa


def _map(sa, fa, files, read_length=None, **kw):
    refs = sa.References.from_fasta(fa)
    r1 = sa.Reads.from_file(files[0])
    if read_length is None:
        n = min(500, len(r1))
        read_length = int(r1.seq_offsets[n] // n) if n else 0
    idx = sa.StrobemerIndex.build(refs, sa.SeedingParameters.from_read_length(read_length))
    m = sa.Mapper(idx, refs, **kw)
    r2 = sa.Reads.from_file(files[1]) if len(files) > 1 else None
    return sa.sam_header(refs) + m.map(r1, r2)


def _diff(a: bytes, b: bytes) -> str:
    la, lb = a.split(b"\n"), b.split(b"\n")
    for i, (x, y) in enumerate(zip(la, lb)):
        if x != y:
            return f"line {i}:\n gpu    {x[:300]!r}\n oracle {y[:300]!r}"
    return f"lengths {len(la)} vs {len(lb)}"


def _secondary(sam: bytes) -> int:
    return sum(1 for line in sam.split(b"\n") if line and not line.startswith(b"@")
               and int(line.split(b"\t")[1]) & 0x100)


def _primary_only(sam: bytes) -> bytes:
    return b"".join(line + b"\n" for line in sam.split(b"\n") if line and
                    (line.startswith(b"@") or not int(line.split(b"\t")[1]) & 0x100))


@pytest.fixture(scope="module")
def repeated_phix(tmp_path_factory):
    # phiX followed by a second copy of itself under another name (tests/run.sh:88-91)
    d = tmp_path_factory.mktemp("rphix")
    src = (GOLDEN / "phix.fasta").read_bytes()
    body = src.split(b"\n", 1)[1]
    fa = d / "repeated-phix.fasta"
    fa.write_bytes(src + b">repeated_NC_001422\n" + body)
    return str(fa)


def test_secondary_alignments_phix(sa):
    fa, fq = str(GOLDEN / "phix.fasta"), str(GOLDEN / "phix.1.fastq")
    with_sec = _map(sa, fa, [fq], max_secondary=5)
    assert _secondary(with_sec) == 0
    assert with_sec == run_oracle_cli(["--no-PG", "-N", "5", fa, fq])


def test_secondary_alignments_repeated_phix(sa, repeated_phix):
    fq = str(GOLDEN / "phix.1.fastq")
    no_sec = _map(sa, repeated_phix, [fq])
    with_sec = _map(sa, repeated_phix, [fq], max_secondary=5)
    assert _secondary(with_sec) > 0
    # removing the secondary alignments gives the output without them
    assert _primary_only(with_sec) == no_sec
    want = run_oracle_cli(["--no-PG", "-N", "5", repeated_phix, fq])
    assert with_sec == want, _diff(with_sec, want)
    # single-end with SSW extension and paired-end, with secondaries
    want = run_oracle_cli(["--no-PG", "-N", "5", "--ssw", repeated_phix, fq])
    got = _map(sa, repeated_phix, [fq], max_secondary=5, use_ssw=1)
    assert got == want, _diff(got, want)
    fq2 = str(GOLDEN / "phix.2.fastq")
    want = run_oracle_cli(["--no-PG", "-N", "3", repeated_phix, fq, fq2])
    got = _map(sa, repeated_phix, [fq, fq2], max_secondary=3)
    assert got == want, _diff(got, want)


@pytest.fixture(scope="module")
def synth(tmp_path_factory):
    from strobealign_gb300 import synthetic as syn
    d = tmp_path_factory.mktemp("branches")
    g = syn.make_genome(41, 600_000, 3, gc=0.41, segdup_fraction=0.10, segdup_div=0.02, repeat_fraction=0.2,
                        family_len=(300, 1000), family_div=(0.02, 0.08))
    fa = str(d / "ref.fa")
    g.write_fasta(fa)
    r1, r2 = syn.make_paired_end(42, g, 2000, 150, 300, 30, 0.01, 0.002, rescue_fraction=0.03)
    f1, f2 = str(d / "r1.fq"), str(d / "r2.fq")
    r1.write_fastq(f1)
    r2.write_fastq(f2)
    se = syn.make_single_end(43, g, 1500, (60, 400), 0.015, 0.002)
    fse = str(d / "se.fq")
    se.write_fastq(fse)
    return dict(fa=fa, f1=f1, f2=f2, fse=fse, genome=g, dir=d)


def test_details_tags_paired_end(sa, synth):
    want = run_oracle_cli(["--no-PG", "--details", synth["fa"], synth["f1"], synth["f2"]])
    got = _map(sa, synth["fa"], [synth["f1"], synth["f2"]], details=1)
    assert b"\tna:i:" in got and b"\tmr:i:" in got
    assert got == want, _diff(got, want)


def test_details_tags_single_end(sa, synth):
    for extra, kw in ((["--ssw"], dict(use_ssw=1)), ([], {})):
        want = run_oracle_cli(["--no-PG", "--details", *extra, synth["fa"], synth["fse"]])
        got = _map(sa, synth["fa"], [synth["fse"]], details=1, **kw)
        assert b"\tna:i:" in got and b"\tmr:i:" not in got
        assert got == want, _diff(got, want)


def test_secondary_alignments_synthetic(sa, synth):
    want = run_oracle_cli(["--no-PG", "-N", "4", synth["fa"], synth["f1"], synth["f2"]])
    got = _map(sa, synth["fa"], [synth["f1"], synth["f2"]], max_secondary=4)
    assert got == want, _diff(got, want)
    want = run_oracle_cli(["--no-PG", "-N", "4", synth["fa"], synth["fse"]])
    got = _map(sa, synth["fa"], [synth["fse"]], max_secondary=4)
    assert got == want, _diff(got, want)


@pytest.fixture(scope="module")
def wildcard(tmp_path_factory, synth):
    # the synthetic genome with runs of N, single IUPAC codes and lower-case stretches;
    # reads sampled from it keep their wildcards as N
    rng = np.random.default_rng(51)
    d = tmp_path_factory.mktemp("wildcard")
    seqs = []
    for s in synth["genome"].seqs:
        a = s.copy()
        for _ in range(40):  # N runs of 1-60
            p = int(rng.integers(0, len(a) - 60))
            a[p:p + int(rng.integers(1, 61))] = ord("N")
        iupac = np.frombuffer(b"RYKMSWBDHVN", dtype=np.uint8)
        pos = rng.integers(0, len(a), 400)
        a[pos] = iupac[rng.integers(0, len(iupac), len(pos))]
        for _ in range(20):  # lower case
            p = int(rng.integers(0, len(a) - 500))
            a[p:p + 500] = np.frombuffer(a[p:p + 500].tobytes().lower(), dtype=np.uint8)
        seqs.append(a)
    fa = str(d / "wild.fa")
    with open(fa, "wb") as f:
        for i, s in enumerate(seqs):
            f.write(f">chr{i + 1} wildcard test\n".encode())
            b = s.tobytes()
            for j in range(0, len(b), 70):
                f.write(b[j:j + 70] + b"\n")
    # reads: fragments of the wildcard genome, wildcards written as N
    names, r1, r2 = [], [], []
    up = bytes.maketrans(b"acgtRYKMSWBDHVrykmswbdhvn", b"ACGTNNNNNNNNNNNNNNNNNNNNN")
    for i in range(1500):
        c = int(rng.integers(0, len(seqs)))
        s = seqs[c]
        p = int(rng.integers(0, len(s) - 400))
        frag = s[p:p + int(rng.integers(250, 400))].tobytes().translate(up)
        comp = bytes.maketrans(b"ACGTN", b"TGCAN")
        names.append(f"w{i}")
        r1.append(frag[:150])
        r2.append(frag[-150:].translate(comp)[::-1])
    f1, f2 = str(d / "w1.fq"), str(d / "w2.fq")
    for path, rs in ((f1, r1), (f2, r2)):
        with open(path, "wb") as f:
            for n, s in zip(names, rs):
                f.write(b"@" + n.encode() + b"\n" + s + b"\n+\n" + b"I" * len(s) + b"\n")
    return dict(fa=fa, f1=f1, f2=f2)


def test_wildcard_reference_index_identical_to_oracle(sa, wildcard):
    refs = sa.References.from_fasta(wildcard["fa"])
    idx = sa.StrobemerIndex.build(refs, sa.SeedingParameters.from_read_length(150))
    rs, bs = idx.to_host()
    o = OracleIndex(wildcard["fa"], 150)
    ors, obs = o.arrays()
    n, bits, cutoff = o.info()
    assert idx.bits == bits and idx.filter_cutoff == cutoff and len(rs) == n
    assert (rs.view(np.uint8) == ors.view(np.uint8)).all() and (bs == obs).all()


def test_wildcard_reference_sam_identical_to_oracle(sa, wildcard):
    want = run_oracle_cli(["--no-PG", "--eqx", wildcard["fa"], wildcard["f1"], wildcard["f2"]])
    got = _map(sa, wildcard["fa"], [wildcard["f1"], wildcard["f2"]], eqx=1)
    assert got == want, _diff(got, want)
    want = run_oracle_cli(["--no-PG", wildcard["fa"], wildcard["f1"]])
    got = _map(sa, wildcard["fa"], [wildcard["f1"]])
    assert got == want, _diff(got, want)


def test_index_identical_to_oracle_at_24_bits(sa):
    # 200 Mbp: pick_bits gives 24 (the size class of the uneven-length workload); the
    # bucket-0 quirk, the directory and the cutoff quantile at that size
    from oracle.binding import OracleIndex as MemIndex
    from strobealign_gb300 import synthetic as syn
    g = syn.make_genome(3, 200_000_000, 8, gc=0.41, repeat_fraction=0.20, family_len=(300, 6000),
                        family_div=(0.10, 0.20))
    refs = sa.References.from_sequences(g.names, [s.tobytes() for s in g.seqs])
    p = sa.SeedingParameters.from_read_length(150)
    idx = sa.StrobemerIndex.build(refs, p)
    assert idx.bits == 24
    gt, gd = idx.to_host()
    o = MemIndex(g.names, g.seqs, 150, threads=os.cpu_count() or 1)
    n, bits, cutoff = o.info()
    ot, od = o.arrays()
    assert (idx.bits, idx.filter_cutoff, len(gt)) == (bits, cutoff, n)
    assert np.array_equal(gd, od)
    assert np.array_equal(gt.view(np.uint8), ot.view(np.uint8))
