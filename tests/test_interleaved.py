"""Interleaved (mixed single-end / paired-end) input: the oracle and the library's
pairing, CPU only.

The pairing rule is the reference's InterleavedIterator (src/io/reads.rs:68-113) and its
unit tests (:178-225: tests/interleaved.fq gives six records, the first two pairs, the
third single-end; a/1 followed by a/2 is one pair named a).  A file that interleaves
phix.1.fastq and phix.2.fastq maps to the paired-end golden, phix.1.fastq alone to the
single-end golden, and a mixed file with one record per chunk to the records of the
paired-end and single-end runs in file order.  The library pairs reads
(sa_reads_pair_interleaved, the rule its interleaved mapping and streaming use) as the
reference's unit tests and a restatement of the rule on random names say.
"""
import random

import pytest

from conftest import GOLDEN
from oracle_lib import run_oracle_cli

RG = ["--rg-id=1", "--rg=SM:sample", "--rg=LB:library"]


def _records(path):
    lines = path.read_bytes().splitlines(keepends=True)
    return [b"".join(lines[i:i + 4]) for i in range(0, len(lines), 4)]


def _sam_body(out: bytes) -> list[bytes]:
    return [l for l in out.splitlines() if not l.startswith(b"@")]


def test_pairing_of_reference_interleaved_file():
    body = _sam_body(run_oracle_cli(["--interleaved", "phix.fasta", "interleaved.fq"], cwd=GOLDEN))
    names = [l.split(b"\t")[0] for l in body]
    flags = [int(l.split(b"\t")[1]) for l in body]
    # records: (.2, .2) (.3, .3) .13852607 .13852608 .13852609 .13852610
    assert names[:5] == [b"SRR4052021.2", b"SRR4052021.2", b"SRR4052021.3", b"SRR4052021.3",
                         b"SRR4052021.13852607"]
    assert all(f & 1 for f in flags[:4])
    assert flags[0] & 0x40 and flags[1] & 0x80
    assert not any(f & 1 for f in flags[4:])
    assert names[4:] == [b"SRR4052021.13852607", b"SRR4052021.13852608", b"SRR4052021.13852609",
                         b"SRR4052021.13852610"]
    seqs = {(n, f & 0xc0): l.split(b"\t")[9] for n, f, l in zip(names, flags, body)}
    # a mate that maps to the reverse strand is written reverse-complemented
    comp = bytes.maketrans(b"ACGTN", b"TGCAN")

    def fwd(n, bit):
        f = [x for x, nm in zip(flags, names) if nm == n and x & 0xc0 == bit][0]
        s = seqs[(n, bit)]
        return s.translate(comp)[::-1] if f & 0x10 else s

    assert fwd(b"SRR4052021.2", 0x40).startswith(b"GTCGCCCA")
    assert fwd(b"SRR4052021.2", 0x80).startswith(b"ATGTATTA")


def test_slash_suffixes_pair(tmp_path):
    (tmp_path / "a.fq").write_bytes(b"@a/1\nAACC\n+\n####\n@a/2\nGGTT\n+n\n####\n")
    (tmp_path / "ref.fa").write_bytes((GOLDEN / "phix.fasta").read_bytes())
    body = _sam_body(run_oracle_cli(["--interleaved", "ref.fa", "a.fq"], cwd=tmp_path))
    assert [l.split(b"\t")[0] for l in body] == [b"a", b"a"]
    assert [int(l.split(b"\t")[1]) for l in body] == [77, 141]


def test_interleaved_pairs_equal_two_files(tmp_path):
    r1, r2 = _records(GOLDEN / "phix.1.fastq"), _records(GOLDEN / "phix.2.fastq")
    (tmp_path / "il.fq").write_bytes(b"".join(a + b for a, b in zip(r1, r2)))
    (tmp_path / "phix.fasta").write_bytes((GOLDEN / "phix.fasta").read_bytes())
    # the read length comes from the first 500 records of the file, here both mates
    n = min(len(r1), 250)
    rl = sum(len(r.splitlines()[1]) for rr in zip(r1[:n], r2[:n]) for r in rr) // (2 * n)
    rl1 = sum(len(r.splitlines()[1]) for r in r1[:500]) // min(len(r1), 500)
    out = run_oracle_cli(["--interleaved", "--no-PG", "--eqx", *RG, "-r", str(rl1), "phix.fasta", "il.fq"],
                         cwd=tmp_path)
    assert out == (GOLDEN / "phix.pe.sam").read_bytes()
    # without -r the estimate covers both mates; the output is the paired-end run's at that length
    out_est = run_oracle_cli(["--interleaved", "--no-PG", "--eqx", *RG, "phix.fasta", "il.fq"], cwd=tmp_path)
    pe_at = run_oracle_cli(["--no-PG", "--eqx", *RG, "-r", str(rl), "phix.fasta", "phix.1.fastq", "phix.2.fastq"],
                           cwd=GOLDEN)
    assert out_est == pe_at


def test_interleaved_singles_equal_single_end():
    out = run_oracle_cli(["--interleaved", "--chunk-size=3", "--no-PG", "--eqx", *RG, "phix.fasta", "phix.1.fastq"],
                         cwd=GOLDEN)
    assert out == (GOLDEN / "phix.se.sam").read_bytes()


@pytest.mark.parametrize("mode", [[], ["-x"], ["--ssw"]])
def test_mixed_records_one_per_chunk(tmp_path, mode):
    r1, r2 = _records(GOLDEN / "phix.1.fastq"), _records(GOLDEN / "phix.2.fastq")
    single = [i % 3 == 0 for i in range(len(r1))]
    (tmp_path / "mixed.fq").write_bytes(b"".join(a if s else a + b for a, b, s in zip(r1, r2, single)))
    (tmp_path / "s.fq").write_bytes(b"".join(a for a, s in zip(r1, single) if s))
    (tmp_path / "p1.fq").write_bytes(b"".join(a for a, s in zip(r1, single) if not s))
    (tmp_path / "p2.fq").write_bytes(b"".join(b for b, s in zip(r2, single) if not s))
    (tmp_path / "phix.fasta").write_bytes((GOLDEN / "phix.fasta").read_bytes())
    common = [*mode, "--chunk-size=0", "--no-PG", *RG, "-r", "150"]
    mixed = _sam_body(run_oracle_cli([*common, "--interleaved", "phix.fasta", "mixed.fq"], cwd=tmp_path))
    se = _sam_body(run_oracle_cli([*common, "phix.fasta", "s.fq"], cwd=tmp_path))
    pe = _sam_body(run_oracle_cli([*common, "phix.fasta", "p1.fq", "p2.fq"], cwd=tmp_path))
    # each record's lines (found by its name, unique in phiX) from the run of its kind,
    # in file order
    def by_name(lines):
        d = {}
        for l in lines:
            n = l.split(b"\t")[0]
            d.setdefault(n[:-2] if n[-2:] in (b"/1", b"/2") else n, []).append(l)  # PAF names carry /1 /2
        return d

    se_d, pe_d = by_name(se), by_name(pe)
    expect = []
    for a, s in zip(r1, single):
        name = a.splitlines()[0][1:].split()[0]
        if name[-2:] in (b"/1", b"/2"):
            name = name[:-2]
        expect += (se_d if s else pe_d).pop(name, [])
    assert not se_d and not pe_d
    assert mixed == expect


def _lib_pairs(reads) -> list[int]:
    return [int(x) for x in reads.interleaved_records()]


def test_library_pairing_of_reference_interleaved_file():
    from strobealign_gb300 import Reads
    r = Reads.from_file(str(GOLDEN / "interleaved.fq"))
    assert len(r) == 8
    # records (.2, .2) (.3, .3) .13852607 .13852608 .13852609 .13852610
    assert _lib_pairs(r) == [0, 2, 4, 5, 6, 7, 8]
    first = r.seq[int(r.seq_offsets[0]):int(r.seq_offsets[1])]
    second = r.seq[int(r.seq_offsets[1]):int(r.seq_offsets[2])]
    assert first.startswith(b"GTCGCCCA") and second.startswith(b"ATGTATTA")


def test_library_pairing_slash_suffixes(tmp_path):
    from strobealign_gb300 import Reads
    (tmp_path / "a.fq").write_bytes(b"@a/1\nAACC\n+\n####\n@a/2\nGGTT\n+n\n####\n")
    assert _lib_pairs(Reads.from_file(str(tmp_path / "a.fq"))) == [0, 2]


def test_library_pairing_random_names():
    from strobealign_gb300 import Reads
    rnd = random.Random(11)
    for n in [0, 1, 2, 3, 17, 200]:
        names = [rnd.choice(["a", "b", "c"]) for _ in range(n)]
        r = Reads.from_lists(names, ["ACGT"] * n)
        # InterleavedIterator: greedy, a read pairs with the next when the names are equal
        expect, i = [], 0
        while i < n:
            expect.append(i)
            i += 2 if i + 1 < n and names[i] == names[i + 1] else 1
        expect.append(n)
        assert _lib_pairs(r) == expect
