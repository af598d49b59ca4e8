"""Input files without a GPU: gzip (single and multi-member, src/io/xopen.rs:9-20) reads
the same records as the plain file, FASTA reads and references load from .gz, and
broken inputs fail with an error (src/io/fastq.rs:37-86) instead of a crash."""
import gzip

import numpy as np
import pytest

from conftest import GOLDEN


@pytest.fixture(scope="module")
def sa():
    import strobealign_gb300 as sa
    sa.lib()
    return sa


def _same(a, b):
    assert len(a) == len(b)
    assert a.seq == b.seq and a.names == b.names and a.qual == b.qual and a.comments == b.comments
    assert np.array_equal(a.seq_offsets, b.seq_offsets) and np.array_equal(a.name_offsets, b.name_offsets)
    assert np.array_equal(a.comment_offsets, b.comment_offsets)


def _members(data: bytes, parts: int) -> bytes:
    cut = [len(data) * i // parts for i in range(parts + 1)]
    return b"".join(gzip.compress(data[cut[i]:cut[i + 1]], compresslevel=1 + i % 9) for i in range(parts))


@pytest.mark.parametrize("name", ["phix.1.fastq", "phix.tags.fastq", "interleaved.fq"])
def test_gzip_fastq_matches_plain(sa, tmp_path, name):
    src = GOLDEN / name
    plain = sa.Reads.from_file(str(src))
    assert len(plain) > 0
    one = tmp_path / (name + ".gz")
    one.write_bytes(gzip.compress(src.read_bytes()))
    _same(plain, sa.Reads.from_file(str(one)))
    # several members, split anywhere (inside records and lines)
    multi = tmp_path / ("multi." + name + ".gz")
    multi.write_bytes(_members(src.read_bytes(), 7))
    _same(plain, sa.Reads.from_file(str(multi)))


def test_gzip_fasta_reads_and_references(sa, tmp_path):
    src = GOLDEN / "phix.fasta"
    gz = tmp_path / "phix.fasta.gz"
    gz.write_bytes(_members(src.read_bytes(), 3))
    _same(sa.Reads.from_file(str(src)), sa.Reads.from_file(str(gz)))
    a, b = sa.References.from_fasta(str(src)), sa.References.from_fasta(str(gz))
    assert len(a) == len(b) and a.total_length == b.total_length > 5000


def test_fasta_reads_multiline_lowercase(sa, tmp_path):
    f = tmp_path / "r.fa"
    f.write_bytes(b">r1 first read\nacgt\nACGN\n\n>r2\nTTTT\r\n>r3\n")
    r = sa.Reads.from_file(str(f))
    assert len(r) == 3 and r.qual is None
    assert r.seq == b"ACGTACGNTTTT" and list(r.seq_offsets) == [0, 8, 12, 12]
    assert r.names == b"r1r2r3" and r.comments == b"first read"


def test_fastq_record_rules(sa, tmp_path):
    f = tmp_path / "r.fq"
    f.write_bytes(b"@a/1 c1\nacgt\n+\nIIII\n@b/2\nGG\r\n+\nII\r\n@c/3\nA\n+\nI\n")
    r = sa.Reads.from_file(str(f))
    assert r.names == b"abc/3" and r.seq == b"ACGTGGA" and r.qual == b"IIIIIII" and r.comments == b"c1"


@pytest.mark.parametrize("body,msg", [
    (b"@a\nACGT\n+\nIII\n", "quality"),
    (b"a\nACGT\n+\nIIII\n", "'@'"),
    (b"@\nACGT\n+\nIIII\n", "identifier"),
    # no newline after the last quality line: its last byte goes as the line end
    (b"@a\nACGT\n+\nIIII", "quality"),
])
def test_fastq_errors(sa, tmp_path, body, msg):
    f = tmp_path / "bad.fq"
    f.write_bytes(body)
    with pytest.raises(sa.SaError, match=msg):
        sa.Reads.from_file(str(f))


def test_gzip_errors(sa, tmp_path):
    data = gzip.compress((GOLDEN / "phix.1.fastq").read_bytes())
    t = tmp_path / "trunc.fq.gz"
    t.write_bytes(data[: len(data) // 2])
    with pytest.raises(sa.SaError, match="gzip"):
        sa.Reads.from_file(str(t))
    c = tmp_path / "corrupt.fq.gz"
    c.write_bytes(data[:20] + bytes(b ^ 0x5A for b in data[20:200]) + data[200:])
    with pytest.raises(sa.SaError):
        sa.Reads.from_file(str(c))
    g = tmp_path / "garbage.fq.gz"
    g.write_bytes(data + b"not a gzip member")
    with pytest.raises(sa.SaError, match="gzip"):
        sa.Reads.from_file(str(g))
    e = tmp_path / "empty.fq.gz"
    e.write_bytes(b"")
    assert len(sa.Reads.from_file(str(e))) == 0
    with pytest.raises(sa.SaError, match="cannot open"):
        sa.Reads.from_file(str(tmp_path / "missing.fq.gz"))


def test_reads_from_standard_input(tmp_path):
    # "-" reads standard input (src/io/xopen.rs:11-12)
    import subprocess
    import sys
    from conftest import ROOT
    src = GOLDEN / "phix.1.fastq"
    code = ("import sys; sys.path.insert(0, %r); import strobealign_gb300 as sa; r = sa.Reads.from_file('-'); "
            "print(len(r), len(r.seq))" % str(ROOT))
    with open(src, "rb") as f:
        out = subprocess.run([sys.executable, "-c", code], stdin=f, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    import strobealign_gb300 as sa
    want = sa.Reads.from_file(str(src))
    assert out.stdout.split() == [str(len(want)), str(len(want.seq))]


def test_estimate_read_length(tmp_path):
    # src/main.rs:1042-1046: the first 500 records of phix.1.fastq give 289
    import strobealign_gb300 as sa
    assert sa.estimate_read_length(str(GOLDEN / "phix.1.fastq")) == 289
    data = (GOLDEN / "phix.1.fastq").read_bytes()
    (tmp_path / "r.fq.gz").write_bytes(gzip.compress(data))
    assert sa.estimate_read_length(str(tmp_path / "r.fq.gz")) == 289
    # only the first 500 records count; the mean is rounded down
    rec = [b"@r%d\n%s\n+\n%s\n" % (i, b"A" * (10 if i < 500 else 1000), b"I" * (10 if i < 500 else 1000))
           for i in range(600)]
    (tmp_path / "long.fq").write_bytes(b"".join(rec))
    assert sa.estimate_read_length(str(tmp_path / "long.fq")) == 10
    (tmp_path / "odd.fa").write_bytes(b">a\nACG\n>b\nACGTAC\n")
    assert sa.estimate_read_length(str(tmp_path / "odd.fa")) == 4
    (tmp_path / "empty.fq").write_bytes(b"")
    assert sa.estimate_read_length(str(tmp_path / "empty.fq")) == 0
    with pytest.raises(sa.SaError, match="standard input"):
        sa.estimate_read_length("-")


# The reference's own reader unit tests (src/io/fasta.rs:174-306, src/io/fastq.rs:97-120,
# src/io/mod.rs:40-58) on the library's readers.

def _refs(sa, tmp_path, data: bytes):
    f = tmp_path / "ref.fa"
    f.write_bytes(data)
    return sa.References.from_fasta(str(f))


def test_reference_fasta_phix(sa):
    r = sa.References.from_fasta(str(GOLDEN / "phix.fasta"))
    assert len(r) == 1 and r.contig(0) == ("NC_001422.1", 5386)
    assert r.decode(0, 0, 5) == b"GAGTT"


def test_reference_fasta_parse(sa, tmp_path):
    r = _refs(sa, tmp_path, b">ref1 a comment\nacgt\n\n>ref2\naacc\ngg\n\ntt\n>empty\n>empty_at_end_of_file")
    assert [r.contig(i)[0] for i in range(len(r))] == ["ref1", "ref2", "empty", "empty_at_end_of_file"]
    assert [r.decode(i) for i in range(len(r))] == [b"ACGT", b"AACCGGTT", b"", b""]


@pytest.mark.parametrize("data,names", [
    (b"><>;abc\nAAAA\n>abc\nCCCC\n", ["<>;abc", "abc"]),
    (b">ab c\nACGT\n>de\tf\nACGT\n", ["ab", "de"]),
])
def test_reference_fasta_names(sa, tmp_path, data, names):
    r = _refs(sa, tmp_path, data)
    assert [r.contig(i)[0] for i in range(len(r))] == names


@pytest.mark.parametrize("data", [
    b">name\x08\n",               # a control character in the name
    b">\x00x80\nACGT\n",           # a NUL in the name
    b">abc\nAAAA\n>abc\nCCCC\n",   # duplicate names
    b"bla",                        # no '>' first
    b">a\nAC\xffGT\n",             # not UTF-8 (read_line fails)
])
def test_reference_fasta_errors(sa, tmp_path, data):
    with pytest.raises(sa.SaError):
        _refs(sa, tmp_path, data)


def test_reference_fasta_error_on_fastq(sa):
    with pytest.raises(sa.SaError):
        sa.References.from_fasta(str(GOLDEN / "phix.1.fastq"))


def test_reference_fasta_wildcards_and_blanks(sa, tmp_path):
    # a vertical tab is not ASCII whitespace to trim_ascii_end: it stays, as a wildcard
    # base; a two-byte UTF-8 character is two wildcard bases; each wildcard takes the
    # value encode_wildcard gives its position (src/packed_seq.rs:50-59)
    r = _refs(sa, tmp_path, b">a\nAC\x0b\nG\xc3\xa9NT \t\r\n")
    assert r.contig(0) == ("a", 8)

    def wild(pos):
        h = (pos * 0x9E3779B97F4A7C15) & (2 ** 64 - 1)
        return b"ACGT"[(h ^ (h >> 30)) & 3:][:1]

    assert r.decode(0) == b"AC" + wild(2) + b"G" + wild(4) + wild(5) + wild(6) + b"T"


def test_fasta_reads_reference_cases(sa, tmp_path):
    r = sa.Reads.from_file(str(GOLDEN / "phix.fasta"))
    assert len(r) == 1 and r.names == b"NC_001422.1" and len(r.seq) == 5386 and r.seq[:5] == b"GAGTT"
    f = tmp_path / "only_name.fa"
    f.write_bytes(b">name\n")
    r = sa.Reads.from_file(str(f))
    assert len(r) == 1 and r.names == b"name" and r.seq == b""
    f = tmp_path / "upper.fa"
    f.write_bytes(b">name\r\nacgt\n>name2\nTgCa")
    r = sa.Reads.from_file(str(f))
    assert r.names == b"namename2" and list(r.name_offsets) == [0, 4, 9]
    assert r.seq == b"ACGTTGCA" and list(r.seq_offsets) == [0, 4, 8]
    f = tmp_path / "empty.fa"
    f.write_bytes(b"")
    assert len(sa.Reads.from_file(str(f))) == 0
    f = tmp_path / "bad.fa"
    f.write_bytes(b">a\nACGT\n>b\xfe\nACGT\n")
    with pytest.raises(sa.SaError, match="UTF-8"):
        sa.Reads.from_file(str(f))


def test_fastq_reference_cases(sa, tmp_path):
    f = tmp_path / "start.fq"
    f.write_bytes(b"@a\nA\n+\n#\n>b")
    with pytest.raises(sa.SaError):
        sa.Reads.from_file(str(f))
    # split_header: "id comment", "id comment ", "id", "id ", "id  "
    f = tmp_path / "hdr.fq"
    f.write_bytes(b"@id comment\nA\n+\nI\n@id comment \nA\n+\nI\n@id\nA\n+\nI\n@id \nA\n+\nI\n@id  \nA\n+\nI\n")
    r = sa.Reads.from_file(str(f))
    assert r.names == b"id" * 5 and r.comments == b"comment" * 2 and list(r.comment_offsets) == [0, 7, 14, 14, 14, 14]
    # a vertical tab is kept in the name; bytes that are not UTF-8 are fine in sequence and
    # quality lines (read as bytes) but not in the header (read as a String)
    f = tmp_path / "vt.fq"
    f.write_bytes(b"@id\x0b\nA\xffC\n+\nI\xfeI\n")
    r = sa.Reads.from_file(str(f))
    assert r.names == b"id\x0b" and r.seq == b"A\xffC" and r.qual == b"I\xfeI"
    f = tmp_path / "bad.fq"
    f.write_bytes(b"@a\nACGT\n+\nIIII\n@b\xc0\xaf\nACGT\n+\nIIII\n")
    with pytest.raises(sa.SaError, match="UTF-8"):
        sa.Reads.from_file(str(f))
