"""The library's read parser against a restatement of the reference's readers on random
files, without a GPU: FastqReader (src/io/fastq.rs:22-94: four lines per record, the
last byte of the sequence and quality lines dropped as the line end and a '\\r' before
it, header split by split_header of src/io/mod.rs:32-38, a trailing /1 or /2 dropped,
sequences upper-cased) and FastaReader (src/io/fasta.rs:64-113).  Whole files through
sa_reads_from_file and the same files in batches through sa_read_file_next, with CRLF
line ends, lower case, comments with tabs, '+' lines with text, empty sequences, a
missing last newline and lines longer than the reader's buffer."""
import gzip
import random

import pytest


def _split_header(h: bytes):
    t = h.rstrip(b" \t\n\r\x0c")
    for i, c in enumerate(t):
        if c in b" \t":
            return t[:i], t[i + 1:]
    return t, None


def _upper(s: bytes) -> bytes:
    return bytes(c - 32 if 97 <= c <= 122 else c for c in s)


def ref_fastq(data: bytes):
    """(name, comment or None, seq, qual) per record, or raises ValueError."""
    pos, n, out = 0, len(data), []

    def until_nl():
        nonlocal pos
        if pos >= n:
            return b""
        j = data.find(b"\n", pos)
        j = n - 1 if j < 0 else j
        line = data[pos:j + 1]
        pos = j + 1
        return line

    def strip_end(line):
        line = line[:-1]  # the line end, or the last byte at the end of the input
        return line[:-1] if line.endswith(b"\r") else line

    while True:
        head = until_nl()
        if not head:
            return out
        if not head.startswith(b"@"):
            raise ValueError("start")
        head.decode("utf-8")
        name, comment = _split_header(head[1:])
        if not name:
            raise ValueError("empty name")
        if name.endswith(b"/1") or name.endswith(b"/2"):
            name = name[:-2]
        seq = strip_end(until_nl())
        until_nl().decode("utf-8")
        qual = strip_end(until_nl())
        if len(seq) != len(qual):
            raise ValueError("quality")
        out.append((name, comment, _upper(seq), qual))


def ref_fasta(data: bytes):
    out, cur = [], None
    for line in data.splitlines(keepends=True):
        line.decode("utf-8")
        if line.startswith(b">"):
            if cur is not None:
                out.append(cur)
            name, comment = _split_header(line[1:])
            cur = (name, comment, b"", None)
        else:
            cur = (cur[0], cur[1], cur[2] + _upper(line.rstrip(b" \t\n\r\x0c")), None)
    if cur is not None:
        out.append(cur)
    return out


def _records_of(reads):
    out = []
    for i in range(len(reads)):
        s0, s1 = int(reads.seq_offsets[i]), int(reads.seq_offsets[i + 1])
        n0, n1 = int(reads.name_offsets[i]), int(reads.name_offsets[i + 1])
        c0, c1 = int(reads.comment_offsets[i]), int(reads.comment_offsets[i + 1])
        q = reads.qual[s0:s1] if reads.qual is not None else None
        out.append((reads.names[n0:n1], reads.comments[c0:c1], reads.seq[s0:s1], q))
    return out


def _norm(recs):
    # the library keeps an absent and an empty comment alike (both print nothing)
    return [(n, c or b"", s, q) for n, c, s, q in recs]


def random_fastq(rnd: random.Random, n: int, long_line: int = 0) -> bytes:
    out = []
    for i in range(n):
        name = b"r%d" % i + rnd.choice([b"", b"/1", b"/2", b"/3", b"x"])
        head = b"@" + name
        r = rnd.random()
        if r < 0.2:
            head += b" comment %d" % i
        elif r < 0.3:
            head += b"\tBC:Z:ACGT\tx"
        elif r < 0.35:
            head += b"  "
        L = long_line if (long_line and i == n // 2) else rnd.choice([0, 1, 5, 50, 150, 151, 300])
        seq = bytes(rnd.choice(b"ACGTNacgtn") for _ in range(L))
        qual = bytes(rnd.choice(b"!#5?IJ") for _ in range(L))
        crlf = rnd.random() < 0.2
        nl = b"\r\n" if crlf else b"\n"
        plus = rnd.choice([b"+", b"+", b"+" + name])
        out.append(head + nl + seq + nl + plus + nl + qual + nl)
    data = b"".join(out)
    if rnd.random() < 0.5 and data.endswith(b"\n") and not data.endswith(b"\r\n"):
        # no newline after the last quality line: add one byte the reader drops instead
        data = data[:-1] + b"X"
    return data


def random_fasta(rnd: random.Random, n: int) -> bytes:
    out = []
    for i in range(n):
        out.append(b">s%d" % i + rnd.choice([b"", b" a comment", b"\tx"]) + b"\n")
        for _ in range(rnd.choice([0, 1, 3])):
            out.append(bytes(rnd.choice(b"ACGTNacgt") for _ in range(rnd.choice([0, 7, 60]))) +
                       rnd.choice([b"\n", b"\r\n", b" \n"]))
    return b"".join(out)


def _batched(sa, path, step):
    f = sa.ReadFile(str(path))
    got = []
    while True:
        b = f.next(step)
        if len(b) == 0:
            return got
        assert len(b) <= step
        got += _records_of(b)


@pytest.mark.parametrize("seed", range(6))
def test_fastq_matches_reference_rules(tmp_path, seed):
    import strobealign_gb300 as sa
    rnd = random.Random(seed)
    data = random_fastq(rnd, rnd.choice([1, 17, 300, 3000]), long_line=(5 << 20) if seed == 5 else 0)
    want = _norm(ref_fastq(data))
    path = tmp_path / "r.fq"
    path.write_bytes(data)
    assert _norm(_records_of(sa.Reads.from_file(str(path)))) == want
    for step in (1, 7, 1000, 1 << 20):
        assert _norm(_batched(sa, path, step)) == want
    gz = tmp_path / "r.fq.gz"
    gz.write_bytes(gzip.compress(data, 1))
    assert _norm(_records_of(sa.Reads.from_file(str(gz)))) == want


@pytest.mark.parametrize("seed", range(4))
def test_fasta_reads_match_reference_rules(tmp_path, seed):
    import strobealign_gb300 as sa
    rnd = random.Random(100 + seed)
    data = random_fasta(rnd, rnd.choice([1, 20, 500]))
    want = _norm(ref_fasta(data))
    path = tmp_path / "r.fa"
    path.write_bytes(data)
    assert _norm(_records_of(sa.Reads.from_file(str(path)))) == want
    for step in (1, 3, 1 << 20):
        assert _norm(_batched(sa, path, step)) == want


def test_fastq_errors_in_batches(tmp_path):
    # the error of the first bad record, wherever the batches are cut
    import strobealign_gb300 as sa
    rnd = random.Random(7)
    good = random_fastq(rnd, 200)
    if not good.endswith(b"\n"):
        good = good[:-1] + b"\n"
    for bad, msg in [(b"@b\nACGT\n+\nIII\n", "quality"), (b"b\nACGT\n+\nIIII\n", "'@'"),
                     (b"@\nACGT\n+\nIIII\n", "identifier"), (b"@\xff\nA\n+\nI\n", "UTF-8")]:
        path = tmp_path / "bad.fq"
        path.write_bytes(good + bad + good)
        with pytest.raises(ValueError):
            ref_fastq(good + bad + good)
        with pytest.raises(sa.SaError, match=msg):
            sa.Reads.from_file(str(path))
        for step in (1, 64, 1 << 20):
            with pytest.raises(sa.SaError, match=msg):
                _batched(sa, path, step)


def test_read_file_errors(tmp_path):
    import strobealign_gb300 as sa
    with pytest.raises(sa.SaError, match="cannot open"):
        sa.ReadFile(str(tmp_path / "missing.fq"))
    (tmp_path / "e.fq").write_bytes(b"")
    assert len(sa.ReadFile(str(tmp_path / "e.fq")).next(10)) == 0


def test_header_utf8_rule_matches_python(tmp_path):
    # a header line the reference reads into a String fails exactly when it is not UTF-8
    import strobealign_gb300 as sa
    rnd = random.Random(21)
    alphabet = [0x41, 0x7F, 0x80, 0xBF, 0xC0, 0xC1, 0xC2, 0xDF, 0xE0, 0xED, 0xEF, 0xF0, 0xF4, 0xF5, 0xFF, 0x9F,
                0xA0, 0x8F, 0x90]
    path = tmp_path / "h.fq"
    for _ in range(400):
        body = bytes(rnd.choice(alphabet) for _ in range(rnd.randint(1, 6)))
        head = b"@a" + body
        path.write_bytes(head + b"\nA\n+\nI\n")
        try:
            head.decode("utf-8")
            ok = True
        except UnicodeDecodeError:
            ok = False
        if ok:
            assert len(sa.Reads.from_file(str(path))) == 1
        else:
            with pytest.raises(sa.SaError, match="UTF-8"):
                sa.Reads.from_file(str(path))
