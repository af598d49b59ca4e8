"""File-to-file mapping (sa_map_files): parsing, mapping and writing overlapped in
batches of whole chunks give the bytes of one sa_map_batch over all records, for plain
and gzip inputs, paired-end and single-end, SAM / PAF / abundance output, and pairs that
end with the shorter file as zip pairs them (src/io/reads.rs:56-62)."""
import gzip

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(tmp_path_factory):
    import strobealign_gb300 as sa
    from strobealign_gb300 import synthetic as syn
    d = tmp_path_factory.mktemp("stream")
    g = syn.make_genome(61, 800_000, 3, gc=0.42, segdup_fraction=0.08, repeat_fraction=0.15)
    fa = str(d / "ref.fa")
    g.write_fasta(fa)
    r1, r2 = syn.make_paired_end(62, g, 6000, 150, 300, 30, 0.01, 0.002, rescue_fraction=0.03)
    f1, f2 = str(d / "r1.fq"), str(d / "r2.fq")
    r1.write_fastq(f1)
    r2.write_fastq(f2)
    se = syn.make_single_end(63, g, 4000, (60, 400), 0.015, 0.002)
    fse = str(d / "se.fq")
    se.write_fastq(fse)
    for f in (f1, f2, fse):
        data = open(f, "rb").read()
        cut = len(data) // 3
        # two gzip members, the split inside a record
        open(f + ".gz", "wb").write(gzip.compress(data[:cut], 1) + gzip.compress(data[cut:], 6))
    refs = sa.References.from_fasta(fa)
    idx = sa.StrobemerIndex.build(refs, sa.SeedingParameters.from_read_length(150))
    return dict(sa=sa, refs=refs, idx=idx, fa=fa, f1=f1, f2=f2, fse=fse, dir=d)


def _whole(s, files, **kw):
    sa = s["sa"]
    m = sa.Mapper(s["idx"], s["refs"], **kw)
    r1 = sa.Reads.from_file(files[0])
    r2 = sa.Reads.from_file(files[1]) if len(files) > 1 else None
    return m.map(r1, r2), m


@pytest.mark.parametrize("gz", [False, True])
@pytest.mark.parametrize("paired", [True, False])
def test_map_files_matches_one_batch(setup, gz, paired):
    s, sa = setup, setup["sa"]
    files = [s["f1"], s["f2"]] if paired else [s["fse"]]
    want, _ = _whole(s, files, chunk_size=40_000)
    head = sa.sam_header(s["refs"])
    ext = ".gz" if gz else ""
    for batch_bases in (1, 150_000, 0):  # one chunk per batch, a few chunks, all in one
        m = sa.Mapper(s["idx"], s["refs"], chunk_size=40_000)
        out = str(s["dir"] / f"out_{paired}_{gz}_{batch_bases}.sam")
        st = m.map_files(files[0] + ext, files[1] + ext if paired else None, out, header=head,
                         batch_bases=batch_bases)
        got = open(out, "rb").read()
        assert got == head + want
        assert st["n_records"] == (6000 if paired else 4000) and st["bytes_out"] == len(got)
        if batch_bases == 1:
            assert st["n_batches"] > 10
        if batch_bases == 0:
            assert st["n_batches"] == 1


def test_map_files_paf_and_abundances(setup):
    s, sa = setup, setup["sa"]
    want, _ = _whole(s, [s["f1"], s["f2"]], mode=sa.MODE_PAF)
    m = sa.Mapper(s["idx"], s["refs"], mode=sa.MODE_PAF)
    out = str(s["dir"] / "o.paf")
    m.map_files(s["f1"] + ".gz", s["f2"] + ".gz", out, batch_bases=100_000)
    assert open(out, "rb").read() == want
    _, mw = _whole(s, [s["fse"]], mode=sa.MODE_ABUNDANCE)
    names = [l[1:].split()[0].decode() for l in open(s["fa"], "rb") if l.startswith(b">")]
    table = "".join(f"{n}\t{a:.6f}\n" for n, a in zip(names, mw.abundances())).encode()
    m = sa.Mapper(s["idx"], s["refs"], mode=sa.MODE_ABUNDANCE)
    out = str(s["dir"] / "o.abun")
    m.map_files(s["fse"], None, out, batch_bases=60_000)
    assert open(out, "rb").read() == table


def test_map_files_pairs_end_with_shorter_file(setup):
    s, sa = setup, setup["sa"]
    lines = open(s["f2"], "rb").read().split(b"\n")
    short = str(s["dir"] / "r2_short.fq")
    open(short, "wb").write(b"\n".join(lines[: 4 * 4500]) + b"\n")
    r1 = sa.Reads.from_file(s["f1"])
    r2 = sa.Reads.from_file(short)
    assert len(r2) == 4500
    import numpy as np
    n = 4500
    so, no = r1.seq_offsets[: n + 1], r1.name_offsets[: n + 1]
    co = r1.comment_offsets[: n + 1]
    cut = sa.Reads(r1.seq[: int(so[-1])], np.ascontiguousarray(so), r1.names[: int(no[-1])], np.ascontiguousarray(no),
                   r1.qual[: int(so[-1])], r1.comments[: int(co[-1])], np.ascontiguousarray(co))
    want = sa.Mapper(s["idx"], s["refs"]).map(cut, r2)
    m = sa.Mapper(s["idx"], s["refs"])
    out = str(s["dir"] / "short.sam")
    st = m.map_files(s["f1"], short, out, batch_bases=200_000)
    assert st["n_records"] == 4500
    assert open(out, "rb").read() == want


def test_map_files_errors(setup):
    s, sa = setup, setup["sa"]
    m = sa.Mapper(s["idx"], s["refs"])
    with pytest.raises(sa.SaError, match="cannot open"):
        m.map_files(str(s["dir"] / "missing.fq"), None, str(s["dir"] / "x.sam"))
    bad = str(s["dir"] / "bad.fq")
    data = open(s["fse"], "rb").read()
    open(bad, "wb").write(data + b"@broken\nACGT\n+\nII\n")
    with pytest.raises(sa.SaError, match="quality"):
        m.map_files(bad, None, str(s["dir"] / "y.sam"), batch_bases=50_000)
    # the mapper still works after a failed stream
    out = str(s["dir"] / "z.sam")
    m.map_files(s["fse"], None, out)
    assert open(out, "rb").read() == _whole(s, [s["fse"]])[0]
