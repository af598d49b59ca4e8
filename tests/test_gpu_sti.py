""".sti index files (format version 7, src/index.rs:345-538).

A file is laid out here by the reference's own writer order (StrobemerIndex::write,
src/index.rs:374-409: magic, version, the reserved chunk, filter cutoff, bits, profile,
k, s, w_min, w_max, q, max_dist, main hash mask, then the randstrobe and bucket vectors
as u64 length + raw data) from the oracle's index; the library must read it into the
same table, write it back byte for byte, and map identically from it."""
import struct

import numpy as np
import pytest

from conftest import GOLDEN
from oracle_lib import OracleIndex

pytestmark = pytest.mark.gpu


def reference_layout(params, cutoff, bits, rs: np.ndarray, bs: np.ndarray) -> bytes:
    out = bytearray(b"STI\x01")
    out += struct.pack("<I", 7)
    out += struct.pack("<QQ", 8, 0)
    out += struct.pack("<9I", cutoff, bits, params.profile, params.k, params.s, params.w_min, params.w_max,
                       params.q & 0xFFFFFFFF, params.max_dist)
    out += struct.pack("<Q", params.main_hash_mask)
    out += struct.pack("<Q", len(rs)) + rs.tobytes()
    out += struct.pack("<Q", len(bs)) + bs.tobytes()
    return bytes(out)


@pytest.fixture(scope="module")
def sa():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import strobealign_gb300
    return strobealign_gb300


@pytest.mark.parametrize("read_length", [150, 250])
def test_reads_reference_layout_and_writes_it_back(sa, tmp_path, read_length):
    fa = GOLDEN / "phix.fasta"
    o = OracleIndex(fa, read_length)
    n, bits, cutoff = o.info()
    rs, bs = o.arrays()
    params = sa.SeedingParameters.from_read_length(read_length)
    ref_file = tmp_path / "ref.sti"
    ref_file.write_bytes(reference_layout(params.c, cutoff, bits, rs, bs))
    idx = sa.StrobemerIndex.read_sti(ref_file, params)
    assert idx.info.n_randstrobes == n and idx.info.bits == bits and idx.filter_cutoff == cutoff
    grs, gbs = idx.to_host()
    assert grs.tobytes() == rs.tobytes() and np.array_equal(gbs, bs)
    out = tmp_path / "out.sti"
    idx.write_sti(out)
    assert out.read_bytes() == ref_file.read_bytes()
    # the GPU-built index writes the same file
    refs = sa.References.from_fasta(fa)
    built = sa.StrobemerIndex.build(refs, params)
    out2 = tmp_path / "built.sti"
    built.write_sti(out2)
    assert out2.read_bytes() == ref_file.read_bytes()


def test_round_trip_maps_identically_and_rejects_mismatch(sa, tmp_path):
    fa = GOLDEN / "phix.fasta"
    refs = sa.References.from_fasta(fa)
    params = sa.SeedingParameters.from_read_length(150)
    idx = sa.StrobemerIndex.build(refs, params)
    path = tmp_path / "phix.sti"
    idx.write_sti(path)
    back = sa.StrobemerIndex.read_sti(path, params)
    r1 = sa.Reads.from_file(GOLDEN / "phix.1.fastq")
    r2 = sa.Reads.from_file(GOLDEN / "phix.2.fastq")
    a = sa.Mapper(idx, refs).map(r1, r2)
    b = sa.Mapper(back, refs).map(r1, r2)
    assert a == b and len(a) > 0
    with pytest.raises(sa.SaError):
        sa.StrobemerIndex.read_sti(path, sa.SeedingParameters.from_read_length(250))
    with pytest.raises(sa.SaError):
        sa.StrobemerIndex.read_sti(path, params, bits=idx.info.bits + 1)
    bad = tmp_path / "bad.sti"
    bad.write_bytes(path.read_bytes()[:100])
    with pytest.raises(sa.SaError):
        sa.StrobemerIndex.read_sti(bad, params)
