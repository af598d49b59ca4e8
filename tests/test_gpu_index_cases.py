"""The reference's index unit tests on the GPU-built index: a phiX index has
randstrobes and the index of an empty reference has none, looking nothing up
(src/indexer.rs:374-396); every randstrobe of phiX is found by its partial hash in the
index of phiX's reverse complement, and with the orientation bit flipped by a forward
partial lookup (src/index.rs partial_orientation)."""
import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

HASH_MASK = np.uint64(0xFFFFFFFFFFFFFF00)
COMP = bytes.maketrans(b"ACGT", b"TGCA")


@pytest.fixture(scope="module")
def sa():
    import strobealign_gb300 as sa
    return sa


def test_index_phix_and_empty_reference(sa):
    p = sa.SeedingParameters.from_read_length(150)
    refs = sa.References.from_fasta(str(GOLDEN / "phix.fasta"))
    idx = sa.StrobemerIndex.build(refs, p, refs.pick_bits(p), 0.1)
    assert idx.info.n_randstrobes > 0
    empty = sa.References.from_sequences(["name"], [b""])
    e = sa.StrobemerIndex.build(empty, p, empty.pick_bits(p), 0.1)
    assert e.info.n_randstrobes == 0
    rs, bs = e.to_host()
    assert len(rs) == 0 and not bs.any()
    h = np.array([0, 1 << 40, (1 << 64) - 256], dtype=np.uint64)
    for kind in (0, 1, 2):
        assert (e.lookup(h, kind=kind) == -1).all()


def test_partial_orientation(sa):
    p = sa.SeedingParameters.from_read_length(300)
    refs = sa.References.from_fasta(str(GOLDEN / "phix.fasta"))
    seq = refs.decode(0)
    rc = sa.References.from_sequences(["phix_rc"], [seq.translate(COMP)[::-1]])
    bits = refs.pick_bits(p)
    fwd = sa.StrobemerIndex.build(refs, p, bits, 0.0000001)
    rev = sa.StrobemerIndex.build(rc, p, bits, 0.0000001)
    t_f, _ = fwd.to_host()
    t_r, _ = rev.to_host()
    assert len(t_f) == len(t_r) > 0
    h = t_f["hash_offset"] & HASH_MASK
    assert (rev.lookup(h, kind=1) >= 0).all()
    flipped = h ^ np.uint64(1 << p.partial_orientation_pos)
    assert (rev.lookup(flipped, kind=2) >= 0).all()
