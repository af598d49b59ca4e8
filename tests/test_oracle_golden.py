"""The oracle against the reference's own goldens (tests/phix.*) and against the
reference's compiled SSW library.  CPU only."""
import random

import pytest

from oracle_lib import (aligner_oracle, randstrobes_oracle, reference_ssw, run_oracle_cli, ssw_oracle,
                        ssw_reference)
from conftest import GOLDEN

RG = ["--rg-id=1", "--rg=SM:sample", "--rg=LB:library"]


def _g(name):
    return (GOLDEN / name).read_bytes()


def test_paired_end_sam_golden():
    out = run_oracle_cli(["--no-PG", "--eqx", *RG, "phix.fasta", "phix.1.fastq", "phix.2.fastq"], cwd=GOLDEN)
    assert out == _g("phix.pe.sam")


def test_single_end_sam_golden():
    out = run_oracle_cli(["--chunk-size=3", "--no-PG", "--eqx", *RG, "phix.fasta", "phix.1.fastq"], cwd=GOLDEN)
    assert out == _g("phix.se.sam")


def test_fastq_comment_tags_golden():
    out = run_oracle_cli(["-C", "--no-PG", *RG, "phix.fasta", "phix.tags.fastq"], cwd=GOLDEN)
    assert out == _g("phix.tags.sam")


def _tail(b: bytes, n: int) -> bytes:
    return b"".join(b.splitlines(keepends=True)[-n:])


def test_single_end_paf_golden():
    assert _tail(run_oracle_cli(["-x", "phix.fasta", "phix.1.fastq"], cwd=GOLDEN), 11) == _g("phix.se.paf")


def test_mcs_rescue_paf_golden():
    out = run_oracle_cli(["-x", "--mcs=rescue", "phix.fasta", "phix.1.fastq"], cwd=GOLDEN)
    assert _tail(out, 11) == _g("phix.mcsrescue.se.paf")


def test_abundance_goldens():
    assert run_oracle_cli(["--aemb", "phix.fasta", "phix.1.fastq"], cwd=GOLDEN) == _g("phix.abun.se.txt")
    assert run_oracle_cli(["--aemb", "phix.fasta", "phix.1.fastq", "phix.2.fastq"], cwd=GOLDEN) == \
        _g("phix.abun.pe.txt")


def test_paired_end_paf_coordinates():
    # the reference disables this golden (tests/run.sh:46-52): its matching-base
    # and MAPQ columns and /1 /2 suffixes predate the current output; the
    # coordinates must still agree
    out = _tail(run_oracle_cli(["-x", "phix.fasta", "phix.1.fastq", "phix.2.fastq"], cwd=GOLDEN), 11)
    mine = [l.split(b"\t")[1:9] for l in out.splitlines()]
    gold = [l.split(b"\t")[1:9] for l in _g("phix.pe.paf").splitlines()]
    assert mine == gold


def test_randstrobe_count_equals_syncmer_count_and_orientation():
    # src/seeding/strobes.rs:216-238 (one randstrobe per syncmer) and the
    # forward/reverse-complement symmetry of canonical syncmers
    seq = b"".join(l.strip() for l in (GOLDEN / "phix.fasta").read_bytes().splitlines()[1:])[:2000]
    fwd, rc = randstrobes_oracle(seq, 150)
    assert len(fwd) == len(rc) > 300
    assert all(fwd[:, 2] <= fwd[:, 3])


def test_ssw_no_result_case():
    # src/ssw.rs:194-201: no alignment between these sequences
    q = b"TCTCTCCCTCTCTCTCTCTCCCTCCCTCTCTCTCCCTCTCTCTCTCTCTCTCCCTCCCTT"
    r = b"GAGGGAGAGAGAGAGAGGGAGAGAGAGAGAGAG"
    assert aligner_oracle(q, r) is None


def _mutate(rnd, s, sub, indel):
    out = bytearray()
    for c in s:
        x = rnd.random()
        if x < sub:
            out.append(rnd.choice(b"ACGT"))
        elif x < sub + indel / 2:
            pass
        elif x < sub + indel:
            out += bytes([c, rnd.choice(b"ACGT")])
        else:
            out.append(c)
    return bytes(out)


@pytest.mark.skipif(reference_ssw() is None, reason="reference ext/ssw/ssw.c not available here")
def test_ssw_restatement_matches_reference_library():
    rnd = random.Random(7)
    n = 0
    for _ in range(1500):
        L = rnd.choice([8, 16, 17, 31, 64, 100, 150, 151, 250, 500])
        q = bytes(rnd.choice(b"ACGT") for _ in range(L))
        if rnd.random() < 0.1:
            q = q[: L // 2] + b"N" * rnd.randint(1, 4) + q[L // 2:]
        core = _mutate(rnd, q, rnd.choice([0, 0.01, 0.05, 0.2, 0.6]), rnd.choice([0, 0.02, 0.08]))
        r = bytes(rnd.choice(b"ACGT") for _ in range(rnd.randint(0, 40))) + core + \
            bytes(rnd.choice(b"ACGT") for _ in range(rnd.randint(0, 40)))
        if not r:
            continue
        assert ssw_oracle(q, r) == ssw_reference(q, r), (q, r)
        n += 1
    assert n > 1000
