"""Copy the reference's own phiX test fixtures and goldens into tests/golden/.

These files are the strobealign test suite's inputs and expected outputs
(tests/phix.fasta, tests/phix.{1,2}.fastq, tests/phix.tags.fastq and the
goldens tests/phix.{se,pe,tags}.sam, tests/phix.{se,mcsrescue.se,pe}.paf,
tests/phix.abun.{se,pe}.txt).  They pin the oracle; the commands that produce
each golden are listed in GOLDEN_COMMANDS (from the reference's tests/test.rs
and tests/run.sh).  Run this where the reference tree is available:

    python tests/golden/fetch_reference_fixtures.py /path/to/strobealign
"""
import shutil
import sys
from pathlib import Path

FILES = [
    "phix.fasta", "phix.1.fastq", "phix.2.fastq", "phix.tags.fastq", "interleaved.fq",
    "phix.se.sam", "phix.pe.sam", "phix.tags.sam", "phix.se.paf", "phix.mcsrescue.se.paf",
    "phix.pe.paf", "phix.abun.se.txt", "phix.abun.pe.txt",
]

# golden file -> (arguments, post-processing); paths relative to tests/golden
GOLDEN_COMMANDS = {
    "phix.se.sam": (["--chunk-size=3", "--no-PG", "--eqx", "--rg-id=1", "--rg=SM:sample",
                     "--rg=LB:library", "phix.fasta", "phix.1.fastq"], None),
    "phix.pe.sam": (["--no-PG", "--eqx", "--rg-id=1", "--rg=SM:sample", "--rg=LB:library",
                     "phix.fasta", "phix.1.fastq", "phix.2.fastq"], None),
    "phix.tags.sam": (["-C", "--no-PG", "--rg-id=1", "--rg=SM:sample", "--rg=LB:library",
                       "phix.fasta", "phix.tags.fastq"], None),
    "phix.se.paf": (["-x", "phix.fasta", "phix.1.fastq"], "tail11"),
    "phix.mcsrescue.se.paf": (["-x", "--mcs=rescue", "phix.fasta", "phix.1.fastq"], "tail11"),
    "phix.abun.se.txt": (["--aemb", "phix.fasta", "phix.1.fastq"], None),
    "phix.abun.pe.txt": (["--aemb", "phix.fasta", "phix.1.fastq", "phix.2.fastq"], None),
}


def main() -> None:
    if len(sys.argv) != 2:
        sys.exit("usage: fetch_reference_fixtures.py REFERENCE_TREE (the strobealign source checkout)")
    src = Path(sys.argv[1]) / "tests"
    dst = Path(__file__).resolve().parent
    for name in FILES:
        shutil.copyfile(src / name, dst / name)
        print("copied", name)


if __name__ == "__main__":
    main()
