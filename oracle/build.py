"""Build recipe for the oracle (test infrastructure only).

* oracle/_build/sa_oracle       -- CLI: the reference's mapping path restated in C++
* oracle/_build/liboracle.so    -- the same code behind ctypes entry points (capi.cpp)
* oracle/_ref/libssw_ref.so     -- the reference's own ext/ssw/ssw.c compiled from where
                                   it lies in the reference tree, only when a tree is named
                                   (argument, or STROBEALIGN_REFERENCE in the environment);
                                   used to fuzz the SSW restatement

    python oracle/build.py [REFERENCE_TREE]

All objects are compiled with -ffp-contract=off so f32/f64 expressions round as
the reference's Rust code does.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
SOURCES = ["seeding.cpp", "nams.cpp", "ssw.cpp", "mapper.cpp", "piecewise.cpp", "io.cpp", "driver.cpp"]
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-Wall"]


def reference_tree(tree: str | os.PathLike | None = None) -> Path | None:
    """The strobealign source checkout to compile ext/ssw/ssw.c from: the argument, else
    STROBEALIGN_REFERENCE; None when neither names one."""
    t = tree if tree is not None else os.environ.get("STROBEALIGN_REFERENCE")
    return Path(t) if t else None


def cli_path() -> Path:
    return BUILD / "sa_oracle"


def lib_path() -> Path:
    return BUILD / "liboracle.so"


def ref_ssw_path() -> Path:
    return REF_OUT / "libssw_ref.so"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, reference: str | os.PathLike | None = None) -> None:
    BUILD.mkdir(exist_ok=True)
    srcs = [HERE / s for s in SOURCES]
    deps = srcs + [HERE / "oracle.hpp", HERE / "main.cpp", HERE / "capi.cpp"]
    newest = max(d.stat().st_mtime for d in deps)
    objs = []
    jobs = []
    for s in srcs + [HERE / "main.cpp", HERE / "capi.cpp"]:
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if force or not o.exists() or o.stat().st_mtime < max(s.stat().st_mtime, (HERE / "oracle.hpp").stat().st_mtime):
            jobs.append(["g++", *FLAGS, "-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    core = [str(BUILD / (Path(s).stem + ".o")) for s in SOURCES]
    if force or jobs or not cli_path().exists() or cli_path().stat().st_mtime < newest:
        _run(["g++", *FLAGS, "-o", str(cli_path()), *core, str(BUILD / "main.o"), "-lpthread"])
    if force or jobs or not lib_path().exists() or lib_path().stat().st_mtime < newest:
        _run(["g++", *FLAGS, "-shared", "-o", str(lib_path()), *core, str(BUILD / "capi.o"), "-lpthread"])
    tree = reference_tree(reference)
    ssw = tree / "ext" / "ssw" / "ssw.c" if tree is not None else None
    if ssw is not None and ssw.exists():
        REF_OUT.mkdir(exist_ok=True)
        if force or not ref_ssw_path().exists():
            _run(["gcc", "-O2", "-fPIC", "-shared", "-o", str(ref_ssw_path()), str(ssw), "-lm"])


if __name__ == "__main__":
    import sys
    build(force=True, reference=sys.argv[1] if len(sys.argv) > 1 else None)
    print(cli_path(), lib_path(), ref_ssw_path() if ref_ssw_path().exists() else "(no reference tree)")
