"""Build recipe for the sm_103a library (libstrobealign_gb300.so), in-tree.

Compiles every translation unit under csrc/ in parallel with nvcc (CUDA sources)
and g++ (host sources), then links one shared library next to this file in
_lib/.  Host and device code are compiled without floating-point contraction so
that f32 arithmetic rounds exactly as the reference's Rust code does.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIBDIR = HERE / "_lib"
LIBNAME = "libstrobealign_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home() -> Path:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and Path(c, "bin", "nvcc").exists():
            return Path(c)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found")


def library_path() -> Path:
    return LIBDIR / LIBNAME


def synth_library_path() -> Path:
    return LIBDIR / "libsa_synth.so"


def build_synth(force: bool = False) -> Path:
    """The workload generator (synth.cpp), a host-only library of its own."""
    LIBDIR.mkdir(exist_ok=True)
    src, lib = HERE / "synth.cpp", synth_library_path()
    if force or _needs(lib, [src]):
        tmp = lib.with_suffix(".so.tmp")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-Wall", "-o", str(tmp), str(src)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    return lib


def _needs(obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [HERE.parent / "include" / "strobealign_gb300.h"]
    common = ["-O3", "-std=c++17", f"-I{CSRC}", f"-I{HERE.parent / 'include'}"]
    cu_flags = [ARCH, "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                "-diag-suppress=177"]
    cpp_flags = ["-fPIC", "-ffp-contract=off", f"-I{cuda / 'include'}", "-Wall"]
    jobs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.stem + ".cu.o")
        if force or _needs(obj, [src] + headers):
            jobs.append([nvcc, *common, *cu_flags, "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cpp")):
        obj = BUILD / (src.stem + ".cpp.o")
        if force or _needs(obj, [src] + headers):
            jobs.append(["g++", *common, *cpp_flags, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return cmd[-1]

    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        for f in [ex.submit(run, j) for j in jobs]:
            f.result()
    objs = sorted(str(p) for p in BUILD.glob("*.o"))
    lib = library_path()
    if force or jobs or not lib.exists():
        tmp = lib.with_suffix(".so.tmp")
        cmd = [nvcc, ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", str(tmp), *objs, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    build_synth(force)
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
