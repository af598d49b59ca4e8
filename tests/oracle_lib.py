"""ctypes access to the oracle (oracle/_build/liboracle.so) and, where it was built,
to the reference's own compiled ext/ssw/ssw.c (oracle/_ref/libssw_ref.so).
Test infrastructure: used only as the checker."""
from __future__ import annotations

import ctypes as C
import functools
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

from oracle import build as oracle_build  # noqa: E402


class SswOut(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("score1", "ref_begin1", "ref_end1", "read_begin1", "read_end1", "flag",
                                         "cigar_len")]


class OraAlignment(C.Structure):
    _fields_ = [("valid", C.c_int32)] + [(n, C.c_uint32) for n in ("score", "query_start", "query_end", "ref_start",
                                                                     "ref_end", "edit_distance", "cigar_len")]


class OraNam(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("nam_id", "ref_id", "ref_start", "ref_end", "query_start", "query_end",
                                          "matching_bases", "n_anchors")] + [("score", C.c_float),
                                                                             ("is_revcomp", C.c_uint32)]


class OraNamDetails(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("full_not_found", "full_filtered", "full_found", "partial_not_found",
                                          "partial_filtered", "partial_found", "rescued", "n_randstrobes",
                                          "n_anchors", "n_nams", "both_orientations")]


class SAlign(C.Structure):  # ext/ssw/ssw.h s_align
    _fields_ = [("score1", C.c_uint16), ("score2", C.c_uint16), ("ref_begin1", C.c_int32), ("ref_end1", C.c_int32),
                ("read_begin1", C.c_int32), ("read_end1", C.c_int32), ("ref_end2", C.c_int32),
                ("cigar", C.POINTER(C.c_uint32)), ("cigarLen", C.c_int32), ("flag", C.c_uint16)]


@functools.lru_cache(None)
def oracle() -> C.CDLL:
    oracle_build.build()
    lib = C.CDLL(str(oracle_build.lib_path()))
    lib.ora_ssw_align.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_uint8,
                                  C.c_uint8, C.POINTER(SswOut), C.POINTER(C.c_uint32), C.c_int32]
    lib.ora_aligner_align.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t, C.c_uint8, C.c_uint8, C.c_uint8,
                                      C.c_uint8, C.c_uint32, C.POINTER(OraAlignment), C.POINTER(C.c_uint32),
                                      C.c_size_t]
    lib.ora_randstrobes.argtypes = [C.c_size_t, C.c_char_p, C.c_size_t, C.POINTER(C.c_uint64), C.c_size_t,
                                    C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
    lib.ora_index_from_fasta.restype = C.c_void_p
    lib.ora_index_from_fasta.argtypes = [C.c_char_p, C.c_size_t, C.c_int32, C.c_double]
    lib.ora_index_free.argtypes = [C.c_void_p]
    lib.ora_index_info.argtypes = [C.c_void_p, C.POINTER(C.c_uint64)]
    lib.ora_index_arrays.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64)]
    lib.ora_nams.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t, C.c_int32, C.c_uint32, C.POINTER(OraNam),
                             C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(OraNamDetails)]
    return lib


@functools.lru_cache(None)
def reference_ssw() -> C.CDLL | None:
    oracle_build.build()
    p = oracle_build.ref_ssw_path()
    if not p.exists():
        return None
    lib = C.CDLL(str(p))
    lib.ssw_init.restype = C.c_void_p
    lib.ssw_init.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int8]
    lib.ssw_align.restype = C.POINTER(SAlign)
    lib.ssw_align.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_uint8, C.c_uint8, C.c_uint8, C.c_uint16,
                              C.c_int32, C.c_int32]
    lib.align_destroy.argtypes = [C.POINTER(SAlign)]
    lib.init_destroy.argtypes = [C.c_void_p]
    return lib


TRANSLATE = np.full(256, 4, dtype=np.int8)
for _c, _v in zip(b"ACGTUacgtu", [0, 1, 2, 3, 0, 0, 1, 2, 3, 0]):
    TRANSLATE[_c] = _v


def score_matrix(match=2, mismatch=8) -> np.ndarray:
    m = np.full((5, 5), -mismatch, dtype=np.int8)
    for i in range(4):
        m[i, i] = match
    return m.reshape(-1).copy()


def ssw_oracle(q: bytes, r: bytes, match=2, mismatch=8, go=12, ge=1):
    lib = oracle()
    tq = TRANSLATE[np.frombuffer(q, dtype=np.uint8)]
    tr = TRANSLATE[np.frombuffer(r, dtype=np.uint8)]
    mat = score_matrix(match, mismatch)
    out = SswOut()
    cig = (C.c_uint32 * (len(q) + len(r) + 8))()
    rc = lib.ora_ssw_align(tq.ctypes.data, len(q), tr.ctypes.data, len(r), mat.ctypes.data, 5, go, ge,
                           C.byref(out), cig, len(cig))
    assert rc == 0
    return (out.score1, out.ref_begin1, out.ref_end1, out.read_begin1, out.read_end1, out.flag,
            tuple(cig[i] for i in range(out.cigar_len)))


def ssw_reference(q: bytes, r: bytes, match=2, mismatch=8, go=12, ge=1):
    lib = reference_ssw()
    tq = TRANSLATE[np.frombuffer(q, dtype=np.uint8)].copy()
    tr = TRANSLATE[np.frombuffer(r, dtype=np.uint8)].copy()
    mat = score_matrix(match, mismatch)
    prof = lib.ssw_init(tq.ctypes.data, len(q), mat.ctypes.data, 5, 2)
    mask = max(len(q) // 2, 15)
    a = lib.ssw_align(prof, tr.ctypes.data, len(r), go, ge, 0x0F, 0, 2**31 - 1, mask)
    s = a.contents
    res = (s.score1, s.ref_begin1, s.ref_end1, s.read_begin1, s.read_end1, s.flag,
           tuple(s.cigar[i] for i in range(s.cigarLen)) if s.cigar else ())
    lib.align_destroy(a)
    lib.init_destroy(prof)
    return res


def aligner_oracle(q: bytes, r: bytes, match=2, mismatch=8, go=12, ge=1, bonus=10):
    lib = oracle()
    out = OraAlignment()
    cig = (C.c_uint32 * (2 * len(q) + len(r) + 8))()
    rc = lib.ora_aligner_align(q, len(q), r, len(r), match, mismatch, go, ge, bonus, C.byref(out), cig, len(cig))
    assert rc == 0
    if not out.valid:
        return None
    ops = "MIDNSHP=X"
    return dict(score=out.score, query_start=out.query_start, query_end=out.query_end, ref_start=out.ref_start,
                ref_end=out.ref_end, edit_distance=out.edit_distance,
                cigar="".join(f"{cig[i] >> 4}{ops[cig[i] & 15]}" for i in range(out.cigar_len)))


def randstrobes_oracle(seq: bytes, read_length_for_params: int):
    lib = oracle()
    cap = 2 * len(seq) + 2
    out = (C.c_uint64 * (4 * cap))()
    nf, nr = C.c_size_t(), C.c_size_t()
    assert lib.ora_randstrobes(read_length_for_params, seq, len(seq), out, cap, C.byref(nf), C.byref(nr)) == 0
    a = np.ctypeslib.as_array(out)[: 4 * (nf.value + nr.value)].reshape(-1, 4)
    return a[: nf.value], a[nf.value:]


class OracleIndex:
    def __init__(self, fasta: str, read_length: int, bits: int = -1, filter_fraction: float = 0.0002):
        self.lib = oracle()
        self.h = self.lib.ora_index_from_fasta(str(fasta).encode(), read_length, bits, filter_fraction)
        assert self.h

    def info(self):
        o = (C.c_uint64 * 3)()
        self.lib.ora_index_info(self.h, o)
        return int(o[0]), int(o[1]), int(o[2])

    def arrays(self):
        n, bits, _ = self.info()
        rs = np.zeros(n, dtype=np.dtype([("hash_offset", "<u8"), ("position", "<u4"), ("ref_index", "<u4")]))
        bs = np.zeros((1 << bits) + 1, dtype=np.uint64)
        self.lib.ora_index_arrays(self.h, rs.ctypes.data_as(C.c_void_p), bs.ctypes.data_as(C.POINTER(C.c_uint64)))
        return rs, bs

    def nams(self, seq: bytes, mcs: int = 0, rescue_distance: int = 100):
        cap = 4 * len(seq) + 16
        n = C.c_size_t()
        det = OraNamDetails()
        while True:
            out = (OraNam * cap)()
            rc = self.lib.ora_nams(self.h, seq, len(seq), mcs, rescue_distance, out, cap, C.byref(n), C.byref(det))
            if rc == 0:
                break
            assert n.value > cap  # the only failure: more NAMs than room; n holds the count
            cap = n.value
        rows = [tuple(getattr(out[i], f) for f, _ in OraNam._fields_) for i in range(n.value)]
        return rows, {f: getattr(det, f) for f, _ in OraNamDetails._fields_}

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ora_index_free(self.h)
            self.h = None


def run_oracle_cli(args: list[str], cwd: str | Path | None = None) -> bytes:
    import subprocess
    oracle_build.build()
    r = subprocess.run([str(oracle_build.cli_path()), *args], capture_output=True, cwd=cwd)
    if r.returncode != 0:
        raise RuntimeError(r.stderr.decode())
    return r.stdout
