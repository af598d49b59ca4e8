"""ctypes binding of the oracle's in-memory entry points (oracle/capi.cpp).

TEST INFRASTRUCTURE ONLY: bench.py's parity, cpu_baseline and reference legs and the
tests use it as the checker and as the timed CPU restatement of the reference path.
The product never imports it.
"""
from __future__ import annotations

import ctypes as C
import functools
import os

import numpy as np

from . import build as _build

RS_DTYPE = np.dtype([("hash_offset", "<u8"), ("position", "<u4"), ("ref_index", "<u4")])


class ReadBatch(C.Structure):
    _fields_ = [("n", C.c_size_t), ("seq", C.c_void_p), ("seq_offsets", C.c_void_p), ("qual", C.c_void_p),
                ("names", C.c_void_p), ("name_offsets", C.c_void_p)]


class MapOpts(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("max_secondary", C.c_uint32), ("dropoff", C.c_float),
                ("rescue_distance", C.c_uint32), ("max_tries", C.c_uint32), ("mcs", C.c_uint32),
                ("output_unmapped", C.c_uint32), ("use_ssw", C.c_uint32), ("eqx", C.c_uint32),
                ("details", C.c_uint32), ("chunk_size", C.c_uint64), ("threads", C.c_uint32)]


@functools.lru_cache(None)
def lib() -> C.CDLL:
    _build.build()
    L = C.CDLL(str(_build.lib_path()))
    L.ora_index_from_buffers.restype = C.c_void_p
    L.ora_index_from_buffers.argtypes = [C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_int32,
                                         C.c_double, C.c_uint32, C.POINTER(C.c_double)]
    L.ora_index_free.argtypes = [C.c_void_p]
    L.ora_index_info.argtypes = [C.c_void_p, C.POINTER(C.c_uint64)]
    L.ora_index_view.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
    L.ora_map_batch.restype = C.c_int32
    L.ora_map_batch.argtypes = [C.c_void_p, C.POINTER(ReadBatch), C.POINTER(ReadBatch), C.POINTER(MapOpts),
                                C.POINTER(C.c_void_p), C.POINTER(C.c_size_t), C.POINTER(C.c_double)]
    L.ora_map_interleaved.restype = C.c_int32
    L.ora_map_interleaved.argtypes = [C.c_void_p, C.POINTER(ReadBatch), C.POINTER(MapOpts), C.POINTER(C.c_void_p),
                                      C.POINTER(C.c_size_t), C.POINTER(C.c_double)]
    L.ora_output_free.argtypes = [C.c_void_p]
    L.ora_lookup_sectors.restype = C.c_int32
    L.ora_lookup_sectors.argtypes = [C.c_void_p, C.POINTER(ReadBatch), C.c_int32, C.c_uint32, C.POINTER(C.c_uint64)]
    return L


def _batch(seq: np.ndarray, offsets: np.ndarray, names: bytes, name_offsets: np.ndarray, qual, keep: list):
    seq = np.ascontiguousarray(seq, dtype=np.uint8)
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    noff = np.ascontiguousarray(name_offsets, dtype=np.uint64)
    nb = C.create_string_buffer(names, len(names) + 1)
    qb = C.create_string_buffer(qual, len(qual) + 1) if qual is not None else None
    keep.extend([seq, off, noff, nb, qb])
    b = ReadBatch(len(off) - 1, seq.ctypes.data, off.ctypes.data, C.addressof(qb) if qb is not None else None,
                  C.addressof(nb), noff.ctypes.data)
    return b


def _take_output(out: C.c_void_p, n: C.c_size_t) -> bytes:
    """The bytes of an oracle output buffer, which is then freed."""
    try:
        m = n.value
        return (C.string_at(out.value, m) if m < (1 << 31) else
                np.ctypeslib.as_array((C.c_uint8 * m).from_address(out.value)).tobytes()) if m else b""
    finally:
        lib().ora_output_free(out)


class OracleIndex:
    """The oracle's make_index over contigs in memory (ASCII uint8 arrays)."""

    def __init__(self, names: list[str], seqs: list[np.ndarray], read_length: int, bits: int = -1,
                 filter_fraction: float = 0.0002, threads: int = 0):
        n = len(names)
        self._names = [x.encode() for x in names]
        self._seqs = [np.ascontiguousarray(s, dtype=np.uint8) for s in seqs]
        an = (C.c_char_p * n)(*self._names)
        aseq = (C.c_void_p * n)(*[s.ctypes.data for s in self._seqs])
        alen = (C.c_size_t * n)(*[len(s) for s in self._seqs])
        sec = C.c_double()
        self.threads = threads or os.cpu_count() or 1
        self.h = lib().ora_index_from_buffers(n, an, aseq, alen, read_length, bits, filter_fraction, self.threads,
                                              C.byref(sec))
        self.build_seconds = sec.value

    def info(self) -> tuple[int, int, int]:
        out = (C.c_uint64 * 3)()
        lib().ora_index_info(self.h, out)
        return int(out[0]), int(out[1]), int(out[2])

    def arrays(self) -> tuple[np.ndarray, np.ndarray]:
        """(table, bucket directory) as views of the oracle's own memory."""
        n, bits, _ = self.info()
        rs, bs = C.c_void_p(), C.c_void_p()
        lib().ora_index_view(self.h, C.byref(rs), C.byref(bs))
        t = np.ctypeslib.as_array((C.c_uint8 * (16 * n)).from_address(rs.value)).view(RS_DTYPE) if n else \
            np.zeros(0, RS_DTYPE)
        d = np.ctypeslib.as_array((C.c_uint64 * ((1 << bits) + 1)).from_address(bs.value))
        return t, d

    def map_batch(self, r1, r2=None, mode: int = 0, threads: int = 0, chunk_size: int = 1_000_000, eqx: bool = False,
                  use_ssw: bool = False, max_secondary: int = 0, details: bool = False) -> tuple[bytes, float]:
        """(SAM / PAF bytes without header, mapping seconds) for ReadSet-like batches
        (seq, offsets, names, name_offsets, qual)."""
        keep: list = []
        b1 = _batch(r1.seq, r1.offsets, r1.names, r1.name_offsets, r1.qual, keep)
        b2 = _batch(r2.seq, r2.offsets, r2.names, r2.name_offsets, r2.qual, keep) if r2 is not None else None
        o = self._opts(mode, threads, chunk_size, eqx, use_ssw, max_secondary, details)
        out, n, sec = C.c_void_p(), C.c_size_t(), C.c_double()
        r = lib().ora_map_batch(self.h, C.byref(b1), C.byref(b2) if b2 is not None else None, C.byref(o),
                                C.byref(out), C.byref(n), C.byref(sec))
        if r != 0:
            raise RuntimeError(f"ora_map_batch failed ({r})")
        return _take_output(out, n), sec.value

    def map_interleaved(self, reads, mode: int = 0, threads: int = 0, chunk_size: int = 1_000_000,
                        eqx: bool = False, use_ssw: bool = False, max_secondary: int = 0,
                        details: bool = False) -> tuple[bytes, float]:
        """As map_batch for one ReadSet-like batch in file order, consecutive records with
        equal names mapped as pairs and the others as single-end reads (--interleaved)."""
        keep: list = []
        b = _batch(reads.seq, reads.offsets, reads.names, reads.name_offsets, reads.qual, keep)
        o = self._opts(mode, threads, chunk_size, eqx, use_ssw, max_secondary, details)
        out, n, sec = C.c_void_p(), C.c_size_t(), C.c_double()
        r = lib().ora_map_interleaved(self.h, C.byref(b), C.byref(o), C.byref(out), C.byref(n), C.byref(sec))
        if r != 0:
            raise RuntimeError(f"ora_map_interleaved failed ({r})")
        return _take_output(out, n), sec.value

    def _opts(self, mode, threads, chunk_size, eqx, use_ssw, max_secondary, details) -> MapOpts:
        return MapOpts(mode, max_secondary, 0.5, 100, 20, 0, 1, 1 if use_ssw else 0, 1 if eqx else 0,
                       1 if details else 0, chunk_size, threads or self.threads)

    def lookup_sectors(self, reads, mcs: int = 0, rescue_distance: int = 100) -> dict:
        """Distinct 32-byte index sectors the reference's lookups read per read, summed
        over a ReadSet-like batch: directory, table, and the randstrobes probed."""
        keep: list = []
        b = _batch(reads.seq, reads.offsets, reads.names, reads.name_offsets, None, keep)
        out = (C.c_uint64 * 3)()
        lib().ora_lookup_sectors(self.h, C.byref(b), mcs, rescue_distance, out)
        return {"reads": len(reads), "dir_sectors": int(out[0]), "table_sectors": int(out[1]),
                "randstrobes": int(out[2])}

    def __del__(self):
        if getattr(self, "h", None):
            lib().ora_index_free(self.h)
            self.h = None
