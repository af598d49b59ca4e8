"""strobealign_gb300: strobealign's per-read mapping path on one GB300 GPU.

Python face of the C ABI (include/strobealign_gb300.h), mirroring the reference's
library surface:

* ``SeedingParameters.from_read_length`` -- SeedingParameters::new (src/seeding/parameters.rs)
* ``References`` -- reference contigs (src/io/fasta.rs, src/packed_seq.rs)
* ``StrobemerIndex.build`` / ``.read_sti`` / ``.write_sti`` / lookups -- make_index
  (src/indexer.rs) and StrobemerIndex (src/index.rs)
* ``randstrobes_batch`` / ``nams_batch`` / ``align_batch`` -- randstrobes_query,
  get_nams_by_chaining, Aligner::align for whole batches
* ``Mapper.map`` -- align_single_end_read / align_paired_end_read /
  map_*_read / abundances_*_read (src/mapper.rs, src/maponly.rs) per chunk as
  Mapper::map_chunk does (src/main.rs)

All compute runs on the GPU through the compiled library; nothing here falls
back to the CPU.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from ._lib import SaError  # noqa: F401  (raised by every entry point)

MODE_SAM, MODE_PAF, MODE_ABUNDANCE = 0, 1, 2
MCS = {"always": 0, "rescue": 1, "off": 2, "first-strobe": 3}


def lib() -> C.CDLL:
    return L.load()


def _p(arr, ctype):
    return arr.ctypes.data_as(C.POINTER(ctype))


def _bytes(ptr, n: int) -> bytes:
    """n bytes at ptr (ctypes.string_at takes a C int size, so large buffers go
    through numpy)."""
    if not n:
        return b""
    if n < (1 << 31):
        return C.string_at(ptr, n)
    return np.ctypeslib.as_array((C.c_uint8 * n).from_address(ptr)).tobytes()


class SeedingParameters:
    """SeedingParameters (src/seeding/parameters.rs:164-221)."""

    def __init__(self, c: L.SeedingParams):
        self.c = c

    @classmethod
    def from_read_length(cls, read_length: int) -> "SeedingParameters":
        c = L.SeedingParams()
        L.check(lib().sa_seeding_params_from_read_length(read_length, C.byref(c)))
        return cls(c)

    def __getattr__(self, name):
        return getattr(self.c, name)


class References:
    """Reference contigs held as 2-bit PackedSeq on the host (uploaded by the index/mapper)."""

    def __init__(self, handle: int):
        self.h = C.c_void_p(handle)

    @classmethod
    def from_fasta(cls, path: str) -> "References":
        h = C.c_void_p()
        L.check(lib().sa_refs_from_fasta(str(path).encode(), C.byref(h)))
        return cls(h.value)

    @classmethod
    def from_sequences(cls, names: list[str], seqs: list[bytes | str]) -> "References":
        n = len(names)
        bn = [x.encode() for x in names]
        bs = [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]
        an = (C.c_char_p * n)(*bn)
        aseq = (C.c_char_p * n)(*bs)
        alen = (C.c_size_t * n)(*[len(s) for s in bs])
        h = C.c_void_p()
        L.check(lib().sa_refs_from_buffers(n, an, aseq, alen, C.byref(h)))
        r = cls(h.value)
        r._keep = (bn, bs)
        return r

    def __len__(self):
        return lib().sa_refs_count(self.h)

    @property
    def total_length(self) -> int:
        return lib().sa_refs_total_length(self.h)

    def contig(self, i: int) -> tuple[str, int]:
        """sa_refs_contig: (name, length) of contig i."""
        name, n = C.c_char_p(), C.c_uint64()
        L.check(lib().sa_refs_contig(self.h, i, C.byref(name), C.byref(n)))
        return name.value.decode(), n.value

    def decode(self, i: int, start: int = 0, end: int | None = None) -> bytes:
        """sa_refs_decode: bases [start, end) of contig i as A/C/G/T."""
        if end is None:
            end = self.contig(i)[1]
        buf = C.create_string_buffer(max(end - start, 1))
        L.check(lib().sa_refs_decode(self.h, i, start, end, buf))
        return buf.raw[:end - start]

    def pick_bits(self, params: SeedingParameters) -> int:
        return lib().sa_refs_pick_bits(self.h, C.byref(params.c))

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            lib().sa_refs_free(self.h)
            self.h = C.c_void_p()


RS_DTYPE = np.dtype([("hash_offset", "<u8"), ("position", "<u4"), ("ref_index", "<u4")])


class StrobemerIndex:
    """Device-resident StrobemerIndex (src/index.rs:66-338)."""

    FULL_FORWARD, PARTIAL, PARTIAL_FORWARD = 0, 1, 2

    def __init__(self, handle: int, params: SeedingParameters):
        self.h = C.c_void_p(handle)
        self.params = params

    @classmethod
    def build(cls, refs: References, params: SeedingParameters, bits: int = -1,
              filter_fraction: float = 0.0002) -> "StrobemerIndex":
        h = C.c_void_p()
        L.check(lib().sa_index_build(refs.h, C.byref(params.c), bits, filter_fraction, C.byref(h)))
        return cls(h.value, params)

    @classmethod
    def read_sti(cls, path: str, params: SeedingParameters, bits: int = -1) -> "StrobemerIndex":
        h = C.c_void_p()
        L.check(lib().sa_index_read_sti(str(path).encode(), C.byref(params.c), bits, C.byref(h)))
        return cls(h.value, params)

    def write_sti(self, path: str) -> None:
        L.check(lib().sa_index_write_sti(self.h, str(path).encode()))

    @property
    def info(self) -> L.IndexInfo:
        i = L.IndexInfo()
        L.check(lib().sa_index_get_info(self.h, C.byref(i)))
        return i

    @property
    def filter_cutoff(self) -> int:
        return self.info.filter_cutoff

    @property
    def bits(self) -> int:
        return self.info.bits

    def __len__(self):
        return self.info.n_randstrobes

    def to_host(self) -> tuple[np.ndarray, np.ndarray]:
        info = self.info
        rs = np.zeros(info.n_randstrobes, dtype=RS_DTYPE)
        bs = np.zeros((1 << info.bits) + 1, dtype=np.uint64)
        L.check(lib().sa_index_copy_to_host(self.h, rs.ctypes.data_as(C.c_void_p), _p(bs, C.c_uint64)))
        return rs, bs

    def lookup(self, hashes, kind: int = 0, counts: bool = False):
        """get_full_forward / get_partial / get_partial_forward for many hashes at once."""
        h = np.ascontiguousarray(hashes, dtype=np.uint64)
        pos = np.zeros(h.size, dtype=np.int64)
        cnt = np.zeros(h.size, dtype=np.uint32) if counts else None
        L.check(lib().sa_index_lookup_batch(self.h, _p(h, C.c_uint64), h.size, kind, _p(pos, C.c_int64),
                                            _p(cnt, C.c_uint32) if counts else None))
        return (pos, cnt) if counts else pos

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            lib().sa_index_free(self.h)
            self.h = C.c_void_p()


class ReadFile:
    """sa_read_file_*: a read file read in batches (next(n) gives up to n more records,
    an empty batch at the end)."""

    def __init__(self, path: str):
        self.h = C.c_void_p()
        L.check(lib().sa_read_file_open(os.fsencode(path), C.byref(self.h)))

    def next(self, max_records: int) -> "Reads":
        h = C.c_void_p()
        L.check(lib().sa_read_file_next(self.h, max_records, C.byref(h)))
        return Reads._take(h)

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            lib().sa_read_file_close(self.h)
            self.h = C.c_void_p()


@dataclass
class Reads:
    """A batch of reads as concatenated buffers (the C ABI's sa_read_batch)."""

    seq: bytes
    seq_offsets: np.ndarray
    names: bytes
    name_offsets: np.ndarray
    qual: bytes | None = None
    comments: bytes | None = None
    comment_offsets: np.ndarray | None = None

    @classmethod
    def from_lists(cls, names, seqs, quals=None, comments=None) -> "Reads":
        bs = [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]
        bn = [x.encode() if isinstance(x, str) else bytes(x) for x in names]
        so = np.zeros(len(bs) + 1, dtype=np.uint64)
        so[1:] = np.cumsum([len(s) for s in bs])
        no = np.zeros(len(bn) + 1, dtype=np.uint64)
        no[1:] = np.cumsum([len(s) for s in bn])
        q = None
        if quals is not None:
            q = b"".join(x.encode() if isinstance(x, str) else bytes(x) for x in quals)
        cm = co = None
        if comments is not None:
            bc = [(c or "").encode() if isinstance(c or "", str) else bytes(c) for c in comments]
            co = np.zeros(len(bc) + 1, dtype=np.uint64)
            co[1:] = np.cumsum([len(s) for s in bc])
            cm = b"".join(bc)
        return cls(b"".join(bs), so, b"".join(bn), no, q, cm, co)

    @classmethod
    def from_arrays(cls, seq: np.ndarray, seq_offsets: np.ndarray, names: bytes, name_offsets: np.ndarray,
                    qual: bytes | None = None) -> "Reads":
        return cls(seq.tobytes() if isinstance(seq, np.ndarray) else seq, np.ascontiguousarray(seq_offsets, np.uint64),
                   names, np.ascontiguousarray(name_offsets, np.uint64), qual)

    @classmethod
    def from_file(cls, path: str) -> "Reads":
        h = C.c_void_p()
        L.check(lib().sa_reads_from_file(str(path).encode(), C.byref(h)))
        return cls._take(h)

    @classmethod
    def _take(cls, h: C.c_void_p) -> "Reads":
        """A copy of an owned sa_reads batch, which is then freed."""
        try:
            v = L.ReadBatch()
            L.check(lib().sa_reads_view(h, C.byref(v)))
            n = v.n
            so = np.ctypeslib.as_array(v.seq_offsets, shape=(n + 1,)).copy()
            no = np.ctypeslib.as_array(v.name_offsets, shape=(n + 1,)).copy()
            co = np.ctypeslib.as_array(v.comment_offsets, shape=(n + 1,)).copy()
            seq = _bytes(v.seq, int(so[-1]))
            names = _bytes(v.names, int(no[-1]))
            qual = _bytes(v.qual, int(so[-1])) if v.qual else None
            comments = _bytes(v.comments, int(co[-1]))
            return cls(seq, so, names, no, qual, comments, co)
        finally:
            lib().sa_reads_free(h)

    def __len__(self):
        return len(self.seq_offsets) - 1

    def interleaved_records(self) -> np.ndarray:
        """sa_reads_pair_interleaved: each record's first read, then the read count (a
        record of two reads is a pair, of one read single-end)."""
        out = np.zeros(len(self) + 1, dtype=np.uint32)
        n = C.c_size_t()
        b = self.c()
        L.check(lib().sa_reads_pair_interleaved(C.byref(b), _p(out, C.c_uint32), len(out), C.byref(n)))
        return out[:n.value + 1].copy()

    def c(self) -> L.ReadBatch:
        b = L.ReadBatch()
        self._bufs = [self.seq, self.names, self.qual, self.comments]
        b.n = len(self)
        b.seq = C.cast(C.c_char_p(self.seq), C.c_void_p)
        b.seq_offsets = _p(self.seq_offsets, C.c_uint64)
        b.qual = C.cast(C.c_char_p(self.qual), C.c_void_p) if self.qual is not None else None
        b.names = C.cast(C.c_char_p(self.names), C.c_void_p)
        b.name_offsets = _p(self.name_offsets, C.c_uint64)
        if self.comments is not None and self.comment_offsets is not None:
            b.comments = C.cast(C.c_char_p(self.comments), C.c_void_p)
            b.comment_offsets = _p(self.comment_offsets, C.c_uint64)
        return b


def chaining_defaults() -> L.ChainingParams:
    c = L.ChainingParams()
    lib().sa_chaining_params_default(C.byref(c))
    return c


def mapping_defaults(**kw) -> L.MappingParams:
    m = L.MappingParams()
    lib().sa_mapping_params_default(C.byref(m))
    for k, v in kw.items():
        if k == "rg_id":
            v = v.encode() if isinstance(v, str) else v
        if k == "mcs_strategy" and isinstance(v, str):
            v = MCS[v]
        setattr(m, k, v)
    return m


def randstrobes_batch(index: StrobemerIndex, reads: Reads):
    """randstrobes_query for each read: list of (forward, reverse-complement) arrays."""
    n = len(reads)
    cap = int(reads.seq_offsets[-1]) * 2 + 1
    out = (L.QueryRandstrobe * cap)()
    offs = np.zeros(2 * n, dtype=np.uint64)
    cnt = np.zeros(2 * n, dtype=np.uint32)
    b = reads.c()
    L.check(lib().sa_randstrobes_batch(index.h, C.byref(b), out, cap, _p(offs, C.c_uint64), _p(cnt, C.c_uint32)))
    arr = np.ctypeslib.as_array(out).view(np.dtype([("hash", "<u8"), ("hash_revcomp", "<u8"), ("start", "<u4"),
                                                     ("end", "<u4")]))
    return [(arr[offs[2 * r]:offs[2 * r] + cnt[2 * r]].copy(), arr[offs[2 * r + 1]:offs[2 * r + 1] + cnt[2 * r + 1]].copy())
            for r in range(n)]


NAM_DTYPE = np.dtype([("nam_id", "<u4"), ("ref_id", "<u4"), ("ref_start", "<u4"), ("ref_end", "<u4"),
                      ("query_start", "<u4"), ("query_end", "<u4"), ("matching_bases", "<u4"),
                      ("n_anchors", "<u4"), ("score", "<f4"), ("is_revcomp", "<u4")])
DETAILS_DTYPE = np.dtype([(n, "<u4") for n in ("full_not_found", "full_filtered", "full_found", "partial_not_found",
                                               "partial_filtered", "partial_found", "rescued", "n_randstrobes",
                                               "n_anchors", "n_nams", "both_orientations")])


def nams_batch(index: StrobemerIndex, reads: Reads, chaining: L.ChainingParams | None = None,
               mapping: L.MappingParams | None = None):
    """get_nams_by_chaining for each read: NAM arrays sorted by score (stable), and details."""
    n = len(reads)
    cap = max(1, int(reads.seq_offsets[-1]) * 4)
    out = np.zeros(cap, dtype=NAM_DTYPE)
    offs = np.zeros(n, dtype=np.uint64)
    cnt = np.zeros(n, dtype=np.uint32)
    det = np.zeros(n, dtype=DETAILS_DTYPE)
    b = reads.c()
    cpar = chaining or chaining_defaults()
    mpar = mapping or mapping_defaults()
    L.check(lib().sa_nams_batch(index.h, C.byref(cpar), C.byref(mpar), C.byref(b),
                                out.ctypes.data_as(C.POINTER(L.Nam)), cap, _p(offs, C.c_uint64), _p(cnt, C.c_uint32),
                                det.ctypes.data_as(C.POINTER(L.NamDetails))))
    return [out[offs[r]:offs[r] + cnt[r]].copy() for r in range(n)], det


ALN_DTYPE = np.dtype([("valid", "<i4"), ("score", "<u4"), ("query_start", "<u4"), ("query_end", "<u4"),
                      ("ref_start", "<u4"), ("ref_end", "<u4"), ("edit_distance", "<u4"), ("cigar_offset", "<u4"),
                      ("cigar_len", "<u4")])
CIGAR_OPS = "MIDNSHP=X"


def cigar_str(ops) -> str:
    return "".join(f"{int(v) >> 4}{CIGAR_OPS[int(v) & 15]}" for v in ops)


def align_batch(queries, refs, mapping: L.MappingParams | None = None):
    """Aligner::align (SSW + end bonus) for (query, reference) pairs.  Returns a list of
    dicts, or None where the reference returns None."""
    bq = [q.encode() if isinstance(q, str) else bytes(q) for q in queries]
    br = [r.encode() if isinstance(r, str) else bytes(r) for r in refs]
    n = len(bq)
    qo = np.zeros(n + 1, dtype=np.uint64)
    qo[1:] = np.cumsum([len(x) for x in bq])
    ro = np.zeros(n + 1, dtype=np.uint64)
    ro[1:] = np.cumsum([len(x) for x in br])
    out = np.zeros(max(n, 1), dtype=ALN_DTYPE)
    cap = int(qo[-1] * 2 + ro[-1] + 4 * n + 8)
    cig = np.zeros(cap, dtype=np.uint32)
    Q, R = b"".join(bq), b"".join(br)
    m = mapping or mapping_defaults()
    L.check(lib().sa_align_batch(C.byref(m), n, C.c_char_p(Q), _p(qo, C.c_uint64), C.c_char_p(R),
                                 _p(ro, C.c_uint64), out.ctypes.data_as(C.POINTER(L.AlignmentC)),
                                 _p(cig, C.c_uint32), cap))
    res = []
    for i in range(n):
        a = out[i]
        if not a["valid"]:
            res.append(None)
            continue
        ops = cig[a["cigar_offset"]:a["cigar_offset"] + a["cigar_len"]]
        res.append(dict(score=int(a["score"]), query_start=int(a["query_start"]), query_end=int(a["query_end"]),
                        ref_start=int(a["ref_start"]), ref_end=int(a["ref_end"]),
                        edit_distance=int(a["edit_distance"]), cigar=cigar_str(ops)))
    return res


def _pairs(queries, refs):
    bq = [q.encode() if isinstance(q, str) else bytes(q) for q in queries]
    br = [r.encode() if isinstance(r, str) else bytes(r) for r in refs]
    n = len(bq)
    qo = np.zeros(n + 1, dtype=np.uint64)
    qo[1:] = np.cumsum([len(x) for x in bq])
    ro = np.zeros(n + 1, dtype=np.uint64)
    ro[1:] = np.cumsum([len(x) for x in br])
    return b"".join(bq), qo, b"".join(br), ro


def _stage_results(out, cig, n) -> list:
    res = []
    for i in range(n):
        a = out[i]
        if not a.valid:
            res.append(None)
            continue
        ops = cig[a.cigar_offset:a.cigar_offset + a.cigar_len]
        res.append(dict(score=int(a.score), query_start=int(a.query_start), query_end=int(a.query_end),
                        ref_start=int(a.ref_start), ref_end=int(a.ref_end), edit_distance=int(a.edit_distance),
                        cigar=cigar_str(ops)))
    return res


def _stage(fn, kinds, queries, refs, mapping):
    Q, qo, R, ro = _pairs(queries, refs)
    n = len(qo) - 1
    k = np.ascontiguousarray(kinds, dtype=np.uint32)
    out = (L.StageAlignment * max(n, 1))()
    cap = int(qo[-1] + ro[-1] + 4 * n + 8)
    cig = np.zeros(cap, dtype=np.uint32)
    m = mapping or mapping_defaults()
    L.check(fn(C.byref(m), n, _p(k, C.c_uint32), C.c_char_p(Q), _p(qo, C.c_uint64), C.c_char_p(R),
               _p(ro, C.c_uint64), out, _p(cig, C.c_uint32), cap))
    return _stage_results(out, cig, n)


def hamming_batch(queries, refs, kinds, mapping: L.MappingParams | None = None):
    """hamming_align (kind 0) / hamming_align_global (kind 1) of (query, reference)
    pairs on the GPU; dicts, or None where the reference returns None."""
    return _stage(lib().sa_hamming_batch, kinds, queries, refs, mapping)


PIECE_GLOBAL, PIECE_AFTER_LAST, PIECE_BEFORE_FIRST = 0, 1, 2


def piecewise_pieces(queries, refs, kinds, mapping: L.MappingParams | None = None):
    """One piecewise-extension piece per pair: global (0), x-drop GlobalStartLocalEnd
    (1) or LocalStartGlobalEnd (2)."""
    return _stage(lib().sa_piecewise_pieces, kinds, queries, refs, mapping)


def remove_spurious_anchors(chains):
    """remove_spurious_anchors on chains of (query_start, ref_start) pairs."""
    off = np.zeros(len(chains) + 1, dtype=np.uint64)
    off[1:] = np.cumsum([len(c) for c in chains])
    anc = np.array([v for c in chains for a in c for v in a] or [0], dtype=np.int32)
    cnt = np.zeros(max(1, len(chains)), dtype=np.uint32)
    L.check(lib().sa_remove_spurious_anchors(len(chains), _p(anc, C.c_int32), _p(off, C.c_uint64),
                                             _p(cnt, C.c_uint32)))
    return [[(int(anc[2 * j]), int(anc[2 * j + 1])) for j in range(int(off[i]), int(off[i]) + int(cnt[i]))]
            for i in range(len(chains))]


def piecewise_batch(queries, refs, anchors, k: int, mapping: L.MappingParams | None = None):
    """extend_piecewise (with remove_spurious_anchors) per (query, window, anchors last
    to first as (query_start, ref_start) pairs)."""
    Q, qo, R, ro = _pairs(queries, refs)
    n = len(qo) - 1
    aoff = np.zeros(n + 1, dtype=np.uint64)
    aoff[1:] = np.cumsum([len(a) for a in anchors])
    anc = np.array([v for a in anchors for x in a for v in x] or [0], dtype=np.uint32)
    out = (L.StageAlignment * max(n, 1))()
    cap = int(2 * qo[-1] + ro[-1] + 4 * n + 8)
    cig = np.zeros(cap, dtype=np.uint32)
    m = mapping or mapping_defaults()
    L.check(lib().sa_piecewise_batch(C.byref(m), k, n, C.c_char_p(Q), _p(qo, C.c_uint64), C.c_char_p(R),
                                     _p(ro, C.c_uint64), _p(anc, C.c_uint32), _p(aoff, C.c_uint64), out,
                                     _p(cig, C.c_uint32), cap))
    return _stage_results(out, cig, n)


class Mapper:
    """Maps batches of reads; keeps the index and its device arenas resident."""

    def __init__(self, index: StrobemerIndex, refs: References, chaining: L.ChainingParams | None = None,
                 mapping: L.MappingParams | None = None, **kw):
        self.index, self.refs = index, refs
        self.cp = chaining or chaining_defaults()
        self.mp = mapping or mapping_defaults(**kw)
        h = C.c_void_p()
        L.check(lib().sa_mapper_create(index.h, refs.h, C.byref(self.cp), C.byref(self.mp), C.byref(h)))
        self.h = h
        self.last = None

    def map(self, r1: Reads, r2: Reads | None = None, copy: bool = True):
        """Output bytes; with copy=False only their length (the bytes stay in the
        library's buffer, which is freed: for timing runs)."""
        o = L.Output()
        b1 = r1.c()
        b2 = r2.c() if r2 is not None else None
        L.check(lib().sa_map_batch(self.h, C.byref(b1), C.byref(b2) if b2 is not None else None, C.byref(o)))
        try:
            data = _bytes(o.data, o.len) if copy else o.len
            self.last = dict(n_reads=o.n_reads, n_mapped=o.n_mapped, n_waves=o.n_waves,
                             n_gpu_launches=o.n_gpu_launches)
            return data
        finally:
            lib().sa_output_free(C.byref(o))

    def map_interleaved(self, reads: Reads, copy: bool = True):
        """sa_map_batch_interleaved: reads in file order, consecutive reads with equal
        names mapped as pairs and the others as single-end records."""
        o = L.Output()
        b = reads.c()
        L.check(lib().sa_map_batch_interleaved(self.h, C.byref(b), C.byref(o)))
        try:
            data = _bytes(o.data, o.len) if copy else o.len
            self.last = dict(n_reads=o.n_reads, n_mapped=o.n_mapped, n_waves=o.n_waves,
                             n_gpu_launches=o.n_gpu_launches)
            return data
        finally:
            lib().sa_output_free(C.byref(o))

    def upload(self, r1: Reads, r2: Reads | None = None) -> None:
        """Copy a batch to the device; map it with map_uploaded()."""
        self._b1 = r1.c()
        self._b2 = r2.c() if r2 is not None else None
        self._keep = (r1, r2)
        L.check(lib().sa_mapper_upload(self.h, C.byref(self._b1),
                                       C.byref(self._b2) if self._b2 is not None else None))

    def map_uploaded(self, copy: bool = True):
        o = L.Output()
        L.check(lib().sa_map_uploaded(self.h, C.byref(o)))
        try:
            self.last = dict(n_reads=o.n_reads, n_mapped=o.n_mapped, n_waves=o.n_waves,
                             n_gpu_launches=o.n_gpu_launches)
            if not copy:
                return o.len
            return _bytes(o.data, o.len)
        finally:
            lib().sa_output_free(C.byref(o))

    def stats(self) -> dict:
        s = L.MapperStats()
        L.check(lib().sa_mapper_get_stats(self.h, C.byref(s)))
        d = {f: getattr(s, f) for f, _ in L.MapperStats._fields_ if not f.startswith("kernel_")}
        d["kernel_ms"] = {n: s.kernel_ms[i] for i, n in enumerate(L.KERNEL_SLOTS)}
        d["kernel_launches"] = {n: s.kernel_launches[i] for i, n in enumerate(L.KERNEL_SLOTS)}
        d["sw_cells"] = dict(zip(("canonical", "forward_byte", "forward_word", "reverse_byte", "reverse_word"),
                                 list(s.sw_cells)))
        d["sw_cells"].update(band_computed=int(s.band_cells[0]), band_canonical=int(s.band_cells[1]))
        d.pop("band_cells", None)
        return d

    def set_profiling(self, on: bool = True) -> None:
        L.check(lib().sa_mapper_set_profiling(self.h, 1 if on else 0))

    def set_parts(self, parts: int) -> None:
        """NAM-pipeline parts a large batch is cut into (output does not depend on it)."""
        L.check(lib().sa_mapper_set_parts(self.h, parts))

    def set_schedule(self, parts: int = 0, overlap: bool = True, wave_min_jobs: int = 0,
                     max_wave_jobs: int = 0) -> None:
        """Batch scheduling (sa_mapper_set_schedule); output bytes do not depend on it.
        parts=0 takes the library's default (8); overlap=False is the plain,
        stage-synchronous form."""
        sp = L.ScheduleParams()
        lib().sa_schedule_params_default(C.byref(sp))
        sp.parts = parts
        sp.overlap = 1 if overlap else 0
        if wave_min_jobs:
            sp.wave_min_jobs = wave_min_jobs
        if max_wave_jobs:
            sp.max_wave_jobs = max_wave_jobs
        L.check(lib().sa_mapper_set_schedule(self.h, C.byref(sp)))

    def tuning(self) -> dict:
        t = L.Tuning()
        L.check(lib().sa_mapper_get_tuning(self.h, C.byref(t)))
        return {f: int(getattr(t, f)) for f, _ in L.Tuning._fields_}

    def set_tuning(self, **kw) -> None:
        t = L.Tuning()
        L.check(lib().sa_mapper_get_tuning(self.h, C.byref(t)))
        for k, v in kw.items():
            setattr(t, k, v)
        L.check(lib().sa_mapper_set_tuning(self.h, C.byref(t)))

    def autotune(self, r1: Reads, r2: Reads | None = None, rounds: int = 2) -> dict:
        """sa_mapper_autotune on a calibration batch (it stays uploaded): the chosen knobs
        and the batch's time under the defaults and under them."""
        rep = L.TuneReport()
        self._b1 = r1.c()
        self._b2 = r2.c() if r2 is not None else None
        self._keep = (r1, r2)
        L.check(lib().sa_mapper_autotune(self.h, C.byref(self._b1), C.byref(self._b2) if self._b2 is not None else None,
                                         rounds, C.byref(rep)))
        return {"chosen": {f: int(getattr(rep.chosen, f)) for f, _ in L.Tuning._fields_},
                "seconds_default": rep.seconds_default, "seconds_tuned": rep.seconds_tuned, "trials": rep.trials}

    def map_files(self, reads1: str, reads2: str | None, out: str, header: bytes = b"", batch_bases: int = 0,
                  read_ahead: int = 0, append: bool = False, interleaved: bool = False) -> dict:
        """sa_map_files: reads1 (and reads2) mapped into the file out, parsing, mapping and
        writing overlapped; header (the SAM header) is written first; interleaved: reads1
        holds mixed single-end and paired records.  Returns the stream statistics."""
        p = L.StreamParams()
        lib().sa_stream_params_default(C.byref(p))
        if batch_bases:
            p.batch_bases = batch_bases
        if read_ahead:
            p.read_ahead = read_ahead
        p.append = int(append)
        p.interleaved = int(interleaved)
        p.header = header or None
        p.header_len = len(header)
        st = L.StreamStats()
        L.check(lib().sa_map_files(self.h, os.fsencode(reads1), os.fsencode(reads2) if reads2 else None,
                                   os.fsencode(out), C.byref(p), C.byref(st)))
        return {f: getattr(st, f) for f, _ in L.StreamStats._fields_}

    def abundances(self) -> np.ndarray:
        n = len(self.refs)
        out = np.zeros(n, dtype=np.float64)
        L.check(lib().sa_mapper_abundances(self.h, _p(out, C.c_double), n))
        return out

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            lib().sa_mapper_free(self.h)
            self.h = C.c_void_p()


class Session:
    """Serving session: requests are mapped with continuous batching on the GPU.

    Each request is mapped as its own chunk stream, so its bytes equal
    Mapper.map on the same records alone."""

    def __init__(self, index: StrobemerIndex, refs: References, chaining: L.ChainingParams | None = None,
                 mapping: L.MappingParams | None = None, max_inflight_bases: int = 0, max_inflight_requests: int = 0,
                 policy_threads: int = 0, admission_streams: int = 0, borrow_inputs: bool = False,
                 device_reserve_bytes: int = 0, **kw):
        self.index, self.refs = index, refs
        # borrow_inputs: the session reads the submitted Reads in place; they are kept
        # referenced here until wait() returns for their ticket
        self.borrow = bool(borrow_inputs)
        self._borrowed: dict[int, tuple] = {}
        self.cp = chaining or chaining_defaults()
        self.mp = mapping or mapping_defaults(**kw)
        sp = L.SessionParams()
        lib().sa_session_params_default(C.byref(sp))
        if max_inflight_bases:
            sp.max_inflight_bases = max_inflight_bases
        sp.max_inflight_requests = max_inflight_requests
        sp.policy_threads = policy_threads
        if admission_streams:
            sp.admission_streams = admission_streams
        sp.borrow_inputs = 1 if self.borrow else 0
        sp.device_reserve_bytes = device_reserve_bytes
        h = C.c_void_p()
        L.check(lib().sa_session_create(index.h, refs.h, C.byref(self.cp), C.byref(self.mp), C.byref(sp),
                                        C.byref(h)))
        self.h = h

    def submit(self, r1: Reads, r2: Reads | None = None) -> int:
        b1 = r1.c()
        b2 = r2.c() if r2 is not None else None
        t = C.c_uint64()
        L.check(lib().sa_session_submit(self.h, C.byref(b1), C.byref(b2) if b2 is not None else None, C.byref(t)))
        if self.borrow:
            self._borrowed[t.value] = (r1, r2, b1, b2)
        return t.value

    def submit_interleaved(self, reads: Reads) -> int:
        """sa_session_submit_interleaved: mixed single-end and paired records in file
        order, paired by name."""
        b = reads.c()
        t = C.c_uint64()
        L.check(lib().sa_session_submit_interleaved(self.h, C.byref(b), C.byref(t)))
        if self.borrow:
            self._borrowed[t.value] = (reads, None, b, None)
        return t.value

    @property
    def info(self) -> dict:
        """The device read arena (bases) and memory reserve the session chose, and the
        requests refused for lack of device memory."""
        i = L.SessionInfo()
        L.check(lib().sa_session_get_info(self.h, C.byref(i)))
        return {f: int(getattr(i, f)) for f, _ in L.SessionInfo._fields_}

    def poll(self, ticket: int) -> bool:
        d = C.c_int32()
        L.check(lib().sa_session_poll(self.h, ticket, C.byref(d)))
        return bool(d.value)

    def wait(self, ticket: int, timeout_ms: int = -1, abundances: bool = False, copy: bool = True):
        """(output bytes, stats dict[, abundances]); copy=False gives the output length instead."""
        o = L.Output()
        st = L.RequestStats()
        ab = np.zeros(len(self.refs), dtype=np.float64) if abundances else None
        L.check(lib().sa_session_wait(self.h, ticket, timeout_ms, C.byref(o), C.byref(st),
                                      _p(ab, C.c_double) if ab is not None else None, len(ab) if ab is not None else 0))
        self._borrowed.pop(ticket, None)
        try:
            data = _bytes(o.data, o.len) if copy else o.len
        finally:
            lib().sa_output_free(C.byref(o))
        stats = {f: getattr(st, f) for f, _ in L.RequestStats._fields_}
        stats["n_mapped"] = o.n_mapped
        return (data, stats, ab) if abundances else (data, stats)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().sa_session_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        self.close()


def measure_int_alu() -> dict:
    """sa_measure_int_alu: the device's integer instruction rates (per second)."""
    out = (C.c_double * 2)()
    L.check(lib().sa_measure_int_alu(out))
    return {"viaddmax_per_s": out[0], "max_xor_per_s": out[1]}


def estimate_read_length(path: str) -> int:
    """sa_estimate_read_length: mean length of the first 500 records of a read file."""
    n = C.c_size_t()
    L.check(lib().sa_estimate_read_length(os.fsencode(path), C.byref(n)))
    return n.value


def sam_header(refs: References, cmd_line: str | None = None, rg_id: str | None = None,
               rg_fields: list[str] = ()) -> bytes:
    o = L.Output()
    f = [x.encode() for x in rg_fields]
    arr = (C.c_char_p * max(1, len(f)))(*f)
    L.check(lib().sa_sam_header(refs.h, cmd_line.encode() if cmd_line else None, rg_id.encode() if rg_id else None,
                                arr, len(f), C.byref(o)))
    try:
        return _bytes(o.data, o.len)
    finally:
        lib().sa_output_free(C.byref(o))
