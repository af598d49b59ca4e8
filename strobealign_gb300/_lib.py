"""ctypes binding of libstrobealign_gb300.so (declarations: include/strobealign_gb300.h).

The library is built in-tree by strobealign_gb300/build.py.  Loading fails loudly
when it is missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from .build import library_path

u8, u32, i32, u64, i64, f32, f64, sz = (C.c_uint8, C.c_uint32, C.c_int32, C.c_uint64, C.c_int64, C.c_float,
                                        C.c_double, C.c_size_t)
P = C.POINTER
vp = C.c_void_p
cp = C.c_char_p


class SeedingParams(C.Structure):
    _fields_ = [("profile", u32), ("k", u32), ("s", u32), ("t", u32), ("w_min", u32), ("w_max", u32),
                ("q", u64), ("max_dist", u32), ("partial_orientation_pos", u32), ("main_hash_mask", u64),
                ("forward_main_hash_mask", u64)]


class ChainingParams(C.Structure):
    _fields_ = [("max_lookback", u32), ("diag_diff_penalty", f32), ("gap_length_penalty", f32),
                ("valid_score_threshold", f32), ("max_ref_gap", u32), ("matches_weight", f32),
                ("max_diagonal_ratio", f32)]


class MappingParams(C.Structure):
    _fields_ = [("max_secondary", u32), ("dropoff_threshold", f32), ("rescue_distance", u32), ("max_tries", u32),
                ("mcs_strategy", u32), ("output_unmapped", u32), ("use_ssw", u32), ("xdrop", i32), ("match", u8),
                ("mismatch", u8), ("gap_open", u8), ("gap_extend", u8), ("end_bonus", u32), ("mode", u32),
                ("eqx", u32), ("details", u32), ("fastq_comments", u32), ("rg_id", cp), ("chunk_size", sz)]


class IndexInfo(C.Structure):
    _fields_ = [("bits", u32), ("filter_cutoff", u32), ("n_randstrobes", u64), ("device_bytes", u64),
                ("params", SeedingParams)]


class ReadBatch(C.Structure):
    _fields_ = [("n", sz), ("seq", vp), ("seq_offsets", P(u64)), ("qual", vp), ("names", vp),
                ("name_offsets", P(u64)), ("comments", vp), ("comment_offsets", P(u64))]


class QueryRandstrobe(C.Structure):
    _fields_ = [("hash", u64), ("hash_revcomp", u64), ("start", u32), ("end", u32)]


class Nam(C.Structure):
    _fields_ = [("nam_id", u32), ("ref_id", u32), ("ref_start", u32), ("ref_end", u32), ("query_start", u32),
                ("query_end", u32), ("matching_bases", u32), ("n_anchors", u32), ("score", f32),
                ("is_revcomp", u32)]


class NamDetails(C.Structure):
    _fields_ = [(n, u32) for n in ("full_not_found", "full_filtered", "full_found", "partial_not_found",
                                   "partial_filtered", "partial_found", "rescued", "n_randstrobes", "n_anchors",
                                   "n_nams", "both_orientations")]


class AlignmentC(C.Structure):
    _fields_ = [("valid", i32), ("score", u32), ("query_start", u32), ("query_end", u32), ("ref_start", u32),
                ("ref_end", u32), ("edit_distance", u32), ("cigar_offset", u32), ("cigar_len", u32)]


class StageAlignment(C.Structure):
    _fields_ = [("valid", i32), ("score", i32), ("query_start", u32), ("query_end", u32), ("ref_start", u32),
                ("ref_end", u32), ("edit_distance", u32), ("cigar_offset", u32), ("cigar_len", u32)]


class Output(C.Structure):
    _fields_ = [("data", vp), ("len", sz), ("n_reads", u64), ("n_mapped", u64), ("n_waves", u32),
                ("n_gpu_launches", u32)]


class SessionParams(C.Structure):
    _fields_ = [("max_inflight_bases", u64), ("max_inflight_requests", u32), ("policy_threads", u32),
                ("admission_streams", u32), ("borrow_inputs", u32), ("device_reserve_bytes", u64)]


class SessionInfo(C.Structure):
    _fields_ = [("arena_bases", u64), ("device_reserve_bytes", u64), ("refused_requests", u64)]


class ScheduleParams(C.Structure):
    _fields_ = [("parts", u32), ("overlap", u32), ("wave_min_jobs", u64), ("max_wave_jobs", u64)]


class Tuning(C.Structure):
    _fields_ = [("parts", u32), ("wave_min_jobs", u64), ("max_wave_jobs", u64), ("ssw_wave_max_qlen", u32),
                ("chain_lane_cluster_max", u32), ("l2_fetch_bytes", u32)]


class TuneReport(C.Structure):
    _fields_ = [("chosen", Tuning), ("seconds_default", f64), ("seconds_tuned", f64), ("trials", u32)]


class StreamParams(C.Structure):
    _fields_ = [("batch_bases", u64), ("read_ahead", u32), ("append", i32), ("header", cp), ("header_len", sz),
                ("interleaved", i32)]


class StreamStats(C.Structure):
    _fields_ = [("n_reads", u64), ("n_records", u64), ("n_mapped", u64), ("n_batches", u64), ("bytes_in", u64),
                ("bytes_out", u64), ("seconds_total", f64), ("seconds_map", f64), ("seconds_wait_input", f64)]


class RequestStats(C.Structure):
    _fields_ = [("seconds_queued", f64), ("seconds_service", f64), ("seconds_total", f64), ("n_reads", u64),
                ("n_waves", u32), ("h2d_bytes", u64), ("d2h_bytes", u64)]


class MapperStats(C.Structure):
    _fields_ = [("seconds_upload", f64), ("seconds_nams", f64), ("seconds_extension", f64),
                ("seconds_policy", f64), ("seconds_total", f64), ("n_jobs", u64), ("n_waves", u64),
                ("n_launches", u64), ("h2d_bytes", u64), ("d2h_bytes", u64), ("n_nams", u64), ("n_anchors", u64),
                ("kernel_ms", f64 * 16), ("kernel_launches", u64 * 16), ("sw_cells", u64 * 5),
                ("n_bases", u64), ("n_randstrobes", u64), ("n_anchor_total", u64), ("band_cells", u64 * 2)]


KERNEL_SLOTS = ["seed", "hits", "anchors", "sort", "chain", "nams_other", "prepare", "fill", "sw_byte", "sw_word",
                "banded_traceback", "finalize", "ext_other"]


# name -> (restype, argtypes)
SIGNATURES = {
    "sa_session_params_default": (None, [P(SessionParams)]),
    "sa_session_create": (i32, [vp, vp, P(ChainingParams), P(MappingParams), P(SessionParams), P(vp)]),
    "sa_session_submit": (i32, [vp, P(ReadBatch), P(ReadBatch), P(u64)]),
    "sa_session_submit_interleaved": (i32, [vp, P(ReadBatch), P(u64)]),
    "sa_session_poll": (i32, [vp, u64, P(i32)]),
    "sa_session_wait": (i32, [vp, u64, i64, P(Output), P(RequestStats), P(f64), sz]),
    "sa_session_free": (None, [vp]),
    "sa_session_get_info": (i32, [vp, P(SessionInfo)]),
    "sa_last_error": (cp, []),
    "sa_version": (cp, []),
    "sa_seeding_params_from_read_length": (i32, [sz, P(SeedingParams)]),
    "sa_chaining_params_default": (None, [P(ChainingParams)]),
    "sa_mapping_params_default": (None, [P(MappingParams)]),
    "sa_refs_from_fasta": (i32, [cp, P(vp)]),
    "sa_refs_from_buffers": (i32, [sz, P(cp), P(cp), P(sz), P(vp)]),
    "sa_refs_count": (sz, [vp]),
    "sa_refs_total_length": (sz, [vp]),
    "sa_refs_contig": (i32, [vp, sz, P(cp), P(u64)]),
    "sa_refs_decode": (i32, [vp, sz, u64, u64, vp]),
    "sa_refs_pick_bits": (u32, [vp, P(SeedingParams)]),
    "sa_refs_free": (None, [vp]),
    "sa_index_build": (i32, [vp, P(SeedingParams), i32, f64, P(vp)]),
    "sa_index_read_sti": (i32, [cp, P(SeedingParams), i32, P(vp)]),
    "sa_index_write_sti": (i32, [vp, cp]),
    "sa_index_get_info": (i32, [vp, P(IndexInfo)]),
    "sa_index_copy_to_host": (i32, [vp, vp, P(u64)]),
    "sa_index_lookup_batch": (i32, [vp, P(u64), sz, i32, P(i64), P(u32)]),
    "sa_index_free": (None, [vp]),
    "sa_reads_from_file": (i32, [cp, P(vp)]),
    "sa_reads_view": (i32, [vp, P(ReadBatch)]),
    "sa_reads_free": (None, [vp]),
    "sa_read_file_open": (i32, [cp, P(vp)]),
    "sa_read_file_next": (i32, [vp, sz, P(vp)]),
    "sa_read_file_close": (None, [vp]),
    "sa_reads_pair_interleaved": (i32, [P(ReadBatch), vp, sz, P(sz)]),
    "sa_estimate_read_length": (i32, [cp, P(sz)]),
    "sa_randstrobes_batch": (i32, [vp, P(ReadBatch), P(QueryRandstrobe), sz, P(u64), P(u32)]),
    "sa_randstrobes_device_noalloc": (i32, [vp, vp, vp, u32, u64, vp, vp, vp, vp, vp, vp]),
    "sa_nams_batch": (i32, [vp, P(ChainingParams), P(MappingParams), P(ReadBatch), P(Nam), sz, P(u64), P(u32),
                            P(NamDetails)]),
    "sa_align_batch": (i32, [P(MappingParams), sz, vp, P(u64), vp, P(u64), P(AlignmentC), P(u32), sz]),
    "sa_mapper_create": (i32, [vp, vp, P(ChainingParams), P(MappingParams), P(vp)]),
    "sa_mapper_free": (None, [vp]),
    "sa_map_batch": (i32, [vp, P(ReadBatch), P(ReadBatch), P(Output)]),
    "sa_map_batch_interleaved": (i32, [vp, P(ReadBatch), P(Output)]),
    "sa_output_free": (None, [P(Output)]),
    "sa_mapper_abundances": (i32, [vp, P(f64), sz]),
    "sa_sam_header": (i32, [vp, cp, cp, P(cp), sz, P(Output)]),
    "sa_mapper_upload": (i32, [vp, P(ReadBatch), P(ReadBatch)]),
    "sa_map_uploaded": (i32, [vp, P(Output)]),
    "sa_mapper_get_stats": (i32, [vp, P(MapperStats)]),
    "sa_mapper_set_profiling": (i32, [vp, i32]),
    "sa_mapper_set_parts": (i32, [vp, u32]),
    "sa_schedule_params_default": (None, [P(ScheduleParams)]),
    "sa_hamming_batch": (i32, [P(MappingParams), sz, P(u32), vp, P(u64), vp, P(u64), P(StageAlignment), P(u32), sz]),
    "sa_piecewise_pieces": (i32, [P(MappingParams), sz, P(u32), vp, P(u64), vp, P(u64), P(StageAlignment), P(u32),
                                  sz]),
    "sa_remove_spurious_anchors": (i32, [sz, P(i32), P(u64), P(u32)]),
    "sa_piecewise_batch": (i32, [P(MappingParams), u32, sz, vp, P(u64), vp, P(u64), P(u32), P(u64),
                                 P(StageAlignment), P(u32), sz]),
    "sa_mapper_set_schedule": (i32, [vp, P(ScheduleParams)]),
    "sa_tuning_default": (None, [P(Tuning)]),
    "sa_mapper_set_tuning": (i32, [vp, P(Tuning)]),
    "sa_mapper_get_tuning": (i32, [vp, P(Tuning)]),
    "sa_mapper_autotune": (i32, [vp, P(ReadBatch), P(ReadBatch), u32, P(TuneReport)]),
    "sa_measure_int_alu": (i32, [P(f64)]),
    "sa_stream_params_default": (None, [P(StreamParams)]),
    "sa_map_files": (i32, [vp, cp, cp, cp, P(StreamParams), P(StreamStats)]),
}

_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Load the library (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else library_path()
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class SaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def check(status: int) -> None:
    if status != 0:
        raise SaError(status, load().sa_last_error().decode())
