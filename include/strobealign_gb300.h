/*
 * strobealign_gb300 -- C ABI of the GB300 (sm_103a) read-mapping library.
 *
 * The library is a drop-in for strobealign's per-read mapping path: index
 * construction and StrobemerIndex lookups, NAM finding (seeding -> hits ->
 * anchors -> collinear chaining), base-level extension (SSW-exact Smith-Waterman,
 * Hamming fast path, mate rescue) and SAM / PAF / abundance output.  Every call
 * returns an int32 status (SA_OK or a negative SA_ERR_*); it never aborts.  The
 * message of the last failure on the calling thread is sa_last_error().
 *
 * Buffers passed in are borrowed for the duration of the call (the library copies
 * what it keeps).  Output buffers returned through sa_output are owned by the
 * library until sa_output_free().  Handles are not thread-safe unless stated.
 *
 * Reference interfaces each entry point replaces are cited as file:line of the
 * strobealign source tree (Rust, v0.18.0-alpha).
 */
#ifndef STROBEALIGN_GB300_H
#define STROBEALIGN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define SA_OK 0
#define SA_ERR_INVALID (-1)      /* bad argument or parameter                 */
#define SA_ERR_CUDA (-2)         /* CUDA runtime error or no usable device      */
#define SA_ERR_OOM (-3)          /* device or host allocation failed            */
#define SA_ERR_IO (-4)           /* file could not be read or written           */
#define SA_ERR_STI_MISMATCH (-5) /* .sti magic/version/parameters differ        */
#define SA_ERR_TIMEOUT (-6)      /* a bounded device wait gave up               */
#define SA_ERR_CANCELLED (-7)    /* request cancelled                           */
#define SA_ERR_FORMAT (-8)       /* malformed FASTA/FASTQ input                 */
#define SA_ERR_BUSY (-9)         /* admission refused: not enough free memory   */

/* Message describing the last failure on this thread (never NULL). */
const char* sa_last_error(void);
/* Library version string. */
const char* sa_version(void);

/* ---------------------------------------------------------------- parameters */
/* SeedingParameters (src/seeding/parameters.rs:164-171; presets :102-159). */
typedef struct {
    uint32_t profile; /* Profile discriminant: 0 noisy, 1 r50, ... 7 r400 */
    uint32_t k, s, t;
    uint32_t w_min, w_max;
    uint64_t q;
    uint32_t max_dist;
    uint32_t partial_orientation_pos;
    uint64_t main_hash_mask;
    uint64_t forward_main_hash_mask;
} sa_seeding_params;

/* SeedingParameters::new(read_length) (src/seeding/parameters.rs:181-221). */
int32_t sa_seeding_params_from_read_length(size_t read_length, sa_seeding_params* out);
/* estimate_read_length over the first 500 records of a read file (src/main.rs:351,
 * :1003-1012): the mean sequence length, rounded down; 0 for an empty file.  Plain or
 * gzip FASTQ/FASTA; standard input ("-") is refused, since its records would be used up. */
int32_t sa_estimate_read_length(const char* path, size_t* out);

/* ChainingParameters (src/chainer.rs:16-44), MappingParameters (src/mapper.rs:31-55),
 * Scores (src/aligner.rs:11-30) and SAM output options (src/mapper.rs:87-112). */
typedef struct {
    uint32_t max_lookback;        /* 50 */
    float diag_diff_penalty;      /* 0.1 */
    float gap_length_penalty;     /* 0.05 */
    float valid_score_threshold;  /* 0.7 */
    uint32_t max_ref_gap;         /* 0 = read length */
    float matches_weight;         /* 0.01 */
    float max_diagonal_ratio;     /* 10.0 */
} sa_chaining_params;

enum { SA_MCS_ALWAYS = 0, SA_MCS_RESCUE = 1, SA_MCS_OFF = 2, SA_MCS_FIRST_STROBE = 3 };
enum { SA_MODE_SAM = 0, SA_MODE_PAF = 1, SA_MODE_ABUNDANCE = 2 };

typedef struct {
    uint32_t max_secondary;  /* -N, 0 */
    float dropoff_threshold; /* -S, 0.5 */
    uint32_t rescue_distance;/* -R, 100 */
    uint32_t max_tries;      /* -M, 20 */
    uint32_t mcs_strategy;   /* SA_MCS_* */
    uint32_t output_unmapped;/* !-U, 1 */
    uint32_t use_ssw;        /* --ssw: single-end extension by SSW instead of piecewise */
    int32_t xdrop;           /* 500 */
    uint8_t match, mismatch, gap_open, gap_extend; /* 2 8 12 1 */
    uint32_t end_bonus;      /* 10 */
    uint32_t mode;           /* SA_MODE_* */
    uint32_t eqx;            /* --eqx */
    uint32_t details;        /* --details */
    uint32_t fastq_comments; /* -C */
    const char* rg_id;       /* RG:Z: value or NULL */
    size_t chunk_size;       /* nucleotides per chunk (1000000) */
} sa_mapping_params;

/* Fill the reference's defaults. */
void sa_chaining_params_default(sa_chaining_params* p);
void sa_mapping_params_default(sa_mapping_params* p);

/* ---------------------------------------------------------------- references */
/* Reference contigs as PackedSeq (src/packed_seq.rs) plus names; read_fasta
 * (src/io/fasta.rs:116-165). */
typedef struct sa_refs sa_refs;
int32_t sa_refs_from_fasta(const char* path, sa_refs** out);
int32_t sa_refs_from_buffers(size_t n_contigs, const char* const* names, const char* const* seqs,
                             const size_t* lens, sa_refs** out);
size_t sa_refs_count(const sa_refs* refs);
size_t sa_refs_total_length(const sa_refs* refs);
/* Contig i's name (NUL-terminated, owned by refs) and length in bases. */
int32_t sa_refs_contig(const sa_refs* refs, size_t i, const char** name, uint64_t* length);
/* PackedSeq::decode (src/packed_seq.rs:103-126): bases [start, end) of contig i as ASCII
 * A/C/G/T into out (end - start bytes; a wildcard base decodes to its pseudo-random
 * 2-bit value, src/packed_seq.rs:50-59). */
int32_t sa_refs_decode(const sa_refs* refs, size_t i, uint64_t start, uint64_t end, char* out);
/* SyncmerParameters::pick_bits (src/indexer.rs:294-300). */
uint32_t sa_refs_pick_bits(const sa_refs* refs, const sa_seeding_params* p);
void sa_refs_free(sa_refs* refs);

/* ---------------------------------------------------------------- index */
/* StrobemerIndex resident in device memory (src/index.rs:66-90). */
typedef struct sa_index sa_index;

typedef struct {
    uint32_t bits;
    uint32_t filter_cutoff;
    uint64_t n_randstrobes;
    uint64_t device_bytes;
    sa_seeding_params params;
} sa_index_info;

/* make_index (src/indexer.rs:18-170) built on the GPU; bits < 0 picks
 * automatically.  The sorted table and directory are identical to the reference's. */
int32_t sa_index_build(const sa_refs* refs, const sa_seeding_params* p, int32_t bits, double filter_fraction,
                       sa_index** out);
/* read_index (src/index.rs:412-495) straight into device memory. */
int32_t sa_index_read_sti(const char* path, const sa_seeding_params* p, int32_t bits, sa_index** out);
/* StrobemerIndex::write (src/index.rs:374-409), .sti format version 7. */
int32_t sa_index_write_sti(const sa_index* idx, const char* path);
int32_t sa_index_get_info(const sa_index* idx, sa_index_info* out);
/* Copy the sorted RefRandstrobe table (16 B each: u64 hash_offset, u32 position,
 * u32 ref_index) and the (2^bits + 1) bucket starts to host memory. */
int32_t sa_index_copy_to_host(const sa_index* idx, void* randstrobes, uint64_t* bucket_starts);

/* Batched StrobemerIndex lookups (src/index.rs:127-205, :254-338).
 * kind: 0 get_full_forward, 1 get_partial, 2 get_partial_forward.
 * out_position[i] = table index of the first match or -1; out_count[i] (may be
 * NULL) = get_count for the matched mask. Host buffers. */
int32_t sa_index_lookup_batch(const sa_index* idx, const uint64_t* hashes, size_t n, int32_t kind,
                              int64_t* out_position, uint32_t* out_count);
void sa_index_free(sa_index* idx);

/* ---------------------------------------------------------------- reads */
/* A batch of reads in host memory.  Sequence i is seq[seq_offsets[i] ..
 * seq_offsets[i+1]); qual (optional, same offsets), names and comments
 * (optional) likewise.  For paired-end input, r1 and r2 batches have equal n. */
typedef struct {
    size_t n;
    const char* seq;
    const uint64_t* seq_offsets; /* n + 1 */
    const char* qual;            /* NULL for FASTA input */
    const char* names;
    const uint64_t* name_offsets; /* n + 1 */
    const char* comments;         /* NULL if none */
    const uint64_t* comment_offsets;
} sa_read_batch;

/* Parse a FASTQ/FASTA read file (src/io/fastq.rs:19-100) into an owned batch; gzip
 * when the name ends in ".gz" (src/io/xopen.rs:9-20), "-" for standard input. */
typedef struct sa_reads sa_reads;
int32_t sa_reads_from_file(const char* path, sa_reads** out);
int32_t sa_reads_view(const sa_reads* reads, sa_read_batch* view);
void sa_reads_free(sa_reads* reads);
/* A read file read in batches, as the reference's record iterator yields records
 * (src/io/reads.rs:121-132 over FastqReader / FastaReader): sa_read_file_next parses up
 * to max_records more records into a new owned batch (release with sa_reads_free); a
 * batch of 0 records marks the end of the input.  Same formats and rules as
 * sa_reads_from_file. */
typedef struct sa_read_file sa_read_file;
int32_t sa_read_file_open(const char* path, sa_read_file** out);
int32_t sa_read_file_next(sa_read_file* f, size_t max_records, sa_reads** out);
void sa_read_file_close(sa_read_file* f);
/* The records InterleavedIterator forms from reads in file order (src/io/reads.rs:68-113):
 * a read and the next one are a pair when their names are equal, any other read is
 * single-end.  first_read[r] = record r's first read, for r < *n_records, then
 * first_read[*n_records] = reads->n; capacity entries (reads->n + 1 suffice). */
int32_t sa_reads_pair_interleaved(const sa_read_batch* reads, uint32_t* first_read, size_t capacity,
                                  size_t* n_records);

/* ---------------------------------------------------------------- stage entry points */
/* randstrobes_query (src/seeding/mod.rs:19-75) for every read of the batch.
 * Output arrays are sized by the caller: capacity entries each; per read r the
 * forward randstrobes are at [out_offsets[2r], +out_counts[2r]) and the
 * reverse-complement ones at [out_offsets[2r+1], +out_counts[2r+1]). */
typedef struct {
    uint64_t hash;
    uint64_t hash_revcomp;
    uint32_t start;
    uint32_t end;
} sa_query_randstrobe;
int32_t sa_randstrobes_batch(const sa_index* idx, const sa_read_batch* reads, sa_query_randstrobe* out,
                             size_t capacity, uint64_t* out_offsets, uint32_t* out_counts);

/* Allocation-free seeding.  No counterpart in the reference: it computes what
 * sa_randstrobes_batch computes, for reads already in device memory, into device
 * buffers the caller owns, and allocates nothing (no cudaMalloc/cudaFree, no
 * pinned or pooled memory).  It is for callers that cannot allocate on the device
 * at this point: cudaMalloc and cudaFree synchronise the whole device, which
 * stalls a caller keeping other streams busy, and a caller that has reserved all
 * device memory up front (index, batches, a memory pool of its own) has none left
 * to give.
 *
 * The syncmer scratch is a static device array of SA_RANDSTROBES_NOALLOC_MAX_BASES
 * bases (12 bytes per base, 12 MiB), one per device, so a batch holds at most that
 * many bases; larger batches are rejected with SA_ERR_INVALID.  Nothing needs to
 * start at zero, neither the scratch nor the output buffers.
 *
 * Calls share the one scratch array of their device: two calls whose kernels
 * overlap in time on the same device (different streams, or different host
 * threads) race and corrupt each other's results.  Serialise them, e.g. on one
 * stream.
 *
 * The first call on each device looks up the scratch address
 * (cudaGetSymbolAddress; this may load the library's device code), so make that
 * call outside any stream capture; a call with n_reads = 0 does only this setup
 * and launches nothing.  Later calls only launch.  The address is kept per device
 * and CUDA context: the first call in a context created anew (for instance after
 * cudaDeviceReset) looks it up again.
 *
 * Runs on the calling thread's current device, asynchronously on `stream` (a
 * cudaStream_t; NULL = legacy default stream).  idx supplies only the seeding
 * parameters.  Device inputs: d_seq (total_bases bytes of ASCII bases),
 * d_seq_offsets (n_reads + 1 values, d_seq_offsets[0] = 0, read r is
 * [d_seq_offsets[r], d_seq_offsets[r+1])).  Device outputs, 2 * total_bases
 * entries each: the forward randstrobes of read r at
 * [d_seq_offsets[r], + d_counts[2r]) and the reverse-complement ones at
 * [total_bases + d_seq_offsets[r], + d_counts[2r+1]), with the values of the
 * hash / hash_revcomp / start / end fields of sa_query_randstrobe.  A read whose
 * offsets decrease, end past total_bases or span more than 2048 bases gets
 * d_counts = UINT32_MAX in both orientations.  d_seq_offsets must not decrease:
 * each read is checked on its own, so in an array that decreases somewhere two
 * reads that are each well-formed can overlap, and overlapping reads race on their
 * output and scratch slots.  Only argument errors are reported
 * by the return value; kernel results are ready when the stream reaches them. */
#define SA_RANDSTROBES_NOALLOC_MAX_BASES 1048576u
int32_t sa_randstrobes_device_noalloc(const sa_index* idx, const uint8_t* d_seq, const uint64_t* d_seq_offsets,
                                      uint32_t n_reads, uint64_t total_bases, uint64_t* d_hash,
                                      uint64_t* d_hash_revcomp, uint32_t* d_start, uint32_t* d_end,
                                      uint32_t* d_counts, void* stream);

/* get_nams_by_chaining (src/nam.rs:138-166) for every read; NAMs in the order the
 * reference produces them (before sort_nams). */
typedef struct {
    uint32_t nam_id;
    uint32_t ref_id;
    uint32_t ref_start, ref_end;
    uint32_t query_start, query_end;
    uint32_t matching_bases;
    uint32_t n_anchors;
    float score;
    uint32_t is_revcomp;
} sa_nam;
/* per-read statistics (NamDetails, src/details.rs:7-32) */
typedef struct {
    uint32_t full_not_found, full_filtered, full_found;
    uint32_t partial_not_found, partial_filtered, partial_found;
    uint32_t rescued;
    uint32_t n_randstrobes, n_anchors, n_nams;
    uint32_t both_orientations;
} sa_nam_details;
int32_t sa_nams_batch(const sa_index* idx, const sa_chaining_params* cp, const sa_mapping_params* mp,
                      const sa_read_batch* reads, sa_nam* out, size_t capacity, uint64_t* out_offsets,
                      uint32_t* out_counts, sa_nam_details* out_details);

/* Aligner::align (src/aligner.rs:80-151) = ssw_align (ext/ssw/ssw.c:818-922) plus
 * end-bonus extension, for independent (query, reference) pairs.  CIGAR ops use
 * the reference encoding len << 4 | op (src/cigar.rs:5-16), =/X form. */
typedef struct {
    int32_t valid; /* 0 where the reference returns None */
    uint32_t score;
    uint32_t query_start, query_end, ref_start, ref_end;
    uint32_t edit_distance;
    uint32_t cigar_offset, cigar_len; /* into the cigar output array */
} sa_alignment;
int32_t sa_align_batch(const sa_mapping_params* mp, size_t n, const char* queries, const uint64_t* query_offsets,
                       const char* refs, const uint64_t* ref_offsets, sa_alignment* out, uint32_t* cigar,
                       size_t cigar_capacity);

/* Stage entry points on caller-given bytes, for parity tests against the reference's
 * unit vectors.  They run the device functions of the mapping path's extension
 * kernels on (query, reference) pairs given here instead of on a batch's reads and
 * the index's reference.  Host buffers; synchronous; CIGAR ops in the reference
 * encoding len << 4 | op (src/cigar.rs:5-16), =/X form, at
 * cigar[cigar_offset .. + cigar_len).  score is signed: global pieces can score
 * below zero.  SA_ERR_INVALID when cigar_capacity is too small (sum over items of
 * |query| + |reference| + 4 always suffices). */
typedef struct {
    int32_t valid; /* 0 where the reference returns None */
    int32_t score;
    uint32_t query_start, query_end, ref_start, ref_end;
    uint32_t edit_distance;
    uint32_t cigar_offset, cigar_len;
} sa_stage_alignment;
/* kind 0: hamming_align (src/aligner.rs:218-259; its segment is
 * highest_scoring_segment, :180-216), kind 1: hamming_align_global (:261-291).  Scores
 * from mp (match, mismatch, end_bonus); NULL = defaults. */
int32_t sa_hamming_batch(const sa_mapping_params* mp, size_t n, const uint32_t* kinds, const char* queries,
                         const uint64_t* query_offsets, const char* refs, const uint64_t* ref_offsets,
                         sa_stage_alignment* out, uint32_t* cigar, size_t cigar_capacity);
/* One piece of single-end piecewise extension per item (src/piecewisealigner.rs):
 * kind 0 global_alignment (:68-130), kind 1 xdrop_alignment GlobalStartLocalEnd (the
 * piece after the last anchor), kind 2 xdrop_alignment LocalStartGlobalEnd (the piece
 * before the first anchor) (:132-240).  The pieces are full affine DPs (the
 * reference's block-aligner 0.5.1 runs them in adaptive blocks; x-drop does not
 * trigger on reads of up to 2048 nt at the default x-drop of 500). */
int32_t sa_piecewise_pieces(const sa_mapping_params* mp, size_t n, const uint32_t* kinds, const char* queries,
                            const uint64_t* query_offsets, const char* refs, const uint64_t* ref_offsets,
                            sa_stage_alignment* out, uint32_t* cigar, size_t cigar_capacity);
/* remove_spurious_anchors (src/piecewisealigner.rs:596-719) on n chains in place.
 * anchors: (query_start, ref_start) int32 pairs, chain t at pairs [offsets[t],
 * offsets[t+1]); out_counts[t] = anchors kept (the first out_counts[t] pairs of the
 * chain's range). */
int32_t sa_remove_spurious_anchors(size_t n, int32_t* anchors, const uint64_t* offsets, uint32_t* out_counts);
/* extend_piecewise (src/piecewisealigner.rs:396-510) per item, with
 * remove_spurious_anchors first, as single-end mapping runs it: query against the
 * reference window, anchors (query_start, ref_start in the window) u32 pairs listed
 * last to first at pairs [anchor_offsets[i], anchor_offsets[i+1]) (at least one),
 * k the seeding k-mer length, padding = |query| / 10 (src/mapper.rs:586-593).  Scores
 * from mp. */
int32_t sa_piecewise_batch(const sa_mapping_params* mp, uint32_t k, size_t n, const char* queries,
                           const uint64_t* query_offsets, const char* refs, const uint64_t* ref_offsets,
                           const uint32_t* anchors, const uint64_t* anchor_offsets, sa_stage_alignment* out,
                           uint32_t* cigar, size_t cigar_capacity);

/* ---------------------------------------------------------------- mapping */
typedef struct sa_mapper sa_mapper;
/* The mapper keeps the index and per-batch arenas resident on the device. */
int32_t sa_mapper_create(const sa_index* idx, const sa_refs* refs, const sa_chaining_params* cp,
                         const sa_mapping_params* mp, sa_mapper** out);
void sa_mapper_free(sa_mapper* m);

typedef struct {
    char* data;     /* SAM records (no header) / PAF lines; owned by the library */
    size_t len;
    uint64_t n_reads;
    uint64_t n_mapped;
    uint32_t n_waves;      /* extension waves the batch needed */
    uint32_t n_gpu_launches;
} sa_output;

/* Map a batch (Mapper::map_chunk, src/main.rs:873-988).  The batch is cut into
 * chunks exactly as the reference cuts its input (records until the nucleotide
 * count exceeds chunk_size), each with a fresh RNG and insert-size estimate, so
 * a batch that starts at the beginning of an input reproduces the reference's
 * output bytes for those records.  r2 = NULL for single-end. */
int32_t sa_map_batch(sa_mapper* m, const sa_read_batch* r1, const sa_read_batch* r2, sa_output* out);
/* Map one batch of mixed single-end and paired-end records, as --interleaved reads them
 * (src/main.rs:580-581, InterleavedIterator src/io/reads.rs:68-113): reads in file order,
 * a read and the next one a pair (r1, r2) when their names are equal, any other read a
 * single-end record.  Chunks count both mates of a pair; each record is mapped as
 * sa_map_batch maps its kind, with the chunk's RNG and insert-size estimate shared
 * between the kinds (src/main.rs:873-988). */
int32_t sa_map_batch_interleaved(sa_mapper* m, const sa_read_batch* reads, sa_output* out);
void sa_output_free(sa_output* out);
/* Abundances accumulated over all batches (--aemb), one per contig, already
 * divided by the contig length as output_abundances does (src/main.rs:990-1001). */
int32_t sa_mapper_abundances(const sa_mapper* m, double* out, size_t n);
/* ---------------------------------------------------------------- serving
 * Continuous batching of mapping requests (the reference maps one input stream
 * per process; a session serves many).  A request is a read batch; the session
 * copies it, admits it onto the device when its reads fit in the in-flight read
 * arena, and maps it as its own chunk stream (src/main.rs:591-604,873-988), so
 * its output is byte-identical to sa_map_batch on the same records, whatever else
 * is in flight.  Requests admitted together share extension waves.
 * submit/poll/wait may be called from any thread. */
typedef struct sa_session sa_session;
typedef struct {
    uint64_t max_inflight_bases;    /* device read arena in bases; 0 = an eighth of the free
                                       device memory beyond the reserve (2^24..2^33) */
    uint32_t max_inflight_requests; /* 0 = no limit */
    uint32_t policy_threads;        /* host threads for the mapping policy; 0 = all */
    uint32_t admission_streams;     /* requests whose NAM pipelines run at once; 0 = 2 */
    uint32_t borrow_inputs;         /* 1: sa_session_submit keeps pointers to the batch's
                                       sequences, qualities, names and comments instead of
                                       copying them; the caller keeps them unchanged until
                                       sa_session_wait returns for that request (also when it
                                       returns an error: by then no session thread reads
                                       them). 0 (default): copied, the caller may free them
                                       after submit. */
    uint64_t device_reserve_bytes;  /* device memory admission leaves free for everything
                                       else; 0 = max(2 GiB, 5% of the device).  A request is
                                       admitted when its reads fit in the arena and the free
                                       device memory beyond this reserve covers the NAM
                                       workspace its admission group needs (160 bytes per
                                       base); one that cannot fit while nothing else is in
                                       flight fails with SA_ERR_BUSY. */
} sa_session_params;
typedef struct {
    double seconds_queued;  /* submit -> admitted */
    double seconds_service; /* admitted -> done */
    double seconds_total;   /* submit -> done */
    uint64_t n_reads;
    uint32_t n_waves; /* extension waves the request took part in */
    uint64_t h2d_bytes, d2h_bytes; /* host<->device bytes moved for this request */
} sa_request_stats;
void sa_session_params_default(sa_session_params* p);
int32_t sa_session_create(const sa_index* idx, const sa_refs* refs, const sa_chaining_params* cp,
                          const sa_mapping_params* mp, const sa_session_params* sp, sa_session** out);
/* Copies the batch (or, with borrow_inputs, refers to it) and queues it; r2 = NULL for
 * single-end.  SA_ERR_INVALID if the request can never fit in the arena. */
int32_t sa_session_submit(sa_session* s, const sa_read_batch* r1, const sa_read_batch* r2, uint64_t* ticket);
/* As sa_session_submit for mixed single-end and paired records in file order, paired by
 * name as sa_map_batch_interleaved pairs them; the output equals sa_map_batch_interleaved
 * on the same records alone. */
int32_t sa_session_submit_interleaved(sa_session* s, const sa_read_batch* reads, uint64_t* ticket);
/* *done = 1 once the request's output is ready. */
int32_t sa_session_poll(sa_session* s, uint64_t ticket, int32_t* done);
/* Waits up to timeout_ms (< 0: no limit; SA_ERR_TIMEOUT when it runs out) and
 * hands over the request's output (release with sa_output_free).  stats may be
 * NULL.  In abundance mode abundances (n_abundances >= contig count) receives the
 * request's per-contig abundances divided by contig length; it may be NULL
 * otherwise.  The ticket is invalid afterwards. */
int32_t sa_session_wait(sa_session* s, uint64_t ticket, int64_t timeout_ms, sa_output* out, sa_request_stats* stats,
                        double* abundances, size_t n_abundances);
/* What the session chose at creation. */
typedef struct {
    uint64_t arena_bases;          /* device read arena (bases) */
    uint64_t device_reserve_bytes; /* device memory admission leaves free */
    uint64_t refused_requests;     /* requests refused for lack of device memory so far */
} sa_session_info;
int32_t sa_session_get_info(const sa_session* s, sa_session_info* out);
/* Finishes the admitted requests, cancels the queued ones, frees the session. */
void sa_session_free(sa_session* s);

/* Two-step form of sa_map_batch: upload a batch to the device, then map it.  The
 * host buffers of the batch must stay valid until the last sa_map_uploaded call
 * (names, qualities and comments are read from them when records are written).
 * Mapping the same uploaded batch again reproduces the same bytes. */
int32_t sa_mapper_upload(sa_mapper* m, const sa_read_batch* r1, const sa_read_batch* r2);
int32_t sa_map_uploaded(sa_mapper* m, sa_output* out);

/* Stage timings and counters of the last mapped batch.  A large batch is cut into
 * parts whose NAM pipelines overlap the extension waves and the policy:
 * seconds_nams sums the parts' pipelines, seconds_extension the waves, and
 * seconds_policy is the rest of seconds_total after the waves and the first part's
 * pipeline. */
typedef struct {
    double seconds_upload, seconds_nams, seconds_extension, seconds_policy, seconds_total;
    uint64_t n_jobs, n_waves, n_launches;
    uint64_t h2d_bytes, d2h_bytes;
    uint64_t n_nams, n_anchors;
    /* per-stage device time (CUDA events on the mapper's stream) when profiling is
     * on: seed, hits, anchors, sort, chain, other NAM, prepare, fill, SW byte,
     * SW word, banded traceback, finalize, other extension */
    double kernel_ms[16];
    uint64_t kernel_launches[16];
    /* Smith-Waterman cells (query x reference).  [0]: canonical cells, |query| x
     * |reference window| once per SSW call.  [1..4]: cells the striped passes
     * computed (up to an early stop): forward byte, forward word (byte overflow
     * reruns), reverse byte, reverse word */
    uint64_t sw_cells[5];
    /* work counts of the NAM stages: read bases, randstrobes (both orientations; one
     * index probe each), anchors */
    uint64_t n_bases, n_randstrobes, n_anchor_total;
    /* banded traceback cells (banded_sw, ext/ssw/ssw.c:598-769): [0] every pass of the
     * band doubling, [1] the final pass, (2bw+1)-wide band rows clipped to the window */
    uint64_t band_cells[2];
} sa_mapper_stats;
int32_t sa_mapper_get_stats(const sa_mapper* m, sa_mapper_stats* out);
/* Record CUDA events around each stage's launches (off by default). */
int32_t sa_mapper_set_profiling(sa_mapper* m, int32_t enable);
/* Parts a large batch is cut into (runs of whole chunks, at least 4 chunks each): the
 * NAM pipeline of one part runs while the earlier parts are extended and written.
 * Output bytes do not depend on it.  Default 8; batches of more than 2^27 bases get
 * as many parts as hold at most 2^27 bases each. */
int32_t sa_mapper_set_parts(sa_mapper* m, uint32_t parts);

/* How a batch is scheduled on the device and the host.  No counterpart in the
 * reference (it maps chunks on CPU threads); output bytes never depend on it.
 *   parts          NAM-pipeline parts (runs of whole chunks, at least 4 chunks each);
 *                  0 = 8.  Batches of more than 2^27 bases get more parts, so that a
 *                  part holds at most 2^27 bases.  With overlap, part p + 1's pipeline
 *                  runs while earlier parts are extended.
 *   overlap        1 (default): continuous batching -- policy threads run the chunks
 *                  whose results are in while the next extension wave runs, and the
 *                  output is copied into place while mapping.  0: the plain,
 *                  stage-synchronous form -- each stage is launched over everything
 *                  waiting for it and the host and device take turns: a wave starts
 *                  only when no chunk can proceed, and chunks resume only when every
 *                  waiting request has run.
 *   wave_min_jobs  waiting jobs that start a wave while policy threads are busy
 *                  (overlap = 1); 0 = 32768.
 *   max_wave_jobs  jobs per wave at most; 0 = 262144. */
typedef struct {
    uint32_t parts;
    uint32_t overlap;
    uint64_t wave_min_jobs;
    uint64_t max_wave_jobs;
} sa_schedule_params;
void sa_schedule_params_default(sa_schedule_params* p);
int32_t sa_mapper_set_schedule(sa_mapper* m, const sa_schedule_params* p);

/* Tuning knobs of a mapper, chosen by sa_mapper_autotune.  No counterpart in the
 * reference; output bytes never depend on them.
 *   parts, wave_min_jobs, max_wave_jobs  as in sa_schedule_params
 *   ssw_wave_max_qlen       SSW tasks of reads up to this length (at most 192) run on
 *                           the lane-wavefront kernel, longer ones a warp per task
 *   chain_lane_cluster_max  clusters of a long read orientation's anchors up to this
 *                           size are chained by one thread, larger ones by a warp
 *   l2_fetch_bytes          the context's L2 fetch granularity for DRAM reads
 *                           (cudaLimitMaxL2FetchGranularity: 32, 64 or 128; 0 keeps the
 *                           value the context had when the mapper was created).  It is a
 *                           limit of the calling process's CUDA context on the mapper's
 *                           device, so it applies to every kernel of the process. */
typedef struct {
    uint32_t parts;
    uint64_t wave_min_jobs;
    uint64_t max_wave_jobs;
    uint32_t ssw_wave_max_qlen;
    uint32_t chain_lane_cluster_max;
    uint32_t l2_fetch_bytes;
} sa_tuning;
typedef struct {
    sa_tuning chosen;
    double seconds_default; /* the calibration batch under the defaults (median of rounds) */
    double seconds_tuned;   /* under the chosen knobs */
    uint32_t trials;
} sa_tune_report;
void sa_tuning_default(sa_tuning* t);
int32_t sa_mapper_set_tuning(sa_mapper* m, const sa_tuning* t);
int32_t sa_mapper_get_tuning(const sa_mapper* m, sa_tuning* t);
/* Autotuner: uploads the calibration batch (it stays uploaded, replacing any earlier
 * one), maps it under the default knobs, then tries a short list of values for one
 * knob after another (coordinate descent; each trial the median of `rounds` maps, a
 * change kept only when 2% faster), checks that every trial writes the same bytes
 * (SA_ERR_INVALID otherwise) and applies the choice to the mapper.  The batch should
 * have the shape of the workload (read lengths, genome). */
int32_t sa_mapper_autotune(sa_mapper* m, const sa_read_batch* r1, const sa_read_batch* r2, uint32_t rounds,
                           sa_tune_report* out);

/* ---------------------------------------------------------------- file to file
 * The reference CLI's read → map → write loop (src/main.rs:555-700): a reader thread
 * parses reads1 (and reads2 for paired-end; pairs end with the shorter file, as zip
 * pairs them) into batches of whole chunks, the calling thread maps each batch, and a
 * writer thread appends the outputs to out_path in input order, so parsing, mapping and
 * writing overlap.  Inputs are FASTQ or FASTA, gzip when the name ends in ".gz" (every
 * member, src/io/xopen.rs:9-20), "-" for standard input; out_path "-" is standard
 * output.  The bytes written are header followed by what sa_map_batch returns for all
 * records at once; in abundance mode the per-contig table ("name\tabundance" with six
 * decimals, src/main.rs:990-1001) of the mapper's accumulated abundances follows. */
typedef struct {
    uint64_t batch_bases;  /* nucleotides per mapped batch, rounded up to whole chunks (0: 2^29) */
    uint32_t read_ahead;   /* parsed batches queued ahead of the mapper (0: 2) */
    int32_t append;        /* 1: append to out_path instead of truncating it */
    const char* header;    /* bytes written first (the SAM header); may be NULL */
    size_t header_len;
    int32_t interleaved;   /* 1: reads1 holds mixed single-end and paired records (reads2 NULL),
                              paired as sa_map_batch_interleaved pairs them */
} sa_stream_params;
typedef struct {
    uint64_t n_reads, n_records, n_mapped, n_batches;
    uint64_t bytes_in;     /* bytes read from the input files (compressed size for .gz) */
    uint64_t bytes_out;
    double seconds_total, seconds_map, seconds_wait_input;
} sa_stream_stats;
void sa_stream_params_default(sa_stream_params* p);
int32_t sa_map_files(sa_mapper* m, const char* reads1, const char* reads2, const char* out_path,
                     const sa_stream_params* p, sa_stream_stats* stats);

/* ---------------------------------------------------------------- measurement
 * Integer-ALU instruction rate of the current device, measured by a kernel of eight
 * independent chains per thread over every SM (the median of five launches):
 * out[0] add-then-max instructions per second (the fused form the SSW and banded
 * kernels use), out[1] max and xor instructions per second.  The denominator of the
 * Smith-Waterman rooflines; no reference counterpart. */
int32_t sa_measure_int_alu(double* out);

/* SAM header (src/io/sam.rs:176-200); cmd_line NULL omits the @PG line. */
int32_t sa_sam_header(const sa_refs* refs, const char* cmd_line, const char* rg_id, const char* const* rg_fields,
                      size_t n_rg_fields, sa_output* out);

#ifdef __cplusplus
}
#endif
#endif /* STROBEALIGN_GB300_H */
