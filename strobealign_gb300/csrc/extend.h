// Extension pipeline (extend.cu): extend_seed / rescue_align / Aligner::align for a
// list of jobs.
#pragma once
#include "host_util.h"
#include "pipeline.h"

namespace sa {

struct AlignScores {
    uint8_t match, mismatch, gap_open, gap_extend;
    uint32_t end_bonus;
};

// Per-job device-side description of the work (filled by the prepare kernel).
struct PrepRec {
    uint32_t type;        // 0 none, 1 hamming, 2 ssw
    uint32_t read;
    uint32_t rc;          // query is the read's reverse complement
    uint32_t qlen;
    uint32_t ref_id;
    uint32_t wstart, wlen;  // reference window (contig coordinates)
    uint64_t arena_off;   // query bytes then window bytes
    uint64_t cigar_off;   // first op of this job's CIGAR
    uint64_t h_off;       // banded-DP scratch (ints)
    uint32_t cigar_cap;
    // SSW task of a NAM extension: the window column of query position 0 on the NAM's
    // diagonal (NO_DIAG for rescue and stage tasks)
    uint32_t diag;
};
constexpr uint32_t NO_DIAG = 0xffffffffu;

// SSW task state (ext/ssw/ssw.c:818-922 results).
struct SswTask {
    uint32_t job;
    int32_t score1;
    int32_t ref_end1, read_end1;
    int32_t ref_begin1, read_begin1;
    int32_t word;
    int32_t flag;
    int32_t band_width;
    uint32_t raw_len;
    uint64_t dir_off;
    uint64_t raw_off;
};

struct ExtWorkspace {
    DevBuf<ExtJob> jobs;
    DevBuf<ExtResult> results;
    DevBuf<PrepRec> prep;
    DevBuf<uint64_t> sizes;     // 3 per job: arena bytes, cigar ops, h ints
    DevBuf<uint64_t> offs;      // 3 per job (+3)
    DevBuf<uint8_t> arena;
    DevBuf<uint32_t> cigar;
    DevBuf<int32_t> hscratch;
    DevBuf<SswTask> tasks;
    DevBuf<uint32_t> band_list, wide_list;  // tasks left by k_band_small / by k_band_warp
    DevBuf<uint32_t> band_buckets;          // tasks by starting band width, then the counts
    DevBuf<uint32_t> counters;  // [0] n_tasks [1] n_word [2] n_rev_byte [3] n_rev_word [4] n_rescue, u64 cells at [8], u64 band cells at [24], band list sizes at [28] and [29]
    DevBuf<uint32_t> rescue_list;
    DevBuf<uint32_t> list_word, list_rev_byte, list_rev_word;
    DevBuf<uint32_t> order;  // task order of the fused SSW kernel
    DevBuf<uint32_t> pw_list;     // piecewise jobs
    DevBuf<uint8_t> pw_scratch;   // per-warp DP directions, ops and anchors of k_piecewise
    DevBuf<uint32_t> anchors;     // the wave's piecewise anchors (uploaded by the caller)
    DevBuf<uint64_t> dir_size, dir_off;
    DevBuf<uint8_t> dir;
    DevBuf<uint64_t> raw_size, raw_off;
    DevBuf<uint32_t> raw;
    DevBuf<uint8_t> cub_tmp;
    // host mirrors (capacity kept across waves; the callers swap them with pooled
    // wave buffers)
    PodArray<ExtResult> h_results;
    PodArray<uint32_t> h_cigar;
    uint64_t total_cigar = 0;
    // tuning (output-invariant): SSW tasks of reads up to wave_qmax nt (at most 192) run
    // on the lane-wavefront kernel, longer ones a warp per task
    uint32_t wave_qmax = 192;
    // SW cells: canonical, then computed forward byte / word, reverse byte / word; then
    // banded cells: every pass's, and the final pass's
    uint64_t cells[7] = {0, 0, 0, 0, 0, 0, 0};
};

// Runs jobs (already in ws.jobs, n of them) against the reads in nws.seq/nws.off.
// Results and CIGARs are copied back into ws.h_results / ws.h_cigar.  Returns the
// number of kernel launches.
// anchors: device (query start, reference start) pairs of the piecewise jobs
// (ExtJob::anc_off / anc_n), max_anchors their largest count; null when no job has
// use_ssw == 0.
uint32_t run_extension(const DevRefs& refs, const NamWorkspace& nws, uint32_t k, const AlignScores& sc, uint32_t n,
                       ExtWorkspace& ws, uint32_t max_qlen, cudaStream_t st, KernelTimers* kt = nullptr,
                       const uint32_t* anchors = nullptr, uint32_t max_anchors = 0);
// The same for reads at seq + off[read] (off holds n_reads + 1 absolute offsets);
// raw_refs / raw_off give the reference bytes of JOB_ALIGN jobs (may be null).
uint32_t run_extension_raw(const DevRefs& refs, const uint8_t* seq, const uint64_t* off, const uint8_t* raw_refs,
                           const uint64_t* raw_off, uint32_t k, const AlignScores& sc, uint32_t n, ExtWorkspace& ws,
                           uint32_t max_qlen, cudaStream_t st, KernelTimers* kt = nullptr,
                           const uint32_t* anchors = nullptr, uint32_t max_anchors = 0);

// Result of a stage entry point (sa_stage_alignment): signed score, since global
// pieces can score below zero.
struct StageAlignment {
    int32_t valid;
    int32_t score;
    uint32_t query_start, query_end, ref_start, ref_end;
    uint32_t edit_distance;
    uint32_t cigar_offset, cigar_len;
};

// Stage entry points (extend.cu) on caller-given bytes; synchronous on st.
// kinds: 0 hamming_align, 1 hamming_align_global.
void stage_hamming(uint32_t n, const uint32_t* kinds, const uint8_t* q, const uint64_t* qo, const uint8_t* r,
                   const uint64_t* ro, const AlignScores& sc, StageAlignment* out, uint32_t* cigar, size_t cap,
                   cudaStream_t st);
// kinds: 0 global piece, 1 x-drop piece after the last anchor, 2 before the first.
void stage_pieces(uint32_t n, const uint32_t* kinds, const uint8_t* q, const uint64_t* qo, const uint8_t* r,
                  const uint64_t* ro, const AlignScores& sc, StageAlignment* out, uint32_t* cigar, size_t cap,
                  cudaStream_t st);
// anchors: (query start, reference start) pairs, chain t at [off[t], off[t+1]); pruned in place.
void stage_prune(uint32_t n, int32_t* anchors, const uint64_t* off, uint32_t* counts, cudaStream_t st);
// extend_piecewise per (query, reference window, anchors last to first).
void stage_piecewise(uint32_t n, const uint8_t* q, const uint64_t* qo, const uint8_t* r, const uint64_t* ro,
                     const uint32_t* anchors, const uint64_t* anc_off, uint32_t k, const AlignScores& sc,
                     StageAlignment* out, uint32_t* cigar, size_t cap, cudaStream_t st);

}  // namespace sa
