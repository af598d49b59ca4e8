// Device pipelines: NAM finding (nams.cu) and extension (extend.cu).
#pragma once
#include "host_state.h"
#include "ktimer.h"

namespace sa {

struct ChainParams {
    uint32_t max_lookback;
    float diag_diff_penalty, gap_length_penalty, valid_score_threshold;
    uint32_t max_ref_gap;  // 0 = read length
    float matches_weight, max_diagonal_ratio;
};

constexpr uint32_t MAX_READ_LEN = 2048;  // longest read the warp-per-read kernels accept
constexpr uint32_t LOG2_LUT_SIZE = 4096; // log2(d + 1) table used by chaining, d < MAX_READ_LEN * 2

// Device buffers of the NAM pipeline; grow-only, reused across batches.
struct NamWorkspace {
    DevBuf<uint8_t> seq;
    DevBuf<uint64_t> off;
    DevBuf<uint64_t> syn_hash;
    DevBuf<uint32_t> syn_pos;  // position << 1 | is_forward
    DevBuf<uint64_t> qr_hash, qr_hash_rc;   // [2][total] forward / reverse complement
    DevBuf<uint32_t> qr_start, qr_end;
    DevBuf<uint32_t> n_rs;                  // 2 per read
    DevBuf<uint64_t> hit_pos;               // [2][total]
    DevBuf<uint32_t> hit_info;              // randstrobe index << 3 | filtered << 2 | partial << 1
    DevBuf<uint32_t> hit_count_cache;
    DevBuf<uint32_t> n_hits;                // 2 per read
    DevBuf<uint32_t> hit_anchors;           // anchors produced per hit
    DevBuf<uint8_t> orient;                 // bit0 forward chained, bit1 reverse chained
    DevBuf<NamDetailsRec> details;
    DevBuf<uint64_t> seg_off;               // 2n + 1
    DevBuf<uint64_t> seg_count;
    DevBuf<uint64_t> anchors, anchors_sorted;
    DevBuf<float> dp;
    DevBuf<uint32_t> pred;
    DevBuf<uint32_t> aux;                   // candidates / used flags scratch
    DevBuf<NamRec> nam_scratch;
    DevBuf<uint32_t> nam_seg_count;         // 2n
    DevBuf<uint64_t> nam_off;               // n + 1
    DevBuf<uint64_t> nam_count;             // n (u64 for the scan)
    DevBuf<NamRec> nams;
    // reads with more than 32 NAMs: push-order copy, sort keys / permutation (in, out),
    // and the list of such reads with their output ranges; long_reads[n] counts them
    DevBuf<NamRec> nam_tmp;
    DevBuf<uint32_t> nam_keys, nam_vals;
    DevBuf<uint32_t> long_reads;
    // read orientations with anchors (2n slots), their count in slot 2n and the count of
    // those sorted by the segmented sort in slot 2n + 1; that sort's ranges
    DevBuf<uint32_t> seg_list;
    // seg_list's anchor counts, and the lists ordered by them (descending) for k_chain4
    DevBuf<uint32_t> seg_key, seg_key_alt, seg_sorted;
    // long orientations' large clusters queued for k_chain_big: [0] count, then
    // (orientation, cluster) pairs
    DevBuf<uint32_t> chain_big;
    DevBuf<uint64_t> sort_begin, sort_end;
    DevBuf<uint64_t> long_begin, long_end;
    // with NamConfig::nam_anchors: the anchors of each NAM's chain, last to first
    // (src/chainer.rs:420-440), as packed anchor keys; NAM t's are at
    // nam_anc[nam_anc_off[t] .. nam_anc_off[t + 1])
    DevBuf<uint64_t> anc_sparse, anc_start, nam_anc_src, nam_anc_off, nam_anc;
    uint64_t last_total_nam_anchors = 0;
    DevBuf<uint8_t> cub_tmp;
    DevBuf<float> log2_lut;
    uint64_t last_total_nams = 0;
    uint32_t anchor_qbits = 0, anchor_pbits = 0;
};

struct NamConfig {
    ChainParams cp;
    uint32_t mcs;
    uint32_t rescue_distance;
    bool nam_anchors = false;  // also keep each NAM's chain anchors (single-end piecewise extension)
    // tuning (output-invariant): clusters of a long read orientation up to this many
    // anchors are scored by one thread, larger ones by a warp
    uint32_t chain_lane_max = 48;
};

// Runs seeding -> hits -> rescue -> anchors -> sort -> chaining -> NAM compaction for
// the reads already in ws.seq / ws.off (n reads, total bases).  Leaves per-read
// NAMs (stable-sorted by score, descending) in ws.nams at ws.nam_off, and per-read
// statistics in ws.details.  Returns the number of kernel launches issued.
uint32_t run_nam_pipeline(const DevIndex& ix, const DevRefs& refs, const NamConfig& cfg, uint32_t n, uint64_t total,
                          uint32_t max_contig_len, uint32_t n_contigs, NamWorkspace& ws, cudaStream_t st,
                          KernelTimers* kt = nullptr);

// Randstrobes only (stage entry point).
uint32_t run_seeding(const SeedParams& sp, uint32_t n, uint64_t total, NamWorkspace& ws, cudaStream_t st,
                     KernelTimers* kt = nullptr);
// Seeding with the syncmer scratch in a static device array and every other buffer
// supplied by the caller (k_seed<true>); allocates nothing.
void run_seeding_noalloc(const SeedParams& sp, const uint8_t* seq, const uint64_t* off, uint32_t n, uint64_t total,
                         uint64_t* qr_hash, uint64_t* qr_hash_rc, uint32_t* qr_start, uint32_t* qr_end,
                         uint32_t* counts, cudaStream_t st);

}  // namespace sa
