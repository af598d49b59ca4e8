// Internal definitions shared by the host runtime and the CUDA kernels.
#pragma once
#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>
#include <stdexcept>

#include "../../include/strobealign_gb300.h"

#ifdef __CUDACC__
#define SA_HD __host__ __device__ __forceinline__
#else
#define SA_HD inline
#endif

namespace sa {

// Error carrying an SA_ERR_* status; caught at the C-ABI boundary.
struct Error : std::runtime_error {
    int32_t code;
    Error(int32_t c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

constexpr uint64_t HASH_MASK = 0xFFFFFFFFFFFFFF00ULL;  // REF_RANDSTROBE_HASH_MASK, src/index.rs:41

// Seeding parameters in the form the kernels read them.
struct SeedParams {
    uint32_t k, s, t, w_min, w_max, max_dist, pop;
    uint64_t q, main_mask, fwd_main_mask;
};

// RefRandstrobe (src/index.rs:15-30): same 16-byte layout as the reference.
struct RefRandstrobe {
    uint64_t hash_offset;
    uint32_t position;
    uint32_t ref_index;
};
static_assert(sizeof(RefRandstrobe) == 16, "RefRandstrobe layout");

// Read-only view of the device-resident index.
struct DevIndex {
    const RefRandstrobe* rs;
    uint64_t n;
    const uint64_t* buckets;
    uint32_t bits;
    uint32_t filter_cutoff;
    SeedParams p;
};

// Read-only view of the device-resident 2-bit reference (contigs start on u64 words).
struct DevRefs {
    const uint64_t* words;
    const uint64_t* word_off;  // per contig
    const uint32_t* len;       // per contig
    uint32_t n;
};

SA_HD uint64_t xxh64_u64(uint64_t input) {
    const uint64_t P1 = 0x9E3779B185EBCA87ULL, P2 = 0xC2B2AE3D27D4EB4FULL, P3 = 0x165667B19E3779F9ULL,
                   P4 = 0x85EBCA77C2B2AE63ULL, P5 = 0x27D4EB2F165667C5ULL;
    uint64_t r = P5 + 8;
    uint64_t x = input * P2;
    x = (x << 31) | (x >> 33);
    r ^= x * P1;
    r = ((r << 27) | (r >> 37)) * P1 + P4;
    r ^= r >> 33;
    r *= P2;
    r ^= r >> 29;
    r *= P3;
    r ^= r >> 32;
    return r;
}

// Randstrobe::hash (src/seeding/strobes.rs:112-124)
SA_HD uint64_t randstrobe_hash(uint64_t h1, uint64_t h2, uint64_t f1, uint64_t f2, const SeedParams& p) {
    return ((h1 & p.main_mask) | (h2 & ~p.fwd_main_mask) | (f1 << p.pop) | (f2 << 8)) & (HASH_MASK << 1);
}

SeedParams to_seed_params(const sa_seeding_params& p);

// Query read batch resident on the device.
struct DevReads {
    const uint8_t* seq;
    const uint64_t* off;  // n + 1
    uint32_t n;
};

// NAM as produced by the chaining kernel (device and host layout).
struct NamRec {
    uint32_t nam_id, ref_id, ref_start, ref_end, query_start, query_end, matching_bases, n_anchors;
    float score;
    uint32_t is_revcomp;
};
static_assert(sizeof(NamRec) == 40, "NamRec layout");

struct NamDetailsRec {
    uint32_t full_not_found, full_filtered, full_found;
    uint32_t partial_not_found, partial_filtered, partial_found;
    uint32_t rescued;
    uint32_t n_randstrobes, n_anchors, n_nams;
    uint32_t both_orientations;
};
static_assert(sizeof(NamDetailsRec) == sizeof(sa_nam_details), "details layout");

// Extension job (one extend_seed or rescue_align call of the reference).
enum JobKind : uint32_t { JOB_EXTEND_FAST = 0, JOB_EXTEND_FULL = 1, JOB_RESCUE = 2, JOB_ALIGN = 3 };
struct ExtJob {
    uint32_t kind;
    uint32_t read;        // read index in the device batch
    uint32_t ref_id;
    uint32_t ref_start;   // NAM ref_start, or rescue window start
    uint32_t ref_end;     // NAM ref_end, or rescue window end
    uint32_t query_start; // NAM only
    uint32_t query_end;   // NAM only
    uint32_t is_revcomp;  // NAM orientation; for rescue: 1 = align the read's reverse complement
    uint32_t use_ssw;     // extend_seed use_ssw (1 for all paired-end extension)
    uint32_t tag;         // caller bookkeeping
    uint32_t nam;         // the NAM's index in its read's NAM list (piecewise anchors)
    uint32_t anc_off, anc_n;  // piecewise: the NAM's anchors in the wave's anchor array
};

// Result of one job.  CIGAR (=/X/I/D, no soft clips) lives in the cigar arena.
struct ExtResult {
    int32_t valid;        // 0 = None
    uint32_t consistent;  // consistency flag the extension used
    uint32_t flipped;     // reverse_nam_if_needed flipped the NAM
    uint32_t nam_query_start, nam_query_end, nam_is_revcomp;  // NAM after the flip
    uint32_t ref_start;   // alignment start on the contig
    uint32_t length;      // reference span
    uint32_t soft_clip_left, soft_clip_right;
    uint32_t edit_distance;
    uint32_t score;
    uint32_t is_revcomp;
    uint32_t gapped;
    uint32_t cigar_offset, cigar_len;
};

}  // namespace sa
