// Host-side mapping policy: the sequential, per-chunk part of the reference's
// mapping (src/mapper.rs, src/maponly.rs) that consumes GPU NAMs and GPU
// extension results.  Missing extension results raise Miss; the batch driver then
// runs another extension wave and resumes the chunk at the read that missed.
#pragma once
#include <cstdint>
#include <deque>
#include <memory>
#include <string>
#include <vector>

#include "extend.h"

namespace sa {

// fastrand 2.3.0 (wyrand + Lemire bounded integers), the RNG the reference seeds
// per chunk (src/main.rs:878) and draws from on ties (src/shuffle.rs:21,
// src/mapper.rs:461,716).
struct Rng {
    uint64_t state = 0;
    uint64_t gen_u64();
    uint32_t gen_mod_u32(uint32_t n);
    uint64_t gen_mod_u64(uint64_t n);
};

// InsertSizeDistribution (src/insertsize.rs:1-50)
struct InsertSize {
    uint64_t sample_size = 0;
    float mu = 300.0f, sigma = 100.0f, variance = 10000.0f, sse = 10000.0f;
    void update(uint64_t insert_size);
};

struct Details {
    NamDetailsRec nam{};
    uint32_t inconsistent_nams = 0, mate_rescue = 0, tried_alignment = 0, gapped = 0, best_alignments = 0;
};

struct Alignment {
    uint32_t reference_id = 0, ref_start = 0, edit_distance = 0, soft_clip_left = 0, soft_clip_right = 0;
    uint32_t score = 0, length = 0;
    bool is_revcomp = false, gapped = false;
    const uint32_t* cigar = nullptr;
    uint32_t cigar_len = 0;
    uint32_t global_edit_distance() const { return edit_distance + soft_clip_left + soft_clip_right; }
};

struct JobKey {
    uint32_t kind, a, b, c, d;
    bool operator==(const JobKey& o) const {
        return kind == o.kind && a == o.a && b == o.b && c == o.c && d == o.d;
    }
};

struct Miss {};

// One extension result as the host keeps it: the device record plus the address
// of its CIGAR in the wave's host copy.
struct StoredResult : ExtResult {
    const uint32_t* cigar = nullptr;
};

// Extension results of one batch, accumulated over waves.  Storage is stable:
// waves append (deque elements never move), so policy threads keep reading the
// results they hold while the extension thread appends the next wave.  An entry of
// per_read[r] is written only by the thread that runs the chunk owning read r, or
// by the extension thread while that chunk waits for the wave.
struct ResultStore {
    struct Entry {
        JobKey key;
        const StoredResult* result;  // nullptr while pending
    };
    std::vector<std::vector<Entry>> per_read;
    std::deque<StoredResult> results;
    std::vector<std::shared_ptr<const std::vector<uint32_t>>> cigars;  // the waves' CIGAR copies referenced here
};

struct ReadView {
    const char* seq;
    uint32_t len;
    const char* qual;  // nullptr if absent
    const char* name;
    uint32_t name_len;
    const char* comment;  // nullptr if absent
    uint32_t comment_len;
};

struct PolicyConfig {
    sa_mapping_params mp;
    std::string rg_id;
    bool has_rg = false;
    uint32_t k = 0;
};

struct ContigInfo {
    const std::string* name;
    uint64_t len;
};

// Per-read inputs the policy reads
struct BatchView {
    std::vector<ReadView> reads;         // device read order (pairs interleaved)
    const NamRec* nams = nullptr;
    const uint64_t* nam_off = nullptr;
    const NamDetailsRec* details = nullptr;
    bool paired = false;
};

struct ChunkState {
    uint64_t first = 0, next = 0, end = 0;  // record range [first, end), cursor next
    Rng rng;
    InsertSize isd;
    std::string out;
    uint64_t mapped = 0;
    bool done = false;
    std::vector<ExtJob> pending;                          // requests raised by this chunk
    std::vector<std::pair<uint32_t, double>> abundance;   // (contig, weight) in read order
    bool lookahead_started = false;
    std::vector<uint64_t> lookahead_todo;                 // reads that missed in the last lookahead
};

class Policy {
  public:
    Policy(const PolicyConfig& cfg, const std::vector<ContigInfo>& contigs, const BatchView& bv, ResultStore& store)
        : cfg_(cfg), contigs_(contigs), bv_(bv), store_(store) {}
    // Advance one chunk as far as the available results allow.  On a miss, the
    // rest of the chunk is evaluated speculatively (state copies, output dropped)
    // so that the jobs of later reads join the next wave.
    void run_chunk(ChunkState& cs);
    // Speculative first-wave requests for the reads of one chunk.
    void seed_requests(ChunkState& cs);

  private:
    const PolicyConfig& cfg_;
    const std::vector<ContigInfo>& contigs_;
    const BatchView& bv_;
    ResultStore& store_;
    ChunkState* cur_ = nullptr;
    bool speculative_ = false;
    void add_abundance(uint32_t ref_id, double w) {
        if (!speculative_) cur_->abundance.emplace_back(ref_id, w);
    }

    void want(uint32_t read, const ExtJob& job, const JobKey& key);
    const StoredResult* lookup(uint32_t read, const JobKey& key) const;
    const StoredResult& get(uint32_t read, const ExtJob& job, const JobKey& key);

    void se_record(uint64_t rec, Rng& rng, std::string& out, uint64_t& mapped);
    void pe_record(uint64_t rec, Rng& rng, InsertSize& isd, std::string& out, uint64_t& mapped);
    void paf_se(uint64_t rec, Rng& rng, std::string& out);
    void paf_pe(uint64_t rec, Rng& rng, InsertSize& isd, std::string& out);
    void aemb_se(uint64_t rec, Rng& rng);
    void aemb_pe(uint64_t rec, Rng& rng, InsertSize& isd);

  public:
    // helpers used by the implementation file
    std::vector<NamRec> sorted_nams(uint32_t read, Rng& rng) const;
    ExtJob nam_job(uint32_t read, const NamRec& n, uint32_t kind) const;
    static JobKey nam_key(const NamRec& n, uint32_t kind) { return JobKey{kind, n.nam_id, 0, 0, 0}; }
    Alignment to_alignment(const StoredResult& r, uint32_t ref_id) const;
    const PolicyConfig& cfg() const { return cfg_; }
    const std::vector<ContigInfo>& contigs() const { return contigs_; }
    const BatchView& bv() const { return bv_; }
    // extend_seed with the given consistency semantics; applies the flip to nam
    bool extend(uint32_t read, NamRec& nam, uint32_t kind, Alignment& out, bool& consistent);
    bool rescue(uint32_t read, const NamRec& mate, float mu, float sigma, Alignment& out);
    void want_nam(uint32_t read, const NamRec& n, uint32_t kind);
};

}  // namespace sa
