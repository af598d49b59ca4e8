// Host-side mapping policy: the sequential, per-chunk part of the reference's
// mapping (src/mapper.rs, src/maponly.rs) that consumes GPU NAMs and GPU
// extension results.  A record whose extension result is missing requests it and
// stops (the functions return MISSING / false up to the chunk loop); the batch driver
// then runs another extension wave and resumes the chunk at the read that missed.
#pragma once
#include <cstdint>
#include <cstring>
#include <deque>
#include <memory>
#include <string>
#include <vector>

#include "extend.h"
#include "host_util.h"

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
    uint64_t last = 0;  // value of the last accepted update (replayed by the lookahead)
    void update(uint64_t insert_size);
    bool same_state(const InsertSize& o) const {
        auto bits = [](float f) {
            uint32_t u;
            std::memcpy(&u, &f, 4);
            return u;
        };
        return sample_size == o.sample_size && bits(mu) == bits(o.mu) && bits(sigma) == bits(o.sigma) &&
               bits(variance) == bits(o.variance) && bits(sse) == bits(o.sse);
    }
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


// Results of one extension wave copied back from the device: one ExtResult per
// job, and the CIGAR ops they point into (ExtResult::cigar_offset).
struct WaveResults {
    PodArray<ExtResult> results;
    PodArray<uint32_t> cigar;
};

// Wave result buffers reused once no chunk refers to them any more (the pool holds
// the only reference), so that a wave's copy back lands in memory already paged in.
struct WavePool {
    std::vector<std::shared_ptr<WaveResults>> items;
    std::shared_ptr<WaveResults> take() {
        for (auto& w : items)
            if (w.use_count() == 1) return w;
        auto w = std::make_shared<WaveResults>();
        if (items.size() < 64) items.push_back(w);
        return w;
    }
};

// One extension result as the policy reads it: the device record plus the address
// of its CIGAR.
struct StoredResult : ExtResult {
    const uint32_t* cigar = nullptr;
};

// Requests and results of one batch, per device read.  An entry is written only by
// the thread that runs the chunk owning the read (chunks run on one thread at a
// time), so no locking is needed.
struct ResultStore {
    static constexpr uint32_t NONE = 0xffffffffu;
    struct Entry {
        JobKey key;
        uint32_t next;            // the read's next entry in its chunk's pool, or NONE
        const ExtResult* result;  // nullptr while pending
        const uint32_t* cigar;    // CIGAR base of the wave that produced the result
    };
    // per read: its first entry in the owning chunk's pool (ChunkState::entries)
    std::vector<uint32_t> head;
    void reset(size_t n_reads) { head.assign(n_reads, NONE); }
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
    bool timing = false;  // accumulate ChunkState::seconds_* (diagnostics)
};

struct ContigInfo {
    const std::string* name;
    uint64_t len;
};

// Per-read inputs the policy reads
// A batch's read views: a view into an array its owner keeps (the mapper, a session
// request), so that batch parts share it without copies
struct ReadSpan {
    const ReadView* p = nullptr;
    size_t n = 0;
    const ReadView& operator[](size_t i) const { return p[i]; }
    size_t size() const { return n; }
};

struct BatchView {
    ReadSpan reads;                      // device read order (pairs interleaved)
    const NamRec* nams = nullptr;
    const uint64_t* nam_off = nullptr;
    const NamDetailsRec* details = nullptr;
    bool paired = false;
    // mixed input (interleaved files, src/io/reads.rs:68-113): record r's reads are
    // rec_read[r] - rec_read_base up to rec_read[r + 1] - rec_read_base, one read
    // (single-end) or two (a pair); null: every record is a pair (paired) or every
    // record one read
    const uint32_t* rec_read = nullptr;
    uint32_t rec_read_base = 0;
    uint32_t first_read(uint64_t rec) const {
        return rec_read ? rec_read[rec] - rec_read_base : (uint32_t)(paired ? 2 * rec : rec);
    }
    bool rec_paired(uint64_t rec) const { return rec_read ? rec_read[rec + 1] - rec_read[rec] == 2 : paired; }
    // single-end piecewise extension: chain anchors of NAM t (index into nams) are the
    // packed keys nam_anc[nam_anc_off[t] .. nam_anc_off[t + 1]), last to first
    const uint64_t* nam_anc_off = nullptr;
    const uint64_t* nam_anc = nullptr;
    uint32_t anc_qbits = 0, anc_pbits = 0;
};

// The anchors of piecewise jobs (use_ssw == 0) as (query start, reference start)
// pairs of a wave's anchor array, in two passes: offsets points the jobs at
// consecutive ranges from anchor `first` on (returns how many anchors they take and
// raises max_n to the largest count); fill writes them (independent per job, so
// callers may split it over threads).  Other jobs are untouched.
uint64_t piecewise_anchor_offsets(const BatchView& bv, ExtJob* jobs, size_t n, uint64_t first, uint32_t& max_n);
void piecewise_anchor_fill(const BatchView& bv, const ExtJob* jobs, size_t n, uint32_t* anchors);

struct ChunkState {
    uint64_t first = 0, next = 0, end = 0;  // record range [first, end), cursor next
    uint32_t part = 0;                      // the batch part whose reads these are (Mapper)
    bool keep_buffers = false;              // done: clear the buffers but keep their memory (pooled)
    Rng rng;
    InsertSize isd;
    OutBuf out;
    uint64_t mapped = 0;
    bool done = false;
    std::vector<ResultStore::Entry> entries;              // requests and results of this chunk's reads
    std::vector<ExtJob> pending;                          // requests raised by this chunk (tag: entry)
    // the wave that ran `pending`: its results start at wave_first, in pending's
    // order; the thread that resumes the chunk points the entries at them
    std::shared_ptr<const WaveResults> wave;
    uint64_t wave_first = 0;
    std::vector<std::shared_ptr<const WaveResults>> waves;  // keeps the results the entries use
    uint64_t result_bytes = 0;  // device->host bytes of this chunk's results and CIGARs
    std::vector<std::pair<uint32_t, double>> abundance;   // (contig, weight) in read order
    bool lookahead_started = false;
    std::vector<uint64_t> lookahead_todo;                 // reads that missed in the last lookahead
    // what each record did to the RNG and the insert-size estimate when the last
    // lookahead evaluated it; later lookaheads replay it instead of evaluating again
    struct Effect {
        uint64_t rng_delta = 0;
        uint64_t isd_value = 0;
        bool known = false, isd_update = false;
        // SAM / PAF: the record's output from that evaluation and the state it started
        // from; the real run reuses it when it reaches the record in the same state
        bool has_output = false;
        uint64_t pre_rng = 0;
        InsertSize pre_isd, post_isd;
        uint64_t out_off = 0, out_len = 0, mapped = 0;
    };
    std::vector<Effect> effects;
    OutBuf spec_out;  // outputs captured by the lookahead
    // the chunk's output in record order: ranges of `out` (records the real run
    // formatted) and of `spec_out` (captured records it reused), copied once into the
    // final buffer
    struct Piece {
        bool spec;
        uint64_t off, len;
    };
    std::vector<Piece> pieces;
    uint64_t out_bytes = 0;
    void add_piece(bool spec, uint64_t off, uint64_t len) {
        if (!len) return;
        if (!pieces.empty() && pieces.back().spec == spec && pieces.back().off + pieces.back().len == off)
            pieces.back().len += len;
        else
            pieces.push_back(Piece{spec, off, len});
        out_bytes += len;
    }
    uint64_t evals_reused = 0;
    // real-run misses on a record the lookahead had evaluated to the end under another
    // state (mispredicted), and on one it had not (unknown)
    uint64_t miss_mispredicted = 0, miss_unknown = 0;
    // captured outputs not reused: the RNG state, the insert-size state differed
    uint64_t stale_rng = 0, stale_isd = 0;
    // host time by phase when PolicyConfig::timing is set
    double seconds_real = 0, seconds_spec = 0, seconds_seed = 0, seconds_format = 0;
    uint64_t evals_real = 0, evals_spec = 0, runs = 0;
};

// Output and bookkeeping buffers of a finished chunk, kept for a later chunk (their
// memory is paged in already): lend() moves them into a new chunk, reclaim() takes
// them back, emptied, when a chunk's output has been gathered.
struct ChunkBuffers {
    OutBuf out, spec_out;
    std::vector<ChunkState::Effect> effects;
    std::vector<ResultStore::Entry> entries;
    std::vector<ChunkState::Piece> pieces;
    void lend(ChunkState& cs) {
        std::swap(cs.out, out);
        std::swap(cs.spec_out, spec_out);
        std::swap(cs.effects, effects);
        std::swap(cs.entries, entries);
        std::swap(cs.pieces, pieces);
        cs.keep_buffers = true;
    }
    void reclaim(ChunkState& cs) {
        cs.out.clear();
        cs.spec_out.clear();
        cs.effects.clear();
        cs.entries.clear();
        cs.pieces.clear();
        std::swap(cs.out, out);
        std::swap(cs.spec_out, spec_out);
        std::swap(cs.effects, effects);
        std::swap(cs.entries, entries);
        std::swap(cs.pieces, pieces);
    }
};

class Policy {
  public:
    Policy(const PolicyConfig& cfg, const std::vector<ContigInfo>& contigs, const BatchView& bv, ResultStore& store);
    ~Policy();
    Policy(const Policy&) = delete;
    Policy& operator=(const Policy&) = delete;
    // Advance one chunk as far as the available results allow.  On a miss, the
    // rest of the chunk is evaluated speculatively (state copies, output dropped)
    // so that the jobs of later reads join the next wave.
    void run_chunk(ChunkState& cs);
    // Speculative first-wave requests for the reads of one chunk.
    void seed_requests(ChunkState& cs);

  private:
    const PolicyConfig& cfg_;
    const std::vector<ContigInfo>& contigs_;
    const BatchView* bv_;
    ResultStore* store_;
    ChunkState* cur_ = nullptr;
    bool speculative_ = false;
    bool pe_ = false;  // the record being evaluated is a pair (its extensions use SSW)
    struct Scratch;
    std::unique_ptr<Scratch> sc_;
    void add_abundance(uint32_t ref_id, double w) {
        if (!speculative_) cur_->abundance.emplace_back(ref_id, w);
    }

    void want(uint32_t read, const ExtJob& job, const JobKey& key);
    const ResultStore::Entry* lookup(uint32_t read, const JobKey& key) const;
    // the result of a job, or false after requesting it
    bool get(uint32_t read, const ExtJob& job, const JobKey& key, StoredResult& out);
    void resolve(ChunkState& cs);

    // false: stopped on a missing result (the record is evaluated again later)
    bool se_record(uint64_t rec, Rng& rng, OutBuf& out, uint64_t& mapped);
    bool pe_record(uint64_t rec, Rng& rng, InsertSize& isd, OutBuf& out, uint64_t& mapped);
    void paf_se(uint64_t rec, Rng& rng, OutBuf& out);
    void paf_pe(uint64_t rec, Rng& rng, InsertSize& isd, OutBuf& out);
    void aemb_se(uint64_t rec, Rng& rng);
    void aemb_pe(uint64_t rec, Rng& rng, InsertSize& isd);

  public:
    // helpers used by the implementation file
    std::vector<NamRec> sorted_nams(uint32_t read, Rng& rng) const;
    void sorted_nams(uint32_t read, Rng& rng, std::vector<NamRec>& out) const;
    ExtJob nam_job(uint32_t read, const NamRec& n, uint32_t kind) const;
    static JobKey nam_key(const NamRec& n, uint32_t kind) { return JobKey{kind, n.nam_id, 0, 0, 0}; }
    Alignment to_alignment(const StoredResult& r, uint32_t ref_id) const;
    const PolicyConfig& cfg() const { return cfg_; }
    const std::vector<ContigInfo>& contigs() const { return contigs_; }
    const BatchView& bv() const { return *bv_; }
    // point the policy at another batch (a session's request) between chunk runs
    void bind(const BatchView& bv, ResultStore& store) {
        bv_ = &bv;
        store_ = &store;
    }
    // results of extend / rescue: aligned, not aligned, or the job's result is missing
    // (it has been requested)
    enum { MISSING = -1, UNALIGNED = 0, ALIGNED = 1 };
    // extend_seed with the given consistency semantics; applies the flip to nam
    int extend(uint32_t read, NamRec& nam, uint32_t kind, Alignment& out, bool& consistent);
    int rescue(uint32_t read, const NamRec& mate, float mu, float sigma, Alignment& out);
    bool rescue_job(uint32_t read, const NamRec& mate, float mu, float sigma, ExtJob& j, JobKey& key) const;
    void want_rescue_chain(uint32_t read, const NamRec& nam, uint32_t mate, float mu, float sigma, bool need_valid);
    void want_nam(uint32_t read, const NamRec& n, uint32_t kind);
};

}  // namespace sa
