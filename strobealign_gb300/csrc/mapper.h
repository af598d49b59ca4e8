// Batch driver state behind sa_mapper.
#pragma once
#include <atomic>
#include <chrono>
#include <thread>

#include "host_util.h"
#include "policy.h"

namespace sa {

class Mapper {
  public:
    static constexpr uint64_t MAX_PART_BASES = 1ULL << 27;
    Mapper(const sa_index* idx, const sa_refs* refs, const sa_chaining_params& cp, const sa_mapping_params& mp);
    ~Mapper();
    void map(const sa_read_batch* r1, const sa_read_batch* r2, sa_output* out);
    void upload(const sa_read_batch* r1, const sa_read_batch* r2);
    // mixed input: one batch of reads in file order, a read and the next one a pair when
    // their names are equal, any other read single-end (src/io/reads.rs:68-113)
    void map_interleaved(const sa_read_batch* reads, sa_output* out);
    void upload_interleaved(const sa_read_batch* reads);
    void map_uploaded(sa_output* out);
    const sa_mapper_stats& stats() const { return stats_; }
    const sa_mapping_params& mapping_params() const { return mp_; }
    const std::vector<ContigInfo>& contigs() const { return contigs_; }
    const std::vector<double>& abundances() const { return abundances_; }
    std::vector<uint64_t> contig_lengths() const {
        std::vector<uint64_t> v;
        for (auto& c : contigs_) v.push_back(c.len);
        return v;
    }
    const DevRefs& refs_view() const { return refs_view_; }
    NamWorkspace& nam_ws() { return nws_; }
    ExtWorkspace& ext_ws() { return ews_; }
    cudaStream_t stream() const { return st_; }
    void upload_reads(const ReadSpan& reads);
    uint32_t n_reads() const { return n_reads_; }
    uint64_t total_bases() const { return total_bases_; }
    uint64_t h2d_bytes() const { return h2d_bytes_; }
    uint64_t d2h_bytes() const { return d2h_bytes_; }
    uint32_t last_launches() const { return last_launches_; }
    uint32_t last_waves() const { return last_waves_; }
    uint64_t jobs_run() const { return jobs_run_; }
    void set_policy_threads(unsigned n) { policy_threads_ = n ? n : 1; }
    void set_profiling(bool on) { kt_.enabled = kt_nam_.enabled = on; }
    void set_parts(uint32_t n) { parts_target_ = n ? n : 1; }
    void set_wave_min_jobs(uint64_t n) { wave_min_jobs_ = n; }
    void set_max_wave_jobs(uint64_t n) { max_wave_jobs_ = n ? n : 1; }
    // false: stage-synchronous (plain) form: the policy and the extension waves
    // alternate, every waiting request goes into the waves before any chunk resumes,
    // and the output is gathered after the last chunk
    void set_overlap(bool on) { overlap_ = on; }
    // output-invariant knobs the autotuner chooses
    struct Tuning {
        uint32_t parts = 8;
        uint64_t wave_min_jobs = 32768, max_wave_jobs = 262144;
        uint32_t wave_qmax = 192, chain_lane_max = 48;
        uint32_t l2_fetch = 0;  // 0: the context's value at construction
    };
    struct TuneReport {
        Tuning chosen;
        double seconds_default = 0, seconds_tuned = 0;
        uint32_t trials = 0;
    };
    void set_tuning(const Tuning& t);
    Tuning tuning() const;
    // Times the batch under the default knobs, then one knob after another over a short
    // list of values (coordinate descent, each trial the median of `rounds` maps), keeps a
    // change only when it is 2% faster, checks that every trial writes the same bytes,
    // and applies the choice.  The batch stays uploaded.
    TuneReport autotune(const sa_read_batch* r1, const sa_read_batch* r2, uint32_t rounds);

  private:
    TuneReport autotune_run(const sa_read_batch* r1, const sa_read_batch* r2, uint32_t rounds);

  public:

  private:
    // One NAM-pipeline part of a batch: a run of whole chunks with their reads' NAMs on
    // the host, and the part's own read view and result store (read and record indices
    // local to the part).  The NAM pipeline of part p + 1 runs while the chunks of
    // parts <= p are in the policy and extension waves.
    struct Part {
        uint64_t rec_lo = 0, rec_hi = 0;
        uint32_t read_lo = 0, read_hi = 0;
        size_t chunk_lo = 0, chunk_hi = 0;
        BatchView bv;
        ResultStore store;
        PinnedBuf<uint64_t> nam_off;
        PinnedBuf<NamRec> nams;
        PinnedBuf<NamDetailsRec> details;
        PinnedBuf<uint64_t> anc_off, anc;  // single-end piecewise: NAM chain anchors
        uint64_t n_nams = 0;
        double seconds = 0;
    };
    void part_nams(Part& p, uint32_t& launches);
    std::shared_ptr<const WaveResults> run_wave(const ExtJob* jobs, uint32_t nj, uint32_t max_qlen,
                                                uint32_t& launches, const uint32_t* anchors, size_t anchor_words,
                                                uint32_t max_anchors);
    uint32_t schedule(std::vector<ChunkState>& chunks, uint32_t& launches, uint32_t& nam_launches);
    PodArray<ReadView> reads_;  // the uploaded batch's read views (device read order)
    BatchView bv_;
    // mixed input: record r's reads are rec_read_[r] .. rec_read_[r + 1] (n + 1 entries);
    // empty for uniform batches
    std::vector<uint32_t> rec_read_;
    bool have_batch_ = false;
    uint32_t max_qlen_ = 1;
    sa_mapper_stats stats_{};
    double t_ext_ = 0;
    KernelTimers kt_, kt_nam_;
    uint64_t sw_cells_[7] = {0, 0, 0, 0, 0, 0, 0};  // SW cells, then banded cells
    unsigned policy_threads_ = std::max(1u, std::thread::hardware_concurrency());
    uint64_t wave_min_jobs_ = 32768;
    uint64_t max_wave_jobs_ = 262144;
    bool overlap_ = true;
    uint32_t chain_lane_max_ = 48;
    uint32_t l2_fetch_ = 0;           // applied by set_tuning (0: untouched)
    size_t l2_fetch_default_ = 0;     // the context's limit at construction
    bool trace_ = false;

    const sa_index* idx_;
    const sa_refs* refs_;
    sa_chaining_params cp_;
    sa_mapping_params mp_;
    std::string rg_id_;
    PolicyConfig pcfg_;
    cudaStream_t st_ = nullptr;   // uploads and extension waves
    cudaStream_t stn_ = nullptr;  // NAM pipelines of the parts (highest priority)
    DevBuf<uint64_t> d_words_, d_woff_;
    DevBuf<uint32_t> d_clen_;
    DevRefs refs_view_{};
    uint32_t max_contig_len_ = 0;
    std::vector<ContigInfo> contigs_;
    std::vector<double> abundances_;
    bool single_end_piecewise_ = false;
    NamWorkspace nws_;
    ExtWorkspace ews_;
    PinnedBuf<uint8_t> h_seq_;
    PinnedBuf<uint64_t> h_off_;
    PinnedBuf<ExtJob> h_jobs_;
    std::vector<std::unique_ptr<Part>> parts_;  // grow-only; pinned buffers reused across batches
    size_t n_parts_ = 0;
    uint32_t parts_target_ = 8;
    NamWorkspace pws_;            // NAM pipeline buffers of one part
    PinnedBuf<uint64_t> h_poff_;  // a part's local read offsets
    double t_nams_ = 0;
    std::chrono::steady_clock::time_point t_map0_;  // start of the current map (trace times)
    PodArray<uint32_t> wave_anchors_;  // a wave's piecewise anchors (query, reference start pairs)
    WavePool wave_pool_;
    std::vector<ChunkBuffers> chunk_pool_;  // the last batch's chunk buffers, lent to the next
    // Output copied while the batch is mapped: idle policy threads copy each chunk whose
    // predecessors are all done into `dst` (sized from the previous batch's bytes per
    // record); the rest is gathered at the end.  Without room it falls back to one
    // gather into an exact buffer.
    struct StreamOut {
        char* dst = nullptr;
        size_t cap = 0;
        bool overflow = false;
        std::vector<size_t> off;       // chunk c's output offset, for c <= done_prefix
        std::vector<char> done;        // chunk finished (set under the schedule lock)
        size_t done_prefix = 0;        // chunks [0, done_prefix) are all done
        size_t next_claim = 0;         // chunks [0, next_claim) copied or being copied
    } so_;
    double bytes_per_record_ = 0;  // previous batch, for the output estimate
    uint32_t n_reads_ = 0;
    uint64_t total_bases_ = 0;
    std::atomic<uint64_t> h2d_bytes_{0}, d2h_bytes_{0};
    uint32_t last_launches_ = 0, last_waves_ = 0;
    uint64_t jobs_run_ = 0;
    double last_seconds_ = 0;
};

}  // namespace sa

struct sa_mapper {
    sa::Mapper* m;
};
