// Serving engine behind sa_session: requests (read batches) are admitted into a
// device read arena as memory frees up, get their NAMs from one pass of the device
// pipeline, and then share the chunk scheduler and the extension waves with every
// other request in flight.  Each request is its own chunk stream (chunks cut from
// the request's records, fresh RNG and insert-size state per chunk,
// src/main.rs:591-604,873-880), so its output does not depend on what else is in
// flight.
#pragma once
#include <chrono>
#include <cstdlib>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "host_util.h"
#include "policy.h"

namespace sa {

// First-fit allocator of [0, capacity) ranges with coalescing on free.
class RangeAllocator {
  public:
    explicit RangeAllocator(uint64_t capacity = 0) { reset(capacity); }
    void reset(uint64_t capacity) {
        free_.clear();
        if (capacity) free_[0] = capacity;
        capacity_ = capacity;
    }
    bool alloc(uint64_t n, uint64_t& at);
    void release(uint64_t at, uint64_t n);
    uint64_t capacity() const { return capacity_; }
    uint64_t largest_free() const;

  private:
    std::map<uint64_t, uint64_t> free_;  // start -> length
    uint64_t capacity_ = 0;
};

struct Request {
    uint64_t id = 0;
    bool paired = false;
    // mixed single-end and paired records (interleaved input): reads in file order,
    // record r's reads from rec_read[r] to rec_read[r + 1]
    bool mixed = false;
    std::vector<uint32_t> rec_read;
    // admission groups share one NAM pipeline configuration: single-end, paired, mixed
    int kind() const { return mixed ? 2 : paired ? 1 : 0; }
    // owned copies of the records (empty when the session borrows the caller's batch)
    RawBytes seq, qual, names, comments;
    // sequences in device read order (mates interleaved) with per-read offsets;
    // qualities, names and comments one block per mate (read views point into them)
    std::vector<uint64_t> seq_off;
    bool has_qual = false, has_comments = false;
    PodArray<ReadView> read_views;  // device read order; bv.reads views them
    BatchView bv;
    uint64_t nrec = 0, n_reads = 0, total_bases = 0;
    uint32_t max_qlen = 1;
    std::mutex max_qlen_mu;  // guards max_qlen while submit's copy threads run
    // device placement (arena units: bases, offset slots)
    uint64_t seq_base = 0, read_base = 0;
    // NAMs copied back from the device
    std::vector<NamRec> nams;
    std::vector<uint64_t> nam_off;
    std::vector<NamDetailsRec> details;
    std::vector<uint64_t> nam_anc_off, nam_anc;  // single-end piecewise: NAM chain anchors
    ResultStore store;
    std::vector<ChunkState> chunks;
    std::vector<uint8_t> seeded;
    size_t n_done = 0;
    // result: malloc'd, handed over to the caller by sa_session_wait
    char* out = nullptr;
    size_t out_len = 0;
    uint64_t mapped = 0;
    std::vector<double> abundance;
    uint32_t waves = 0;
    uint64_t h2d_bytes = 0, d2h_bytes = 0;  // this request's share of the transfers
    int state = 0;  // 0 queued, 1 admitted, 2 done, 3 failed
    // threads reading the request's records outside the session lock (admission lanes,
    // policy workers); a failed request's wait returns only once this is 0, so that a
    // caller's borrowed buffers are no longer read when it frees them
    int users = 0;
    std::string error;
    int32_t error_code = 0;
    std::chrono::steady_clock::time_point t_submit, t_admit, t_done;
    ~Request() { release_output(out); }
};

struct SessionConfig {
    uint64_t max_inflight_bases = 0;      // 0 = sized from free device memory
    uint64_t device_reserve_bytes = 0;    // 0 = max(2 GiB, 5% of the device)
    uint32_t max_inflight_requests = 0;  // 0 = no limit
    uint32_t policy_threads = 0;         // 0 = all host threads
    uint32_t admission_streams = 2;      // requests admitted concurrently (NAM pipelines in flight)
    bool borrow_inputs = false;          // read views point into the caller's batch (no copies)
};

// One admission lane: a thread with its own stream, NAM workspace and staging, so that
// the NAM pipelines of several requests run at once (a request's pipeline ends with its
// slowest read orientation; concurrent lanes fill the GPU meanwhile).
struct AdmitLane {
    cudaStream_t st = nullptr;
    NamWorkspace nws;
    uint64_t ws_bases = 0;  // bases the lane's NAM workspace has grown to (admission estimate)
    PinnedBuf<uint8_t> h_seq;
    PinnedBuf<uint64_t> h_off;
    std::vector<uint64_t> h_goff;
    // a group's NAMs, statistics and chain anchors as copied back, before the split
    PinnedBuf<uint64_t> h_nam_off, h_anc_off, h_anc;
    PinnedBuf<NamRec> h_nams;
    PinnedBuf<NamDetailsRec> h_details;
    std::thread th;
};

class Session {
  public:
    Session(const sa_index* idx, const sa_refs* refs, const sa_chaining_params& cp, const sa_mapping_params& mp,
            const SessionConfig& sc);
    ~Session();
    uint64_t submit(const sa_read_batch* r1, const sa_read_batch* r2, bool interleaved = false);
    // 1 done, 0 not yet; throws for an unknown ticket
    int poll(uint64_t ticket);
    // Waits up to timeout_ms (< 0: no limit).  Returns false on timeout.  On
    // success the request is released and its output moved out.
    bool wait(uint64_t ticket, int64_t timeout_ms, std::unique_ptr<Request>& out);
    uint64_t in_flight() const;
    // device read arena (bases) and the device memory admission leaves free
    uint64_t arena_bases() const { return cfg_.max_inflight_bases; }
    uint64_t reserve_bytes() const { return reserve_; }
    uint64_t refused() const { return refused_; }
    // NAM workspace bytes per base of an admitted group (estimate: syncmers 12,
    // randstrobes 48, hits 32, anchor counts 8, anchors and chaining state)
    static constexpr uint64_t NAM_BYTES_PER_BASE = 160;
    const std::vector<ContigInfo>& contigs() const { return contigs_; }

  private:
    void engine();
    void admitter(AdmitLane& lane);
    void worker();
    void admit_group(const std::vector<Request*>& group, AdmitLane& lane);
    void run_wave(std::vector<std::pair<Request*, size_t>>& batch);
    void complete(Request& r);
    void fail_all(const std::string& msg, int32_t code);

    const sa_index* idx_;
    const sa_refs* refs_;
    sa_chaining_params cp_;
    sa_mapping_params mp_;
    std::string rg_id_;
    PolicyConfig pcfg_;
    SessionConfig cfg_;
    std::vector<ContigInfo> contigs_;
    uint32_t max_contig_len_ = 0;
    cudaStream_t st_ = nullptr;   // extension waves
    std::vector<std::unique_ptr<AdmitLane>> lanes_;
    DevBuf<uint64_t> d_words_, d_woff_;
    DevBuf<uint32_t> d_clen_;
    DevRefs refs_view_{};
    ExtWorkspace ews_;
    PinnedBuf<ExtJob> h_jobs_;
    PodArray<uint32_t> wave_anchors_;  // a wave's piecewise anchors (query, reference start pairs)
    WavePool wave_pool_;
    // buffers of finished requests' chunks, lent to the chunks of new requests
    std::mutex chunk_pool_mu_;
    std::vector<ChunkBuffers> chunk_pool_;
    // read arena
    DevBuf<uint8_t> arena_seq_;
    DevBuf<uint64_t> arena_off_;
    RangeAllocator seq_alloc_, off_alloc_;

    mutable std::mutex mu_;
    std::condition_variable cv_engine_, cv_admit_, cv_work_, cv_done_;
    std::deque<std::unique_ptr<Request>> queue_;                    // submitted, not admitted
    std::unordered_map<uint64_t, std::unique_ptr<Request>> live_;  // admitted or done
    std::deque<std::pair<Request*, size_t>> ready_;
    std::vector<std::pair<Request*, size_t>> waiting_;
    uint64_t waiting_jobs_ = 0;
    unsigned running_ = 0;
    uint64_t next_id_ = 1;
    uint64_t reserve_ = 0;         // device memory admission keeps free
    uint64_t pending_growth_ = 0;  // workspace growth of groups being admitted (not yet allocated)
    uint64_t refused_ = 0;         // requests refused for lack of device memory
    uint32_t inflight_ = 0;
    bool stop_ = false;
    bool workers_stop_ = false;
    unsigned admitting_ = 0;  // admissions in progress
    bool broken_ = false;  // a device or internal error failed every request
    std::string broken_msg_;
    // failed requests stay allocated until the session is destroyed: queued work
    // items may still point at them
    std::vector<std::unique_ptr<Request>> graveyard_;
    uint64_t wave_min_jobs_ = 32768;
    uint64_t admit_group_reads_ = 262144;  // reads one admission's NAM pipeline takes at most
    uint64_t max_wave_jobs_ = 262144;
    bool trace_ = false;
    std::chrono::steady_clock::time_point t0_;
    std::thread engine_;
    std::vector<std::thread> workers_;
};

}  // namespace sa

struct sa_session {
    sa::Session* s;
};
