// Serving engine: continuous batching of mapping requests on one GPU.
//
// One engine thread owns the device work: it admits queued requests into the
// read arena (upload, NAM pipeline, NAMs copied back) and runs extension waves
// over the requests of every chunk that stopped on a miss, whichever request it
// belongs to.  Policy threads run the chunks whose results are in.  A wave starts
// once enough jobs wait or when the policy threads have nothing left to run; a
// request is admitted when its reads fit in the arena.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "host_input.h"
#include "host_util.h"
#include "session.h"

namespace sa {

bool RangeAllocator::alloc(uint64_t n, uint64_t& at) {
    if (n == 0) n = 1;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
        if (it->second >= n) {
            at = it->first;
            const uint64_t rest = it->second - n;
            const uint64_t start = it->first + n;
            free_.erase(it);
            if (rest) free_[start] = rest;
            return true;
        }
    }
    return false;
}

void RangeAllocator::release(uint64_t at, uint64_t n) {
    if (n == 0) n = 1;
    auto it = free_.emplace(at, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        free_.erase(nx);
    }
    if (it != free_.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            free_.erase(it);
        }
    }
}

uint64_t RangeAllocator::largest_free() const {
    uint64_t m = 0;
    for (auto& f : free_) m = std::max(m, f.second);
    return m;
}

Session::Session(const sa_index* idx, const sa_refs* refs, const sa_chaining_params& cp, const sa_mapping_params& mp,
                 const SessionConfig& sc)
    : idx_(idx), refs_(refs), cp_(cp), mp_(mp), cfg_(sc) {
    if (mp.rg_id) rg_id_ = mp.rg_id;
    mp_.rg_id = nullptr;
    // SA_TRACE_WAVES=1: admissions and extension waves on stderr
    const char* tr = std::getenv("SA_TRACE_WAVES");
    trace_ = tr && *tr && *tr != '0';
    // SA_MAX_WAVE_JOBS: extension jobs per wave at most (tuning)
    if (const char* mw = std::getenv("SA_MAX_WAVE_JOBS")) max_wave_jobs_ = std::max<uint64_t>(1, std::strtoull(mw, nullptr, 10));
    // SA_WAVE_MIN_JOBS: jobs that start a wave while policy threads are still busy;
    // SA_ADMIT_GROUP_READS: reads one admission takes at most (tuning)
    if (const char* mj = std::getenv("SA_WAVE_MIN_JOBS")) wave_min_jobs_ = std::max<uint64_t>(1, std::strtoull(mj, nullptr, 10));
    if (const char* ag = std::getenv("SA_ADMIT_GROUP_READS"))
        admit_group_reads_ = std::max<uint64_t>(1, std::strtoull(ag, nullptr, 10));
    t0_ = std::chrono::steady_clock::now();
    SA_CUDA(cudaSetDevice(idx->device));
    SA_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
    // admissions at the highest stream priority: their blocks are dispatched ahead of
    // queued wave blocks, so a new request's NAM pipeline does not wait behind a wave
    int prio_least = 0, prio_greatest = 0;
    SA_CUDA(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
    const uint32_t n_lanes = std::max<uint32_t>(1, cfg_.admission_streams);
    for (uint32_t l = 0; l < n_lanes; l++) {
        lanes_.push_back(std::make_unique<AdmitLane>());
        SA_CUDA(cudaStreamCreateWithPriority(&lanes_.back()->st, cudaStreamNonBlocking, prio_greatest));
    }
    const auto& cs = refs->contigs;
    const uint32_t nc = (uint32_t)cs.size();
    std::vector<uint64_t> woff(nc);
    std::vector<uint32_t> clen(nc);
    uint64_t nw = 0;
    for (uint32_t c = 0; c < nc; c++) {
        woff[c] = nw;
        nw += cs[c].words.size() + 1;
        clen[c] = (uint32_t)cs[c].len;
        max_contig_len_ = std::max<uint32_t>(max_contig_len_, clen[c]);
        contigs_.push_back(ContigInfo{&cs[c].name, cs[c].len});
    }
    std::vector<uint64_t> hw(nw, 0);
    for (uint32_t c = 0; c < nc; c++) std::copy(cs[c].words.begin(), cs[c].words.end(), hw.begin() + woff[c]);
    d_words_.reserve(std::max<uint64_t>(nw, 1));
    d_woff_.reserve(std::max<uint32_t>(nc, 1));
    d_clen_.reserve(std::max<uint32_t>(nc, 1));
    if (nw) SA_CUDA(cudaMemcpy(d_words_.p, hw.data(), nw * 8, cudaMemcpyHostToDevice));
    if (nc) {
        SA_CUDA(cudaMemcpy(d_woff_.p, woff.data(), nc * 8, cudaMemcpyHostToDevice));
        SA_CUDA(cudaMemcpy(d_clen_.p, clen.data(), nc * 4, cudaMemcpyHostToDevice));
    }
    refs_view_ = DevRefs{d_words_.p, d_woff_.p, d_clen_.p, nc};
    pcfg_.mp = mp_;
    pcfg_.rg_id = rg_id_;
    pcfg_.has_rg = mp.rg_id != nullptr;
    pcfg_.k = idx->sp.k;
    // memory-based admission: the arena and the lanes' workspaces come out of the free
    // device memory, less a reserve kept for everything else on the device
    size_t mem_free = 0, mem_total = 0;
    SA_CUDA(cudaMemGetInfo(&mem_free, &mem_total));
    reserve_ = cfg_.device_reserve_bytes ? cfg_.device_reserve_bytes
                                         : std::max<uint64_t>(2ull << 30, (uint64_t)mem_total / 20);
    if (cfg_.max_inflight_bases == 0) {
        // an eighth of what is usable, the rest left to the NAM and extension workspaces
        const uint64_t usable = mem_free > reserve_ ? (uint64_t)mem_free - reserve_ : 0;
        cfg_.max_inflight_bases = std::min<uint64_t>(1ull << 33, std::max<uint64_t>(1ull << 24, usable / 8));
    }
    const uint64_t slots = cfg_.max_inflight_bases / 32 + 65536;
    arena_seq_.reserve(cfg_.max_inflight_bases + 16);
    arena_off_.reserve(slots);
    seq_alloc_.reset(cfg_.max_inflight_bases);
    off_alloc_.reset(slots);
    unsigned nt = cfg_.policy_threads ? cfg_.policy_threads : std::max(1u, std::thread::hardware_concurrency());
    engine_ = std::thread([this] { engine(); });
    for (auto& l : lanes_) {
        AdmitLane* lp = l.get();
        l->th = std::thread([this, lp] { admitter(*lp); });
    }
    for (unsigned t = 0; t < nt; t++) workers_.emplace_back([this] { worker(); });
}

Session::~Session() {
    {
        std::lock_guard<std::mutex> g(mu_);
        stop_ = true;
        for (auto& q : queue_) {
            q->state = 3;
            q->error = "session destroyed before the request was admitted";
            q->error_code = SA_ERR_CANCELLED;
        }
        queue_.clear();
    }
    cv_engine_.notify_all();
    cv_admit_.notify_all();
    cv_done_.notify_all();
    for (auto& l : lanes_)
        if (l->th.joinable()) l->th.join();
    if (engine_.joinable()) engine_.join();
    {
        std::lock_guard<std::mutex> g(mu_);
        workers_stop_ = true;
    }
    cv_work_.notify_all();
    for (auto& t : workers_) t.join();
    if (st_) cudaStreamDestroy(st_);
    for (auto& l : lanes_)
        if (l->st) cudaStreamDestroy(l->st);
}

uint64_t Session::submit(const sa_read_batch* r1, const sa_read_batch* r2, bool interleaved) {
    if (!r1) throw Error(SA_ERR_INVALID, "null read batch");
    if (interleaved && r2) throw Error(SA_ERR_INVALID, "interleaved input takes one read batch");
    if (interleaved && r1->n >= UINT32_MAX) throw Error(SA_ERR_INVALID, "batch too large");
    const bool paired = r2 != nullptr;
    if (paired && r2->n != r1->n) throw Error(SA_ERR_INVALID, "r1 and r2 batches differ in size");
    auto r = std::make_unique<Request>();
    r->paired = paired;
    r->nrec = r1->n;
    r->n_reads = paired ? 2 * r1->n : r1->n;
    r->has_qual = r1->qual != nullptr && (!paired || r2->qual != nullptr);
    r->has_comments = r1->comments && r1->comment_offsets;
    const sa_read_batch* mates[2] = {r1, r2};
    const int nm = paired ? 2 : 1;
    // qualities, names and comments: one block per mate, copied whole; sequences in
    // device read order (mates interleaved), as the arena and the NAM pipeline take them
    uint64_t seq_total = 0, qual_base[2] = {0, 0}, name_base[2] = {0, 0}, com_base[2] = {0, 0};
    uint64_t qual_total = 0, name_total = 0, com_total = 0;
    for (int m = 0; m < nm; m++) {
        const sa_read_batch* b = mates[m];
        const uint64_t n = b->n;
        const uint64_t sb = n ? b->seq_offsets[n] - b->seq_offsets[0] : 0;
        seq_total += sb;
        qual_base[m] = qual_total;
        if (r->has_qual) qual_total += sb;
        name_base[m] = name_total;
        name_total += n ? b->name_offsets[n] - b->name_offsets[0] : 0;
        com_base[m] = com_total;
        if (b->comments && b->comment_offsets)
            com_total += n ? b->comment_offsets[n] - b->comment_offsets[0] : 0;
    }
    const bool borrow = cfg_.borrow_inputs;
    if (!borrow) {
        r->qual.resize(qual_total);
        r->names.resize(name_total);
        r->comments.resize(com_total);
    }
    for (int m = 0; m < nm && !borrow; m++) {
        const sa_read_batch* b = mates[m];
        const uint64_t n = b->n;
        if (!n) continue;
        if (r->has_qual)
            parallel_memcpy(r->qual.data() + qual_base[m], b->qual + b->seq_offsets[0],
                            b->seq_offsets[n] - b->seq_offsets[0], 8);
        std::memcpy(r->names.data() + name_base[m], b->names + b->name_offsets[0],
                    b->name_offsets[n] - b->name_offsets[0]);
        if (b->comments && b->comment_offsets)
            std::memcpy(r->comments.data() + com_base[m], b->comments + b->comment_offsets[0],
                        b->comment_offsets[n] - b->comment_offsets[0]);
    }
    if (!borrow) r->seq.resize(seq_total);
    r->seq_off.resize(r->n_reads + 1);
    r->read_views.resize(r->n_reads);
    r->bv.paired = paired;
    // offsets first (a prefix sum), then the copies and views in parallel
    uint64_t so = 0;
    for (uint64_t i = 0; i < r1->n; i++) {
        for (int m = 0; m < nm; m++) {
            const sa_read_batch* b = mates[m];
            const uint64_t len = b->seq_offsets[i + 1] - b->seq_offsets[i];
            if (len > MAX_READ_LEN)
                throw Error(SA_ERR_INVALID, "read longer than " + std::to_string(MAX_READ_LEN) + " nt");
            r->seq_off[paired ? 2 * i + m : i] = so;
            so += len;
        }
    }
    const unsigned copy_threads = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
    parallel_ranges(r1->n, copy_threads, [&](uint64_t ia, uint64_t ib) {
        uint32_t mq = 1;
        for (uint64_t i = ia; i < ib; i++) {
            for (int m = 0; m < nm; m++) {
                const sa_read_batch* b = mates[m];
                const uint64_t s0 = b->seq_offsets[i], s1 = b->seq_offsets[i + 1];
                const uint64_t d = paired ? 2 * i + m : i;
                const uint64_t at = r->seq_off[d];
                ReadView& v = r->read_views[d];
                const uint64_t n0 = b->name_offsets[i], n1 = b->name_offsets[i + 1];
                v.len = (uint32_t)(s1 - s0);
                v.name_len = (uint32_t)(n1 - n0);
                v.comment = nullptr;
                v.comment_len = 0;
                const bool com = b->comments && b->comment_offsets && b->comment_offsets[i + 1] > b->comment_offsets[i];
                if (borrow) {
                    v.seq = b->seq + s0;
                    v.qual = r->has_qual ? b->qual + s0 : nullptr;
                    v.name = b->names + n0;
                    if (com) {
                        v.comment = b->comments + b->comment_offsets[i];
                        v.comment_len = (uint32_t)(b->comment_offsets[i + 1] - b->comment_offsets[i]);
                    }
                } else {
                    std::memcpy(r->seq.data() + at, b->seq + s0, s1 - s0);
                    v.seq = r->seq.data() + at;
                    v.qual = r->has_qual ? r->qual.data() + qual_base[m] + (s0 - b->seq_offsets[0]) : nullptr;
                    v.name = r->names.data() + name_base[m] + (n0 - b->name_offsets[0]);
                    if (com) {
                        const uint64_t c0 = b->comment_offsets[i], c1 = b->comment_offsets[i + 1];
                        v.comment = r->comments.data() + com_base[m] + (c0 - b->comment_offsets[0]);
                        v.comment_len = (uint32_t)(c1 - c0);
                    }
                }
                mq = std::max(mq, v.len);
            }
        }
        std::lock_guard<std::mutex> g(r->max_qlen_mu);
        r->max_qlen = std::max(r->max_qlen, mq);
    });
    r->seq_off[r->n_reads] = so;
    r->total_bases = so;
    if (interleaved) {
        // the reads stay in file order; records pair them by name (src/io/reads.rs:68-113)
        pair_records_by_name(*r1, true, r->rec_read);
        r->mixed = true;
        r->nrec = r->rec_read.size() - 1;
        r->bv.rec_read = r->rec_read.data();
    }
    if (r->total_bases > seq_alloc_.capacity() || r->n_reads + 1 > off_alloc_.capacity())
        throw Error(SA_ERR_INVALID, "request larger than the session's in-flight capacity (" +
                                        std::to_string(seq_alloc_.capacity()) + " bases)");
    r->bv.reads = ReadSpan{r->read_views.data(), r->read_views.size()};
    r->t_submit = std::chrono::steady_clock::now();
    uint64_t id;
    {
        std::lock_guard<std::mutex> g(mu_);
        if (broken_) throw Error(SA_ERR_CUDA, "session failed: " + broken_msg_);
        if (stop_) throw Error(SA_ERR_CANCELLED, "session is shutting down");
        id = next_id_++;
        r->id = id;
        queue_.push_back(std::move(r));
    }
    cv_admit_.notify_one();
    return id;
}

int Session::poll(uint64_t ticket) {
    std::lock_guard<std::mutex> g(mu_);
    auto it = live_.find(ticket);
    if (it != live_.end()) return it->second->state >= 2 ? 1 : 0;
    for (auto& q : queue_)
        if (q->id == ticket) return 0;
    throw Error(SA_ERR_INVALID, "unknown ticket");
}

bool Session::wait(uint64_t ticket, int64_t timeout_ms, std::unique_ptr<Request>& out) {
    std::unique_lock<std::mutex> lk(mu_);
    auto known = [&]() {
        if (live_.count(ticket)) return true;
        for (auto& q : queue_)
            if (q->id == ticket) return true;
        return false;
    };
    if (!known()) throw Error(SA_ERR_INVALID, "unknown ticket");
    auto done = [&]() {
        auto it = live_.find(ticket);
        return it != live_.end() && it->second->state >= 2;
    };
    if (timeout_ms < 0) cv_done_.wait(lk, [&] { return done() || !known(); });
    else if (!cv_done_.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return done() || !known(); }))
        return false;
    auto it = live_.find(ticket);
    if (it == live_.end()) throw Error(SA_ERR_CANCELLED, "request was cancelled");
    if (it->second->state == 3 && it->second->users > 0) {
        // a failed request: wait for the threads still reading its records
        Request* rq = it->second.get();
        cv_done_.wait(lk, [&] { return rq->users == 0; });
        it = live_.find(ticket);
        if (it == live_.end()) throw Error(SA_ERR_CANCELLED, "request was cancelled");
    }
    if (it->second->state == 3) {
        const std::string msg = it->second->error;
        const int32_t code = it->second->error_code ? it->second->error_code : SA_ERR_INVALID;
        graveyard_.push_back(std::move(it->second));
        live_.erase(it);
        throw Error(code, msg);
    }
    out = std::move(it->second);
    live_.erase(it);
    return true;
}

uint64_t Session::in_flight() const {
    std::lock_guard<std::mutex> g(mu_);
    return inflight_ + queue_.size();
}

// Extension waves, on the session's main stream.
void Session::engine() {
    std::vector<std::pair<Request*, size_t>> batch;
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
        auto idle = [&]() { return running_ == 0 && ready_.empty(); };
        auto wave_ok = [&]() { return !waiting_.empty() && (waiting_jobs_ >= wave_min_jobs_ || idle()); };
        cv_engine_.wait(lk, [&] { return broken_ || (stop_ && inflight_ == 0 && !admitting_) || wave_ok(); });
        if (broken_ || (stop_ && inflight_ == 0 && !admitting_)) break;
        // at most max_wave_jobs_ per wave (at least one chunk), as in Mapper::schedule
        batch.clear();
        size_t k = 0;
        uint64_t taken = 0;
        while (k < waiting_.size()) {
            const uint64_t nj = waiting_[k].first->chunks[waiting_[k].second].pending.size();
            if (!batch.empty() && taken + nj > max_wave_jobs_) break;
            taken += nj;
            batch.push_back(waiting_[k++]);
        }
        waiting_.erase(waiting_.begin(), waiting_.begin() + (ptrdiff_t)k);
        waiting_jobs_ -= taken;
        lk.unlock();
        try {
            const auto tw = std::chrono::steady_clock::now();
            run_wave(batch);
            if (trace_) {
                std::fprintf(stderr, "sa_swave t=%.4f dur=%.4f chunks=%zu\n",
                             std::chrono::duration<double>(tw - t0_).count(),
                             std::chrono::duration<double>(std::chrono::steady_clock::now() - tw).count(),
                             batch.size());
            }
        } catch (const std::exception& e) {
            lk.lock();
            fail_all(e.what(), dynamic_cast<const Error*>(&e) ? static_cast<const Error&>(e).code : SA_ERR_CUDA);
            return;
        }
        lk.lock();
        for (auto& b : batch) ready_.push_back(b);
        batch.clear();
        cv_work_.notify_all();
    }
}

// Admission: reads into the arena and the NAM pipeline, on a second stream so that
// it overlaps the waves of the requests already in flight.
void Session::admitter(AdmitLane& lane) {
    std::unique_lock<std::mutex> lk(mu_);
    std::vector<Request*> group;
    for (;;) {
        auto fits = [&](const Request& q) {
            if (cfg_.max_inflight_requests && inflight_ >= cfg_.max_inflight_requests) return false;
            return seq_alloc_.largest_free() >= std::max<uint64_t>(q.total_bases, 1) &&
                   off_alloc_.largest_free() >= q.n_reads + 1;
        };
        // device memory for the lane's NAM workspace to grow to `bases` (other lanes'
        // admissions in progress count as taken)
        auto growth = [&](uint64_t bases) {
            return bases > lane.ws_bases ? (bases - lane.ws_bases) * NAM_BYTES_PER_BASE : 0;
        };
        auto mem_ok = [&](uint64_t bases) {
            const uint64_t need = growth(bases);
            if (!need) return true;
            size_t f = 0, t = 0;
            if (cudaMemGetInfo(&f, &t) != cudaSuccess) return false;
            return (uint64_t)f >= reserve_ + pending_growth_ + need;
        };
        // free device memory can grow without a notification (another allocation on the
        // device ends), so the wait polls
        cv_admit_.wait_for(lk, std::chrono::milliseconds(20),
                           [&] { return broken_ || stop_ || (!queue_.empty() && fits(*queue_.front())); });
        if (broken_ || stop_) break;
        if (queue_.empty() || !fits(*queue_.front())) continue;
        if (!mem_ok(queue_.front()->total_bases)) {
            // a lane whose workspace already holds the request takes it instead
            bool other = false;
            for (auto& l : lanes_) other = other || l->ws_bases >= queue_.front()->total_bases;
            if (other) {
                cv_admit_.notify_all();
                cv_admit_.wait_for(lk, std::chrono::milliseconds(20));  // releases the lock meanwhile
            } else if (inflight_ == 0 && admitting_ == 0) {
                // nothing in flight will free memory: refuse the request
                std::unique_ptr<Request> rq = std::move(queue_.front());
                queue_.pop_front();
                rq->state = 3;
                rq->error = "admission refused: the request's " + std::to_string(rq->total_bases) +
                            " bases need more device memory than is free beyond the reserve";
                rq->error_code = SA_ERR_BUSY;
                refused_++;
                live_[rq->id] = std::move(rq);
                cv_done_.notify_all();
            } else {
                // memory frees as admissions and requests in flight finish: wait (the
                // lock is released meanwhile; the predicate wait above would return at
                // once and spin with it held)
                cv_admit_.wait_for(lk, std::chrono::milliseconds(20));
            }
            continue;
        }
        // one NAM pipeline for the queued requests at the front, up to a read budget (the
        // fixed cost of a pipeline run is paid once) and to the device memory free for the
        // workspace, all of one kind (single-end, paired-end or mixed)
        group.clear();
        uint64_t group_reads = 0, group_bases = 0;
        const int kind = queue_.front()->kind();
        while (!queue_.empty() && (group.empty() || (queue_.front()->kind() == kind &&
                                                     group_reads + queue_.front()->n_reads <= admit_group_reads_ &&
                                                     fits(*queue_.front()) &&
                                                     mem_ok(group_bases + queue_.front()->total_bases)))) {
            std::unique_ptr<Request> rq = std::move(queue_.front());
            queue_.pop_front();
            Request* r = rq.get();
            seq_alloc_.alloc(std::max<uint64_t>(r->total_bases, 1), r->seq_base);
            off_alloc_.alloc(r->n_reads + 1, r->read_base);
            inflight_++;
            r->state = 1;
            r->t_admit = std::chrono::steady_clock::now();
            live_[r->id] = std::move(rq);
            group.push_back(r);
            group_reads += r->n_reads;
            group_bases += r->total_bases;
        }
        const uint64_t grow = growth(group_bases);
        pending_growth_ += grow;
        lane.ws_bases = std::max(lane.ws_bases, group_bases);
        admitting_++;
        for (Request* r : group) r->users++;
        auto release_group = [&]() {  // with mu_ held
            pending_growth_ -= grow;  // allocated by now (or failed)
            for (Request* r : group)
                if (--r->users == 0 && r->state == 3) cv_done_.notify_all();
        };
        lk.unlock();
        try {
            const auto ta = std::chrono::steady_clock::now();
            admit_group(group, lane);
            if (trace_)
                std::fprintf(stderr, "sa_admit t=%.4f dur=%.4f id=%llu reads=%llu requests=%zu\n",
                             std::chrono::duration<double>(ta - t0_).count(),
                             std::chrono::duration<double>(std::chrono::steady_clock::now() - ta).count(),
                             (unsigned long long)group[0]->id, (unsigned long long)group_reads, group.size());
        } catch (const std::exception& e) {
            lk.lock();
            admitting_--;
            release_group();
            fail_all(e.what(), dynamic_cast<const Error*>(&e) ? static_cast<const Error&>(e).code : SA_ERR_CUDA);
            return;
        }
        lk.lock();
        admitting_--;
        release_group();
        for (Request* r : group) {
            if (r->chunks.empty()) {
                lk.unlock();
                complete(*r);
                lk.lock();
                continue;
            }
            for (size_t c = 0; c < r->chunks.size(); c++) ready_.emplace_back(r, c);
        }
        cv_work_.notify_all();
        cv_engine_.notify_one();
    }
    cv_engine_.notify_all();
}

// Admission of a group of requests: their reads go to the lane's staging back to back
// and to each request's arena range; one NAM pipeline runs over all of them; the NAMs,
// statistics (and chain anchors) come back once and are split per request, with the
// request's own read indices.
void Session::admit_group(const std::vector<Request*>& group, AdmitLane& lane) {
    const auto ta = std::chrono::steady_clock::now();
    uint64_t n64 = 0, bases = 0;
    for (const Request* r : group) {
        n64 += r->n_reads;
        bases += r->total_bases;
    }
    const uint32_t n = (uint32_t)n64;
    // single-end records (in a single-end or mixed group) extend piecewise on the NAMs' anchors
    const bool nam_anchors = group[0]->kind() != 1 && mp_.mode == SA_MODE_SAM && !mp_.use_ssw;
    if (n > 0) {
        lane.h_seq.reserve(bases + 16);
        lane.h_off.reserve((size_t)n + 1);
        lane.nws.seq.reserve(bases + 16);
        lane.nws.off.reserve((size_t)n + 1);
        uint64_t b0 = 0, i0 = 0;
        for (const Request* r : group) {
            if (!r->seq.size() && r->total_bases) {
                // borrowed batch: the bases from the caller's records, in device read order
                char* dst = (char*)lane.h_seq.p + b0;
                parallel_ranges(r->n_reads, 4, [&](uint64_t a, uint64_t e) {
                    for (uint64_t i = a; i < e; i++)
                        std::memcpy(dst + r->seq_off[i], r->read_views[i].seq, r->read_views[i].len);
                });
            } else {
                std::memcpy(lane.h_seq.p + b0, r->seq.data(), r->total_bases);
            }
            for (uint64_t i = 0; i < r->n_reads; i++) lane.h_off.p[i0 + i] = b0 + r->seq_off[i];
            b0 += r->total_bases;
            i0 += r->n_reads;
        }
        lane.h_off.p[n] = bases;
        SA_CUDA(cudaMemcpyAsync(lane.nws.seq.p, lane.h_seq.p, bases, cudaMemcpyHostToDevice, lane.st));
        SA_CUDA(cudaMemcpyAsync(lane.nws.off.p, lane.h_off.p, ((size_t)n + 1) * 8, cudaMemcpyHostToDevice, lane.st));
        // each request's bases and global offsets into its arena range
        b0 = 0;
        for (const Request* r : group) {
            if (r->n_reads == 0) continue;
            SA_CUDA(cudaMemcpyAsync(arena_seq_.p + r->seq_base, lane.nws.seq.p + b0, r->total_bases,
                                    cudaMemcpyDeviceToDevice, lane.st));
            lane.h_goff.resize(r->n_reads + 1);
            for (uint64_t i = 0; i <= r->n_reads; i++) lane.h_goff[i] = r->seq_base + r->seq_off[i];
            SA_CUDA(cudaMemcpyAsync(arena_off_.p + r->read_base, lane.h_goff.data(), (r->n_reads + 1) * 8,
                                    cudaMemcpyHostToDevice, lane.st));
            b0 += r->total_bases;
        }
    }
    NamConfig cfg;
    cfg.cp = ChainParams{cp_.max_lookback, cp_.diag_diff_penalty, cp_.gap_length_penalty, cp_.valid_score_threshold,
                         cp_.max_ref_gap, cp_.matches_weight, cp_.max_diagonal_ratio};
    cfg.mcs = mp_.mcs_strategy;
    cfg.rescue_distance = mp_.rescue_distance;
    cfg.nam_anchors = nam_anchors;
    if (trace_) SA_CUDA(cudaStreamSynchronize(lane.st));  // the pipeline's time is its own
    const auto tp1 = std::chrono::steady_clock::now();
    uint64_t tn = 0, ta_total = 0;
    if (n > 0) {
        KernelTimers kt;
        kt.enabled = trace_;
        run_nam_pipeline(idx_->view(), refs_view_, cfg, n, bases, max_contig_len_, (uint32_t)refs_->contigs.size(),
                         lane.nws, lane.st, &kt);
        if (trace_) {
            SA_CUDA(cudaStreamSynchronize(lane.st));
            kt.collect();
            std::fprintf(stderr,
                         "sa_admit_kernels id=%llu seed=%.3f hits=%.3f anchors=%.3f sort=%.3f chain=%.3f other=%.3f\n",
                         (unsigned long long)group[0]->id, kt.ms[KS_SEED], kt.ms[KS_HITS], kt.ms[KS_ANCHORS],
                         kt.ms[KS_SORT], kt.ms[KS_CHAIN], kt.ms[KS_NAMS_OTHER]);
        }
        tn = lane.nws.last_total_nams;
        lane.h_nam_off.reserve((size_t)n + 1);
        lane.h_nams.reserve(tn);
        lane.h_details.reserve(n);
        SA_CUDA(cudaMemcpyAsync(lane.h_nam_off.p, lane.nws.nam_off.p, ((size_t)n + 1) * 8, cudaMemcpyDeviceToHost,
                                lane.st));
        if (tn)
            SA_CUDA(cudaMemcpyAsync(lane.h_nams.p, lane.nws.nams.p, tn * sizeof(NamRec), cudaMemcpyDeviceToHost,
                                    lane.st));
        SA_CUDA(cudaMemcpyAsync(lane.h_details.p, lane.nws.details.p, (size_t)n * sizeof(NamDetailsRec),
                                cudaMemcpyDeviceToHost, lane.st));
        if (nam_anchors) {
            ta_total = lane.nws.last_total_nam_anchors;
            lane.h_anc_off.reserve(tn + 1);
            lane.h_anc.reserve(ta_total + 1);
            SA_CUDA(cudaMemcpyAsync(lane.h_anc_off.p, lane.nws.nam_anc_off.p, (tn + 1) * 8, cudaMemcpyDeviceToHost,
                                    lane.st));
            if (ta_total)
                SA_CUDA(cudaMemcpyAsync(lane.h_anc.p, lane.nws.nam_anc.p, ta_total * 8, cudaMemcpyDeviceToHost,
                                        lane.st));
        }
        SA_CUDA(cudaStreamSynchronize(lane.st));
    }
    const auto tp2 = std::chrono::steady_clock::now();
    // split per request
    uint64_t i0 = 0;
    for (Request* rp : group) {
        Request& r = *rp;
        const uint64_t rn = r.n_reads;
        const uint64_t t0 = rn ? lane.h_nam_off.p[i0] : 0, t1 = rn ? lane.h_nam_off.p[i0 + rn] : 0;
        r.nam_off.resize(rn + 1);
        for (uint64_t i = 0; i <= rn; i++) r.nam_off[i] = rn ? lane.h_nam_off.p[i0 + i] - t0 : 0;
        r.nams.assign(lane.h_nams.p + t0, lane.h_nams.p + t1);
        r.details.assign(lane.h_details.p + i0, lane.h_details.p + i0 + rn);
        r.h2d_bytes += r.total_bases + 2 * (rn + 1) * 8;
        r.d2h_bytes += (rn + 1) * 8 + (t1 - t0) * sizeof(NamRec) + rn * sizeof(NamDetailsRec);
        r.bv.nams = r.nams.data();
        r.bv.nam_off = r.nam_off.data();
        r.bv.details = r.details.data();
        if (nam_anchors && rn) {
            const uint64_t a0 = lane.h_anc_off.p[t0], a1 = lane.h_anc_off.p[t1];
            r.nam_anc_off.resize(t1 - t0 + 1);
            for (uint64_t t = t0; t <= t1; t++) r.nam_anc_off[t - t0] = lane.h_anc_off.p[t] - a0;
            r.nam_anc.assign(lane.h_anc.p + a0, lane.h_anc.p + a1);
            r.d2h_bytes += (t1 - t0 + 1) * 8 + (a1 - a0) * 8;
            r.bv.nam_anc_off = r.nam_anc_off.data();
            r.bv.nam_anc = r.nam_anc.data();
            r.bv.anc_qbits = lane.nws.anchor_qbits;
            r.bv.anc_pbits = lane.nws.anchor_pbits;
        }
        i0 += rn;
        if (rn == 0) continue;
        // chunks (src/main.rs:591-604), with buffers of finished requests' chunks
        for (uint64_t i = 0; i < r.nrec;) {
            uint64_t nt = 0, j = i;
            while (j < r.nrec) {
                const uint32_t f = r.bv.first_read(j);
                nt += r.bv.reads[f].len + (r.bv.rec_paired(j) ? r.bv.reads[f + 1].len : 0);
                j++;
                if (nt > mp_.chunk_size) break;
            }
            ChunkState cs;
            cs.first = cs.next = i;
            cs.end = j;
            {
                std::lock_guard<std::mutex> g(chunk_pool_mu_);
                if (!chunk_pool_.empty()) {
                    chunk_pool_.back().lend(cs);
                    chunk_pool_.pop_back();
                }
            }
            cs.keep_buffers = true;
            r.chunks.push_back(std::move(cs));
            i = j;
        }
        r.seeded.assign(r.chunks.size(), 0);
        r.store.reset(rn);
    }
    if (trace_) {
        auto d = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
            return std::chrono::duration<double>(b - a).count();
        };
        std::fprintf(stderr, "sa_admit_parts id=%llu upload=%.4f pipeline=%.4f rest=%.4f\n",
                     (unsigned long long)group[0]->id, d(ta, tp1), d(tp1, tp2),
                     d(tp2, std::chrono::steady_clock::now()));
    }
}

void Session::run_wave(std::vector<std::pair<Request*, size_t>>& batch) {
    std::sort(batch.begin(), batch.end(), [](const std::pair<Request*, size_t>& a, const std::pair<Request*, size_t>& b) {
        return a.first->id != b.first->id ? a.first->id < b.first->id : a.second < b.second;
    });
    size_t nj = 0;
    uint32_t max_qlen = 1;
    for (auto& b : batch) {
        nj += b.first->chunks[b.second].pending.size();
        max_qlen = std::max(max_qlen, b.first->max_qlen);
    }
    if (!nj) return;
    // jobs in pinned staging with batch-global read indices; chunks keep theirs local
    h_jobs_.reserve(nj);
    size_t o = 0;
    Request* last = nullptr;
    uint32_t max_anchors = 0;
    uint64_t n_anc = 0;
    for (auto& b : batch) {
        Request* r = b.first;
        ChunkState& cs = r->chunks[b.second];
        cs.wave_first = o;
        const size_t o0 = o;
        for (const ExtJob& j : cs.pending) h_jobs_.p[o++] = j;
        // anchors are looked up with the request's own read indices
        if (r->bv.nam_anc) n_anc += piecewise_anchor_offsets(r->bv, h_jobs_.p + o0, o - o0, n_anc, max_anchors);
        r->h2d_bytes += cs.pending.size() * sizeof(ExtJob);
        if (r != last) {
            r->waves++;
            last = r;
        }
    }
    wave_anchors_.resize(2 * n_anc);
    if (n_anc)
        parallel_ranges(batch.size(), 8, [&](uint64_t a, uint64_t b) {
            for (uint64_t k = a; k < b; k++) {
                const Request* r = batch[k].first;
                const ChunkState& cs = r->chunks[batch[k].second];
                if (r->bv.nam_anc)
                    piecewise_anchor_fill(r->bv, h_jobs_.p + cs.wave_first, cs.pending.size(), wave_anchors_.data());
            }
        });
    for (auto& b : batch) {
        const ChunkState& cs = b.first->chunks[b.second];
        const uint32_t base = (uint32_t)b.first->read_base;
        for (size_t x = 0; x < cs.pending.size(); x++) h_jobs_.p[cs.wave_first + x].read += base;
    }
    ews_.jobs.reserve(nj);
    SA_CUDA(cudaMemcpyAsync(ews_.jobs.p, h_jobs_.p, nj * sizeof(ExtJob), cudaMemcpyHostToDevice, st_));
    if (wave_anchors_.size()) {
        ews_.anchors.reserve(wave_anchors_.size());
        SA_CUDA(cudaMemcpyAsync(ews_.anchors.p, wave_anchors_.data(), wave_anchors_.size() * 4,
                                cudaMemcpyHostToDevice, st_));
    }
    AlignScores sc{mp_.match, mp_.mismatch, mp_.gap_open, mp_.gap_extend, mp_.end_bonus};
    // the pooled buffers (with their capacity) take the copy back
    std::shared_ptr<WaveResults> w = wave_pool_.take();
    std::swap(w->results, ews_.h_results);
    std::swap(w->cigar, ews_.h_cigar);
    run_extension_raw(refs_view_, arena_seq_.p, arena_off_.p, nullptr, nullptr, idx_->sp.k, sc, (uint32_t)nj, ews_,
                      max_qlen, st_, nullptr, wave_anchors_.size() ? ews_.anchors.p : nullptr, max_anchors);
    std::swap(w->results, ews_.h_results);
    std::swap(w->cigar, ews_.h_cigar);
    for (auto& b : batch) b.first->chunks[b.second].wave = w;
}

void Session::worker() {
    // one policy per thread, bound to each chunk's request in turn (its buffers are
    // reused across records and requests)
    BatchView none;
    ResultStore none_store;
    Policy policy(pcfg_, contigs_, none, none_store);
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
        cv_work_.wait(lk, [&] { return workers_stop_ || !ready_.empty(); });
        if (ready_.empty()) return;
        auto item = ready_.front();
        ready_.pop_front();
        Request* r = item.first;
        if (r->state == 3) continue;
        ChunkState& cs = r->chunks[item.second];
        const bool first = !r->seeded[item.second];
        r->seeded[item.second] = 1;
        running_++;
        r->users++;
        lk.unlock();
        std::string err;
        try {
            policy.bind(r->bv, r->store);
            if (first) policy.seed_requests(cs);
            else policy.run_chunk(cs);
        } catch (const std::exception& e) {
            err = e.what();
        }
        lk.lock();
        running_--;
        if (--r->users == 0 && r->state == 3) cv_done_.notify_all();
        if (r->state == 3) continue;  // failed meanwhile
        if (!err.empty()) {
            fail_all("internal: " + err, SA_ERR_INVALID);
            cv_engine_.notify_all();
            continue;
        }
        bool finished = false;
        if (!first && cs.done) {
            finished = ++r->n_done == r->chunks.size();
        } else if (cs.pending.empty()) {
            if (!first) {
                fail_all("internal: chunk stalled without a pending request", SA_ERR_INVALID);
                cv_engine_.notify_all();
                continue;
            }
            ready_.push_back(item);
            cv_work_.notify_one();
        } else {
            waiting_.push_back(item);
            waiting_jobs_ += cs.pending.size();
        }
        cv_engine_.notify_one();
        if (finished) {
            lk.unlock();
            complete(*r);
            lk.lock();
        }
    }
}

void Session::complete(Request& r) {
    size_t total = 0;
    for (auto& c : r.chunks) {
        total += c.out_bytes;
        r.mapped += c.mapped;
        r.d2h_bytes += c.result_bytes;
    }
    r.out = alloc_output(total + 1);
    if (r.out) {
        gather_chunk_outputs(r.chunks, r.out, total >= (64u << 20) ? 4 : 1);
        r.out[total] = 0;
        r.out_len = total;
    } else {
        r.error = "output allocation failed";
        r.error_code = SA_ERR_OOM;
    }
    if (mp_.mode == SA_MODE_ABUNDANCE) {
        r.abundance.assign(contigs_.size(), 0.0);
        for (auto& c : r.chunks)
            for (auto& a : c.abundance) r.abundance[a.first] += a.second;
    }
    // release what the finished request no longer needs; its chunk buffers go to the pool
    {
        std::lock_guard<std::mutex> g(chunk_pool_mu_);
        for (auto& c : r.chunks) {
            if (chunk_pool_.size() >= 384) break;  // bounds the pooled memory (a few MB per chunk)
            chunk_pool_.emplace_back();
            chunk_pool_.back().reclaim(c);
        }
    }
    r.chunks.clear();
    r.chunks.shrink_to_fit();
    r.store = ResultStore();
    r.nams = std::vector<NamRec>();
    r.nam_off = std::vector<uint64_t>();
    r.nam_anc = std::vector<uint64_t>();
    r.nam_anc_off = std::vector<uint64_t>();
    r.details = std::vector<NamDetailsRec>();
    {
        std::lock_guard<std::mutex> g(mu_);
        seq_alloc_.release(r.seq_base, std::max<uint64_t>(r.total_bases, 1));
        off_alloc_.release(r.read_base, r.n_reads + 1);
        inflight_--;
        r.state = 2;
        r.t_done = std::chrono::steady_clock::now();
    }
    cv_done_.notify_all();
    cv_engine_.notify_one();
    cv_admit_.notify_one();
}

// called with mu_ held
void Session::fail_all(const std::string& msg, int32_t code) {
    broken_ = true;
    broken_msg_ = msg;
    for (auto& kv : live_) {
        Request& r = *kv.second;
        if (r.state < 2) {
            r.state = 3;
            r.error = msg;
            r.error_code = code;
        }
    }
    for (auto& q : queue_) {
        q->state = 3;
        q->error = msg;
        q->error_code = code;
        live_[q->id] = std::move(q);
    }
    queue_.clear();
    ready_.clear();
    waiting_.clear();
    waiting_jobs_ = 0;
    inflight_ = 0;
    cv_done_.notify_all();
    cv_work_.notify_all();
    cv_engine_.notify_all();
    cv_admit_.notify_all();
}

}  // namespace sa
