// Batch driver: Mapper::map_chunk (src/main.rs:873-988) for a whole batch on one
// GPU.  NAMs for every read come from one pass of the device pipeline; the
// sequential per-chunk policy then consumes extension results produced in waves:
// the first requests of a chunk extend each read's best NAMs speculatively, and
// later ones are exactly the jobs the chunk stopped on (plus their likely
// successors).  Waves are batched continuously across chunks (Mapper::schedule).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <exception>
#include <mutex>
#include <thread>

#include "host_input.h"
#include "host_util.h"
#include "mapper.h"

namespace sa {

Mapper::Mapper(const sa_index* idx, const sa_refs* refs, const sa_chaining_params& cp, const sa_mapping_params& mp)
    : idx_(idx), refs_(refs), cp_(cp), mp_(mp) {
    if (mp.rg_id) rg_id_ = mp.rg_id;
    if (cudaDeviceGetLimit(&l2_fetch_default_, cudaLimitMaxL2FetchGranularity) != cudaSuccess) {
        l2_fetch_default_ = 0;
        cudaGetLastError();
    }
    // SA_TRACE_WAVES=1: one line per extension wave on stderr
    const char* tr = std::getenv("SA_TRACE_WAVES");
    trace_ = tr && *tr && *tr != '0';
    // SA_MAX_WAVE_JOBS: extension jobs per wave at most (tuning)
    if (const char* mw = std::getenv("SA_MAX_WAVE_JOBS")) set_max_wave_jobs(std::strtoull(mw, nullptr, 10));
    // SA_WAVE_MIN_JOBS: jobs that start a wave while policy threads are still busy (tuning)
    if (const char* mj = std::getenv("SA_WAVE_MIN_JOBS")) set_wave_min_jobs(std::max<uint64_t>(1, std::strtoull(mj, nullptr, 10)));
    // SA_PARTS: NAM-pipeline parts a large batch is cut into (tuning)
    if (const char* np = std::getenv("SA_PARTS")) set_parts((uint32_t)std::strtoul(np, nullptr, 10));
    SA_CUDA(cudaSetDevice(idx->device));
    SA_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
    int prio_least = 0, prio_greatest = 0;
    SA_CUDA(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
    SA_CUDA(cudaStreamCreateWithPriority(&stn_, cudaStreamNonBlocking, prio_greatest));
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
    d_words_.reserve(nw);
    d_woff_.reserve(nc);
    d_clen_.reserve(nc);
    SA_CUDA(cudaMemcpy(d_words_.p, hw.data(), nw * 8, cudaMemcpyHostToDevice));
    SA_CUDA(cudaMemcpy(d_woff_.p, woff.data(), nc * 8, cudaMemcpyHostToDevice));
    SA_CUDA(cudaMemcpy(d_clen_.p, clen.data(), nc * 4, cudaMemcpyHostToDevice));
    refs_view_ = DevRefs{d_words_.p, d_woff_.p, d_clen_.p, nc};
    abundances_.assign(nc, 0.0);
    pcfg_.mp = mp_;
    pcfg_.rg_id = rg_id_;
    pcfg_.has_rg = mp.rg_id != nullptr;
    pcfg_.k = idx->sp.k;
    pcfg_.timing = trace_;
    if (!mp_.use_ssw && mp_.mode == SA_MODE_SAM) {
        // single-end extension without --ssw is piecewise on the NAM's anchors; paired-end
        // extension always uses SSW (src/mapper.rs:860-870)
        single_end_piecewise_ = true;
    }
}

Mapper::~Mapper() {
    // the fetch granularity is the context's: give back the value found at construction
    if (l2_fetch_ && l2_fetch_default_) cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, l2_fetch_default_);
    if (st_) cudaStreamDestroy(st_);
    if (stn_) cudaStreamDestroy(stn_);
}

void Mapper::upload_reads(const ReadSpan& reads) {
    uint64_t total = 0;
    for (size_t i = 0; i < reads.size(); i++) {
        if (reads[i].len > MAX_READ_LEN)
            throw Error(SA_ERR_INVALID, "read longer than " + std::to_string(MAX_READ_LEN) + " nt");
        total += reads[i].len;
    }
    const uint32_t n = (uint32_t)reads.size();
    h_seq_.reserve(total + 16);
    h_off_.reserve((size_t)n + 1);
    uint64_t o = 0;
    for (uint32_t i = 0; i < n; i++) {
        h_off_.p[i] = o;
        o += reads[i].len;
    }
    h_off_.p[n] = o;
    // the bases into pinned staging, in parallel
    parallel_ranges(n, policy_threads_, [&](uint64_t a, uint64_t b) {
        for (uint64_t i = a; i < b; i++) std::memcpy(h_seq_.p + h_off_.p[i], reads[i].seq, reads[i].len);
    });
    nws_.seq.reserve(total + 16);
    nws_.off.reserve((size_t)n + 1);
    SA_CUDA(cudaMemcpyAsync(nws_.seq.p, h_seq_.p, total, cudaMemcpyHostToDevice, st_));
    SA_CUDA(cudaMemcpyAsync(nws_.off.p, h_off_.p, ((size_t)n + 1) * 8, cudaMemcpyHostToDevice, st_));
    total_bases_ = total;
    n_reads_ = n;
    h2d_bytes_ += total + ((size_t)n + 1) * 8;
}

// The NAM pipeline for one part, on stn_: the part's bases are copied out of the
// uploaded batch with local offsets, and its NAMs, statistics (and for single-end
// piecewise extension the NAMs' chain anchors) come back into the part's pinned buffers.
void Mapper::part_nams(Part& p, uint32_t& launches) {
    const auto t0 = std::chrono::steady_clock::now();
    const uint32_t n = p.read_hi - p.read_lo;
    const uint64_t base = h_off_.p[p.read_lo], total = h_off_.p[p.read_hi] - base;
    NamConfig cfg;
    cfg.cp = ChainParams{cp_.max_lookback, cp_.diag_diff_penalty, cp_.gap_length_penalty, cp_.valid_score_threshold,
                         cp_.max_ref_gap, cp_.matches_weight, cp_.max_diagonal_ratio};
    cfg.mcs = mp_.mcs_strategy;
    cfg.rescue_distance = mp_.rescue_distance;
    cfg.nam_anchors = single_end_piecewise_ && (!bv_.paired || bv_.rec_read);
    cfg.chain_lane_max = chain_lane_max_;
    pws_.seq.reserve(total + 16);
    pws_.off.reserve((size_t)n + 1);
    h_poff_.reserve((size_t)n + 1);
    for (uint32_t i = 0; i <= n; i++) h_poff_.p[i] = h_off_.p[p.read_lo + i] - base;
    if (total) SA_CUDA(cudaMemcpyAsync(pws_.seq.p, nws_.seq.p + base, total, cudaMemcpyDeviceToDevice, stn_));
    SA_CUDA(cudaMemcpyAsync(pws_.off.p, h_poff_.p, ((size_t)n + 1) * 8, cudaMemcpyHostToDevice, stn_));
    launches += run_nam_pipeline(idx_->view(), refs_view_, cfg, n, total, max_contig_len_,
                                 (uint32_t)refs_->contigs.size(), pws_, stn_, &kt_nam_);
    const uint64_t tn = pws_.last_total_nams;
    p.n_nams = tn;
    uint64_t d2h = 0;
    if (cfg.nam_anchors) {
        const uint64_t ta = pws_.last_total_nam_anchors;
        p.anc_off.reserve(tn + 1);
        p.anc.reserve(ta);
        SA_CUDA(cudaMemcpyAsync(p.anc_off.p, pws_.nam_anc_off.p, (tn + 1) * 8, cudaMemcpyDeviceToHost, stn_));
        if (ta) SA_CUDA(cudaMemcpyAsync(p.anc.p, pws_.nam_anc.p, ta * 8, cudaMemcpyDeviceToHost, stn_));
        d2h += (tn + 1) * 8 + ta * 8;
    }
    p.nam_off.reserve((size_t)n + 1);
    p.nams.reserve(tn);
    p.details.reserve(n);
    SA_CUDA(cudaMemcpyAsync(p.nam_off.p, pws_.nam_off.p, ((size_t)n + 1) * 8, cudaMemcpyDeviceToHost, stn_));
    if (tn) SA_CUDA(cudaMemcpyAsync(p.nams.p, pws_.nams.p, tn * sizeof(NamRec), cudaMemcpyDeviceToHost, stn_));
    SA_CUDA(cudaMemcpyAsync(p.details.p, pws_.details.p, (size_t)n * sizeof(NamDetailsRec), cudaMemcpyDeviceToHost,
                            stn_));
    SA_CUDA(cudaStreamSynchronize(stn_));
    d2h += ((size_t)n + 1) * 8 + tn * sizeof(NamRec) + (size_t)n * sizeof(NamDetailsRec);
    p.bv.nams = p.nams.p;
    p.bv.nam_off = p.nam_off.p;
    p.bv.details = p.details.p;
    p.bv.nam_anc_off = cfg.nam_anchors ? p.anc_off.p : nullptr;
    p.bv.nam_anc = cfg.nam_anchors ? p.anc.p : nullptr;
    p.bv.anc_qbits = pws_.anchor_qbits;
    p.bv.anc_pbits = pws_.anchor_pbits;
    p.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    d2h_bytes_ += d2h;  // atomic: the wave thread adds its transfers meanwhile
    h2d_bytes_ += ((size_t)n + 1) * 8;
    if (trace_)
        std::fprintf(stderr, "sa_nams part t=%.4f reads=%u nams=%llu seconds=%.4f\n",
                     std::chrono::duration<double>(t0 - t_map0_).count(), n, (unsigned long long)tn, p.seconds);
}

std::shared_ptr<const WaveResults> Mapper::run_wave(const ExtJob* jobs, uint32_t nj, uint32_t max_qlen,
                                                    uint32_t& launches, const uint32_t* anchors,
                                                    size_t anchor_words, uint32_t max_anchors) {
    std::shared_ptr<WaveResults> w = wave_pool_.take();
    w->results.clear();
    w->cigar.clear();
    if (!nj) return w;
    // the pooled buffers (with their capacity) take the copy back
    std::swap(w->results, ews_.h_results);
    std::swap(w->cigar, ews_.h_cigar);
    ews_.jobs.reserve(nj);
    SA_CUDA(cudaMemcpyAsync(ews_.jobs.p, jobs, (size_t)nj * sizeof(ExtJob), cudaMemcpyHostToDevice, st_));
    h2d_bytes_ += (size_t)nj * sizeof(ExtJob);
    if (anchor_words) {
        ews_.anchors.reserve(anchor_words);
        SA_CUDA(cudaMemcpyAsync(ews_.anchors.p, anchors, anchor_words * 4, cudaMemcpyHostToDevice, st_));
        h2d_bytes_ += anchor_words * 4;
    }
    AlignScores sc{mp_.match, mp_.mismatch, mp_.gap_open, mp_.gap_extend, mp_.end_bonus};
    launches += run_extension(refs_view_, nws_, idx_->sp.k, sc, nj, ews_, max_qlen, st_, &kt_,
                              anchor_words ? ews_.anchors.p : nullptr, max_anchors);
    d2h_bytes_ += (size_t)nj * sizeof(ExtResult) + ews_.total_cigar * 4;
    for (int c = 0; c < 7; c++) sw_cells_[c] += ews_.cells[c];
    std::swap(w->results, ews_.h_results);
    std::swap(w->cigar, ews_.h_cigar);
    jobs_run_ += nj;
    return w;
}

namespace {
ReadView read_view(const sa_read_batch* b, uint64_t i) {
    ReadView v;
    v.seq = b->seq + b->seq_offsets[i];
    v.len = (uint32_t)(b->seq_offsets[i + 1] - b->seq_offsets[i]);
    v.qual = b->qual ? b->qual + b->seq_offsets[i] : nullptr;
    v.name = b->names + b->name_offsets[i];
    v.name_len = (uint32_t)(b->name_offsets[i + 1] - b->name_offsets[i]);
    v.comment = nullptr;
    v.comment_len = 0;
    if (b->comments && b->comment_offsets && b->comment_offsets[i + 1] > b->comment_offsets[i]) {
        v.comment = b->comments + b->comment_offsets[i];
        v.comment_len = (uint32_t)(b->comment_offsets[i + 1] - b->comment_offsets[i]);
    }
    return v;
}
}  // namespace

void Mapper::upload(const sa_read_batch* r1, const sa_read_batch* r2) {
    auto t0 = std::chrono::steady_clock::now();
    const bool paired = r2 != nullptr;
    if (paired && r2->n != r1->n) throw Error(SA_ERR_INVALID, "r1 and r2 batches differ in size");
    const uint64_t nrec = r1->n;
    bv_ = BatchView();
    bv_.paired = paired;
    rec_read_.clear();
    reads_.resize(paired ? 2 * nrec : nrec);
    auto view = read_view;
    parallel_ranges(nrec, policy_threads_, [&](uint64_t a, uint64_t b) {
        for (uint64_t i = a; i < b; i++) {
            if (paired) {
                reads_[2 * i] = view(r1, i);
                reads_[2 * i + 1] = view(r2, i);
            } else {
                reads_[i] = view(r1, i);
            }
        }
    });
    max_qlen_ = 1;
    bv_.reads = ReadSpan{reads_.data(), reads_.size()};
    for (auto& r : reads_) max_qlen_ = std::max(max_qlen_, r.len);
    h2d_bytes_ = 0;
    upload_reads(bv_.reads);
    SA_CUDA(cudaStreamSynchronize(st_));
    have_batch_ = true;
    stats_.seconds_upload = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void Mapper::upload_interleaved(const sa_read_batch* reads) {
    auto t0 = std::chrono::steady_clock::now();
    const uint64_t n = reads->n;
    if (n >= UINT32_MAX) throw Error(SA_ERR_INVALID, "batch too large");
    bv_ = BatchView();
    reads_.resize(n);
    parallel_ranges(n, policy_threads_, [&](uint64_t a, uint64_t b) {
        for (uint64_t i = a; i < b; i++) reads_[i] = read_view(reads, i);
    });
    pair_records_by_name(*reads, true, rec_read_);
    bv_.rec_read = rec_read_.data();
    max_qlen_ = 1;
    bv_.reads = ReadSpan{reads_.data(), reads_.size()};
    for (auto& r : reads_) max_qlen_ = std::max(max_qlen_, r.len);
    h2d_bytes_ = 0;
    upload_reads(bv_.reads);
    SA_CUDA(cudaStreamSynchronize(st_));
    have_batch_ = true;
    stats_.seconds_upload = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void Mapper::map_interleaved(const sa_read_batch* reads, sa_output* out) {
    auto t0 = std::chrono::steady_clock::now();
    upload_interleaved(reads);
    uint64_t h2d = h2d_bytes_;
    double tu = stats_.seconds_upload;
    map_uploaded(out);
    stats_.seconds_upload = tu;
    stats_.h2d_bytes += h2d;
    stats_.seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void Mapper::map(const sa_read_batch* r1, const sa_read_batch* r2, sa_output* out) {
    auto t0 = std::chrono::steady_clock::now();
    upload(r1, r2);
    uint64_t h2d = h2d_bytes_;
    double tu = stats_.seconds_upload;
    map_uploaded(out);
    stats_.seconds_upload = tu;
    stats_.h2d_bytes += h2d;
    stats_.seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// Continuous batching of extension work.  Chunks are independent (fresh RNG and
// insert-size state, src/main.rs:878-880), so policy threads run whichever chunks
// have their results, while this thread gathers the requests of the chunks that
// stopped on a miss into the next extension wave.  A wave starts once enough jobs
// are waiting, or as soon as no policy thread could add more.  Which jobs share a
// wave depends on timing; results do not (each job is a pure function of its
// inputs, and the output of every chunk depends only on the results it reads).
uint32_t Mapper::schedule(std::vector<ChunkState>& chunks, uint32_t& launches, uint32_t& nam_launches) {
    const size_t nchunks = chunks.size();
    const unsigned nthreads = std::max(1u, std::min<unsigned>(policy_threads_, (unsigned)nchunks));
    std::mutex mu;
    std::condition_variable cv_work, cv_ext;
    std::deque<size_t> ready;       // chunks that can run
    std::vector<size_t> waiting;    // chunks whose requests are not yet in a wave
    size_t waiting_jobs = 0, n_done = 0;
    unsigned running = 0;
    std::exception_ptr err;
    bool stop = false;
    std::vector<bool> is_seeded(nchunks, false);
    bool nam_done = false;  // every part's NAMs are in (the plain form waits for it)

    // NAM pipelines part by part; a part's chunks become ready once its NAMs are in
    std::thread nam_thread([&]() {
        try {
            for (size_t pi = 0; pi < n_parts_; pi++) {
                {
                    std::lock_guard<std::mutex> g(mu);
                    if (stop) return;
                }
                Part& p = *parts_[pi];
                part_nams(p, nam_launches);
                if (!overlap_) continue;  // the plain form starts the policy after the last part
                std::lock_guard<std::mutex> g(mu);
                for (size_t c = p.chunk_lo; c < p.chunk_hi; c++) ready.push_back(c);
                cv_work.notify_all();
                cv_ext.notify_one();
            }
            std::lock_guard<std::mutex> g(mu);
            if (!overlap_)
                for (size_t c = 0; c < nchunks; c++) ready.push_back(c);
            nam_done = true;
            cv_work.notify_all();
            cv_ext.notify_one();
        } catch (...) {
            std::lock_guard<std::mutex> g(mu);
            if (!err) err = std::current_exception();
            stop = true;
            cv_work.notify_all();
            cv_ext.notify_all();
        }
    });

    auto worker = [&]() {
        // one policy per thread, bound to each chunk's part in turn
        Policy policy(pcfg_, contigs_, parts_[0]->bv, parts_[0]->store);
        std::unique_lock<std::mutex> lk(mu);
        auto copy_ready = [&] { return so_.dst && !so_.overflow && so_.next_claim < so_.done_prefix; };
        for (;;) {
            cv_work.wait(lk, [&] { return stop || !ready.empty() || copy_ready(); });
            if (stop) return;
            if (ready.empty()) {
                // nothing to map: copy the next finished chunk's output into place
                const size_t cc = so_.next_claim++;
                char* d = so_.dst + so_.off[cc];
                lk.unlock();
                copy_chunk_output(chunks[cc], d);
                lk.lock();
                continue;
            }
            const size_t c = ready.front();
            ready.pop_front();
            running++;
            const bool first = !is_seeded[c];
            is_seeded[c] = true;
            lk.unlock();
            ChunkState& cs = chunks[c];
            try {
                policy.bind(parts_[cs.part]->bv, parts_[cs.part]->store);
                if (first)
                    policy.seed_requests(cs);
                else
                    policy.run_chunk(cs);
            } catch (...) {
                lk.lock();
                if (!err) err = std::current_exception();
                stop = true;
                running--;
                cv_work.notify_all();
                cv_ext.notify_all();
                return;
            }
            lk.lock();
            running--;
            if (!first && cs.done) {
                n_done++;
                if (so_.dst) {
                    so_.done[c] = 1;
                    while (so_.done_prefix < nchunks && so_.done[so_.done_prefix]) {
                        const size_t d = so_.done_prefix;
                        so_.off[d + 1] = so_.off[d] + chunks[d].out_bytes;
                        if (so_.off[d + 1] > so_.cap) so_.overflow = true;
                        so_.done_prefix++;
                    }
                    if (copy_ready()) cv_work.notify_one();
                }
            } else if (cs.pending.empty()) {
                // nothing requested: a seeded chunk runs at once; a stalled one is a bug
                if (!first) {
                    if (!err)
                        err = std::make_exception_ptr(
                            Error(SA_ERR_INVALID, "internal: chunk stalled without a pending request"));
                    stop = true;
                    cv_work.notify_all();
                } else {
                    ready.push_back(c);
                    cv_work.notify_one();
                }
            } else {
                waiting.push_back(c);
                waiting_jobs += cs.pending.size();
            }
            cv_ext.notify_one();
        }
    };
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nthreads; t++) th.emplace_back(worker);

    uint32_t waves = 0;
    std::vector<size_t> batch, held;
    const auto t_sched0 = t_map0_;
    try {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            // start a wave when the policy threads cannot add more, or enough has queued
            cv_ext.wait(lk, [&] {
                if (stop || n_done == nchunks) return true;
                if (waiting.empty()) return false;
                const bool idle = running == 0 && ready.empty();
                if (!overlap_) return idle && nam_done;
                return idle || waiting_jobs >= wave_min_jobs_;
            });
            if (stop || n_done == nchunks) break;
            // at most max_wave_jobs_ per wave (at least one chunk): the policy threads
            // resume the chunks of one wave while the next runs on the device
            batch.clear();
            size_t k = 0, taken = 0;
            while (k < waiting.size() &&
                   (batch.empty() || taken + chunks[waiting[k]].pending.size() <= max_wave_jobs_)) {
                taken += chunks[waiting[k]].pending.size();
                batch.push_back(waiting[k++]);
            }
            waiting.erase(waiting.begin(), waiting.begin() + (ptrdiff_t)k);
            waiting_jobs -= taken;
            lk.unlock();
            // chunk order inside a wave keeps waves reproducible for a given grouping
            std::sort(batch.begin(), batch.end());
            size_t nj = 0;
            for (size_t c : batch) nj += chunks[c].pending.size();
            h_jobs_.reserve(std::max<size_t>(nj, 1));
            nj = 0;
            uint32_t max_anchors = 0;
            uint64_t n_anc = 0;
            for (size_t c : batch) {
                const Part& p = *parts_[chunks[c].part];
                const size_t j0 = nj, cnt = chunks[c].pending.size();
                chunks[c].wave_first = nj;
                std::memcpy(h_jobs_.p + nj, chunks[c].pending.data(), cnt * sizeof(ExtJob));
                nj += cnt;
                // anchors are looked up with the part's read indices
                if (p.bv.nam_anc) n_anc += piecewise_anchor_offsets(p.bv, h_jobs_.p + j0, cnt, n_anc, max_anchors);
            }
            wave_anchors_.resize(2 * n_anc);
            if (n_anc)
                parallel_ranges(batch.size(), policy_threads_, [&](uint64_t a, uint64_t b) {
                    for (uint64_t k = a; k < b; k++) {
                        const ChunkState& cs = chunks[batch[k]];
                        const Part& p = *parts_[cs.part];
                        if (p.bv.nam_anc)
                            piecewise_anchor_fill(p.bv, h_jobs_.p + cs.wave_first, cs.pending.size(),
                                                  wave_anchors_.data());
                    }
                });
            // the device reads of the whole batch are indexed from the part's first read
            for (size_t c : batch) {
                const uint32_t lo = parts_[chunks[c].part]->read_lo;
                ExtJob* j = h_jobs_.p + chunks[c].wave_first;
                for (size_t x = 0; x < chunks[c].pending.size(); x++) j[x].read += lo;
            }
            if (waves > 1000000) throw Error(SA_ERR_INVALID, "internal: extension waves do not converge");
            auto tw = std::chrono::steady_clock::now();
            auto wres = run_wave(h_jobs_.p, (uint32_t)nj, max_qlen_, launches, wave_anchors_.data(),
                                 wave_anchors_.size(), max_anchors);
            for (size_t c : batch) chunks[c].wave = wres;
            const auto tw2 = std::chrono::steady_clock::now();
            t_ext_ += std::chrono::duration<double>(tw2 - tw).count();
            if (trace_) {
                uint64_t kinds[4] = {0, 0, 0, 0};
                for (size_t j = 0; j < nj; j++) kinds[h_jobs_.p[j].kind & 3]++;
                std::fprintf(stderr,
                             "sa_wave %u t=%.4f dur=%.4f chunks=%zu jobs=%zu fast=%llu full=%llu rescue=%llu align=%llu\n",
                             waves, std::chrono::duration<double>(tw - t_sched0).count(),
                             std::chrono::duration<double>(tw2 - tw).count(), batch.size(), nj,
                             (unsigned long long)kinds[0], (unsigned long long)kinds[1],
                             (unsigned long long)kinds[2], (unsigned long long)kinds[3]);
            }
            waves++;
            lk.lock();
            if (!overlap_) {
                // plain form: the chunks resume together once every waiting request has run
                held.insert(held.end(), batch.begin(), batch.end());
                if (!waiting.empty()) continue;
                batch.swap(held);
                held.clear();
            }
            for (size_t c : batch) ready.push_back(c);
            cv_work.notify_all();
        }
        stop = true;
        cv_work.notify_all();
    } catch (...) {
        std::lock_guard<std::mutex> g(mu);
        if (!err) err = std::current_exception();
        stop = true;
        cv_work.notify_all();
    }
    for (auto& t : th) t.join();
    nam_thread.join();
    if (err) std::rethrow_exception(err);
    return waves;
}

void Mapper::map_uploaded(sa_output* out) {
    if (!have_batch_) throw Error(SA_ERR_INVALID, "no uploaded batch");
    auto t0 = std::chrono::steady_clock::now();
    t_map0_ = t0;
    BatchView& bv = bv_;
    const bool paired = bv.paired;
    const bool mixed = bv.rec_read != nullptr;
    const uint64_t nrec = mixed ? rec_read_.size() - 1 : paired ? bv.reads.size() / 2 : bv.reads.size();
    // record j's first read (for j = nrec: the read count)
    auto first_read = [&](uint64_t j) -> uint64_t { return mixed ? rec_read_[j] : paired ? 2 * j : j; };
    uint32_t launches = 0;
    h2d_bytes_ = 0;
    d2h_bytes_ = 0;
    jobs_run_ = 0;
    t_ext_ = 0;
    kt_.reset();
    kt_nam_.reset();
    for (int c = 0; c < 7; c++) sw_cells_[c] = 0;
    // chunks (src/main.rs:591-604), cut on the uploaded read offsets (record j's bases
    // are off[first_read(j + 1)] - off[first_read(j)])
    std::vector<ChunkState> chunks;
    chunks.reserve(total_bases_ / (mp_.chunk_size + 1) + 2);
    const uint64_t* off = h_off_.p;
    for (uint64_t i = 0; i < nrec;) {
        uint64_t j = i;
        const uint64_t base = off[first_read(i)];
        while (j < nrec) {
            j++;
            if (off[first_read(j)] - base > mp_.chunk_size) break;
        }
        ChunkState cs;
        cs.first = cs.next = i;
        cs.end = j;
        // buffers of an earlier batch's chunk: their memory is paged in already
        const size_t c = chunks.size();
        if (c < chunk_pool_.size()) chunk_pool_[c].lend(cs);
        cs.keep_buffers = true;
        chunks.push_back(std::move(cs));
        i = j;
    }
    // parts: runs of whole chunks (at least 4 chunks each), so that chunk semantics and
    // output order are those of the whole batch; read and record indices inside a part
    // are local to it
    const size_t nchunks = chunks.size();
    // at least parts_target_ parts, and enough that a part holds at most
    // MAX_PART_BASES bases (the NAM workspace takes about 100 bytes per base)
    const size_t by_bases = (size_t)((total_bases_ + MAX_PART_BASES - 1) / MAX_PART_BASES);
    n_parts_ = std::max<size_t>(1, std::min<size_t>(std::max<size_t>(parts_target_, by_bases), nchunks / 4));
    while (parts_.size() < n_parts_) parts_.push_back(std::make_unique<Part>());
    // the first part is half the size of the others, so that the policy threads and the
    // first extension wave start sooner
    const size_t first = n_parts_ > 1 ? std::max<size_t>(1, nchunks / (2 * n_parts_ - 1)) : nchunks;
    for (size_t pi = 0, c0 = 0; pi < n_parts_; pi++) {
        const size_t c1 = pi + 1 == n_parts_ ? nchunks
                          : pi == 0       ? first
                                          : first + (nchunks - first) * pi / (n_parts_ - 1);
        Part& p = *parts_[pi];
        p.chunk_lo = c0;
        p.chunk_hi = c1;
        p.rec_lo = c0 < nchunks ? chunks[c0].first : nrec;
        p.rec_hi = c1 > 0 && c1 <= nchunks ? chunks[c1 - 1].end : p.rec_lo;
        p.read_lo = (uint32_t)first_read(p.rec_lo);
        p.read_hi = (uint32_t)first_read(p.rec_hi);
        p.bv = BatchView();
        p.bv.paired = paired;
        if (mixed) {
            p.bv.rec_read = rec_read_.data() + p.rec_lo;
            p.bv.rec_read_base = p.read_lo;
        }
        p.bv.reads = ReadSpan{reads_.data() + p.read_lo, (size_t)(p.read_hi - p.read_lo)};
        p.store.reset(p.read_hi - p.read_lo);
        p.n_nams = 0;
        for (size_t c = c0; c < c1; c++) {
            chunks[c].part = (uint32_t)pi;
            chunks[c].first -= p.rec_lo;
            chunks[c].next -= p.rec_lo;
            chunks[c].end -= p.rec_lo;
        }
        c0 = c1;
    }
    // output buffer sized from the previous batch (large batches only)
    so_ = StreamOut();
    const size_t est = (size_t)(bytes_per_record_ * 1.15 * (double)nrec) + ((size_t)1 << 20);
    if (overlap_ && bytes_per_record_ > 0 && est >= OutputPool::LARGE) {
        so_.cap = (est + OutputPool::LARGE - 1) / OutputPool::LARGE * OutputPool::LARGE;
        so_.dst = alloc_output(so_.cap + 1);
        so_.off.assign(chunks.size() + 1, 0);
        so_.done.assign(chunks.size(), 0);
    }
    uint32_t nam_launches = 0;
    const auto t_sched = std::chrono::steady_clock::now();
    uint32_t waves = 0;
    try {
        waves = schedule(chunks, launches, nam_launches);
    } catch (...) {
        if (so_.dst) release_output(so_.dst);
        so_ = StreamOut();
        throw;
    }
    const auto t_sched_end = std::chrono::steady_clock::now();
    launches += nam_launches;
    double t_nams = 0;
    for (size_t pi = 0; pi < n_parts_; pi++) t_nams += parts_[pi]->seconds;
    if (trace_) {
        double sr = 0, ss = 0, sd = 0, sf = 0;
        uint64_t er = 0, es = 0, runs = 0, eu = 0, mm = 0, mk = 0, sr2 = 0, si = 0;
        for (auto& c : chunks) {
            sr2 += c.stale_rng;
            si += c.stale_isd;
            eu += c.evals_reused;
            mm += c.miss_mispredicted;
            mk += c.miss_unknown;
            sf += c.seconds_format;
            sr += c.seconds_real;
            ss += c.seconds_spec;
            sd += c.seconds_seed;
            er += c.evals_real;
            es += c.evals_spec;
            runs += c.runs;
        }
        std::fprintf(stderr, "sa_policy chunks=%zu runs=%llu cpu_real=%.3f cpu_spec=%.3f cpu_seed=%.3f cpu_format=%.3f "
                             "evals_real=%llu evals_spec=%llu reused=%llu miss_mispredicted=%llu miss_unknown=%llu "
                             "stale_rng=%llu stale_isd=%llu\n",
                     chunks.size(), (unsigned long long)runs, sr, ss, sd, sf, (unsigned long long)er,
                     (unsigned long long)es, (unsigned long long)eu, (unsigned long long)mm, (unsigned long long)mk,
                     (unsigned long long)sr2, (unsigned long long)si);
    }
    for (auto& c : chunks)
        for (auto& a : c.abundance) abundances_[a.first] += a.second;
    size_t total_len = 0;
    uint64_t mapped = 0;
    for (auto& c : chunks) {
        total_len += c.out_bytes;
        mapped += c.mapped;
    }
    if (so_.dst && !so_.overflow && total_len <= so_.cap) {
        // the chunks copied while mapping are in place; gather the rest behind them
        out->data = so_.dst;
        const size_t c0 = so_.next_claim;
        gather_chunk_outputs(chunks, so_.dst + so_.off[c0], policy_threads_, c0);
    } else {
        if (so_.dst) release_output(so_.dst);
        out->data = alloc_output(total_len + 1);
        if (!out->data) throw Error(SA_ERR_OOM, "output allocation failed");
        gather_chunk_outputs(chunks, out->data, policy_threads_);
    }
    so_ = StreamOut();
    if (nrec) bytes_per_record_ = (double)total_len / (double)nrec;
    // keep the chunks' buffers (emptied) for the next batch
    if (chunk_pool_.size() < chunks.size()) chunk_pool_.resize(chunks.size());
    for (size_t c = 0; c < chunks.size(); c++) chunk_pool_[c].reclaim(chunks[c]);
    if (trace_) {
        auto d = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
            return std::chrono::duration<double>(b - a).count();
        };
        std::fprintf(stderr, "sa_map setup=%.4f schedule=%.4f output=%.4f bytes=%zu\n", d(t0, t_sched),
                     d(t_sched, t_sched_end), d(t_sched_end, std::chrono::steady_clock::now()), total_len);
    }
    out->data[total_len] = 0;
    out->len = total_len;
    out->n_reads = bv.reads.size();
    out->n_mapped = mapped;
    out->n_waves = waves;
    out->n_gpu_launches = launches;
    last_launches_ = launches;
    last_waves_ = waves;
    auto t2 = std::chrono::steady_clock::now();
    last_seconds_ = std::chrono::duration<double>(t2 - t0).count();
    // the parts' NAM pipelines overlap the waves and the policy; the policy's share is
    // what neither the waves nor the first part's pipeline cover
    stats_.seconds_nams = t_nams;
    stats_.seconds_extension = t_ext_;
    stats_.seconds_policy = std::max(0.0, last_seconds_ - t_ext_ - parts_[0]->seconds);
    stats_.seconds_total = last_seconds_;
    stats_.n_jobs = jobs_run_;
    stats_.n_waves = waves;
    stats_.n_launches = launches;
    stats_.h2d_bytes = h2d_bytes_;
    stats_.d2h_bytes = d2h_bytes_;
    {
        uint64_t rs = 0, an = 0, nn = 0;
        for (size_t pi = 0; pi < n_parts_; pi++) {
            const Part& p = *parts_[pi];
            nn += p.n_nams;
            for (uint32_t i = 0; i < p.read_hi - p.read_lo; i++) {
                rs += p.details.p[i].n_randstrobes;
                an += p.details.p[i].n_anchors;
            }
        }
        stats_.n_nams = nn;
        stats_.n_anchors = an;
        stats_.n_anchor_total = an;
        stats_.n_randstrobes = rs;
        stats_.n_bases = total_bases_;
    }
    kt_.collect();
    kt_nam_.collect();
    for (int c = 0; c < 5; c++) stats_.sw_cells[c] = sw_cells_[c];
    for (int c = 0; c < 2; c++) stats_.band_cells[c] = sw_cells_[5 + c];
    for (int i = 0; i < 16; i++) {
        stats_.kernel_ms[i] = i < KS_COUNT ? kt_.ms[i] + kt_nam_.ms[i] : 0.0;
        stats_.kernel_launches[i] = i < KS_COUNT ? kt_.launches[i] + kt_nam_.launches[i] : 0;
    }
}

void Mapper::set_tuning(const Tuning& t) {
    set_parts(t.parts);
    set_wave_min_jobs(std::max<uint64_t>(1, t.wave_min_jobs));
    set_max_wave_jobs(t.max_wave_jobs);
    ews_.wave_qmax = std::max<uint32_t>(1, t.wave_qmax);
    chain_lane_max_ = std::max<uint32_t>(1, t.chain_lane_max);
    if (t.l2_fetch != l2_fetch_) {
        const size_t v = t.l2_fetch ? t.l2_fetch : l2_fetch_default_;
        if (v) SA_CUDA(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, v));
        l2_fetch_ = t.l2_fetch;
    }
}

Mapper::Tuning Mapper::tuning() const {
    Tuning t;
    t.parts = parts_target_;
    t.wave_min_jobs = wave_min_jobs_;
    t.max_wave_jobs = max_wave_jobs_;
    t.wave_qmax = ews_.wave_qmax;
    t.chain_lane_max = chain_lane_max_;
    t.l2_fetch = l2_fetch_;
    return t;
}

Mapper::TuneReport Mapper::autotune(const sa_read_batch* r1, const sa_read_batch* r2, uint32_t rounds) {
    const Tuning before = tuning();
    const bool saved_overlap = overlap_;
    try {
        return autotune_run(r1, r2, rounds);
    } catch (...) {
        // a failed tuning leaves the mapper as it found it
        overlap_ = saved_overlap;
        set_tuning(before);
        throw;
    }
}

Mapper::TuneReport Mapper::autotune_run(const sa_read_batch* r1, const sa_read_batch* r2, uint32_t rounds) {
    rounds = std::max<uint32_t>(1, rounds);
    const bool saved_overlap = overlap_;
    overlap_ = true;
    upload(r1, r2);
    std::vector<char> want;
    TuneReport rep;
    // SA_TRACE_TUNE=1: one line per trial on stderr
    const char* tt = std::getenv("SA_TRACE_TUNE");
    const bool trace_tune = tt && *tt && *tt != '0';
    auto run = [&](const Tuning& t) {
        set_tuning(t);
        std::vector<double> secs;
        for (uint32_t r = 0; r < rounds; r++) {
            sa_output o{};
            const auto t0 = std::chrono::steady_clock::now();
            map_uploaded(&o);
            secs.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
            const bool same = want.size() == o.len && (o.len == 0 || std::memcmp(want.data(), o.data, o.len) == 0);
            release_output(o.data);
            if (!same) throw Error(SA_ERR_INVALID, "internal: tuning changed the output bytes");
        }
        rep.trials++;
        std::sort(secs.begin(), secs.end());
        if (trace_tune)
            std::fprintf(stderr, "sa_tune parts=%u wave_min=%llu wave_max=%llu wave_qmax=%u chain_lane=%u l2=%u s=%.4f\n",
                         t.parts, (unsigned long long)t.wave_min_jobs, (unsigned long long)t.max_wave_jobs, t.wave_qmax,
                         t.chain_lane_max, t.l2_fetch, secs[secs.size() / 2]);
        return secs[secs.size() / 2];
    };
    Tuning best;  // the defaults
    set_tuning(best);
    for (int w = 0; w < 2; w++) {
        // two warm-up maps (buffers and pools reach their size), the first one's bytes
        // are what every trial must reproduce
        sa_output o{};
        map_uploaded(&o);
        if (w == 0) want.assign(o.data, o.data + o.len);
        release_output(o.data);
    }
    double best_s = run(best);
    rep.seconds_default = best_s;
    auto knob = [&](auto field, std::initializer_list<uint64_t> values) {
        for (uint64_t v : values) {
            Tuning t = best;
            if ((uint64_t)(t.*field) == v) continue;
            t.*field = (std::remove_reference_t<decltype(t.*field)>)v;
            const double sec = run(t);
            if (sec < 0.98 * best_s) {
                best = t;
                best_s = sec;
            }
        }
    };
    knob(&Tuning::parts, {2, 4, 16});
    knob(&Tuning::max_wave_jobs, {65536, 131072, 524288});
    knob(&Tuning::wave_min_jobs, {8192, 131072});
    if (max_qlen_ > 128) knob(&Tuning::wave_qmax, {128, 160});
    knob(&Tuning::chain_lane_max, {16, 128});
    knob(&Tuning::l2_fetch, {32, 64, 128});
    set_tuning(best);
    overlap_ = saved_overlap;
    rep.chosen = best;
    rep.seconds_tuned = best_s;
    return rep;
}

}  // namespace sa
