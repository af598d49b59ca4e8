// Oracle (test infrastructure only): index lookups, hits, anchors, collinear
// chaining and NAM sorting.  Restates src/index.rs:127-338, src/partition.rs,
// src/hit.rs, src/chainer.rs, src/nam.rs, src/shuffle.rs; fastrand 2.3.0 restated.
#include "oracle.hpp"

#include <algorithm>
#include <cmath>

namespace oracle {

thread_local std::vector<uint64_t>* g_sectors = nullptr;

// src/partition.rs:27-88: a lower bound on a monotone predicate
template <class P>
static size_t partition_point(const RefRandstrobe* s, size_t n, P pred) {
    size_t lo = 0, hi = n;
    while (lo < hi) {
        size_t mid = lo + (hi - lo) / 2;
        touch(s + mid);
        if (pred(s[mid])) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// src/index.rs:159-197
size_t Index::get_masked_from(uint64_t hash, uint64_t mask, size_t start_position, bool has_start) const {
    uint64_t masked = hash & mask;
    size_t top_n = (size_t)(hash >> (64 - bits));
    if (!has_start) touch(&bucket_starts[top_n]);
    touch(&bucket_starts[top_n + 1]);
    size_t ps = has_start ? start_position : (size_t)bucket_starts[top_n];
    size_t pe = (size_t)bucket_starts[top_n + 1];
    if (ps >= pe) return SIZE_MAX;
    size_t len = pe - ps;
    const RefRandstrobe* b = randstrobes.data() + ps;
    if (len < 4) {
        for (size_t i = 0; i < len; i++) {
            touch(b + i);
            uint64_t h = b[i].hash() & mask;
            if (h == masked) return ps + i;
            if (h > masked) return SIZE_MAX;
        }
        return SIZE_MAX;
    }
    size_t pos = partition_point(b, len, [&](const RefRandstrobe& r) { return (r.hash() & mask) < masked; });
    if (pos < len) touch(b + pos);
    if (pos < len && (b[pos].hash() & mask) == masked) return ps + pos;
    return SIZE_MAX;
}

// src/index.rs:272-295
size_t Index::get_count(size_t position, uint64_t mask) const {
    touch(&randstrobes[position]);
    uint64_t key = randstrobes[position].hash();
    uint64_t masked = key & mask;
    size_t top_n = (size_t)(key >> (64 - bits));
    touch(&bucket_starts[top_n + 1]);
    size_t pe = (size_t)bucket_starts[top_n + 1];
    if (pe - position < 8) {
        size_t count = 1;
        for (size_t p = position + 1; p < pe; p++) {
            touch(&randstrobes[p]);
            if ((randstrobes[p].hash() & mask) == masked) count++;
            else break;
        }
        return count;
    }
    return partition_point(randstrobes.data() + position, pe - position,
                           [&](const RefRandstrobe& r) { return (r.hash() & mask) <= masked; });
}

// src/index.rs:254-263
size_t Index::get_count_full(size_t pos, uint64_t hash_revcomp) const {
    size_t rc = get_full_forward(hash_revcomp);
    size_t reverse_count = rc == SIZE_MAX ? 0 : get_count_full_forward(rc);
    return reverse_count + get_count_full_forward(pos);
}

// src/index.rs:298-307 (the guard uses the index's own filter_cutoff)
bool Index::is_too_frequent_forward(size_t pos, size_t cutoff) const {
    if (pos + filter_cutoff < randstrobes.size()) {
        touch(&randstrobes[pos]);
        touch(&randstrobes[pos + cutoff]);
        return randstrobes[pos].hash() == randstrobes[pos + cutoff].hash();
    }
    return false;
}

// src/index.rs:309-323
bool Index::is_too_frequent(size_t pos, size_t cutoff, uint64_t hash_revcomp) const {
    if (is_too_frequent_forward(pos, cutoff)) return true;
    size_t rc = get_full_forward(hash_revcomp);
    if (rc != SIZE_MAX) {
        if (is_too_frequent_forward(rc, cutoff)) return true;
        size_t count = get_count_full_forward(pos) + get_count_full_forward(rc);
        return count > cutoff;
    }
    return false;
}

// src/index.rs:325-337
bool Index::is_too_frequent_partial(size_t pos, size_t cutoff) const {
    if (pos + cutoff < randstrobes.size()) {
        touch(&randstrobes[pos]);
        touch(&randstrobes[pos + cutoff]);
    }
    if (pos + cutoff < randstrobes.size())
        return (randstrobes[pos].hash() & params.main_hash_mask) ==
               (randstrobes[pos + cutoff].hash() & params.main_hash_mask);
    return false;
}

void HitsDetails::add(const HitsDetails& o) {
    full_not_found += o.full_not_found;
    full_filtered += o.full_filtered;
    full_found += o.full_found;
    partial_not_found += o.partial_not_found;
    partial_filtered += o.partial_filtered;
    partial_found += o.partial_found;
    rescued += o.rescued;
}

void NamDetails::add(const NamDetails& o) {
    hits.add(o.hits);
    n_reads += o.n_reads;
    n_randstrobes += o.n_randstrobes;
    n_anchors += o.n_anchors;
    n_nams += o.n_nams;
}

void Details::add(const Details& o) {
    nam.add(o.nam);
    inconsistent_nams += o.inconsistent_nams;
    mate_rescue += o.mate_rescue;
    tried_alignment += o.tried_alignment;
    gapped += o.gapped;
    best_alignments += o.best_alignments;
}

// src/hit.rs:88-125
static size_t rescue_least_frequent(const Index& idx, std::vector<Hit>& hits, size_t start, size_t end,
                                    size_t to_rescue, size_t threshold) {
    std::vector<std::pair<size_t, size_t>> hc;
    for (size_t i = start; i < end; i++) {
        size_t cnt = hits[i].is_partial ? idx.get_count_partial(hits[i].position)
                                        : idx.get_count_full(hits[i].position, hits[i].hash_revcomp);
        if (cnt <= threshold) hc.emplace_back(i, cnt);
    }
    std::stable_sort(hc.begin(), hc.end(), [](auto& a, auto& b) { return a.second < b.second; });
    size_t rescued = 0;
    for (size_t t = 0; t < hc.size() && t < to_rescue; t++) {
        rescued += hits[hc[t].first].is_filtered ? 1 : 0;
        hits[hc[t].first].is_filtered = false;
    }
    return rescued;
}

// src/hit.rs:129-225
static void find_all_hits(const std::vector<QueryRandstrobe>& qr, const Index& idx, size_t cutoff, Mcs mcs,
                          HitsDetails& d, std::vector<Hit>& hits) {
    auto partial = [&](const QueryRandstrobe& r) {
        size_t e = idx.get_partial(r.hash);
        if (e != SIZE_MAX) {
            bool f = idx.is_too_frequent_partial(e, cutoff);
            if (f) d.partial_filtered++;
            else d.partial_found++;
            hits.push_back(Hit{r.start, r.start + idx.params.k, e, r.hash, r.hash_revcomp, true, f});
        } else {
            d.partial_not_found++;
        }
    };
    if (mcs != Mcs::FirstStrobe) {
        for (auto& r : qr) {
            size_t e = idx.get_full_forward(r.hash);
            if (e != SIZE_MAX) {
                bool f = idx.is_too_frequent(e, cutoff, r.hash_revcomp);
                if (f) d.full_filtered++;
                else d.full_found++;
                hits.push_back(Hit{r.start, r.end, e, r.hash, r.hash_revcomp, false, f});
            } else {
                d.full_not_found++;
                if (mcs == Mcs::Always) partial(r);
            }
        }
    }
    if (mcs == Mcs::FirstStrobe || (mcs == Mcs::Rescue && d.full_filtered + d.full_found == 0)) {
        for (auto& r : qr) partial(r);
    }
}

// src/hit.rs:232-268
static size_t rescue_all_least_frequent(const Index& idx, std::vector<Hit>& hits, size_t rescue_distance) {
    size_t last_unfiltered_start = 0, first_filtered = 0;
    struct Iv { size_t s, e, n; };
    std::vector<Iv> iv;
    for (size_t i = 0; i < hits.size(); i++) {
        const Hit& h = hits[i];
        if (h.is_filtered) continue;
        if (h.query_start > last_unfiltered_start + rescue_distance)
            iv.push_back(Iv{first_filtered, i, (h.query_start - last_unfiltered_start) / rescue_distance});
        last_unfiltered_start = h.query_start;
        first_filtered = i + 1;
    }
    if (!hits.empty()) {
        size_t diff = hits.back().query_start - last_unfiltered_start;  // wraps like release-mode usize
        if (diff > rescue_distance) iv.push_back(Iv{first_filtered, hits.size(), diff / rescue_distance});
    }
    size_t rescued = 0;
    for (auto& v : iv) rescued += rescue_least_frequent(idx, hits, v.s, v.e, v.n, 10000);
    return rescued;
}

// src/hit.rs:270-333
void find_hits(const std::vector<QueryRandstrobe>& qr, const Index& idx, Mcs mcs, size_t filter_cutoff,
               size_t rescue_distance, HitsDetails& d, std::vector<Hit>& hits) {
    d = HitsDetails();
    hits.clear();
    find_all_hits(qr, idx, filter_cutoff, mcs, d, hits);
    size_t total = d.total_hits(), nonrep = d.total_found();
    float frac = total > 0 ? (float)nonrep / (float)total : 1.0f;
    if (rescue_distance > 0) {
        if (frac < 0.7f && nonrep < 5) d.rescued += rescue_least_frequent(idx, hits, 0, hits.size(), 5, 1000);
        d.rescued += rescue_all_least_frequent(idx, hits, rescue_distance);
    }
}

// src/chainer.rs:286-302
float chaining_score(size_t dq, size_t dr, size_t k, const ChainingParameters& cp) {
    size_t dd = dr > dq ? dr - dq : dq - dr;
    size_t dg = std::min(dq, dr);
    float score = (float)std::min(k, dg);
    dg = dg > k ? dg - k : 0;
    float lin = cp.diag_diff_penalty * (float)dd + cp.gap_length_penalty * (float)dg;
    float lg = dd >= 1 ? std::log2((float)dd + 1.0f) : 0.0f;
    score -= lin + 0.5f * lg;
    return score;
}

// src/chainer.rs:304-384
std::vector<Anchor> hits_to_anchors(const std::vector<Hit>& hits, const Index& idx) {
    std::vector<Anchor> a;
    const size_t k = idx.params.k;
    for (const Hit& h : hits) {
        if (h.is_filtered) continue;
        if (h.is_partial) {
            size_t e = idx.get_partial_forward_from(h.hash, h.position);
            if (e == SIZE_MAX) continue;
            uint64_t fh = idx.randstrobes[e].hash_offset & idx.params.forward_main_hash_mask;
            for (size_t i = e; i < idx.randstrobes.size(); i++) {
                const RefRandstrobe& r = idx.randstrobes[i];
                touch(&r);
                if ((r.hash_offset & idx.params.forward_main_hash_mask) != fh) break;
                a.push_back(Anchor{r.ref_index, r.position, h.query_start});
            }
        } else {
            size_t min_length_diff = SIZE_MAX;
            uint64_t fh = idx.randstrobes[h.position].hash();
            for (size_t i = h.position; i < idx.randstrobes.size(); i++) {
                const RefRandstrobe& r = idx.randstrobes[i];
                touch(&r);
                if (r.hash() != fh) break;
                size_t ref_start = r.position;
                size_t ref_end = ref_start + r.offset() + k;
                size_t ql = h.query_end - h.query_start, rl = ref_end - ref_start;
                size_t ld = ql > rl ? ql - rl : rl - ql;
                if (ld <= min_length_diff) {
                    a.push_back(Anchor{r.ref_index, ref_start, h.query_start});
                    a.push_back(Anchor{r.ref_index, ref_end - k, h.query_end - k});
                    min_length_diff = ld;
                }
            }
        }
    }
    return a;
}

// src/chainer.rs:85-180 (collinear_chaining): dp[i] the best chain score ending at
// anchor i, pred[i] its predecessor; returns the best score (best_index its anchor).
float collinear_chaining(const std::vector<Anchor>& anchors, size_t k, size_t max_ref_gap,
                         const ChainingParameters& cp, std::vector<float>& dp, std::vector<size_t>& pred,
                         size_t& best_index) {
    size_t n = anchors.size();
    dp.assign(n, (float)k);
    pred.assign(n, SIZE_MAX);
    float best_score = 0.0f;
    best_index = SIZE_MAX;
    for (size_t i = 0; i < n; i++) {
        size_t lookup_end = i > cp.max_lookback ? i - cp.max_lookback : 0;
        const Anchor& ai = anchors[i];
        for (size_t j = i; j-- > lookup_end;) {
            const Anchor& aj = anchors[j];
            if (ai.ref_id != aj.ref_id) break;
            if (ai.query_start < aj.query_start) continue;
            size_t dq = ai.query_start - aj.query_start;
            size_t dr = ai.ref_start - aj.ref_start;
            if (dr >= max_ref_gap) break;
            float ratio = (float)std::max(dq, dr) / (float)std::min(dq, dr);
            if (ratio > cp.max_diagonal_ratio) continue;
            float sc = chaining_score(dq, dr, k, cp);
            float ns = dp[j] + sc;
            if (ns >= dp[i]) {
                dp[i] = ns;
                pred[i] = j;
                if (dq == dr) break;
            }
        }
        if (best_index != SIZE_MAX && ai.ref_id == anchors[best_index].ref_id) {
            const Anchor& aj = anchors[best_index];
            if (ai.query_start > aj.query_start) {
                size_t dq = ai.query_start - aj.query_start;
                size_t dr = ai.ref_start - aj.ref_start;
                float ratio = (float)std::max(dq, dr) / (float)std::min(dq, dr);
                if (dr < max_ref_gap && dr > 0 && ratio <= cp.max_diagonal_ratio) {
                    float ns = dp[best_index] + chaining_score(dq, dr, k, cp);
                    if (ns > dp[i]) {
                        dp[i] = ns;
                        pred[i] = best_index;
                    }
                }
            }
        }
        if (dp[i] > best_score) {
            best_score = dp[i];
            best_index = i;
        }
    }
    return best_score;
}

// src/chainer.rs:386-449 (extract_chains) after collinear_chaining
static void chain_and_extract(std::vector<Anchor>& anchors, size_t read_len, size_t k, const ChainingParameters& cp,
                              bool is_revcomp, std::vector<Nam>& chains) {
    size_t n = anchors.size();
    if (n == 0) return;
    size_t max_ref_gap = cp.has_max_ref_gap ? cp.max_ref_gap : read_len;
    std::vector<float> dp;
    std::vector<size_t> pred;
    size_t best_index;
    float best_score = collinear_chaining(anchors, k, max_ref_gap, cp, dp, pred, best_index);
    (void)best_index;
    float valid = best_score * cp.valid_score_threshold;
    std::vector<std::pair<size_t, float>> cand;
    for (size_t i = 0; i < n; i++)
        if (dp[i] >= valid) cand.emplace_back(i, dp[i]);
    std::stable_sort(cand.begin(), cand.end(), [](auto& a, auto& b) { return a.second > b.second; });
    std::vector<bool> used(n, false);
    for (auto& c : cand) {
        size_t i = c.first;
        if (used[i]) continue;
        size_t j = i;
        bool overlaps = false;
        std::vector<Anchor> ca{anchors[i]};
        size_t matching = k, cov = anchors[i].ref_start;
        while (pred[j] != SIZE_MAX) {
            j = pred[j];
            if (used[j]) {
                overlaps = true;
                break;
            }
            ca.push_back(anchors[j]);
            used[j] = true;
            size_t d = cov > anchors[j].ref_start ? cov - anchors[j].ref_start : 0;
            matching += std::min(d, k);
            cov = anchors[j].ref_start;
        }
        if (overlaps) continue;
        const Anchor& first = anchors[j];
        const Anchor& last = anchors[i];
        Nam nam;
        nam.nam_id = chains.size();
        nam.query_start = first.query_start;
        nam.query_end = last.query_start + k;
        nam.ref_start = first.ref_start;
        nam.ref_end = last.ref_start + k;
        nam.matching_bases = matching;
        nam.ref_id = last.ref_id;
        float w = (float)ca.size() * cp.matches_weight;
        nam.score = c.second + w;
        nam.is_revcomp = is_revcomp;
        nam.anchors = std::move(ca);
        chains.push_back(std::move(nam));
    }
}

// src/nam.rs:138-166 + src/chainer.rs:182-267
std::vector<Nam> get_nams_by_chaining(const std::string& seq, const Index& idx, const ChainingParameters& cp,
                                      size_t rescue_distance, Mcs mcs, NamDetails& det) {
    std::vector<QueryRandstrobe> qr[2];
    randstrobes_query(seq, idx.params, qr);
    std::vector<Hit> hits[2];
    HitsDetails hd[2];
    for (int o = 0; o < 2; o++) find_hits(qr[o], idx, mcs, idx.filter_cutoff, rescue_distance, hd[o], hits[o]);
    int orientations[2], no = 0;
    if (hd[0].is_better_than(hd[1])) orientations[no++] = 0;
    else if (hd[1].is_better_than(hd[0])) orientations[no++] = 1;
    else {
        orientations[no++] = 0;
        orientations[no++] = 1;
    }
    std::vector<Nam> chains;
    size_t n_anchors = 0;
    for (int t = 0; t < no; t++) {
        int o = orientations[t];
        std::vector<Anchor> a = hits_to_anchors(hits[o], idx);
        n_anchors += a.size();
        std::sort(a.begin(), a.end());
        a.erase(std::unique(a.begin(), a.end()), a.end());
        chain_and_extract(a, seq.size(), idx.params.k, cp, o == 1, chains);
    }
    det = NamDetails();
    det.hits = hd[0];
    det.hits.add(hd[1]);
    det.n_reads = 1;
    det.n_randstrobes = qr[0].size() + qr[1].size();
    det.n_anchors = n_anchors;
    det.n_nams = chains.size();
    det.both_orientations = no > 1;
    return chains;
}

// fastrand 2.3.0: wyrand generator and Lemire's bounded integers (restated from
// the published algorithm; parity unpinned by the reference tests)
uint64_t Rng::gen_u64() {
    uint64_t s = state + 0x2d358dccaa6c78a5ULL;
    state = s;
    unsigned __int128 t = (unsigned __int128)s * (unsigned __int128)(s ^ 0x8bb84b93962eacc9ULL);
    return (uint64_t)t ^ (uint64_t)(t >> 64);
}

uint32_t Rng::gen_mod_u32(uint32_t n) {
    uint32_t r = (uint32_t)gen_u64();
    uint64_t m = (uint64_t)r * n;
    uint32_t hi = (uint32_t)(m >> 32), lo = (uint32_t)m;
    if (lo < n) {
        uint32_t t = (0u - n) % n;
        while (lo < t) {
            r = (uint32_t)gen_u64();
            m = (uint64_t)r * n;
            hi = (uint32_t)(m >> 32);
            lo = (uint32_t)m;
        }
    }
    return hi;
}

uint64_t Rng::gen_mod_u64(uint64_t n) {
    uint64_t r = gen_u64();
    unsigned __int128 m = (unsigned __int128)r * n;
    uint64_t hi = (uint64_t)(m >> 64), lo = (uint64_t)m;
    if (lo < n) {
        uint64_t t = (0ULL - n) % n;
        while (lo < t) {
            r = gen_u64();
            m = (unsigned __int128)r * n;
            hi = (uint64_t)(m >> 64);
            lo = (uint64_t)m;
        }
    }
    return hi;
}

// src/nam.rs:168-188 + src/shuffle.rs:7-25
void sort_nams(std::vector<Nam>& nams, Rng& rng) {
    std::stable_sort(nams.begin(), nams.end(), [](const Nam& a, const Nam& b) { return a.score > b.score; });
    if (nams.empty()) return;
    float best = nams[0].score;
    size_t n_best = 0;
    while (n_best < nams.size() && nams[n_best].score == best) n_best++;
    if (n_best > 1) rng.shuffle(nams.data(), n_best);
}

}  // namespace oracle
