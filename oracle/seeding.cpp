// Oracle (test infrastructure only): sequences, hashing and randstrobe seeding.
// Restates src/packed_seq.rs, src/revcomp.rs, src/seeding/{hash,syncmers,strobes,
// parameters,mod}.rs.
#include "oracle.hpp"

#include <algorithm>
#include <atomic>
#include <thread>
#include <deque>
#include <cmath>

namespace oracle {

// src/packed_seq.rs:50-59 (encode_wildcard) and :79-92 (push)
void PackedSeq::push(uint8_t c) {
    uint64_t v;
    switch (c) {
        case 'A': case 'a': v = 0; break;
        case 'C': case 'c': v = 1; break;
        case 'G': case 'g': v = 2; break;
        case 'T': case 't': case 'U': case 'u': v = 3; break;
        default: {
            uint64_t h = (uint64_t)len * 0x9e3779b97f4a7c15ULL;
            v = (h ^ (h >> 30)) & 3;
        }
    }
    size_t bit = (len & 31) * 2;
    if (bit == 0) data.push_back(v);
    else data.back() |= v << bit;
    len++;
}

std::string PackedSeq::decode(size_t start, size_t end) const {
    std::string s;
    s.resize(end > start ? end - start : 0);
    for (size_t i = start; i < end; i++) s[i - start] = decode_at(i);
    return s;
}

// src/revcomp.rs:5-22: ACGTU (any case) complemented, everything else -> 'N'
std::string reverse_complement(const std::string& s) {
    std::string r(s.size(), 'N');
    for (size_t i = 0; i < s.size(); i++) {
        char c = s[s.size() - 1 - i], o;
        switch (c) {
            case 'A': case 'a': o = 'T'; break;
            case 'C': case 'c': o = 'G'; break;
            case 'G': case 'g': o = 'C'; break;
            case 'T': case 't': case 'U': case 'u': o = 'A'; break;
            default: o = 'N';
        }
        r[i] = o;
    }
    return r;
}

static inline uint64_t rotl(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }

// src/seeding/hash.rs:9-27 (single-u64 xxh64)
uint64_t xxh64(uint64_t input) {
    const uint64_t P1 = 0x9E3779B185EBCA87ULL, P2 = 0xC2B2AE3D27D4EB4FULL, P3 = 0x165667B19E3779F9ULL,
                   P4 = 0x85EBCA77C2B2AE63ULL, P5 = 0x27D4EB2F165667C5ULL;
    uint64_t r = P5 + 8;
    r ^= rotl(input * P2, 31) * P1;
    r = rotl(r, 27) * P1 + P4;
    r ^= r >> 33;
    r *= P2;
    r ^= r >> 29;
    r *= P3;
    r ^= r >> 32;
    return r;
}

// src/seeding/parameters.rs:102-159 (READ_LENGTH_SETTINGS) and :181-221 (new)
SeedingParameters SeedingParameters::from_read_length(size_t read_length) {
    struct S { int profile; size_t r_threshold, k, s, w_min, w_max, canonical; };
    static const S table[7] = {
        {1, 70, 18, 14, 1, 4, 50},    {2, 90, 20, 16, 1, 6, 75},     {3, 110, 20, 16, 2, 6, 100},
        {4, 135, 20, 16, 3, 8, 125},  {5, 175, 20, 16, 5, 11, 150},  {6, 375, 22, 18, 6, 16, 250},
        {7, SIZE_MAX, 23, 17, 5, 15, 400},
    };
    const S* sel = &table[6];
    for (const S& e : table)
        if (read_length <= e.r_threshold) { sel = &e; break; }
    // the profile's canonical length selects the row again (always the same row)
    SeedingParameters p;
    p.profile = sel->profile;
    p.k = sel->k;
    p.s = sel->s;
    p.t = (p.k - p.s) / 2 + 1;
    p.w_min = sel->w_min;
    p.w_max = sel->w_max;
    p.q = 255;
    size_t len = sel->canonical;
    size_t md = len > 70 ? len - 70 : 0;
    md = std::max(md, p.k);
    md = std::min<size_t>(md, 255);
    p.max_dist = (uint32_t)md;
    p.main_hash_mask = ~0ULL << (9 + 17);
    p.finish_masks();
    return p;
}

void SeedingParameters::finish_masks() {
    partial_orientation_pos = (uint32_t)__builtin_ctzll(main_hash_mask) - 1;
    forward_main_hash_mask = main_hash_mask | (1ULL << partial_orientation_pos);
}

// src/seeding/syncmers.rs:89-94 (NUCLEOTIDES table): A,C,G,T,U any case; else 4
static inline uint8_t nucleotide(uint8_t c) {
    switch (c) {
        case 'A': case 'a': return 0;
        case 'C': case 'c': return 1;
        case 'G': case 'g': return 2;
        case 'T': case 't': case 'U': case 'u': return 3;
        default: return 4;
    }
}

// src/seeding/syncmers.rs:171-237 (SyncmerIterator::next), generic over the base source
template <class F>
static std::vector<Syncmer> syncmers_generic(size_t n, F base, const SeedingParameters& p) {
    std::vector<Syncmer> out;
    const size_t k = p.k, s = p.s, t = p.t;
    const uint64_t kmask = (k == 32) ? ~0ULL : ((1ULL << (2 * k)) - 1);
    const uint64_t smask = (1ULL << (2 * s)) - 1;
    const int kshift = (int)(k - 1) * 2, sshift = (int)(s - 1) * 2;
    std::deque<uint64_t> qs;
    uint64_t qs_min = UINT64_MAX;
    size_t l = 0;
    uint64_t xk0 = 0, xk1 = 0, xs0 = 0, xs1 = 0;
    for (size_t i = 0; i < n; i++) {
        uint8_t c = base(i);
        if (c < 4) {
            xk0 = ((xk0 << 2) | c) & kmask;
            xk1 = (xk1 >> 2) | ((uint64_t)(3 - c) << kshift);
            xs0 = ((xs0 << 2) | c) & smask;
            xs1 = (xs1 >> 2) | ((uint64_t)(3 - c) << sshift);
            l++;
            if (l < s) continue;
            uint64_t ys = std::min(xs0, xs1);
            uint64_t hs = xxh64(ys);
            qs.push_back(hs);
            if (qs.size() < k - s + 1) continue;
            if (qs.size() == k - s + 1) {
                for (uint64_t v : qs) qs_min = std::min(v, qs_min);
            } else {
                uint64_t front = qs.front();
                qs.pop_front();
                if (front == qs_min) {
                    qs_min = UINT64_MAX;
                    for (uint64_t v : qs) qs_min = std::min(v, qs_min);
                } else if (hs < qs_min) {
                    qs_min = hs;
                }
            }
            if (qs[t - 1] == qs_min) {
                uint64_t yk = std::min(xk0, xk1);
                out.push_back(Syncmer{xxh64(yk), xk0 <= xk1, i + 1 - k});
            }
        } else {
            qs_min = UINT64_MAX;
            l = 0;
            xs0 = xs1 = xk0 = xk1 = 0;
            qs.clear();
        }
    }
    return out;
}

std::vector<Syncmer> syncmers_of_read(const std::string& seq, const SeedingParameters& p) {
    return syncmers_generic(seq.size(), [&](size_t i) { return nucleotide((uint8_t)seq[i]); }, p);
}

std::vector<Syncmer> syncmers_of_ref(const PackedSeq& seq, const SeedingParameters& p) {
    return syncmers_generic(seq.len, [&](size_t i) { return seq.bits(i); }, p);
}

// src/seeding/strobes.rs:112-124 (Randstrobe::hash)
static inline uint64_t randstrobe_hash(uint64_t h1, uint64_t h2, uint64_t f1, uint64_t f2,
                                       const SeedingParameters& p) {
    return ((h1 & p.main_hash_mask) | (h2 & ~p.forward_main_hash_mask) | (f1 << p.partial_orientation_pos) |
            (f2 << 8)) &
           (REF_RANDSTROBE_HASH_MASK << 1);
}

struct Randstrobe {
    uint64_t hash, hash_revcomp;
    size_t strobe1_pos, strobe2_pos;
};

// src/seeding/strobes.rs:145-176 (RandstrobeIterator::next) over a syncmer list
static void randstrobes_from_syncmers(const std::vector<Syncmer>& sy, const SeedingParameters& p,
                                      std::vector<Randstrobe>& out) {
    size_t n = sy.size();
    for (size_t base = 0; base < n; base++) {
        // the deque holds sy[base .. min(base + w_max + 1, n))
        size_t dq_len = std::min(p.w_max + 1, n - base);
        const Syncmer& s1 = sy[base];
        size_t max_position = s1.position + p.max_dist;
        uint64_t min_val = UINT64_MAX;
        const Syncmer* s2 = &sy[base];
        for (size_t i = p.w_min; i < dq_len; i++) {
            const Syncmer& c = sy[base + i];
            if (c.position > max_position) break;
            uint64_t b = (s1.hash ^ c.hash) & p.q;
            uint64_t ones = (uint64_t)__builtin_popcountll(b);
            if (ones < min_val) {
                min_val = ones;
                s2 = &c;
            }
        }
        uint64_t f1 = s1.is_forward, f2 = s2->is_forward;
        out.push_back(Randstrobe{randstrobe_hash(s1.hash, s2->hash, f1, f2, p),
                                 randstrobe_hash(s2->hash, s1.hash, f1 ^ 1, f2 ^ 1, p), s1.position,
                                 s2->position});
    }
}

// src/seeding/mod.rs:19-75
void randstrobes_query(const std::string& seq, const SeedingParameters& p, std::vector<QueryRandstrobe> out[2]) {
    out[0].clear();
    out[1].clear();
    if (seq.size() < p.w_max) return;
    std::vector<Syncmer> sy = syncmers_of_read(seq, p);
    std::vector<Randstrobe> rs;
    randstrobes_from_syncmers(sy, p, rs);
    for (auto& r : rs) out[0].push_back(QueryRandstrobe{r.hash, r.hash_revcomp, r.strobe1_pos, r.strobe2_pos + p.k});
    std::reverse(sy.begin(), sy.end());
    for (auto& s : sy) {
        s.position = seq.size() - s.position - p.k;
        s.is_forward = !s.is_forward;
    }
    rs.clear();
    randstrobes_from_syncmers(sy, p, rs);
    for (auto& r : rs) out[1].push_back(QueryRandstrobe{r.hash, r.hash_revcomp, r.strobe1_pos, r.strobe2_pos + p.k});
}

// ---------------------------------------------------------------- index build
// src/indexer.rs:294-300
uint8_t pick_bits(const std::vector<RefSeq>& refs, const SeedingParameters& p) {
    size_t total = 0;
    for (auto& r : refs) total += r.seq.len;
    size_t est = total / (p.k - p.s + 1) + 1;
    uint32_t lg = (uint32_t)std::log2((double)est);
    lg = std::clamp<uint32_t>(lg, 9, 32);
    return (uint8_t)(lg - 1);
}

// RefRandstrobe order (src/index.rs:15-25: derived Ord over hash_offset, position,
// ref_index).  A total order on distinct records, so any correct sort gives the same
// table.
static inline bool rs_less(const RefRandstrobe& a, const RefRandstrobe& b) {
    if (a.hash_offset != b.hash_offset) return a.hash_offset < b.hash_offset;
    if (a.position != b.position) return a.position < b.position;
    return a.ref_index < b.ref_index;
}

template <class F>
static void parallel_for(size_t n, size_t threads, F f) {
    if (threads <= 1 || n <= 1) {
        for (size_t i = 0; i < n; i++) f(i);
        return;
    }
    std::atomic<size_t> next{0};
    std::vector<std::thread> th;
    for (size_t t = 0; t < std::min(threads, n); t++)
        th.emplace_back([&] {
            for (size_t i; (i = next.fetch_add(1)) < n;) f(i);
        });
    for (auto& t : th) t.join();
}

// The sort of make_index on several threads: records scattered by the top 12 bits
// of hash_offset (the leading key), then every range sorted on its own.
static void sort_randstrobes(std::vector<RefRandstrobe>& rs, size_t threads) {
    if (threads <= 1 || rs.size() < (1u << 20)) {
        std::sort(rs.begin(), rs.end(), rs_less);
        return;
    }
    const int B = 12;
    const size_t NB = (size_t)1 << B, n = rs.size();
    const size_t parts = threads * 4, per = (n + parts - 1) / parts;
    std::vector<std::vector<size_t>> cnt(parts, std::vector<size_t>(NB, 0));
    parallel_for(parts, threads, [&](size_t t) {
        for (size_t i = t * per; i < std::min(n, (t + 1) * per); i++) cnt[t][rs[i].hash_offset >> (64 - B)]++;
    });
    std::vector<size_t> start(NB + 1, 0);
    std::vector<std::vector<size_t>> pos(parts, std::vector<size_t>(NB, 0));
    size_t acc = 0;
    for (size_t b = 0; b < NB; b++) {
        start[b] = acc;
        for (size_t t = 0; t < parts; t++) {
            pos[t][b] = acc;
            acc += cnt[t][b];
        }
    }
    start[NB] = acc;
    std::vector<RefRandstrobe> out(n);
    parallel_for(parts, threads, [&](size_t t) {
        for (size_t i = t * per; i < std::min(n, (t + 1) * per); i++)
            out[pos[t][rs[i].hash_offset >> (64 - B)]++] = rs[i];
    });
    parallel_for(NB, threads, [&](size_t b) { std::sort(out.begin() + start[b], out.begin() + start[b + 1], rs_less); });
    rs.swap(out);
}

// src/indexer.rs:18-170 (make_index) and :222-253 (assign_randstrobes).  Contigs are
// turned into randstrobes on `threads` threads and the records concatenated in
// contig order; the sort is a total order, so the table does not depend on threads.
Index make_index(const std::vector<RefSeq>& refs, const SeedingParameters& p, uint8_t bits, double filter_fraction,
                 size_t threads) {
    Index idx;
    idx.params = p;
    idx.bits = bits;
    std::vector<RefRandstrobe>& rs = idx.randstrobes;
    std::vector<std::vector<RefRandstrobe>> per(refs.size());
    parallel_for(refs.size(), threads, [&](size_t ri) {
        const PackedSeq& seq = refs[ri].seq;
        if (seq.len < p.w_max) return;
        std::vector<Syncmer> sy = syncmers_of_ref(seq, p);
        std::vector<Randstrobe> out;
        randstrobes_from_syncmers(sy, p, out);
        std::vector<Syncmer>().swap(sy);
        per[ri].reserve(out.size());
        for (auto& r : out) {
            uint64_t off = (uint64_t)(uint8_t)(r.strobe2_pos - r.strobe1_pos);
            per[ri].push_back(RefRandstrobe{(r.hash & REF_RANDSTROBE_HASH_MASK) | off, (uint32_t)r.strobe1_pos,
                                            (uint32_t)ri});
        }
    });
    size_t total = 0;
    for (auto& v : per) total += v.size();
    rs.reserve(total);
    for (auto& v : per) {
        rs.insert(rs.end(), v.begin(), v.end());
        std::vector<RefRandstrobe>().swap(v);
    }
    sort_randstrobes(rs, threads);
    std::vector<uint64_t>& starts = idx.bucket_starts;
    starts.reserve(((size_t)1 << bits) + 1);
    std::vector<size_t> counts;
    uint64_t unique = rs.empty() ? 0 : 1;
    uint64_t prev = rs.empty() ? 0 : rs[0].hash();
    size_t count = 1;
    if (!rs.empty()) starts.push_back(0);
    for (size_t pos = 1; pos < rs.size(); pos++) {
        uint64_t cur = rs[pos].hash();
        if (cur == prev) {
            count++;
            continue;
        }
        unique++;
        if (count != 1) counts.push_back(count);
        count = 1;
        uint64_t n = cur >> (64 - bits);
        while (starts.size() <= n) starts.push_back(pos);
        prev = cur;
    }
    if (count != 1) counts.push_back(count);
    while (starts.size() < ((size_t)1 << bits) + 1) starts.push_back(rs.size());
    // counts sorted in descending order (src/indexer.rs:138-155); only the element at
    // index_cutoff (or the last one) is read, so a selection gives the same value
    size_t index_cutoff = (size_t)((double)unique * filter_fraction);
    size_t cutoff;
    if (index_cutoff < counts.size()) {
        std::nth_element(counts.begin(), counts.begin() + index_cutoff, counts.end(), std::greater<size_t>());
        cutoff = counts[index_cutoff];
    } else if (!counts.empty()) {
        cutoff = *std::min_element(counts.begin(), counts.end());
    } else {
        cutoff = 30;
    }
    idx.filter_cutoff = std::clamp<size_t>(cutoff, 30, 100);
    return idx;
}

}  // namespace oracle
