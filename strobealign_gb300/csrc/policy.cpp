// Host-side mapping policy (see policy.h).  Follows src/mapper.rs and
// src/maponly.rs decision by decision; every base-level alignment comes from the
// GPU extension jobs.
#include <chrono>

#include "policy.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace sa {

// ------------------------------------------------------------------ fastrand 2.3.0
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

void InsertSize::update(uint64_t insert_size) {
    if (insert_size >= 2000) return;
    last = insert_size;
    if (sample_size > 0) {
        float x = (float)insert_size;
        float e = x - mu;
        mu += e / (float)sample_size;
        sse += e * (x - mu);
        variance = sample_size > 1 ? sse / ((float)sample_size - 1.0f) : sse;
        sigma = std::sqrt(variance);
    }
    sample_size++;
}

namespace {

constexpr uint16_t PAIRED = 1, PROPER_PAIR = 2, UNMAP = 4, MUNMAP = 8, REVERSE = 0x10, MREVERSE = 0x20, READ1 = 0x40,
                   READ2 = 0x80, SECONDARY = 0x100;

inline uint8_t sat_u8(float f) {
    if (!(f == f) || f <= 0.0f) return 0;
    if (f >= 255.0f) return 255;
    return (uint8_t)f;
}
inline uint64_t sat_usize(float f) {
    if (!(f == f) || f <= 0.0f) return 0;
    if (f >= 1.8446744e19f) return UINT64_MAX;
    return (uint64_t)f;
}
inline uint64_t absdiff(uint64_t a, uint64_t b) { return a > b ? a - b : b - a; }

// src/math.rs:3-7
float normal_pdf(float x, float mu, float sigma) {
    const double INV_SQRT_PI = 0.3989422804014327;
    float a = (x - mu) / sigma;
    return (float)INV_SQRT_PI / sigma * std::exp(-0.5f * a * a);
}

uint32_t projected_ref_start(const NamRec& n) { return n.ref_start > n.query_start ? n.ref_start - n.query_start : 0; }

// ------------------------------------------------------------------ SAM records
struct Sam {
    const ReadView* rv = nullptr;
    uint16_t flags = 0;
    const std::string* rname = nullptr;
    bool has_pos = false;
    uint32_t pos = 0;
    uint8_t mapq = 0;
    const Alignment* aln = nullptr;  // CIGAR source (mapped records)
    const std::string* rnext = nullptr;
    bool has_pnext = false;
    uint32_t pnext = 0;
    bool has_tlen = false;
    int32_t tlen = 0;
    bool seq_rc = false;
    bool has_nm = false;
    uint32_t nm = 0, as = 0;
    const Details* det = nullptr;
    bool is_mapped() const { return (flags & UNMAP) == 0; }
};

const std::string EQUALS = "=";

inline void put_u64(OutBuf& o, uint64_t v) {
    char b[24];
    int n = 0;
    do { b[n++] = (char)('0' + v % 10); v /= 10; } while (v);
    while (n) o.push_back(b[--n]);
}
inline void put_i64(OutBuf& o, int64_t v) {
    if (v < 0) { o.push_back('-'); put_u64(o, (uint64_t)(-v)); }
    else put_u64(o, (uint64_t)v);
}

char comp_char(char c) {
    switch (c) {
        case 'A': case 'a': return 'T';
        case 'C': case 'c': return 'G';
        case 'G': case 'g': return 'C';
        case 'T': case 't': case 'U': case 'u': return 'A';
        default: return 'N';
    }
}

// CIGAR with soft clips, merged like Cigar::push (src/mapper.rs:173-182), in =/X or M form: w_cigar

// Pointer writers for format_sam: the record is written into space reserved for
// its largest possible size, then the string is cut to what was written.
inline char* w_u64(char* p, uint64_t v) {
    char b[24];
    int n = 0;
    do { b[n++] = (char)('0' + v % 10); v /= 10; } while (v);
    while (n) *p++ = b[--n];
    return p;
}
inline char* w_i64(char* p, int64_t v) {
    if (v < 0) {
        *p++ = '-';
        return w_u64(p, (uint64_t)(-v));
    }
    return w_u64(p, (uint64_t)v);
}
inline char* w_str(char* p, const char* s, size_t n) {
    std::memcpy(p, s, n);
    return p + n;
}
inline char* w_lit(char* p, const char* s) { return w_str(p, s, std::strlen(s)); }

struct CompTable {
    char t[256];
    CompTable() {
        for (int i = 0; i < 256; i++) t[i] = comp_char((char)i);
    }
};
const CompTable COMP;

// Reversed copies 16 bytes at a time with GCC vector extensions (portable: TBL on Arm,
// scalar elsewhere).  Reverse complement: the complement of an upper-cased A, C, G, T
// or U is looked up by its low 4 bits; any other byte becomes N, as in comp_char.
typedef unsigned char v16u8 __attribute__((vector_size(16)));
const v16u8 REV16 = {15, 14, 13, 12, 11, 10, 9, 8, 7, 6, 5, 4, 3, 2, 1, 0};

inline char* w_revcomp(char* p, const char* s, uint32_t len) {
    const v16u8 tab = {'N', 'T', 'N', 'G', 'A', 'A', 'N', 'C', 'N', 'N', 'N', 'N', 'N', 'N', 'N', 'N'};
    uint32_t i = len;
    while (i >= 16) {
        v16u8 x;
        std::memcpy(&x, s + i - 16, 16);
        x = __builtin_shuffle(x, REV16);
        const v16u8 up = x & (unsigned char)0xDF;
        const v16u8 ok = (up == 'A') | (up == 'C') | (up == 'G') | (up == 'T') | (up == 'U');
        const v16u8 c = __builtin_shuffle(tab, (v16u8)(x & (unsigned char)15));
        const v16u8 y = (c & ok) | ((unsigned char)'N' & ~ok);
        std::memcpy(p, &y, 16);
        p += 16;
        i -= 16;
    }
    while (i > 0) *p++ = COMP.t[(uint8_t)s[--i]];
    return p;
}

inline char* w_reversed(char* p, const char* s, uint32_t len) {
    uint32_t i = len;
    while (i >= 16) {
        v16u8 x;
        std::memcpy(&x, s + i - 16, 16);
        x = __builtin_shuffle(x, REV16);
        std::memcpy(p, &x, 16);
        p += 16;
        i -= 16;
    }
    while (i > 0) *p++ = s[--i];
    return p;
}

char* w_cigar(char* p, const Alignment& a, bool eqx) {
    static const char ch[] = "MIDNSHP=X";
    uint32_t pend_op = 99, pend_len = 0;
    auto push = [&](uint32_t op, uint32_t len) {
        if (len == 0) return;
        if (!eqx && (op == 7 || op == 8)) op = 0;
        if (op == pend_op) {
            pend_len += len;
            return;
        }
        if (pend_len) {
            p = w_u64(p, pend_len);
            *p++ = ch[pend_op];
        }
        pend_op = op;
        pend_len = len;
    };
    push(4, a.soft_clip_left);
    for (uint32_t i = 0; i < a.cigar_len; i++) push(a.cigar[i] & 15, a.cigar[i] >> 4);
    push(4, a.soft_clip_right);
    if (pend_len) {
        p = w_u64(p, pend_len);
        *p++ = ch[pend_op];
    }
    return p;
}

// src/io/sam.rs:53-138
void format_sam(const Sam& r, const PolicyConfig& cfg, OutBuf& o) {
    const bool secondary = (r.flags & SECONDARY) != 0;
    const ReadView& rv = *r.rv;
    size_t bound = rv.name_len + 2 * (size_t)rv.len + 160;
    if (r.rname) bound += r.rname->size();
    if (r.rnext) bound += r.rnext->size();
    if (r.aln) bound += ((size_t)r.aln->cigar_len + 2) * 11;
    if (cfg.has_rg) bound += 6 + cfg.rg_id.size();
    if (cfg.mp.fastq_comments && rv.comment) bound += 1 + rv.comment_len;
    // written in place at the end of the output (no zero fill of the bound)
    char* p = o.tail(bound);
    p = w_str(p, rv.name, rv.name_len);
    *p++ = '\t';
    p = w_u64(p, r.flags);
    *p++ = '\t';
    if (r.rname) p = w_str(p, r.rname->data(), r.rname->size());
    else *p++ = '*';
    *p++ = '\t';
    p = w_u64(p, r.has_pos ? (uint64_t)r.pos + 1 : 0);
    *p++ = '\t';
    p = w_u64(p, r.mapq);
    *p++ = '\t';
    if (r.aln) p = w_cigar(p, *r.aln, cfg.mp.eqx != 0);
    else *p++ = '*';
    *p++ = '\t';
    if (r.rnext) p = w_str(p, r.rnext->data(), r.rnext->size());
    else *p++ = '*';
    *p++ = '\t';
    p = w_u64(p, r.has_pnext ? (uint64_t)r.pnext + 1 : 0);
    *p++ = '\t';
    p = w_i64(p, r.has_tlen ? r.tlen : 0);
    *p++ = '\t';
    if (!secondary && rv.len > 0) {
        if (r.seq_rc)
            p = w_revcomp(p, rv.seq, rv.len);
        else
            p = w_str(p, rv.seq, rv.len);
    } else {
        *p++ = '*';
    }
    *p++ = '\t';
    if (rv.qual && !secondary && rv.len > 0) {
        if (r.seq_rc)
            p = w_reversed(p, rv.qual, rv.len);
        else
            p = w_str(p, rv.qual, rv.len);
    } else {
        *p++ = '*';
    }
    if (r.has_nm) {
        p = w_lit(p, "\tNM:i:");
        p = w_u64(p, r.nm);
        p = w_lit(p, "\tAS:i:");
        p = w_u64(p, r.as);
    }
    if (cfg.mp.details && r.det) {
        p = w_lit(p, "\tna:i:");
        p = w_u64(p, r.det->nam.n_nams);
        p = w_lit(p, "\tal:i:");
        p = w_u64(p, r.det->tried_alignment);
        p = w_lit(p, "\tga:i:");
        p = w_u64(p, r.det->gapped);
        p = w_lit(p, "\tX0:i:");
        p = w_u64(p, r.det->best_alignments);
        if (r.flags & PAIRED) {
            p = w_lit(p, "\tmr:i:");
            p = w_u64(p, r.det->mate_rescue);
        }
    }
    if (cfg.has_rg) {
        p = w_lit(p, "\tRG:Z:");
        p = w_str(p, cfg.rg_id.data(), cfg.rg_id.size());
    }
    if (cfg.mp.fastq_comments && rv.comment) {
        *p++ = '\t';
        p = w_str(p, rv.comment, rv.comment_len);
    }
    *p++ = '\n';
    o.commit(p);
}

Sam mapped_record(const Policy& P, const Alignment& a, const ReadView& rv, uint8_t mapq, bool secondary,
                  const Details& det) {
    Sam r;
    r.rv = &rv;
    if (a.is_revcomp) r.flags |= REVERSE;
    if (secondary) {
        mapq = 0;
        r.flags |= SECONDARY;
    }
    r.seq_rc = a.is_revcomp;
    r.rname = P.contigs()[a.reference_id].name;
    r.has_pos = true;
    r.pos = a.ref_start;
    r.mapq = mapq;
    r.aln = &a;
    r.has_nm = true;
    r.nm = a.edit_distance;
    r.as = a.score;
    r.det = &det;
    return r;
}

Sam unmapped_record(const ReadView& rv, const Details& det) {
    Sam r;
    r.rv = &rv;
    r.flags = UNMAP;
    r.det = &det;
    return r;
}

// src/mapper.rs:239-345
void paired_records(const Policy& P, const Alignment* al[2], const ReadView* rv[2], const uint8_t mapq[2],
                    const Details det[2], bool secondary, bool proper, std::vector<Sam>& out) {
    Sam s[2];
    for (int i = 0; i < 2; i++)
        s[i] = al[i] ? mapped_record(P, *al[i], *rv[i], mapq[i], secondary, det[i]) : unmapped_record(*rv[i], det[i]);
    s[0].flags |= READ1;
    s[1].flags |= READ2;
    for (int i = 0; i < 2; i++) {
        s[i].flags |= PAIRED;
        if (proper) s[i].flags |= PROPER_PAIR;
        const Alignment* mate = al[1 - i];
        if (mate) {
            if (mate->is_revcomp) s[i].flags |= MREVERSE;
            s[i].has_pnext = true;
            s[i].pnext = mate->ref_start;
            s[i].rnext = P.contigs()[mate->reference_id].name;
            if (al[i]) {
                const Alignment* self = al[i];
                if (self->reference_id == mate->reference_id) {
                    s[i].rnext = &EQUALS;
                    int64_t tl;
                    if (mate->ref_start > self->ref_start)
                        tl = (int64_t)(mate->ref_start - self->ref_start + mate->length);
                    else if (self->ref_start > mate->ref_start)
                        tl = -(int64_t)(self->ref_start - mate->ref_start + self->length);
                    else if (i == 0)
                        tl = -(int64_t)mate->length;
                    else
                        tl = (int64_t)self->length;
                    s[i].has_tlen = true;
                    s[i].tlen = (int32_t)tl;
                }
            } else {
                s[i].rnext = &EQUALS;
                s[i].rname = P.contigs()[mate->reference_id].name;
                s[i].has_pos = true;
                s[i].pos = mate->ref_start;
            }
        } else {
            s[i].flags |= MUNMAP;
            if (al[i]) {
                s[i].rnext = &EQUALS;
                s[i].has_pnext = true;
                s[i].pnext = al[i]->ref_start;
            }
        }
    }
    if (secondary) {
        if (!s[1].is_mapped()) {
            out.push_back(s[0]);
            return;
        }
        if (!s[0].is_mapped()) {
            out.push_back(s[1]);
            return;
        }
    }
    out.push_back(s[0]);
    out.push_back(s[1]);
}

// src/mapper.rs:1200-1218
bool proper_nam_pair(const NamRec& n1, const NamRec& n2, float mu, float sigma) {
    if (n1.ref_id != n2.ref_id || (n1.is_revcomp != 0) == (n2.is_revcomp != 0)) return false;
    uint32_t r1 = projected_ref_start(n1), r2 = projected_ref_start(n2);
    float lim = mu + 10.0f * sigma;
    bool r1_r2 = n2.is_revcomp && r1 <= r2 && (float)(r2 - r1) < lim;
    bool r2_r1 = n1.is_revcomp && r2 <= r1 && (float)(r1 - r2) < lim;
    return r1_r2 || r2_r1;
}

// src/mapper.rs:1180-1197
bool proper_pair(const Alignment& a1, const Alignment& a2, float mu, float sigma) {
    int64_t dist = (int64_t)a2.ref_start - (int64_t)a1.ref_start;
    bool same = a1.reference_id == a2.reference_id;
    bool r1_r2 = !a1.is_revcomp && a2.is_revcomp && dist >= 0;
    bool r2_r1 = !a2.is_revcomp && a1.is_revcomp && dist <= 0;
    bool good = (uint64_t)(dist < 0 ? -dist : dist) <= sat_usize(mu + sigma * 6.0f);
    return same && good && (r1_r2 || r2_r1);
}

// src/mapper.rs:1302-1313
uint8_t mapping_quality(const std::vector<NamRec>& n) {
    if (n.size() <= 1) return 60;
    float s1 = n[0].score, s2 = n[1].score;
    float mm = (float)std::min<uint32_t>(n[0].n_anchors, 10) / 10.0f;
    float u = 40.0f * (1.0f - s2 / s1) * mm * std::log(s1);
    return sat_u8(std::fmin(u, 60.0f));
}

struct ScoredPair {
    double score;
    bool h1, h2;
    Alignment a1, a2;
};

// src/mapper.rs:1440-1458
uint8_t alignment_quality(const std::vector<ScoredPair>& v) {
    if (v.size() <= 1) return 60;
    float s1 = (float)v[0].score, s2 = (float)v[1].score;
    if (s1 > 0.0f && s2 > 0.0f) return sat_u8(std::fmin(s1 - s2, 60.0f));
    if (s1 > 0.0f && s2 <= 0.0f) return 60;
    return 1;
}

// src/mapper.rs:1461-1470
float top_dropoff(const std::vector<NamRec>& n) {
    if (n[0].n_anchors <= 2) return 1.0f;
    if (n.size() > 1) return (float)n[1].n_anchors / (float)n[0].n_anchors;
    return 0.0f;
}

struct NamPair {
    float score;
    bool h1, h2;
    NamRec n1, n2;
};

// src/mapper.rs:1224-1299
// Stable sort for the short lists of one record: insertion sort (no allocation) up
// to 32 elements, std::stable_sort beyond.  `before(a, b)`: a strictly precedes b.
template <class T, class F>
void stable_sort_small(std::vector<T>& v, F before) {
    if (v.size() > 32) {
        std::stable_sort(v.begin(), v.end(), before);
        return;
    }
    for (size_t i = 1; i < v.size(); i++) {
        T x = v[i];
        size_t j = i;
        while (j > 0 && before(x, v[j - 1])) {
            v[j] = v[j - 1];
            j--;
        }
        v[j] = x;
    }
}

void best_scoring_nam_pairs(const std::vector<NamRec>& n1, const std::vector<NamRec>& n2, float mu, float sigma,
                            std::vector<NamPair>& pairs, std::vector<uint32_t>& added1,
                            std::vector<uint32_t>& added2) {
    pairs.clear();
    added1.clear();
    added2.clear();
    if (n1.empty() && n2.empty()) return;
    auto has = [](const std::vector<uint32_t>& v, uint32_t x) { return std::find(v.begin(), v.end(), x) != v.end(); };
    uint32_t best_joint = 0;
    for (size_t a = 0; a < n1.size() && a < 1000; a++) {
        for (size_t b = 0; b < n2.size() && b < 1000; b++) {
            uint32_t joint = n1[a].n_anchors + n2[b].n_anchors;
            if (joint < best_joint / 2) break;
            if (proper_nam_pair(n1[a], n2[b], mu, sigma)) {
                pairs.push_back(NamPair{n1[a].score + n2[b].score, true, true, n1[a], n2[b]});
                if (!has(added1, n1[a].nam_id)) added1.push_back(n1[a].nam_id);
                if (!has(added2, n2[b].nam_id)) added2.push_back(n2[b].nam_id);
                best_joint = std::max(joint, best_joint);
            }
        }
    }
    if (!n1.empty()) {
        uint32_t bj = best_joint > 0 ? best_joint : n1[0].n_anchors;
        for (auto& n : n1) {
            if (n.n_anchors < bj / 2) break;
            if (has(added1, n.nam_id)) continue;
            pairs.push_back(NamPair{n.score, true, false, n, NamRec{}});
        }
    }
    if (!n2.empty()) {
        uint32_t bj = best_joint > 0 ? best_joint : n2[0].n_anchors;
        for (auto& n : n2) {
            if (n.n_anchors < bj / 2) break;
            if (has(added2, n.nam_id)) continue;
            pairs.push_back(NamPair{n.score, false, true, NamRec{}, n});
        }
    }
    stable_sort_small(pairs, [](const NamPair& a, const NamPair& b) { return a.score > b.score; });
}

}  // namespace

// Per-thread buffers of one record's evaluation, reused across records
struct Policy::Scratch {
    std::vector<NamRec> nams[2];
    std::vector<Alignment> alignments, al1;
    std::vector<std::pair<bool, Alignment>> al2;
    std::vector<ScoredPair> pairs;
    std::vector<std::pair<uint32_t, std::pair<bool, Alignment>>> cache[2];
    std::vector<NamPair> np;
    std::vector<uint32_t> added1, added2;
    std::vector<Sam> recs;
};

Policy::Policy(const PolicyConfig& cfg, const std::vector<ContigInfo>& contigs, const BatchView& bv,
               ResultStore& store)
    : cfg_(cfg), contigs_(contigs), bv_(&bv), store_(&store), sc_(new Scratch) {}

Policy::~Policy() = default;

// ------------------------------------------------------------------ result access
const ResultStore::Entry* Policy::lookup(uint32_t read, const JobKey& key) const {
    const uint32_t h = store_->head[read];
    const ResultStore::Entry* pool = cur_->entries.data();
    auto find = [&](const JobKey& k) -> const ResultStore::Entry* {
        for (uint32_t i = h; i != ResultStore::NONE; i = pool[i].next)
            if (pool[i].key == k && pool[i].result) return &pool[i];
        return nullptr;
    };
    if (const ResultStore::Entry* r = find(key)) return r;
    // extend_seed after is_consistent and after reverse_nam_if_needed coincide whenever
    // the latter does not flip the NAM
    if (key.kind == JOB_EXTEND_FULL) {
        const ResultStore::Entry* f = find(JobKey{JOB_EXTEND_FAST, key.a, 0, 0, 0});
        if (f && f->result->consistent) return f;
    } else if (key.kind == JOB_EXTEND_FAST) {
        const ResultStore::Entry* f = find(JobKey{JOB_EXTEND_FULL, key.a, 0, 0, 0});
        if (f && !f->result->flipped) return f;
    }
    return nullptr;
}

void Policy::want(uint32_t read, const ExtJob& job, const JobKey& key) {
    if (lookup(read, key)) return;
    auto& pool = cur_->entries;
    uint32_t& h = store_->head[read];
    for (uint32_t i = h; i != ResultStore::NONE; i = pool[i].next)
        if (pool[i].key == key) return;  // pending
    pool.push_back(ResultStore::Entry{key, h, nullptr, nullptr});
    h = (uint32_t)(pool.size() - 1);
    ExtJob j = job;
    j.tag = h;
    cur_->pending.push_back(j);
}

bool Policy::get(uint32_t read, const ExtJob& job, const JobKey& key, StoredResult& r) {
    if (const ResultStore::Entry* e = lookup(read, key)) {
        static_cast<ExtResult&>(r) = *e->result;
        r.cigar = e->cigar + e->result->cigar_offset;
        return true;
    }
    want(read, job, key);
    return false;
}

void Policy::resolve(ChunkState& cs) {
    if (!cs.wave) return;
    const WaveResults& w = *cs.wave;
    for (size_t j = 0; j < cs.pending.size(); j++) {
        const ExtJob& jb = cs.pending[j];
        auto& e = cs.entries[jb.tag];
        e.result = &w.results[cs.wave_first + j];
        e.cigar = w.cigar.data();
        cs.result_bytes += sizeof(ExtResult) + (e.result->valid ? 4ull * e.result->cigar_len : 0);
    }
    cs.pending.clear();
    cs.waves.push_back(std::move(cs.wave));
    cs.wave.reset();
}

ExtJob Policy::nam_job(uint32_t read, const NamRec& cur, uint32_t kind) const {
    // jobs always carry the NAM as the GPU produced it (before any host-side flip)
    const NamRec* b = bv_->nams + bv_->nam_off[read];
    const NamRec* e = bv_->nams + bv_->nam_off[read + 1];
    const NamRec* f = std::find_if(b, e, [&](const NamRec& x) { return x.nam_id == cur.nam_id; });
    const NamRec& n = f != e ? *f : cur;
    ExtJob j{};
    j.kind = kind;
    j.read = read;
    j.ref_id = n.ref_id;
    j.ref_start = n.ref_start;
    j.ref_end = n.ref_end;
    j.query_start = n.query_start;
    j.query_end = n.query_end;
    j.is_revcomp = n.is_revcomp;
    // paired-end extension always uses SSW (src/mapper.rs:860-870); single-end follows --ssw
    j.use_ssw = (pe_ || cfg_.mp.use_ssw) ? 1 : 0;
    j.nam = (uint32_t)(f != e ? f - b : 0);
    return j;
}

static bool is_piecewise(const BatchView& bv, const ExtJob& j) {
    return !j.use_ssw && (j.kind == JOB_EXTEND_FAST || j.kind == JOB_EXTEND_FULL) && bv.nam_anc;
}

uint64_t piecewise_anchor_offsets(const BatchView& bv, ExtJob* jobs, size_t n, uint64_t first, uint32_t& max_n) {
    uint64_t at = first;
    for (size_t i = 0; i < n; i++) {
        ExtJob& j = jobs[i];
        if (!is_piecewise(bv, j)) continue;
        const uint64_t t = bv.nam_off[j.read] + j.nam;
        j.anc_off = (uint32_t)at;
        j.anc_n = (uint32_t)(bv.nam_anc_off[t + 1] - bv.nam_anc_off[t]);
        max_n = std::max(max_n, j.anc_n);
        at += j.anc_n;
    }
    return at - first;
}

void piecewise_anchor_fill(const BatchView& bv, const ExtJob* jobs, size_t n, uint32_t* anchors) {
    const uint64_t qmask = (1ull << bv.anc_qbits) - 1, pmask = (1ull << bv.anc_pbits) - 1;
    for (size_t i = 0; i < n; i++) {
        const ExtJob& j = jobs[i];
        if (!is_piecewise(bv, j)) continue;
        const uint64_t a0 = bv.nam_anc_off[bv.nam_off[j.read] + j.nam];
        uint32_t* o = anchors + 2 * (uint64_t)j.anc_off;
        for (uint32_t a = 0; a < j.anc_n; a++) {
            const uint64_t key = bv.nam_anc[a0 + a];
            o[2 * a] = (uint32_t)(key & qmask);
            o[2 * a + 1] = (uint32_t)((key >> bv.anc_qbits) & pmask);
        }
    }
}

void Policy::want_nam(uint32_t read, const NamRec& n, uint32_t kind) { want(read, nam_job(read, n, kind), nam_key(n, kind)); }

Alignment Policy::to_alignment(const StoredResult& r, uint32_t ref_id) const {
    Alignment a;
    a.reference_id = ref_id;
    a.ref_start = r.ref_start;
    a.edit_distance = r.edit_distance;
    a.soft_clip_left = r.soft_clip_left;
    a.soft_clip_right = r.soft_clip_right;
    a.score = r.score;
    a.length = r.length;
    a.is_revcomp = r.is_revcomp != 0;
    a.gapped = r.gapped != 0;
    a.cigar = r.cigar;
    a.cigar_len = r.cigar_len;
    return a;
}

int Policy::extend(uint32_t read, NamRec& nam, uint32_t kind, Alignment& out, bool& consistent) {
    StoredResult r;
    if (!get(read, nam_job(read, nam, kind), nam_key(nam, kind), r)) return MISSING;
    consistent = r.consistent != 0;
    if (kind == JOB_EXTEND_FULL) {
        nam.is_revcomp = r.nam_is_revcomp;
        nam.query_start = r.nam_query_start;
        nam.query_end = r.nam_query_end;
    }
    if (!r.valid) return UNALIGNED;
    out = to_alignment(r, nam.ref_id);
    return ALIGNED;
}

// rescue_align (src/mapper.rs:1094-1153): the window is fixed here, the
// has_shared_substring filter and the alignment run on the GPU
bool Policy::rescue_job(uint32_t read, const NamRec& mate, float mu, float sigma, ExtJob& j, JobKey& key) const {
    const uint64_t rl = bv_->reads[read].len;
    const uint64_t w = sat_usize(mu + 5.0f * sigma);
    uint64_t rs, re;
    bool rc;
    if (mate.is_revcomp) {
        rc = false;
        uint64_t p = projected_ref_start(mate);
        rs = p > w ? p - w : 0;
        re = p + rl / 2;
    } else {
        rc = true;
        uint64_t b = (uint64_t)mate.ref_end + rl - mate.query_end;
        rs = b > rl / 2 ? b - rl / 2 : 0;
        re = b + w;
    }
    const uint64_t clen = contigs_[mate.ref_id].len;
    rs = std::min(rs, clen);
    re = std::min(re, clen);
    if (re < rs + cfg_.k) return false;
    j = ExtJob{};
    j.kind = JOB_RESCUE;
    j.read = read;
    j.ref_id = mate.ref_id;
    j.ref_start = (uint32_t)rs;
    j.ref_end = (uint32_t)re;
    j.is_revcomp = rc;
    j.use_ssw = 1;
    key = JobKey{JOB_RESCUE, mate.ref_id, (uint32_t)rs, (uint32_t)re, rc ? 1u : 0u};
    return true;
}

int Policy::rescue(uint32_t read, const NamRec& mate, float mu, float sigma, Alignment& out) {
    ExtJob j;
    JobKey key;
    if (!rescue_job(read, mate, mu, sigma, j, key)) return UNALIGNED;
    StoredResult r;
    if (!get(read, j, key, r)) return MISSING;
    if (!r.valid) return UNALIGNED;
    out = to_alignment(r, mate.ref_id);
    return ALIGNED;
}

// Requests made on a miss for work a record will need once the missing results are
// in: the NAM's full extension if it is unknown, else (need_valid: only when that
// extension aligned) the rescue of the mate from the NAM as the extension flipped it.
// Requests change no result, only which wave computes it.
void Policy::want_rescue_chain(uint32_t read, const NamRec& nam, uint32_t mate, float mu, float sigma,
                               bool need_valid) {
    const ResultStore::Entry* e = lookup(read, nam_key(nam, JOB_EXTEND_FULL));
    if (!e) {
        want_nam(read, nam, JOB_EXTEND_FULL);
        return;
    }
    if (need_valid && !e->result->valid) return;
    NamRec m = nam;
    m.is_revcomp = e->result->nam_is_revcomp;
    m.query_start = e->result->nam_query_start;
    m.query_end = e->result->nam_query_end;
    ExtJob j;
    JobKey key;
    if (rescue_job(mate, m, mu, sigma, j, key)) want(mate, j, key);
}

// sort_nams (src/nam.rs:168-188): the GPU already applied the stable sort
void Policy::sorted_nams(uint32_t read, Rng& rng, std::vector<NamRec>& v) const {
    v.assign(bv_->nams + bv_->nam_off[read], bv_->nams + bv_->nam_off[read + 1]);
    if (!v.empty()) {
        size_t nb = 0;
        while (nb < v.size() && v[nb].score == v[0].score) nb++;
        if (nb > 1)
            for (size_t i = 1; i < nb; i++) std::swap(v[i], v[(size_t)rng.gen_mod_u64(i + 1)]);
    }
}

std::vector<NamRec> Policy::sorted_nams(uint32_t read, Rng& rng) const {
    std::vector<NamRec> v;
    sorted_nams(read, rng, v);
    return v;
}

// ------------------------------------------------------------------ single end
// src/mapper.rs:349-528
bool Policy::se_record(uint64_t rec, Rng& rng, OutBuf& out, uint64_t& mapped) {
    const uint32_t read = bv_->first_read(rec);
    const ReadView& rv = bv_->reads[read];
    std::vector<NamRec>& nams = sc_->nams[0];
    sorted_nams(read, rng, nams);
    Details details;
    details.nam = bv_->details[read];
    if (nams.empty()) {
        if (cfg_.mp.output_unmapped && !speculative_) format_sam(unmapped_record(rv, details), cfg_, out);
        return true;
    }
    const float nam_max = nams[0].score;
    const size_t max_tries = cfg_.mp.max_tries;
    uint64_t best_edit = UINT64_MAX;
    uint32_t best_score = 0, second = 0, n_best = 0;
    size_t best_index = 0;
    bool have_best = false;
    Alignment best;
    std::vector<Alignment>& alignments = sc_->alignments;
    alignments.clear();
    for (size_t tries = 0; tries < nams.size() && tries < max_tries; tries++) {
        NamRec& nam = nams[tries];
        float dropoff = nam.score / nam_max;
        if ((tries > 1 && best_edit == 0) || dropoff < cfg_.mp.dropoff_threshold) break;
        Alignment a;
        bool consistent;
        const int er = extend(read, nam, JOB_EXTEND_FAST, a, consistent);
        if (er == MISSING) {
            // also request the next candidates this read may try
            for (size_t t = tries + 1; t < nams.size() && t < max_tries && t < tries + 4; t++)
                if (nams[t].score / nam_max >= cfg_.mp.dropoff_threshold) want_nam(read, nams[t], JOB_EXTEND_FAST);
            return false;
        }
        const bool ok = er == ALIGNED;
        if (!consistent) {
            details.inconsistent_nams++;
            continue;
        }
        if (!ok) continue;
        details.tried_alignment++;
        details.gapped += a.gapped;
        if (a.score >= best_score) {
            second = best_score;
            bool update = false;
            if (a.score > best_score) {
                n_best = 1;
                update = true;
            } else {
                n_best++;
                if (rng.gen_mod_u32(n_best) == 0) update = true;
            }
            if (update) {
                best_score = a.score;
                best = a;
                have_best = true;
                best_index = alignments.size();
                if (cfg_.mp.max_secondary == 0) best_edit = a.global_edit_distance();
            }
        } else if (a.score > second) {
            second = a.score;
        }
        if (cfg_.mp.max_secondary > 0) alignments.push_back(a);
    }
    if (!have_best) {
        if (cfg_.mp.output_unmapped && !speculative_) format_sam(unmapped_record(rv, details), cfg_, out);
        return true;
    }
    uint8_t mapq = (uint8_t)((60 * (best_score - second) + best_score - 1) / best_score);
    if (!speculative_) format_sam(mapped_record(*this, best, rv, mapq, false, details), cfg_, out);
    mapped++;
    if (cfg_.mp.max_secondary > 0) {
        alignments[best_index] = alignments.back();
        alignments.pop_back();
        std::stable_sort(alignments.begin(), alignments.end(),
                         [](const Alignment& x, const Alignment& y) { return x.score > y.score; });
        uint32_t lim = 2u * cfg_.mp.mismatch + cfg_.mp.gap_open;
        for (size_t t = 0; t < alignments.size() && t < cfg_.mp.max_secondary; t++) {
            const Alignment& a = alignments[t];
            uint32_t d = a.score > best_score ? a.score - best_score : 0;
            if (d > lim) break;
            if (!speculative_) format_sam(mapped_record(*this, a, rv, mapq, true, details), cfg_, out);
        }
    }
    return true;
}

// ------------------------------------------------------------------ paired end
// src/mapper.rs:624-1091
bool Policy::pe_record(uint64_t rec, Rng& rng, InsertSize& isd, OutBuf& out, uint64_t& mapped) {
    const uint32_t rd[2] = {bv_->first_read(rec), bv_->first_read(rec) + 1};
    const ReadView* rv[2] = {&bv_->reads[rd[0]], &bv_->reads[rd[1]]};
    Details det[2];
    std::vector<NamRec>(&nams)[2] = sc_->nams;
    for (int i = 0; i < 2; i++) {
        sorted_nams(rd[i], rng, nams[i]);
        det[i].nam = bv_->details[rd[i]];
    }
    for (int i = 0; i < 2; i++)
        if (!nams[i].empty()) want_nam(rd[i], nams[i][0], JOB_EXTEND_FAST);
    const float mu = isd.mu, sigma = isd.sigma, dropoff = cfg_.mp.dropoff_threshold;
    const size_t max_tries = cfg_.mp.max_tries;
    std::vector<ScoredPair>& pairs = sc_->pairs;
    pairs.clear();
    bool fast = false;
    Alignment proper[2];

    auto rescue_read = [&](int has, int other) -> bool {
        // src/mapper.rs:1018-1091; det[has] / det[other] as the reference passes them
        std::vector<NamRec>& n1 = nams[has];
        float max1 = n1[0].score;
        std::vector<Alignment>& al1 = sc_->al1;
        std::vector<std::pair<bool, Alignment>>& al2 = sc_->al2;
        al1.clear();
        al2.clear();
        for (size_t t = 0; t < n1.size() && t < max_tries; t++) {
            NamRec& nam = n1[t];
            if (nam.score / max1 < dropoff) break;
            Alignment a;
            bool consistent = false;
            // on a miss: every later try is an extension and, when it aligns, a rescue
            auto prefetch_after = [&]() {
                for (size_t u = t + 1; u < n1.size() && u < max_tries; u++)
                    if (n1[u].score / max1 >= dropoff) want_rescue_chain(rd[has], n1[u], rd[other], mu, sigma, true);
            };
            const int er = extend(rd[has], nam, JOB_EXTEND_FULL, a, consistent);
            if (er == MISSING) {
                prefetch_after();
                return false;
            }
            det[has].inconsistent_nams += !consistent;
            if (er == ALIGNED) {
                det[has].gapped += a.gapped;
                al1.push_back(a);
                det[has].tried_alignment++;
                Alignment b;
                const int rr = rescue(rd[other], nam, mu, sigma, b);
                if (rr == MISSING) {
                    prefetch_after();
                    return false;
                }
                if (rr == ALIGNED) det[other].mate_rescue++;
                al2.emplace_back(rr == ALIGNED, b);
            }
        }
        for (auto& a1 : al1) {
            for (auto& a2p : al2) {
                ScoredPair sp;
                if (a2p.first) {
                    const Alignment& a2 = a2p.second;
                    uint64_t dist = absdiff(a1.ref_start, a2.ref_start);
                    float score = (float)(a1.score + a2.score);
                    if ((a1.is_revcomp ^ a2.is_revcomp) && (float)dist < mu + 4.0f * sigma)
                        score += std::log(normal_pdf((float)dist, mu, sigma));
                    else
                        score -= 10.0f;
                    sp.score = (double)score;
                    sp.h1 = sp.h2 = true;
                    sp.a1 = a1;
                    sp.a2 = a2;
                } else {
                    sp.score = (double)a1.score - 10.0;
                    sp.h1 = true;
                    sp.h2 = false;
                    sp.a1 = a1;
                }
                if (has == 1) {  // the mate with NAMs is read 2: swap back
                    std::swap(sp.h1, sp.h2);
                    std::swap(sp.a1, sp.a2);
                }
                pairs.push_back(sp);
            }
        }
        return true;
    };

    if (nams[0].empty() && nams[1].empty()) {
    } else if (!nams[0].empty() && nams[1].empty()) {
        if (!rescue_read(0, 1)) return false;
    } else if (nams[0].empty() && !nams[1].empty()) {
        if (!rescue_read(1, 0)) return false;
    } else {
        bool took_fast = false;
        if (top_dropoff(nams[0]) < dropoff && top_dropoff(nams[1]) < dropoff &&
            proper_nam_pair(nams[0][0], nams[1][0], mu, sigma)) {
            NamRec m1 = nams[0][0], m2 = nams[1][0];
            Alignment a1, a2;
            bool c1, c2;
            want_nam(rd[1], m2, JOB_EXTEND_FAST);
            const int e1 = extend(rd[0], m1, JOB_EXTEND_FAST, a1, c1);
            if (e1 == MISSING) return false;
            const int e2 = extend(rd[1], m2, JOB_EXTEND_FAST, a2, c2);
            if (e2 == MISSING) return false;
            const bool ok1 = e1 == ALIGNED, ok2 = e2 == ALIGNED;
            det[0].inconsistent_nams += !c1;
            det[1].inconsistent_nams += !c2;
            if (ok1 && ok2) {
                det[0].tried_alignment++;
                det[0].gapped += a1.gapped;
                det[1].tried_alignment++;
                det[1].gapped += a2.gapped;
                proper[0] = a1;
                proper[1] = a2;
                fast = took_fast = true;
            }
        }
        if (!took_fast) {
            // full search (src/mapper.rs:882-1013)
            for (int i = 0; i < 2; i++) want_nam(rd[i], nams[i][0], JOB_EXTEND_FULL);
            std::vector<std::pair<uint32_t, std::pair<bool, Alignment>>>(&cache)[2] = sc_->cache;
            cache[0].clear();
            cache[1].clear();
            bool have_indv[2] = {false, false};
            Alignment indv[2];
            for (int i = 0; i < 2; i++) {
                Alignment a;
                bool c;
                const int e = extend(rd[i], nams[i][0], JOB_EXTEND_FULL, a, c);
                if (e == MISSING) return false;
                const bool ok = e == ALIGNED;
                det[i].inconsistent_nams += !c;
                have_indv[i] = ok;
                if (ok) indv[i] = a;
                det[i].tried_alignment++;
                det[i].gapped += ok ? a.gapped : 0;
                cache[i].push_back({nams[i][0].nam_id, {ok, a}});
            }
            std::vector<NamPair>& np = sc_->np;
            best_scoring_nam_pairs(nams[0], nams[1], mu, sigma, np, sc_->added1, sc_->added2);
            float max_score = np[0].score;
            size_t n_out = 0;
            size_t cur = 0;  // the pair being evaluated
            auto prefetch = [&]() {
                // on a miss, also request what the next pairs can need: their NAM
                // extensions, and for a one-sided pair the rescue from its partner
                // (pairs whose alignments fail do not count towards max_tries, so
                // the loop can run through many pairs)
                for (size_t t = cur; t < np.size() && t < cur + max_tries; t++) {
                    if (np[t].score / max_score < dropoff) break;
                    if (np[t].h1 && np[t].h2) {
                        want_nam(rd[0], np[t].n1, JOB_EXTEND_FULL);
                        want_nam(rd[1], np[t].n2, JOB_EXTEND_FULL);
                    } else if (np[t].h1) {
                        want_rescue_chain(rd[0], np[t].n1, rd[1], mu, sigma, false);
                    } else if (np[t].h2) {
                        want_rescue_chain(rd[1], np[t].n2, rd[0], mu, sigma, false);
                    }
                }
            };
            for (; cur < np.size(); cur++) {
                auto& pr = np[cur];
                float sd = pr.score / max_score;
                if (n_out >= max_tries || sd < dropoff) break;
                bool hv[2] = {pr.h1, pr.h2};
                NamRec* nm[2] = {&pr.n1, &pr.n2};
                bool okal[2] = {false, false};
                Alignment al[2];
                for (int i = 0; i < 2; i++) {
                    bool ok = false;
                    Alignment a;
                    if (hv[i]) {
                        NamRec this_nam = *nm[i];
                        auto it = std::find_if(cache[i].begin(), cache[i].end(),
                                               [&](auto& e) { return e.first == this_nam.nam_id; });
                        if (it == cache[i].end()) {
                            bool c = false;
                            const int e = extend(rd[i], this_nam, JOB_EXTEND_FULL, a, c);
                            if (e == MISSING) {
                                prefetch();
                                return false;
                            }
                            ok = e == ALIGNED;
                            det[i].inconsistent_nams += !c;
                            det[i].tried_alignment++;
                            det[i].gapped += ok ? a.gapped : 0;
                            cache[i].push_back({this_nam.nam_id, {ok, a}});
                        } else {
                            ok = it->second.first;
                            a = it->second.second;
                        }
                    } else {
                        NamRec other = *nm[1 - i];
                        // reverse_nam_if_needed on the partner, then rescue from it
                        StoredResult fr;
                        if (!get(rd[1 - i], nam_job(rd[1 - i], other, JOB_EXTEND_FULL),
                                 nam_key(other, JOB_EXTEND_FULL), fr)) {
                            prefetch();
                            return false;
                        }
                        det[1 - i].inconsistent_nams += !fr.consistent;
                        other.is_revcomp = fr.nam_is_revcomp;
                        other.query_start = fr.nam_query_start;
                        other.query_end = fr.nam_query_end;
                        const int rr = rescue(rd[i], other, mu, sigma, a);
                        if (rr == MISSING) {
                            prefetch();
                            return false;
                        }
                        ok = rr == ALIGNED;
                        if (ok) {
                            det[i].mate_rescue++;
                            det[i].tried_alignment++;
                        }
                    }
                    uint32_t s_new = ok ? a.score : 0, s_old = have_indv[i] ? indv[i].score : 0;
                    if (s_new > s_old) {
                        indv[i] = a;
                        have_indv[i] = ok;
                    }
                    okal[i] = ok;
                    al[i] = a;
                }
                if (!okal[0] || !okal[1]) continue;
                const Alignment& a1 = al[0];
                const Alignment& a2 = al[1];
                uint64_t lim = sat_usize(mu + 10.0f * sigma);
                bool r1_r2 = a2.is_revcomp && !a1.is_revcomp && a1.ref_start <= a2.ref_start &&
                             (uint64_t)(a2.ref_start - a1.ref_start) < lim;
                bool r2_r1 = a1.is_revcomp && !a2.is_revcomp && a2.ref_start <= a1.ref_start &&
                             (uint64_t)(a1.ref_start - a2.ref_start) < lim;
                double combined;
                if (r1_r2 || r2_r1) {
                    uint64_t x = absdiff(a1.ref_start, a2.ref_start);
                    double lp = (double)std::log(normal_pdf((float)x, mu, sigma));
                    combined = (double)a1.score + (double)a2.score + std::fmax(-20.0 + 0.001, lp);
                } else {
                    combined = (double)a1.score + (double)a2.score - 20.0;
                }
                ScoredPair sp;
                sp.score = combined;
                sp.h1 = sp.h2 = true;
                sp.a1 = a1;
                sp.a2 = a2;
                pairs.push_back(sp);
                n_out++;
            }
            if (have_indv[0] && have_indv[1]) {
                ScoredPair sp;
                sp.score = (double)indv[0].score + (double)indv[1].score - 20.0;
                sp.h1 = sp.h2 = true;
                sp.a1 = indv[0];
                sp.a2 = indv[1];
                pairs.push_back(sp);
            }
        }
    }
    std::vector<Sam>& recs = sc_->recs;
    recs.clear();
    if (fast) {
        bool ps = proper_pair(proper[0], proper[1], isd.mu, isd.sigma);
        if (ps && isd.sample_size < 400 && proper[0].edit_distance + proper[1].edit_distance < 3)
            isd.update(absdiff(proper[0].ref_start, proper[1].ref_start));
        uint8_t mq[2] = {mapping_quality(nams[0]), mapping_quality(nams[1])};
        det[0].best_alignments = 1;
        det[1].best_alignments = 1;
        const Alignment* al[2] = {&proper[0], &proper[1]};
        paired_records(*this, al, rv, mq, det, false, ps, recs);
    } else {
        stable_sort_small(pairs, [](const ScoredPair& a, const ScoredPair& b) { return a.score > b.score; });
        // deduplicate_scored_pairs (src/mapper.rs:1322-1352)
        if (pairs.size() >= 2) {
            auto same = [](bool ha, const Alignment& a, bool hb, const Alignment& b) {
                if (!ha && !hb) return true;
                if (ha != hb) return false;
                return a.ref_start == b.ref_start && a.reference_id == b.reference_id;
            };
            size_t kk = 0, j = 1;
            for (size_t i = 1; i < pairs.size(); i++) {
                if (!same(pairs[kk].h1, pairs[kk].a1, pairs[i].h1, pairs[i].a1) ||
                    !same(pairs[kk].h2, pairs[kk].a2, pairs[i].h2, pairs[i].a2)) {
                    pairs[j] = pairs[i];
                    j++;
                    kk = i;
                }
            }
            pairs.resize(j);
        }
        size_t nb = 0;
        while (nb < pairs.size() && pairs[nb].score == pairs[0].score) nb++;
        det[0].best_alignments = (uint32_t)nb;
        det[1].best_alignments = (uint32_t)nb;
        if (nb > 1) std::swap(pairs[0], pairs[(size_t)rng.gen_mod_u64(nb)]);
        uint8_t mq[2];
        auto proper_opt = [&](const ScoredPair& p) { return p.h1 && p.h2 && proper_pair(p.a1, p.a2, isd.mu, isd.sigma); };
        if (pairs.size() == 1 && !proper_opt(pairs[0])) {
            mq[0] = mapping_quality(nams[0]);
            mq[1] = mapping_quality(nams[1]);
        } else {
            mq[0] = mq[1] = alignment_quality(pairs);
        }
        // aligned_pairs_to_sam (src/mapper.rs:1365-1437)
        if (pairs.empty()) {
            Sam u[2] = {unmapped_record(*rv[0], det[0]), unmapped_record(*rv[1], det[1])};
            u[0].flags |= PAIRED | READ1 | MUNMAP;
            u[1].flags |= PAIRED | READ2 | MUNMAP;
            recs.push_back(u[0]);
            recs.push_back(u[1]);
        } else if (cfg_.mp.max_secondary == 0) {
            const ScoredPair& b = pairs[0];
            const Alignment* al[2] = {b.h1 ? &b.a1 : nullptr, b.h2 ? &b.a2 : nullptr};
            paired_records(*this, al, rv, mq, det, false, proper_opt(b), recs);
        } else {
            bool secondary = false;
            double s_max = pairs[0].score;
            double sd = 2.0 * cfg_.mp.mismatch + cfg_.mp.gap_open;
            for (size_t t = 0; t < pairs.size() && t < cfg_.mp.max_secondary; t++) {
                const ScoredPair& p = pairs[t];
                if (s_max - p.score < sd) {
                    uint8_t zero[2] = {0, 0};
                    const Alignment* al[2] = {p.h1 ? &p.a1 : nullptr, p.h2 ? &p.a2 : nullptr};
                    paired_records(*this, al, rv, secondary ? zero : mq, det, secondary, proper_opt(p), recs);
                } else {
                    break;
                }
                secondary = true;
            }
        }
    }
    if (!cfg_.mp.output_unmapped && recs.size() >= 2 && !recs[0].is_mapped() && !recs[1].is_mapped()) recs.clear();
    const auto tf = cfg_.timing ? std::chrono::steady_clock::now() : std::chrono::steady_clock::time_point();
    for (auto& r : recs) {
        if (!speculative_) format_sam(r, cfg_, out);
        mapped += r.is_mapped();
    }
    if (cfg_.timing)
        cur_->seconds_format += std::chrono::duration<double>(std::chrono::steady_clock::now() - tf).count();
    return true;
}

// ------------------------------------------------------------------ map-only / aemb
namespace {

void paf_line(const Policy& P, const NamRec& nam, const ReadView& rv, int end, int mapq, OutBuf& o) {
    o.append(rv.name, rv.name_len);
    if (end == 1) o += "/1";
    else if (end == 2) o += "/2";
    o.push_back('\t');
    put_u64(o, rv.len);
    o.push_back('\t');
    put_u64(o, nam.query_start);
    o.push_back('\t');
    put_u64(o, nam.query_end);
    o.push_back('\t');
    o.push_back(nam.is_revcomp ? '-' : '+');
    o.push_back('\t');
    o += *P.contigs()[nam.ref_id].name;
    o.push_back('\t');
    put_u64(o, P.contigs()[nam.ref_id].len);
    o.push_back('\t');
    put_u64(o, nam.ref_start);
    o.push_back('\t');
    put_u64(o, nam.ref_end);
    o.push_back('\t');
    put_u64(o, nam.matching_bases);
    o.push_back('\t');
    put_u64(o, nam.ref_end - nam.ref_start);
    o.push_back('\t');
    put_u64(o, mapq < 0 ? 255 : mapq);
    o.push_back('\n');
}

struct NamPairM {
    NamRec n1, n2;
    double score;
};

bool nam_key_less(const NamRec& a, const NamRec& b) {
    if (a.ref_id != b.ref_id) return a.ref_id < b.ref_id;
    return projected_ref_start(a) < projected_ref_start(b);
}

// src/maponly.rs:366-378
void split_orient(NamRec* n, size_t c, bool both, NamRec*& f, size_t& nf, NamRec*& r, size_t& nr) {
    if (both) {
        size_t left = 0, right = c;
        while (left < right) {
            if (n[left].is_revcomp) {
                right--;
                std::swap(n[left], n[right]);
            } else {
                left++;
            }
        }
        f = n; nf = left; r = n + left; nr = c - left;
    } else if (n[0].is_revcomp) {
        f = n; nf = 0; r = n; nr = c;
    } else {
        f = n; nf = c; r = n + c; nr = 0;
    }
}

// src/maponly.rs:380-458
void find_pairs(const NamRec* fw, size_t nf, const NamRec* rv, size_t nr, float mu, float sigma, bool swap,
                std::vector<NamPairM>& out) {
    uint64_t max_dist = sat_usize(std::ceil(mu + 10.0f * sigma));
    size_t rp = 0;
    bool has_last = false;
    size_t last_id = 0;
    double prev = 0;
    for (size_t fi = 0; fi < nf; fi++) {
        const NamRec& f = fw[fi];
        while (rp < nr && (rv[rp].ref_id < f.ref_id ||
                           (rv[rp].ref_id == f.ref_id && projected_ref_start(rv[rp]) < projected_ref_start(f))))
            rp++;
        if (rp == nr) break;
        if (rv[rp].ref_id > f.ref_id) continue;
        bool hb = false;
        size_t bid = 0;
        double bs = 0;
        for (size_t i = rp; i < nr && rv[i].ref_id == f.ref_id &&
                            (uint64_t)(projected_ref_start(rv[i]) - projected_ref_start(f)) <= max_dist;
             i++) {
            uint64_t x = absdiff(f.ref_start, rv[i].ref_start);
            double sc = (double)f.score + (double)rv[i].score +
                        std::fmax(0.001, (double)std::log(normal_pdf((float)x, mu, sigma) + 1.0f));
            if (!hb || sc > bs) { hb = true; bid = i; bs = sc; }
        }
        if (!hb) continue;
        if (has_last && last_id == bid) {
            if (bs <= prev) continue;
            out.pop_back();
        }
        if (swap) out.push_back(NamPairM{rv[bid], f, bs});
        else out.push_back(NamPairM{f, rv[bid], bs});
        has_last = true;
        last_id = bid;
        prev = bs;
        rp = bid;
    }
}

std::vector<NamPairM> nam_pairs_maponly(std::vector<NamRec>& n1, std::vector<NamRec>& n2, float mu, float sigma,
                                        bool both1, bool both2) {
    std::vector<NamPairM> pairs;
    if (n1.empty() || n2.empty()) return pairs;
    NamRec *f1, *r1, *f2, *r2;
    size_t nf1, nr1, nf2, nr2;
    split_orient(n1.data(), n1.size(), both1, f1, nf1, r1, nr1);
    split_orient(n2.data(), n2.size(), both2, f2, nf2, r2, nr2);
    if (nf1 && nr2) {
        std::stable_sort(f1, f1 + nf1, nam_key_less);
        std::stable_sort(r2, r2 + nr2, nam_key_less);
        find_pairs(f1, nf1, r2, nr2, mu, sigma, false, pairs);
    }
    if (nf2 && nr1) {
        std::stable_sort(f2, f2 + nf2, nam_key_less);
        std::stable_sort(r1, r1 + nr1, nam_key_less);
        find_pairs(f2, nf2, r1, nr1, mu, sigma, true, pairs);
    }
    std::stable_sort(pairs.begin(), pairs.end(), [](const NamPairM& a, const NamPairM& b) { return a.score > b.score; });
    return pairs;
}

// the NAM lists before sort_nams, i.e. in push order (nam_id)
std::vector<NamRec> unsorted_nams(const BatchView& bv, uint32_t read) {
    std::vector<NamRec> v(bv.nams + bv.nam_off[read], bv.nams + bv.nam_off[read + 1]);
    std::sort(v.begin(), v.end(), [](const NamRec& a, const NamRec& b) { return a.nam_id < b.nam_id; });
    return v;
}

// sort_nams on a list whose current order is the pre-sort order
void sort_nams_host(std::vector<NamRec>& v, Rng& rng) {
    std::stable_sort(v.begin(), v.end(), [](const NamRec& a, const NamRec& b) { return a.score > b.score; });
    if (v.empty()) return;
    size_t nb = 0;
    while (nb < v.size() && v[nb].score == v[0].score) nb++;
    if (nb > 1)
        for (size_t i = 1; i < nb; i++) std::swap(v[i], v[(size_t)rng.gen_mod_u64(i + 1)]);
}

int best_paired_location(const std::vector<NamPairM>& pairs, const std::vector<NamRec>& n1,
                         const std::vector<NamRec>& n2, InsertSize& isd) {
    double indiv = (n1.empty() ? 0.0 : (double)n1[0].score) + (n2.empty() ? 0.0 : (double)n2[0].score);
    if (!pairs.empty() && pairs[0].score >= indiv / 2.0) {
        if (isd.sample_size < 400) isd.update(absdiff(pairs[0].n1.ref_start, pairs[0].n2.ref_start));
        return 1;
    }
    return 0;
}

}  // namespace

// src/maponly.rs:18-52
void Policy::paf_se(uint64_t rec, Rng& rng, OutBuf& out) {
    const uint32_t read = bv_->first_read(rec);
    std::vector<NamRec> nams = sorted_nams(read, rng);
    if (!nams.empty()) paf_line(*this, nams[0], bv_->reads[read], 0, mapping_quality(nams), out);
}

// src/maponly.rs:114-195
void Policy::paf_pe(uint64_t rec, Rng& rng, InsertSize& isd, OutBuf& out) {
    uint32_t a = bv_->first_read(rec), b = a + 1;
    std::vector<NamRec> n1 = unsorted_nams(*bv_, a), n2 = unsorted_nams(*bv_, b);
    if (n1.empty() && n2.empty()) return;
    std::vector<NamPairM> pairs = nam_pairs_maponly(n1, n2, isd.mu, isd.sigma, bv_->details[a].both_orientations,
                                                    bv_->details[b].both_orientations);
    sort_nams_host(n1, rng);
    sort_nams_host(n2, rng);
    if (best_paired_location(pairs, n1, n2, isd)) {
        paf_line(*this, pairs[0].n1, bv_->reads[a], 1, -1, out);
        paf_line(*this, pairs[0].n2, bv_->reads[b], 2, -1, out);
    } else {
        if (!n1.empty()) paf_line(*this, n1[0], bv_->reads[a], 1, -1, out);
        if (!n2.empty()) paf_line(*this, n2[0], bv_->reads[b], 2, -1, out);
    }
}

// src/maponly.rs:57-78
void Policy::aemb_se(uint64_t rec, Rng& rng) {
    const uint32_t read = bv_->first_read(rec);
    std::vector<NamRec> nams = sorted_nams(read, rng);
    size_t nb = 0;
    while (nb < nams.size() && nams[nb].score == nams[0].score) nb++;
    double w = (double)bv_->reads[read].len / (double)nb;
    for (size_t i = 0; i < nb; i++) add_abundance(nams[i].ref_id, w);
}

// src/maponly.rs:198-261
void Policy::aemb_pe(uint64_t rec, Rng& rng, InsertSize& isd) {
    uint32_t a = bv_->first_read(rec), b = a + 1;
    std::vector<NamRec> n1 = unsorted_nams(*bv_, a), n2 = unsorted_nams(*bv_, b);
    if (n1.empty() && n2.empty()) return;
    std::vector<NamPairM> pairs = nam_pairs_maponly(n1, n2, isd.mu, isd.sigma, bv_->details[a].both_orientations,
                                                    bv_->details[b].both_orientations);
    sort_nams_host(n1, rng);
    sort_nams_host(n2, rng);
    if (best_paired_location(pairs, n1, n2, isd)) {
        double js = pairs[0].score;
        size_t nb = 0;
        while (nb < pairs.size() && pairs[nb].score == js) nb++;
        double w1 = (double)bv_->reads[a].len / (double)nb, w2 = (double)bv_->reads[b].len / (double)nb;
        for (size_t i = 0; i < nb; i++) {
            add_abundance(pairs[i].n1.ref_id, w1);
            add_abundance(pairs[i].n2.ref_id, w2);
        }
    } else {
        const std::vector<NamRec>* lists[2] = {&n1, &n2};
        uint32_t lens[2] = {bv_->reads[a].len, bv_->reads[b].len};
        for (int t = 0; t < 2; t++) {
            const std::vector<NamRec>& n = *lists[t];
            size_t nb = 0;
            while (nb < n.size() && n[nb].score == n[0].score) nb++;
            double w = (double)lens[t] / (double)nb;
            for (size_t i = 0; i < nb; i++) add_abundance(n[i].ref_id, w);
        }
    }
}

// ------------------------------------------------------------------ chunk driver
void Policy::seed_requests(ChunkState& cs) {
    if (cfg_.mp.mode != SA_MODE_SAM) return;
    cur_ = &cs;
    const auto t0 = cfg_.timing ? std::chrono::steady_clock::now() : std::chrono::steady_clock::time_point();
    struct Acc {
        const PolicyConfig& c;
        ChunkState& cs;
        std::chrono::steady_clock::time_point t0;
        ~Acc() {
            if (c.timing) cs.seconds_seed += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
    } acc{cfg_, cs, t0};
    for (uint64_t rec = cs.first; rec < cs.end; rec++) {
        const bool paired = bv_->rec_paired(rec);
        pe_ = paired;
        for (int m = 0; m < (paired ? 2 : 1); m++) {
            const uint32_t read = bv_->first_read(rec) + m;
            const NamRec* n = bv_->nams + bv_->nam_off[read];
            size_t c = bv_->nam_off[read + 1] - bv_->nam_off[read];
            if (!c) continue;
            size_t nb = 0;
            while (nb < c && n[nb].score == n[0].score) nb++;
            size_t want_n = paired ? std::max<size_t>(nb, 1) : std::max<size_t>(nb, 2);
            want_n = std::min<size_t>(std::min<size_t>(want_n, 16), c);
            for (size_t t = 0; t < want_n; t++)
                if (n[t].score / n[0].score >= cfg_.mp.dropoff_threshold) want_nam(read, n[t], JOB_EXTEND_FAST);
        }
    }
}

void Policy::run_chunk(ChunkState& cs) {
    cur_ = &cs;
    resolve(cs);
    const bool timing = cfg_.timing;
    auto now = [] { return std::chrono::steady_clock::now(); };
    auto since = [&](std::chrono::steady_clock::time_point t) {
        return std::chrono::duration<double>(now() - t).count();
    };
    const auto t_run = timing ? now() : std::chrono::steady_clock::time_point();
    cs.runs++;
    // false: the record stopped on a missing result
    // a record with a mate is a pair (src/main.rs:886-985 matches on r2)
    auto one = [&](uint64_t rec, Rng& rng, InsertSize& isd, OutBuf& out, uint64_t& mapped) -> bool {
        pe_ = bv_->rec_paired(rec);
        switch (cfg_.mp.mode) {
            case SA_MODE_SAM:
                return pe_ ? pe_record(rec, rng, isd, out, mapped) : se_record(rec, rng, out, mapped);
            case SA_MODE_PAF:
                if (pe_) paf_pe(rec, rng, isd, out);
                else paf_se(rec, rng, out);
                return true;
            default:
                if (pe_) aemb_pe(rec, rng, isd);
                else aemb_se(rec, rng);
                return true;
        }
    };
    const bool capture = cfg_.mp.mode == SA_MODE_SAM || cfg_.mp.mode == SA_MODE_PAF;
    while (cs.next < cs.end) {
        if (capture && !cs.effects.empty()) {
            const auto& ef = cs.effects[cs.next - cs.first];
            // A record that drew nothing from the RNG took no path that depends on its
            // state (the path up to a first draw is the same under any state), so its
            // output holds under any RNG state; one that drew needs the same state.
            const bool rng_ok = ef.rng_delta == 0 || ef.pre_rng == cs.rng.state;
            const bool isd_ok = ef.pre_isd.same_state(cs.isd);
            if (ef.has_output) {
                cs.stale_rng += !rng_ok;
                cs.stale_isd += !isd_ok;
            }
            if (ef.has_output && rng_ok && isd_ok) {
                cs.add_piece(true, ef.out_off, ef.out_len);
                cs.rng.state += ef.rng_delta;
                cs.isd = ef.post_isd;
                cs.mapped += ef.mapped;
                cs.next++;
                cs.evals_reused++;
                continue;
            }
        }
        Rng rng = cs.rng;
        InsertSize isd = cs.isd;
        size_t out_len = cs.out.size(), ab_len = cs.abundance.size();
        uint64_t mapped = 0;
        const bool done_rec = one(cs.next, rng, isd, cs.out, mapped);
        if (done_rec) cs.add_piece(false, out_len, cs.out.size() - out_len);
        if (!done_rec) {
            cs.out.resize(out_len);
            cs.abundance.resize(ab_len);
            if (!cs.effects.empty()) {
                if (cs.effects[cs.next - cs.first].known) cs.miss_mispredicted++;
                else cs.miss_unknown++;
            }
            // look ahead: later reads of the chunk with the best-known state, so that
            // their requests join the next wave; after the first lookahead only the
            // reads that missed are evaluated again, the others' effect on the state
            // is replayed
            speculative_ = true;
            // the state as the real run will have it once the missing results are in:
            // the draws made before the miss, no insert-size update (only the fast
            // path updates it, and that path does not miss)
            Rng srng = rng;
            InsertSize sisd = isd;
            OutBuf scratch;
            std::vector<uint64_t> todo;
            if (cs.effects.empty()) {
                cs.effects.resize(cs.end - cs.first);
                if (capture) {
                    // room for the captured records (SEQ and QUAL plus the fixed fields)
                    uint64_t est = 0;
                    for (uint64_t rec = cs.next + 1; rec < cs.end; rec++) {
                        const uint32_t r0 = bv_->first_read(rec);
                        if (bv_->rec_paired(rec)) est += 2ull * (bv_->reads[r0].len + bv_->reads[r0 + 1].len) + 320;
                        else est += 2ull * bv_->reads[r0].len + 160;
                    }
                    cs.spec_out.reserve(est);
                }
            }
            auto visit = [&](uint64_t rec) {
                cs.evals_spec++;
                Rng r2 = srng;
                InsertSize i2 = sisd;
                uint64_t m2 = 0;
                auto& ef = cs.effects[rec - cs.first];
                const size_t o0 = cs.spec_out.size();
                speculative_ = !capture;  // when capturing, records are formatted into spec_out
                if (one(rec, r2, i2, capture ? cs.spec_out : scratch, m2)) {
                    ef.known = true;
                    ef.rng_delta = r2.state - srng.state;
                    ef.isd_update = i2.sample_size != sisd.sample_size;
                    ef.isd_value = i2.last;
                    if (capture) {
                        ef.has_output = true;
                        ef.pre_rng = srng.state;
                        ef.pre_isd = sisd;
                        ef.post_isd = i2;
                        ef.out_off = o0;
                        ef.out_len = cs.spec_out.size() - o0;
                        ef.mapped = m2;
                    }
                } else {
                    // keep the draws made before the miss; see above for the estimate
                    ef.known = false;
                    ef.has_output = false;
                    if (capture) cs.spec_out.resize(o0);
                    todo.push_back(rec);
                }
                speculative_ = true;
                srng = r2;
                sisd = i2;
            };
            const auto t_spec = timing ? now() : std::chrono::steady_clock::time_point();
            if (timing) cs.seconds_real += std::chrono::duration<double>(t_spec - t_run).count();
            if (!cs.lookahead_started) {
                for (uint64_t rec = cs.next + 1; rec < cs.end; rec++) visit(rec);
                cs.lookahead_started = true;
            } else {
                // evaluate the reads that missed last time; replay what the others did
                size_t ti = 0;
                const auto& old = cs.lookahead_todo;
                for (uint64_t rec = cs.next + 1; rec < cs.end; rec++) {
                    while (ti < old.size() && old[ti] < rec) ti++;
                    const auto& ef = cs.effects[rec - cs.first];
                    if ((ti < old.size() && old[ti] == rec) || !ef.known) {
                        visit(rec);
                    } else {
                        srng.state += ef.rng_delta;
                        if (ef.isd_update) sisd.update(ef.isd_value);
                    }
                }
            }
            if (timing) cs.seconds_spec += since(t_spec);
            cs.lookahead_todo.swap(todo);
            speculative_ = false;
            return;
        }
        cs.rng = rng;
        cs.isd = isd;
        cs.mapped += mapped;
        cs.next++;
        cs.evals_real++;
    }
    if (timing) cs.seconds_real += since(t_run);
    cs.done = true;
    if (cs.keep_buffers) {
        cs.effects.clear();
        cs.entries.clear();
    } else {
        std::vector<ChunkState::Effect>().swap(cs.effects);
        std::vector<ResultStore::Entry>().swap(cs.entries);
    }
}

}  // namespace sa
