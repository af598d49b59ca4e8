// Oracle (test infrastructure only): single-end / paired-end mapping policy and
// SAM/PAF record formatting.  Restates src/mapper.rs, src/maponly.rs,
// src/insertsize.rs, src/math.rs, src/io/sam.rs, src/io/paf.rs, src/nam.rs:49-135.
#include "oracle.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <unordered_set>

namespace oracle {

static constexpr uint16_t PAIRED = 1, PROPER_PAIR = 2, UNMAP = 4, MUNMAP = 8, REVERSE = 0x10, MREVERSE = 0x20,
                          READ1 = 0x40, READ2 = 0x80, SECONDARY = 0x100;

// Rust `f as u8` / `f as usize`: saturating, NaN -> 0
static inline uint8_t sat_u8(float f) {
    if (!(f == f) || f <= 0.0f) return 0;
    if (f >= 255.0f) return 255;
    return (uint8_t)f;
}
static inline size_t sat_usize(float f) {
    if (!(f == f) || f <= 0.0f) return 0;
    if (f >= 1.8446744e19f) return SIZE_MAX;
    return (size_t)f;
}

// src/math.rs:3-7
static float normal_pdf(float x, float mu, float sigma) {
    const double INV_SQRT_PI = 0.3989422804014327;
    float a = (x - mu) / sigma;
    return (float)INV_SQRT_PI / sigma * std::exp(-0.5f * a * a);
}

// src/insertsize.rs:29-49
void InsertSizeDistribution::update(size_t insert_size) {
    if (insert_size >= 2000) return;
    if (sample_size > 0) {
        float x = (float)insert_size;
        float e = x - mu;
        mu += e / (float)sample_size;
        sse += e * (x - mu);
        if (sample_size > 1) variance = sse / ((float)sample_size - 1.0f);
        else variance = sse;
        sigma = std::sqrt(variance);
    }
    sample_size++;
}

struct Read {
    const std::string& seq;
    std::string rc;
    explicit Read(const std::string& s) : seq(s), rc(reverse_complement(s)) {}
    size_t len() const { return seq.size(); }
};

// src/nam.rs:49-69
static bool is_consistent(const Nam& nam, const Read& read, const std::vector<RefSeq>& refs, size_t k) {
    const PackedSeq& r = refs[nam.ref_id].seq;
    const std::string& s = nam.is_revcomp ? read.rc : read.seq;
    for (size_t i = 0; i < k; i++)
        if (r.decode_at(nam.ref_start + i) != s[nam.query_start + i]) return false;
    for (size_t i = 0; i < k; i++)
        if (r.decode_at(nam.ref_end - k + i) != s[nam.query_end - k + i]) return false;
    return true;
}

// src/nam.rs:90-135
static bool reverse_nam_if_needed(Nam& nam, const Read& read, const std::vector<RefSeq>& refs, size_t k) {
    if (is_consistent(nam, read, refs, k)) return true;
    const PackedSeq& r = refs[nam.ref_id].seq;
    const std::string& seq_rc = nam.is_revcomp ? read.seq : read.rc;
    size_t qs = read.len() - nam.query_end, qe = read.len() - nam.query_start;
    for (size_t i = 0; i < k; i++)
        if (r.decode_at(nam.ref_start + i) != seq_rc[qs + i]) return false;
    for (size_t i = 0; i < k; i++)
        if (r.decode_at(nam.ref_end - k + i) != seq_rc[qe - k + i]) return false;
    nam.is_revcomp = !nam.is_revcomp;
    nam.query_start = qs;
    nam.query_end = qe;
    return true;
}

struct Alignment {
    size_t reference_id = 0, ref_start = 0;
    Cigar cigar;
    size_t edit_distance = 0, soft_clip_left = 0, soft_clip_right = 0;
    uint32_t score = 0;
    size_t length = 0;
    bool is_revcomp = false, gapped = false;
    size_t global_edit_distance() const { return edit_distance + soft_clip_left + soft_clip_right; }
};

// src/mapper.rs:532-620
static std::optional<Alignment> extend_seed(const Context& ctx, Nam& nam, const Read& read, bool consistent,
                                            bool use_ssw) {
    const std::string& query = nam.is_revcomp ? read.rc : read.seq;
    const PackedSeq& refseq = (*ctx.refs)[nam.ref_id].seq;
    size_t prs = nam.projected_ref_start();
    size_t pre = std::min(nam.ref_end + query.size() - nam.query_end, refseq.len);
    AlignmentInfo info;
    size_t result_ref_start = 0;
    bool gapped = true;
    if (prs + query.size() == pre && consistent) {
        std::string seg = refseq.decode(prs, pre);
        uint32_t hd = 0;
        for (size_t i = 0; i < query.size(); i++) hd += query[i] != seg[i];
        if ((float)hd / (float)query.size() < 0.05f) {
            info = *hamming_align(query, seg, ctx.sc.match, ctx.sc.mismatch, ctx.sc.end_bonus);
            result_ref_start = prs + info.ref_start;
            gapped = false;
        }
    }
    if (gapped) {
        size_t padding = read.len() / 10;
        if (use_ssw) {
            size_t rs = prs > padding ? prs - padding : 0;
            size_t re = std::min(pre + padding, refseq.len);
            std::string seg = refseq.decode(rs, re);
            std::optional<AlignmentInfo> oi = aligner_align(query, seg, ctx.sc);
            if (!oi) return std::nullopt;
            info = *oi;
            result_ref_start = rs + info.ref_start;
        } else {
            remove_spurious_anchors(nam.anchors);
            size_t ds = nam.ref_start > query.size() + padding ? nam.ref_start - (query.size() + padding) : 0;
            size_t de = std::min(nam.ref_end + query.size() + padding, refseq.len);
            std::string dref = refseq.decode(ds, de);
            std::vector<Anchor> adj;
            for (auto& a : nam.anchors) adj.push_back(Anchor{a.ref_id, a.ref_start - ds, a.query_start});
            std::optional<AlignmentInfo> oi =
                extend_piecewise(query, dref, adj, padding, ctx.index->params.k, ctx.sc, ctx.mp.xdrop);
            if (!oi) return std::nullopt;
            info = *oi;
            result_ref_start = info.ref_start + ds;
        }
    }
    Alignment a;
    a.cigar = info.cigar;
    a.edit_distance = info.edit_distance;
    a.soft_clip_left = info.query_start;
    a.soft_clip_right = query.size() - info.query_end;
    a.score = info.score;
    a.ref_start = result_ref_start;
    a.length = info.ref_end - info.ref_start;
    a.is_revcomp = nam.is_revcomp;
    a.reference_id = nam.ref_id;
    a.gapped = gapped;
    return a;
}

// ------------------------------------------------------------------ SAM records
struct SamRecord {
    std::string query_name;
    uint16_t flags = 0;
    const std::string* reference_name = nullptr;
    bool has_pos = false;
    uint32_t pos = 0;
    uint8_t mapq = 0;
    bool has_cigar = false;
    Cigar cigar;
    const std::string* mate_reference_name = nullptr;
    bool has_mate_pos = false;
    uint32_t mate_pos = 0;
    bool has_tlen = false;
    int32_t tlen = 0;
    const std::string* seq = nullptr;
    std::string seq_rc;
    bool seq_is_rc = false;
    const std::string* qual = nullptr;
    bool qual_rev = false;
    bool has_nm = false;
    uint32_t nm = 0;
    bool has_as = false;
    uint32_t as = 0;
    bool has_details = false;
    Details details;
    const std::string* rg_id = nullptr;
    const std::string* extra = nullptr;
    bool is_mapped() const { return (flags & UNMAP) == 0; }
};

static const std::string EQUALS = "=";

// src/io/sam.rs:53-138
static void format_sam(const SamRecord& r, std::string& out) {
    bool secondary = (r.flags & SECONDARY) != 0;
    out += r.query_name;
    out += '\t';
    out += std::to_string(r.flags);
    out += '\t';
    out += r.reference_name ? *r.reference_name : "*";
    out += '\t';
    out += std::to_string(r.has_pos ? (uint64_t)r.pos + 1 : 0);
    out += '\t';
    out += std::to_string(r.mapq);
    out += '\t';
    out += r.has_cigar ? r.cigar.str() : "*";
    out += '\t';
    out += r.mate_reference_name ? *r.mate_reference_name : "*";
    out += '\t';
    out += std::to_string(r.has_mate_pos ? (uint64_t)r.mate_pos + 1 : 0);
    out += '\t';
    out += std::to_string(r.has_tlen ? r.tlen : 0);
    out += '\t';
    const std::string* seq = r.seq_is_rc ? &r.seq_rc : r.seq;
    if (seq && !secondary && !seq->empty()) out += *seq;
    else out += '*';
    out += '\t';
    if (r.qual && !secondary && !r.qual->empty()) {
        if (r.qual_rev) out.append(r.qual->rbegin(), r.qual->rend());
        else out += *r.qual;
    } else {
        out += '*';
    }
    if (r.has_nm) { out += "\tNM:i:"; out += std::to_string(r.nm); }
    if (r.has_as) { out += "\tAS:i:"; out += std::to_string(r.as); }
    if (r.has_details) {
        out += "\tna:i:" + std::to_string(r.details.nam.n_nams) + "\tal:i:" + std::to_string(r.details.tried_alignment) +
               "\tga:i:" + std::to_string(r.details.gapped) + "\tX0:i:" + std::to_string(r.details.best_alignments);
        if (r.flags & PAIRED) out += "\tmr:i:" + std::to_string(r.details.mate_rescue);
    }
    if (r.rg_id) { out += "\tRG:Z:"; out += *r.rg_id; }
    if (r.extra) { out += '\t'; out += *r.extra; }
    out += '\n';
}

// src/mapper.rs:138-204
static SamRecord make_mapped_record(const Context& ctx, const Alignment& a, const SequenceRecord& rec, uint8_t mapq,
                                    bool secondary, const Details& det) {
    SamRecord r;
    r.query_name = rec.name;
    if (a.is_revcomp) r.flags |= REVERSE;
    if (secondary) { mapq = 0; r.flags |= SECONDARY; }
    if (a.is_revcomp) { r.seq_rc = reverse_complement(rec.seq); r.seq_is_rc = true; }
    else r.seq = &rec.seq;
    if (rec.has_qual) { r.qual = &rec.qual; r.qual_rev = a.is_revcomp; }
    Cigar c;
    c.push(OP_S, a.soft_clip_left);
    c.extend(a.cigar);
    c.push(OP_S, a.soft_clip_right);
    r.reference_name = &(*ctx.refs)[a.reference_id].name;
    r.has_cigar = true;
    r.cigar = ctx.so.eqx ? c : c.with_m();
    if (ctx.so.fastq_comments && rec.has_comment) r.extra = &rec.comment;
    r.has_pos = true;
    r.pos = (uint32_t)a.ref_start;
    r.mapq = mapq;
    r.has_nm = true;
    r.nm = (uint32_t)a.edit_distance;
    r.has_as = true;
    r.as = a.score;
    if (ctx.so.details) { r.has_details = true; r.details = det; }
    if (ctx.so.has_rg) r.rg_id = &ctx.so.rg_id;
    return r;
}

// src/mapper.rs:206-223
static SamRecord make_unmapped_record(const Context& ctx, const SequenceRecord& rec, const Details& det) {
    SamRecord r;
    r.query_name = rec.name;
    r.flags = UNMAP;
    r.seq = &rec.seq;
    if (rec.has_qual) r.qual = &rec.qual;
    if (ctx.so.details) { r.has_details = true; r.details = det; }
    if (ctx.so.has_rg) r.rg_id = &ctx.so.rg_id;
    if (ctx.so.fastq_comments && rec.has_comment) r.extra = &rec.comment;
    return r;
}

// src/mapper.rs:239-345
static std::vector<SamRecord> make_paired_records(const Context& ctx, const Alignment* al[2],
                                                  const SequenceRecord* recs[2], const uint8_t mapq[2],
                                                  const Details det[2], bool secondary, bool proper) {
    std::vector<SamRecord> s;
    for (int i = 0; i < 2; i++)
        s.push_back(al[i] ? make_mapped_record(ctx, *al[i], *recs[i], mapq[i], secondary, det[i])
                          : make_unmapped_record(ctx, *recs[i], det[i]));
    s[0].flags |= READ1;
    s[1].flags |= READ2;
    const std::vector<RefSeq>& refs = *ctx.refs;
    for (int i = 0; i < 2; i++) {
        s[i].flags |= PAIRED;
        if (proper) s[i].flags |= PROPER_PAIR;
        const Alignment* mate = al[1 - i];
        if (mate) {
            if (mate->is_revcomp) s[i].flags |= MREVERSE;
            s[i].has_mate_pos = true;
            s[i].mate_pos = (uint32_t)mate->ref_start;
            s[i].mate_reference_name = &refs[mate->reference_id].name;
            if (al[i]) {
                const Alignment* self = al[i];
                if (self->reference_id == mate->reference_id) {
                    s[i].mate_reference_name = &EQUALS;
                    int64_t tl;
                    if (mate->ref_start > self->ref_start) tl = (int64_t)(mate->ref_start - self->ref_start + mate->length);
                    else if (self->ref_start > mate->ref_start)
                        tl = -(int64_t)(self->ref_start - mate->ref_start + self->length);
                    else if (i == 0) tl = -(int64_t)mate->length;
                    else tl = (int64_t)self->length;
                    s[i].has_tlen = true;
                    s[i].tlen = (int32_t)tl;
                }
            } else {
                s[i].mate_reference_name = &EQUALS;
                s[i].reference_name = &refs[mate->reference_id].name;
                s[i].has_pos = true;
                s[i].pos = (uint32_t)mate->ref_start;
            }
        } else {
            s[i].flags |= MUNMAP;
            if (al[i]) {
                s[i].mate_reference_name = &EQUALS;
                s[i].has_mate_pos = true;
                s[i].mate_pos = (uint32_t)al[i]->ref_start;
            }
        }
    }
    if (secondary) {
        if (!s[1].is_mapped()) s.pop_back();
        else if (!s[0].is_mapped()) { s[0] = std::move(s[1]); s.pop_back(); }
    }
    return s;
}

// ------------------------------------------------------------------ single end
// src/mapper.rs:349-528
std::string align_single_end_read(const SequenceRecord& rec, const Context& ctx, Rng& rng, Details& det) {
    std::string out;
    NamDetails nd;
    std::vector<Nam> nams = get_nams_by_chaining(rec.seq, *ctx.index, ctx.cp, ctx.mp.rescue_distance, ctx.mp.mcs, nd);
    sort_nams(nams, rng);
    Details details;
    details.nam = nd;
    if (nams.empty()) {
        SamRecord r = make_unmapped_record(ctx, rec, details);
        if (ctx.mp.output_unmapped) format_sam(r, out);
        det = details;
        return out;
    }
    std::vector<Alignment> alignments;
    float nam_max_score = nams[0].score;
    size_t best_edit = SIZE_MAX;
    uint32_t best_score = 0, second = 0;
    size_t best_index = 0;
    uint32_t n_best = 0;
    std::optional<Alignment> best;
    const size_t k = ctx.index->params.k;
    Read read(rec.seq);
    for (size_t tries = 0; tries < nams.size() && tries < ctx.mp.max_tries; tries++) {
        Nam& nam = nams[tries];
        float dropoff = nam.score / nam_max_score;
        if ((tries > 1 && best_edit == 0) || dropoff < ctx.mp.dropoff_threshold) break;
        bool consistent = is_consistent(nam, read, *ctx.refs, k);
        if (!consistent) {
            details.inconsistent_nams++;
            continue;
        }
        std::optional<Alignment> oa = extend_seed(ctx, nam, read, consistent, ctx.mp.use_ssw);
        if (!oa) continue;
        Alignment& a = *oa;
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
                if (rng.u32_below(n_best) == 0) update = true;
            }
            if (update) {
                best_score = a.score;
                best = a;
                best_index = alignments.size();
                if (ctx.mp.max_secondary == 0) best_edit = a.global_edit_distance();
            }
        } else if (a.score > second) {
            second = a.score;
        }
        if (ctx.mp.max_secondary > 0) alignments.push_back(a);
    }
    if (!best) {
        SamRecord r = make_unmapped_record(ctx, rec, details);
        if (ctx.mp.output_unmapped) format_sam(r, out);
        det = details;
        return out;
    }
    uint8_t mapq = (uint8_t)((60 * (best_score - second) + best_score - 1) / best_score);
    format_sam(make_mapped_record(ctx, *best, rec, mapq, false, details), out);
    if (ctx.mp.max_secondary > 0) {
        // Vec::swap_remove, then a stable sort by score descending (src/mapper.rs:500-524)
        alignments[best_index] = alignments.back();
        alignments.pop_back();
        std::stable_sort(alignments.begin(), alignments.end(),
                         [](const Alignment& a, const Alignment& b) { return a.score > b.score; });
        uint32_t lim = 2u * ctx.sc.mismatch + ctx.sc.gap_open;
        for (size_t t = 0; t < alignments.size() && t < ctx.mp.max_secondary; t++) {
            const Alignment& a = alignments[t];
            uint32_t d = a.score > best_score ? a.score - best_score : 0;
            if (d > lim) break;
            format_sam(make_mapped_record(ctx, a, rec, mapq, true, details), out);
        }
    }
    det = details;
    return out;
}

// ------------------------------------------------------------------ paired end
struct ScoredAlignmentPair {
    double score;
    std::optional<Alignment> a1, a2;
};

struct NamPair {
    float score;
    std::optional<Nam> n1, n2;
};

// src/mapper.rs:1200-1218
static bool is_proper_nam_pair(const Nam& n1, const Nam& n2, float mu, float sigma) {
    if (n1.ref_id != n2.ref_id || n1.is_revcomp == n2.is_revcomp) return false;
    size_t r1 = n1.projected_ref_start(), r2 = n2.projected_ref_start();
    float lim = mu + 10.0f * sigma;
    bool r1_r2 = n2.is_revcomp && r1 <= r2 && (float)(r2 - r1) < lim;
    bool r2_r1 = n1.is_revcomp && r2 <= r1 && (float)(r1 - r2) < lim;
    return r1_r2 || r2_r1;
}

// src/mapper.rs:1180-1197
static bool is_proper_pair(const Alignment& a1, const Alignment& a2, float mu, float sigma) {
    int64_t dist = (int64_t)a2.ref_start - (int64_t)a1.ref_start;
    bool same = a1.reference_id == a2.reference_id;
    bool r1_r2 = !a1.is_revcomp && a2.is_revcomp && dist >= 0;
    bool r2_r1 = !a2.is_revcomp && a1.is_revcomp && dist <= 0;
    bool insert_good = (size_t)(dist < 0 ? -dist : dist) <= sat_usize(mu + sigma * 6.0f);
    return same && insert_good && (r1_r2 || r2_r1);
}

static bool is_proper_pair_opt(const std::optional<Alignment>& a1, const std::optional<Alignment>& a2, float mu,
                               float sigma) {
    if (!a1 || !a2) return false;
    return is_proper_pair(*a1, *a2, mu, sigma);
}

// src/mapper.rs:1224-1299
static std::vector<NamPair> get_best_scoring_nam_pairs(const std::vector<Nam>& n1, const std::vector<Nam>& n2, float mu,
                                                       float sigma) {
    std::vector<NamPair> pairs;
    if (n1.empty() && n2.empty()) return pairs;
    std::unordered_set<size_t> added1, added2;
    size_t best_joint = 0;
    for (size_t a = 0; a < n1.size() && a < 1000; a++) {
        for (size_t b = 0; b < n2.size() && b < 1000; b++) {
            size_t joint = n1[a].anchors.size() + n2[b].anchors.size();
            if (joint < best_joint / 2) break;
            if (is_proper_nam_pair(n1[a], n2[b], mu, sigma)) {
                pairs.push_back(NamPair{n1[a].score + n2[b].score, n1[a], n2[b]});
                added1.insert(n1[a].nam_id);
                added2.insert(n2[b].nam_id);
                best_joint = std::max(joint, best_joint);
            }
        }
    }
    if (!n1.empty()) {
        size_t bj = best_joint > 0 ? best_joint : n1[0].anchors.size();
        for (auto& n : n1) {
            if (n.anchors.size() < bj / 2) break;
            if (added1.count(n.nam_id)) continue;
            pairs.push_back(NamPair{n.score, n, std::nullopt});
        }
    }
    if (!n2.empty()) {
        size_t bj = best_joint > 0 ? best_joint : n2[0].anchors.size();
        for (auto& n : n2) {
            if (n.anchors.size() < bj / 2) break;
            if (added2.count(n.nam_id)) continue;
            pairs.push_back(NamPair{n.score, std::nullopt, n});
        }
    }
    std::stable_sort(pairs.begin(), pairs.end(), [](const NamPair& a, const NamPair& b) { return a.score > b.score; });
    return pairs;
}

// src/mapper.rs:1302-1313
static uint8_t mapping_quality(const std::vector<Nam>& nams) {
    if (nams.size() <= 1) return 60;
    float s1 = nams[0].score, s2 = nams[1].score;
    float mm = (float)std::min<size_t>(nams[0].anchors.size(), 10) / 10.0f;
    float u = 40.0f * (1.0f - s2 / s1) * mm * std::log(s1);
    return sat_u8(std::fmin(u, 60.0f));
}

// src/mapper.rs:1440-1458
static uint8_t alignment_quality(const std::vector<ScoredAlignmentPair>& items) {
    if (items.size() <= 1) return 60;
    float s1 = (float)items[0].score, s2 = (float)items[1].score;
    if (s1 > 0.0f && s2 > 0.0f) return sat_u8(std::fmin(s1 - s2, 60.0f));
    if (s1 > 0.0f && s2 <= 0.0f) return 60;
    return 1;
}

// src/mapper.rs:1461-1470
static float top_dropoff(const std::vector<Nam>& nams) {
    const Nam& m = nams[0];
    if (m.anchors.size() <= 2) return 1.0f;
    if (nams.size() > 1) return (float)nams[1].anchors.size() / (float)m.anchors.size();
    return 0.0f;
}

// src/mapper.rs:1157-1168
bool has_shared_substring(const std::string& read, const std::string& ref, size_t k) {
    size_t sub = 2 * k / 3, step = k / 3;
    size_t lim = read.size() > sub ? read.size() - sub : 0;
    for (size_t i = 0; i < lim; i += step) {
        if (sub == 0) return true;
        if (ref.size() >= sub) {
            const char* hay = ref.data();
            const char* hit = (const char*)memmem(hay, ref.size(), read.data() + i, sub);
            if (hit) return true;
        }
        if (step == 0) break;
    }
    return false;
}

// src/mapper.rs:1094-1153
static std::optional<Alignment> rescue_align(const Context& ctx, const Nam& mate, const Read& read, float mu,
                                             float sigma, size_t k) {
    size_t rl = read.len();
    const std::string* r_tmp;
    size_t rs, re;
    size_t w = sat_usize(mu + 5.0f * sigma);
    if (mate.is_revcomp) {
        r_tmp = &read.seq;
        size_t p = mate.projected_ref_start();
        rs = p > w ? p - w : 0;
        re = p + rl / 2;
    } else {
        r_tmp = &read.rc;
        size_t b = mate.ref_end + rl - mate.query_end;
        rs = b > rl / 2 ? b - rl / 2 : 0;
        re = b + w;
    }
    const PackedSeq& ref = (*ctx.refs)[mate.ref_id].seq;
    rs = std::min(rs, ref.len);
    re = std::min(re, ref.len);
    if (re < rs + k) return std::nullopt;
    std::string seg = ref.decode(rs, re);
    if (!has_shared_substring(*r_tmp, seg, k)) return std::nullopt;
    std::optional<AlignmentInfo> oi = aligner_align(*r_tmp, seg, ctx.sc);
    if (!oi) return std::nullopt;
    Alignment a;
    a.reference_id = mate.ref_id;
    a.ref_start = rs + oi->ref_start;
    a.edit_distance = oi->edit_distance;
    a.soft_clip_left = oi->query_start;
    a.soft_clip_right = rl - oi->query_end;
    a.score = oi->score;
    a.length = oi->ref_end - oi->ref_start;
    a.cigar = oi->cigar;
    a.is_revcomp = !mate.is_revcomp;
    a.gapped = true;
    return a;
}

// src/mapper.rs:1018-1091
static std::vector<ScoredAlignmentPair> rescue_read(const Context& ctx, const Read& read2, const Read& read1,
                                                    std::vector<Nam>& nams1, Details det[2], size_t k, float mu,
                                                    float sigma) {
    float max1 = nams1[0].score;
    std::vector<Alignment> al1;
    std::vector<std::optional<Alignment>> al2;
    for (size_t t = 0; t < nams1.size() && t < ctx.mp.max_tries; t++) {
        Nam& nam = nams1[t];
        if (nam.score / max1 < ctx.mp.dropoff_threshold) break;
        bool consistent = reverse_nam_if_needed(nam, read1, *ctx.refs, k);
        det[0].inconsistent_nams += !consistent;
        std::optional<Alignment> a = extend_seed(ctx, nam, read1, consistent, true);
        if (a) {
            det[0].gapped += a->gapped;
            al1.push_back(*a);
            det[0].tried_alignment++;
            std::optional<Alignment> b = rescue_align(ctx, nam, read2, mu, sigma, k);
            if (b) det[1].mate_rescue++;
            al2.push_back(b);
        }
    }
    std::vector<ScoredAlignmentPair> pairs;
    for (auto& a1 : al1) {
        for (auto& a2 : al2) {
            if (a2) {
                size_t dist = a1.ref_start > a2->ref_start ? a1.ref_start - a2->ref_start : a2->ref_start - a1.ref_start;
                float score = (float)(a1.score + a2->score);
                if ((a1.is_revcomp ^ a2->is_revcomp) && (float)dist < mu + 4.0f * sigma)
                    score += std::log(normal_pdf((float)dist, mu, sigma));
                else
                    score -= 10.0f;
                pairs.push_back(ScoredAlignmentPair{(double)score, a1, a2});
            } else {
                pairs.push_back(ScoredAlignmentPair{(double)a1.score - 10.0, a1, std::nullopt});
            }
        }
    }
    return pairs;
}

// src/mapper.rs:1322-1352
static void deduplicate_scored_pairs(std::vector<ScoredAlignmentPair>& p) {
    if (p.size() < 2) return;
    auto same = [](const std::optional<Alignment>& a, const std::optional<Alignment>& b) {
        if (!a && !b) return true;
        if (!a || !b) return false;
        return a->ref_start == b->ref_start && a->reference_id == b->reference_id;
    };
    size_t k = 0, j = 1;
    for (size_t i = 1; i < p.size(); i++) {
        if (!same(p[k].a1, p[i].a1) || !same(p[k].a2, p[i].a2)) {
            p[j] = p[i];
            j++;
            k = i;
        }
    }
    p.resize(j);
}

// src/mapper.rs:1360-1369: the pairs that share the first (best) score of a sorted list
static size_t count_best_alignment_pairs(const std::vector<ScoredAlignmentPair>& p) {
    size_t nb = 0;
    while (nb < p.size() && p[nb].score == p[0].score) nb++;
    return nb;
}

// src/mapper.rs:778-1014 (returns true for the Proper fast path)
static bool extend_paired_seeds(const Context& ctx, std::vector<Nam> nams[2], const Read& read1, const Read& read2,
                                size_t k, Details det[2], const InsertSizeDistribution& isd, Alignment proper[2],
                                std::vector<ScoredAlignmentPair>& out) {
    const float mu = isd.mu, sigma = isd.sigma, dropoff = ctx.mp.dropoff_threshold;
    const size_t max_tries = ctx.mp.max_tries;
    out.clear();
    if (nams[0].empty() && nams[1].empty()) return false;
    if (!nams[0].empty() && nams[1].empty()) {
        out = rescue_read(ctx, read2, read1, nams[0], det, k, mu, sigma);
        return false;
    }
    if (nams[0].empty() && !nams[1].empty()) {
        Details sw[2] = {det[1], det[0]};
        out = rescue_read(ctx, read1, read2, nams[1], sw, k, mu, sigma);
        det[0] = sw[1];
        det[1] = sw[0];
        for (auto& p : out) std::swap(p.a1, p.a2);
        return false;
    }
    if (top_dropoff(nams[0]) < dropoff && top_dropoff(nams[1]) < dropoff &&
        is_proper_nam_pair(nams[0][0], nams[1][0], mu, sigma)) {
        Nam m1 = nams[0][0], m2 = nams[1][0];
        bool c1 = is_consistent(m1, read1, *ctx.refs, k);
        det[0].inconsistent_nams += !c1;
        bool c2 = is_consistent(m2, read2, *ctx.refs, k);
        det[1].inconsistent_nams += !c2;
        std::optional<Alignment> a1 = extend_seed(ctx, m1, read1, c1, true);
        std::optional<Alignment> a2 = extend_seed(ctx, m2, read2, c2, true);
        if (a1 && a2) {
            det[0].tried_alignment++;
            det[0].gapped += a1->gapped;
            det[1].tried_alignment++;
            det[1].gapped += a2->gapped;
            proper[0] = *a1;
            proper[1] = *a2;
            return true;
        }
    }
    const Read* reads[2] = {&read1, &read2};
    std::unordered_map<size_t, std::optional<Alignment>> cache[2];
    std::optional<Alignment> indv[2];
    for (int i = 0; i < 2; i++) {
        bool c = reverse_nam_if_needed(nams[i][0], *reads[i], *ctx.refs, k);
        det[i].inconsistent_nams += !c;
        indv[i] = extend_seed(ctx, nams[i][0], *reads[i], c, true);
        det[i].tried_alignment++;
        det[i].gapped += indv[i] ? indv[i]->gapped : 0;
        cache[i][nams[i][0].nam_id] = indv[i];
    }
    std::vector<NamPair> np = get_best_scoring_nam_pairs(nams[0], nams[1], mu, sigma);
    float max_score = np[0].score;
    for (auto& pair : np) {
        float sd = pair.score / max_score;
        if (out.size() >= max_tries || sd < dropoff) break;
        std::optional<Nam>* namsp[2] = {&pair.n1, &pair.n2};
        std::optional<Alignment> al[2];
        for (int i = 0; i < 2; i++) {
            std::optional<Alignment> a;
            if (*namsp[i]) {
                Nam this_nam = **namsp[i];
                auto it = cache[i].find(this_nam.nam_id);
                if (it == cache[i].end()) {
                    bool c = reverse_nam_if_needed(this_nam, *reads[i], *ctx.refs, k);
                    det[i].inconsistent_nams += !c;
                    a = extend_seed(ctx, this_nam, *reads[i], c, true);
                    det[i].tried_alignment++;
                    det[i].gapped += a ? a->gapped : 0;
                    cache[i][this_nam.nam_id] = a;
                } else {
                    a = it->second;
                }
            } else {
                Nam other = **namsp[1 - i];
                det[1 - i].inconsistent_nams += !reverse_nam_if_needed(other, *reads[1 - i], *ctx.refs, k);
                a = rescue_align(ctx, other, *reads[i], mu, sigma, k);
                if (a) {
                    det[i].mate_rescue++;
                    det[i].tried_alignment++;
                }
            }
            if ((a ? a->score : 0) > (indv[i] ? indv[i]->score : 0)) indv[i] = a;
            al[i] = a;
        }
        if (!al[0] || !al[1]) continue;
        const Alignment& a1 = *al[0];
        const Alignment& a2 = *al[1];
        size_t lim = sat_usize(mu + 10.0f * sigma);
        bool r1_r2 = a2.is_revcomp && !a1.is_revcomp && a1.ref_start <= a2.ref_start && (a2.ref_start - a1.ref_start) < lim;
        bool r2_r1 = a1.is_revcomp && !a2.is_revcomp && a2.ref_start <= a1.ref_start && (a1.ref_start - a2.ref_start) < lim;
        double combined;
        if (r1_r2 || r2_r1) {
            size_t x = a1.ref_start > a2.ref_start ? a1.ref_start - a2.ref_start : a2.ref_start - a1.ref_start;
            double lp = (double)std::log(normal_pdf((float)x, mu, sigma));
            combined = (double)a1.score + (double)a2.score + std::fmax(-20.0 + 0.001, lp);
        } else {
            combined = (double)a1.score + (double)a2.score - 20.0;
        }
        out.push_back(ScoredAlignmentPair{combined, a1, a2});
    }
    if (indv[0] && indv[1]) {
        out.push_back(ScoredAlignmentPair{(double)indv[0]->score + (double)indv[1]->score - 20.0, indv[0], indv[1]});
    }
    return false;
}

// src/mapper.rs:1365-1437
static void aligned_pairs_to_sam(const Context& ctx, const std::vector<ScoredAlignmentPair>& hs,
                                 const SequenceRecord* recs[2], float mu, float sigma, const Details det[2],
                                 const uint8_t mapqs[2], std::vector<SamRecord>& records) {
    if (hs.empty()) {
        for (int i = 0; i < 2; i++) records.push_back(make_unmapped_record(ctx, *recs[i], det[i]));
        records[records.size() - 2].flags |= PAIRED | READ1 | MUNMAP;
        records[records.size() - 1].flags |= PAIRED | READ2 | MUNMAP;
        return;
    }
    const ScoredAlignmentPair& best = hs[0];
    double secondary_dropoff = 2.0 * ctx.sc.mismatch + ctx.sc.gap_open;
    if (ctx.mp.max_secondary == 0) {
        const Alignment* al[2] = {best.a1 ? &*best.a1 : nullptr, best.a2 ? &*best.a2 : nullptr};
        bool proper = is_proper_pair_opt(best.a1, best.a2, mu, sigma);
        for (auto& r : make_paired_records(ctx, al, recs, mapqs, det, false, proper)) records.push_back(std::move(r));
    } else {
        bool secondary = false;
        double s_max = best.score;
        for (size_t t = 0; t < hs.size() && t < ctx.mp.max_secondary; t++) {
            const ScoredAlignmentPair& p = hs[t];
            if (s_max - p.score < secondary_dropoff) {
                bool proper = is_proper_pair_opt(p.a1, p.a2, mu, sigma);
                uint8_t zero[2] = {0, 0};
                const Alignment* al[2] = {p.a1 ? &*p.a1 : nullptr, p.a2 ? &*p.a2 : nullptr};
                for (auto& r : make_paired_records(ctx, al, recs, secondary ? zero : mapqs, det, secondary, proper))
                    records.push_back(std::move(r));
            } else {
                break;
            }
            secondary = true;
        }
    }
}

// src/mapper.rs:624-768
std::string align_paired_end_read(const SequenceRecord& r1, const SequenceRecord& r2, const Context& ctx,
                                  InsertSizeDistribution& isd, Rng& rng, Details& det_out) {
    Details det[2];
    std::vector<Nam> nams[2];
    const SequenceRecord* recs[2] = {&r1, &r2};
    for (int i = 0; i < 2; i++) {
        NamDetails nd;
        nams[i] = get_nams_by_chaining(recs[i]->seq, *ctx.index, ctx.cp, ctx.mp.rescue_distance, ctx.mp.mcs, nd);
        sort_nams(nams[i], rng);
        det[i].nam = nd;
    }
    Read read1(r1.seq), read2(r2.seq);
    Alignment proper[2];
    std::vector<ScoredAlignmentPair> pairs;
    bool is_proper_fast =
        extend_paired_seeds(ctx, nams, read1, read2, ctx.index->params.k, det, isd, proper, pairs);
    std::vector<SamRecord> records;
    if (is_proper_fast) {
        bool ps = is_proper_pair(proper[0], proper[1], isd.mu, isd.sigma);
        if (ps && isd.sample_size < 400 && proper[0].edit_distance + proper[1].edit_distance < 3) {
            size_t a = proper[0].ref_start, b = proper[1].ref_start;
            isd.update(a > b ? a - b : b - a);
        }
        uint8_t mapq[2] = {mapping_quality(nams[0]), mapping_quality(nams[1])};
        det[0].best_alignments = 1;
        det[1].best_alignments = 1;
        const Alignment* al[2] = {&proper[0], &proper[1]};
        records = make_paired_records(ctx, al, recs, mapq, det, false, ps);
    } else {
        std::stable_sort(pairs.begin(), pairs.end(),
                         [](const ScoredAlignmentPair& a, const ScoredAlignmentPair& b) { return a.score > b.score; });
        deduplicate_scored_pairs(pairs);
        const size_t nb = count_best_alignment_pairs(pairs);
        det[0].best_alignments = nb;
        det[1].best_alignments = nb;
        if (nb > 1) {
            size_t ri = rng.usize_below(nb);
            std::swap(pairs[0], pairs[ri]);
        }
        uint8_t mapqs[2];
        if (pairs.size() == 1 && !is_proper_pair_opt(pairs[0].a1, pairs[0].a2, isd.mu, isd.sigma)) {
            mapqs[0] = mapping_quality(nams[0]);
            mapqs[1] = mapping_quality(nams[1]);
        } else {
            uint8_t j = alignment_quality(pairs);
            mapqs[0] = mapqs[1] = j;
        }
        aligned_pairs_to_sam(ctx, pairs, recs, isd.mu, isd.sigma, det, mapqs, records);
    }
    std::string out;
    bool any_mapped = false;
    for (auto& r : records) any_mapped |= r.is_mapped();
    if (!ctx.mp.output_unmapped && !records[0].is_mapped() && !records[1].is_mapped()) records.clear();
    (void)any_mapped;
    for (auto& r : records) format_sam(r, out);
    det_out = det[0];
    det_out.add(det[1]);
    return out;
}

// ------------------------------------------------------------------ map-only / aemb
// src/io/paf.rs:37-61 + src/maponly.rs:80-105
static void paf_record(const Nam& nam, const std::string& name, int end, const std::vector<RefSeq>& refs, size_t qlen,
                       int mapq, std::string& out) {
    out += name;
    if (end == 1) out += "/1";
    else if (end == 2) out += "/2";
    out += '\t' + std::to_string(qlen) + '\t' + std::to_string(nam.query_start) + '\t' + std::to_string(nam.query_end) +
           '\t' + (nam.is_revcomp ? "-" : "+") + '\t' + refs[nam.ref_id].name + '\t' +
           std::to_string(refs[nam.ref_id].seq.len) + '\t' + std::to_string(nam.ref_start) + '\t' +
           std::to_string(nam.ref_end) + '\t' + std::to_string(nam.matching_bases) + '\t' +
           std::to_string(nam.ref_end - nam.ref_start) + '\t' + std::to_string(mapq < 0 ? 255 : mapq) + '\n';
}

// src/maponly.rs:18-52
std::string map_single_end_read(const SequenceRecord& rec, const Context& ctx, Rng& rng, Details& det) {
    NamDetails nd;
    std::vector<Nam> nams = get_nams_by_chaining(rec.seq, *ctx.index, ctx.cp, ctx.mp.rescue_distance, ctx.mp.mcs, nd);
    sort_nams(nams, rng);
    det = Details();
    det.nam = nd;
    std::string out;
    if (!nams.empty()) paf_record(nams[0], rec.name, 0, *ctx.refs, rec.seq.size(), mapping_quality(nams), out);
    return out;
}

// src/maponly.rs:366-378
static void split_by_orientation(Nam* nams, size_t n, bool both, Nam*& fwd, size_t& nf, Nam*& rev, size_t& nr) {
    if (both) {
        size_t left = 0, right = n;
        while (left < right) {
            if (nams[left].is_revcomp) {
                right--;
                std::swap(nams[left], nams[right]);
            } else {
                left++;
            }
        }
        fwd = nams;
        nf = left;
        rev = nams + left;
        nr = n - left;
    } else if (nams[0].is_revcomp) {
        fwd = nams; nf = 0; rev = nams; nr = n;
    } else {
        fwd = nams; nf = n; rev = nams + n; nr = 0;
    }
}

struct NamPairM {
    Nam n1, n2;
    double score;
};

// src/maponly.rs:380-458
static void find_pairs(const Nam* fwd, size_t nf, const Nam* rev, size_t nr, float mu, float sigma, bool swap,
                       std::vector<NamPairM>& out) {
    size_t max_dist = sat_usize(std::ceil(mu + 10.0f * sigma));
    size_t rp = 0;
    bool has_last = false;
    size_t last_id = 0;
    double prev_score = 0;
    size_t base = out.size();
    (void)base;
    for (size_t fi = 0; fi < nf; fi++) {
        const Nam& f = fwd[fi];
        while (rp < nr && (rev[rp].ref_id < f.ref_id ||
                           (rev[rp].ref_id == f.ref_id && rev[rp].projected_ref_start() < f.projected_ref_start())))
            rp++;
        if (rp == nr) break;
        if (rev[rp].ref_id > f.ref_id) continue;
        bool has_best = false;
        size_t best_id = 0;
        double best_score = 0;
        for (size_t i = rp; i < nr && rev[i].ref_id == f.ref_id &&
                            (rev[i].projected_ref_start() - f.projected_ref_start()) <= max_dist;
             i++) {
            const Nam& r = rev[i];
            size_t x = f.ref_start > r.ref_start ? f.ref_start - r.ref_start : r.ref_start - f.ref_start;
            double sc = (double)f.score + (double)r.score +
                        std::fmax(0.001, (double)std::log(normal_pdf((float)x, mu, sigma) + 1.0f));
            if (!has_best || sc > best_score) {
                has_best = true;
                best_id = i;
                best_score = sc;
            }
        }
        if (!has_best) continue;
        const Nam& r = rev[best_id];
        if (has_last && last_id == best_id) {
            if (best_score <= prev_score) continue;
            out.pop_back();
        }
        if (swap) out.push_back(NamPairM{r, f, best_score});
        else out.push_back(NamPairM{f, r, best_score});
        has_last = true;
        last_id = best_id;
        prev_score = best_score;
        rp = best_id;
    }
}

static bool nam_key_less(const Nam& a, const Nam& b) {
    if (a.ref_id != b.ref_id) return a.ref_id < b.ref_id;
    return a.projected_ref_start() < b.projected_ref_start();
}

// src/maponly.rs:314-345 (unstable sorts restated as stable; identical when keys differ)
static std::vector<NamPairM> get_nam_pairs(std::vector<Nam>& n1, std::vector<Nam>& n2, float mu, float sigma, bool both1,
                                           bool both2) {
    std::vector<NamPairM> pairs;
    if (n1.empty() || n2.empty()) return pairs;
    Nam *f1, *r1, *f2, *r2;
    size_t nf1, nr1, nf2, nr2;
    split_by_orientation(n1.data(), n1.size(), both1, f1, nf1, r1, nr1);
    split_by_orientation(n2.data(), n2.size(), both2, f2, nf2, r2, nr2);
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

// src/maponly.rs:277-304; returns 1 for Pair, 0 for Individual
static int best_paired_location(const std::vector<NamPairM>& pairs, const std::vector<Nam>& n1,
                                const std::vector<Nam>& n2, InsertSizeDistribution& isd) {
    double indiv = (n1.empty() ? 0.0 : (double)n1[0].score) + (n2.empty() ? 0.0 : (double)n2[0].score);
    if (!pairs.empty() && pairs[0].score >= indiv / 2.0) {
        if (isd.sample_size < 400) {
            size_t a = pairs[0].n1.ref_start, b = pairs[0].n2.ref_start;
            isd.update(a > b ? a - b : b - a);
        }
        return 1;
    }
    return 0;
}

// src/maponly.rs:114-195
std::string map_paired_end_read(const SequenceRecord& r1, const SequenceRecord& r2, const Context& ctx,
                                InsertSizeDistribution& isd, Rng& rng, Details& det) {
    NamDetails d1, d2;
    std::vector<Nam> n1 = get_nams_by_chaining(r1.seq, *ctx.index, ctx.cp, ctx.mp.rescue_distance, ctx.mp.mcs, d1);
    std::vector<Nam> n2 = get_nams_by_chaining(r2.seq, *ctx.index, ctx.cp, ctx.mp.rescue_distance, ctx.mp.mcs, d2);
    det = Details();
    det.nam = d1;
    det.nam.add(d2);
    std::string out;
    if (n1.empty() && n2.empty()) return out;
    std::vector<NamPairM> pairs = get_nam_pairs(n1, n2, isd.mu, isd.sigma, d1.both_orientations, d2.both_orientations);
    sort_nams(n1, rng);
    sort_nams(n2, rng);
    if (best_paired_location(pairs, n1, n2, isd)) {
        paf_record(pairs[0].n1, r1.name, 1, *ctx.refs, r1.seq.size(), -1, out);
        paf_record(pairs[0].n2, r2.name, 2, *ctx.refs, r2.seq.size(), -1, out);
    } else {
        if (!n1.empty()) paf_record(n1[0], r1.name, 1, *ctx.refs, r1.seq.size(), -1, out);
        if (!n2.empty()) paf_record(n2[0], r2.name, 2, *ctx.refs, r2.seq.size(), -1, out);
    }
    return out;
}

// src/maponly.rs:57-78
void abundances_single_end_read(const SequenceRecord& rec, const Context& ctx, std::vector<double>& ab, Rng& rng) {
    NamDetails nd;
    std::vector<Nam> nams = get_nams_by_chaining(rec.seq, *ctx.index, ctx.cp, ctx.mp.rescue_distance, ctx.mp.mcs, nd);
    sort_nams(nams, rng);
    size_t nb = 0;
    while (nb < nams.size() && nams[nb].score == nams[0].score) nb++;
    double w = (double)rec.seq.size() / (double)nb;
    for (size_t i = 0; i < nb; i++) ab[nams[i].ref_id] += w;
}

// src/maponly.rs:198-261
void abundances_paired_end_read(const SequenceRecord& r1, const SequenceRecord& r2, const Context& ctx,
                                std::vector<double>& ab, InsertSizeDistribution& isd, Rng& rng) {
    NamDetails d1, d2;
    std::vector<Nam> n1 = get_nams_by_chaining(r1.seq, *ctx.index, ctx.cp, ctx.mp.rescue_distance, ctx.mp.mcs, d1);
    std::vector<Nam> n2 = get_nams_by_chaining(r2.seq, *ctx.index, ctx.cp, ctx.mp.rescue_distance, ctx.mp.mcs, d2);
    if (n1.empty() && n2.empty()) return;
    std::vector<NamPairM> pairs = get_nam_pairs(n1, n2, isd.mu, isd.sigma, d1.both_orientations, d2.both_orientations);
    sort_nams(n1, rng);
    sort_nams(n2, rng);
    if (best_paired_location(pairs, n1, n2, isd)) {
        double js = pairs[0].score;
        size_t nb = 0;
        while (nb < pairs.size() && pairs[nb].score == js) nb++;
        double w1 = (double)r1.seq.size() / (double)nb, w2 = (double)r2.seq.size() / (double)nb;
        for (size_t i = 0; i < nb; i++) {
            ab[pairs[i].n1.ref_id] += w1;
            ab[pairs[i].n2.ref_id] += w2;
        }
    } else {
        const std::vector<Nam>* lists[2] = {&n1, &n2};
        size_t lens[2] = {r1.seq.size(), r2.seq.size()};
        for (int t = 0; t < 2; t++) {
            const std::vector<Nam>& n = *lists[t];
            size_t nb = 0;
            while (nb < n.size() && n[nb].score == n[0].score) nb++;
            double w = (double)lens[t] / (double)nb;
            for (size_t i = 0; i < nb; i++) ab[n[i].ref_id] += w;
        }
    }
}

}  // namespace oracle

// Hooks for the reference's unit tests of the pair helpers (src/mapper.rs tests
// is_proper_pair_*, deduplicate_scored_pairs_works, count_best_alignment_pairs_works)
extern "C" {

int32_t ora_is_proper_pair(uint64_t ref1, uint64_t start1, int32_t rc1, uint64_t ref2, uint64_t start2, int32_t rc2,
                           float mu, float sigma) {
    oracle::Alignment a, b;
    a.reference_id = ref1;
    a.ref_start = start1;
    a.is_revcomp = rc1 != 0;
    b.reference_id = ref2;
    b.ref_start = start2;
    b.is_revcomp = rc2 != 0;
    return oracle::is_proper_pair(a, b, mu, sigma) ? 1 : 0;
}

// n pairs: score, then per mate present / reference / start (ref_start < 0: absent);
// deduplicated in place; returns how many are left and their scores in out_score
size_t ora_deduplicate_scored_pairs(size_t n, const double* score, const int64_t* ref1, const int64_t* start1,
                                    const int64_t* ref2, const int64_t* start2, double* out_score) {
    std::vector<oracle::ScoredAlignmentPair> v(n);
    for (size_t i = 0; i < n; i++) {
        v[i].score = score[i];
        if (start1[i] >= 0) {
            v[i].a1 = oracle::Alignment();
            v[i].a1->reference_id = (size_t)ref1[i];
            v[i].a1->ref_start = (size_t)start1[i];
        }
        if (start2[i] >= 0) {
            v[i].a2 = oracle::Alignment();
            v[i].a2->reference_id = (size_t)ref2[i];
            v[i].a2->ref_start = (size_t)start2[i];
        }
    }
    oracle::deduplicate_scored_pairs(v);
    for (size_t i = 0; i < v.size(); i++) out_score[i] = v[i].score;
    return v.size();
}

size_t ora_count_best_alignment_pairs(size_t n, const double* score) {
    std::vector<oracle::ScoredAlignmentPair> v(n);
    for (size_t i = 0; i < n; i++) v[i].score = score[i];
    return oracle::count_best_alignment_pairs(v);
}

}  // extern "C"
