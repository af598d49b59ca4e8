// Oracle (test infrastructure only): C entry points used by the tests through
// ctypes to compare stage outputs (randstrobes, index arrays, NAMs, alignments)
// with the GPU library.
#include <algorithm>
#include <cstring>

#include "oracle.hpp"

using namespace oracle;

namespace {
struct OraIndex {
    std::vector<RefSeq> refs;
    Index index;
};
}  // namespace

extern "C" {

struct ora_ssw_out {
    int32_t score1, ref_begin1, ref_end1, read_begin1, read_end1, flag, cigar_len;
};

// ext/ssw/ssw.c ssw_align restated, same arguments as the library call src/ssw.rs makes
int32_t ora_ssw_align(const int8_t* read, int32_t read_len, const int8_t* ref, int32_t ref_len, const int8_t* mat,
                      int32_t n, uint8_t gap_open, uint8_t gap_extend, ora_ssw_out* out, uint32_t* cigar,
                      int32_t cap) {
    SswResult r = ssw_align(read, read_len, ref, ref_len, mat, n, gap_open, gap_extend);
    out->score1 = r.score1;
    out->ref_begin1 = r.ref_begin1;
    out->ref_end1 = r.ref_end1;
    out->read_begin1 = r.read_begin1;
    out->read_end1 = r.read_end1;
    out->flag = r.flag;
    out->cigar_len = (int32_t)r.cigar.size();
    if ((int32_t)r.cigar.size() > cap) return -1;
    for (size_t i = 0; i < r.cigar.size(); i++) cigar[i] = r.cigar[i];
    return 0;
}

struct ora_alignment {
    int32_t valid;
    uint32_t score, query_start, query_end, ref_start, ref_end, edit_distance, cigar_len;
};

// Aligner::align (src/aligner.rs:80-151)
int32_t ora_aligner_align(const char* q, size_t ql, const char* r, size_t rl, uint8_t match, uint8_t mismatch,
                          uint8_t gap_open, uint8_t gap_extend, uint32_t end_bonus, ora_alignment* out,
                          uint32_t* cigar, size_t cap) {
    Scores sc;
    sc.match = match;
    sc.mismatch = mismatch;
    sc.gap_open = gap_open;
    sc.gap_extend = gap_extend;
    sc.end_bonus = end_bonus;
    std::optional<AlignmentInfo> a = aligner_align(std::string(q, ql), std::string(r, rl), sc);
    std::memset(out, 0, sizeof(*out));
    if (!a) return 0;
    out->valid = 1;
    out->score = a->score;
    out->query_start = (uint32_t)a->query_start;
    out->query_end = (uint32_t)a->query_end;
    out->ref_start = (uint32_t)a->ref_start;
    out->ref_end = (uint32_t)a->ref_end;
    out->edit_distance = (uint32_t)a->edit_distance;
    out->cigar_len = (uint32_t)a->cigar.ops.size();
    if (a->cigar.ops.size() > cap) return -1;
    for (size_t i = 0; i < a->cigar.ops.size(); i++) cigar[i] = a->cigar.ops[i];
    return 0;
}

// randstrobes_query (src/seeding/mod.rs:19-75); out holds 4 u64 per randstrobe
int32_t ora_randstrobes(size_t read_length_for_params, const char* seq, size_t len, uint64_t* out, size_t cap,
                        size_t* n_fwd, size_t* n_rc) {
    SeedingParameters p = SeedingParameters::from_read_length(read_length_for_params);
    std::vector<QueryRandstrobe> qr[2];
    randstrobes_query(std::string(seq, len), p, qr);
    *n_fwd = qr[0].size();
    *n_rc = qr[1].size();
    if (qr[0].size() + qr[1].size() > cap) return -1;
    size_t w = 0;
    for (int o = 0; o < 2; o++)
        for (auto& r : qr[o]) {
            out[4 * w] = r.hash;
            out[4 * w + 1] = r.hash_revcomp;
            out[4 * w + 2] = r.start;
            out[4 * w + 3] = r.end;
            w++;
        }
    return 0;
}

void* ora_index_from_fasta(const char* path, size_t read_length, int32_t bits, double filter_fraction) {
    auto* o = new OraIndex();
    std::string err;
    if (!read_fasta(path, o->refs, err)) {
        delete o;
        return nullptr;
    }
    SeedingParameters p = SeedingParameters::from_read_length(read_length);
    uint8_t b = bits < 0 ? pick_bits(o->refs, p) : (uint8_t)bits;
    o->index = make_index(o->refs, p, b, filter_fraction);
    return o;
}

void ora_index_free(void* h) { delete (OraIndex*)h; }

// sizes: [n_randstrobes, bits, filter_cutoff]
void ora_index_info(void* h, uint64_t* out3) {
    auto* o = (OraIndex*)h;
    out3[0] = o->index.randstrobes.size();
    out3[1] = o->index.bits;
    out3[2] = o->index.filter_cutoff;
}

void ora_index_arrays(void* h, void* randstrobes, uint64_t* buckets) {
    auto* o = (OraIndex*)h;
    std::memcpy(randstrobes, o->index.randstrobes.data(), o->index.randstrobes.size() * 16);
    std::memcpy(buckets, o->index.bucket_starts.data(), o->index.bucket_starts.size() * 8);
}

struct ora_nam {
    uint32_t nam_id, ref_id, ref_start, ref_end, query_start, query_end, matching_bases, n_anchors;
    float score;
    uint32_t is_revcomp;
};

struct ora_nam_details {
    uint32_t full_not_found, full_filtered, full_found, partial_not_found, partial_filtered, partial_found, rescued;
    uint32_t n_randstrobes, n_anchors, n_nams, both_orientations;
};

// get_nams_by_chaining (src/nam.rs:138-166) followed by the stable sort of sort_nams
// (without the tie shuffle); mcs: 0 always, 1 rescue, 2 off, 3 first-strobe
int32_t ora_nams(void* h, const char* seq, size_t len, int32_t mcs, uint32_t rescue_distance, ora_nam* out,
                 size_t cap, size_t* n_out, ora_nam_details* det) {
    auto* o = (OraIndex*)h;
    ChainingParameters cp;
    NamDetails nd;
    std::vector<Nam> nams =
        get_nams_by_chaining(std::string(seq, len), o->index, cp, rescue_distance, (Mcs)mcs, nd);
    std::stable_sort(nams.begin(), nams.end(), [](const Nam& a, const Nam& b) { return a.score > b.score; });
    *n_out = nams.size();
    if (det) {
        det->full_not_found = (uint32_t)nd.hits.full_not_found;
        det->full_filtered = (uint32_t)nd.hits.full_filtered;
        det->full_found = (uint32_t)nd.hits.full_found;
        det->partial_not_found = (uint32_t)nd.hits.partial_not_found;
        det->partial_filtered = (uint32_t)nd.hits.partial_filtered;
        det->partial_found = (uint32_t)nd.hits.partial_found;
        det->rescued = (uint32_t)nd.hits.rescued;
        det->n_randstrobes = (uint32_t)nd.n_randstrobes;
        det->n_anchors = (uint32_t)nd.n_anchors;
        det->n_nams = (uint32_t)nd.n_nams;
        det->both_orientations = nd.both_orientations;
    }
    if (nams.size() > cap) return -1;
    for (size_t i = 0; i < nams.size(); i++) {
        const Nam& n = nams[i];
        out[i] = ora_nam{(uint32_t)n.nam_id, (uint32_t)n.ref_id, (uint32_t)n.ref_start, (uint32_t)n.ref_end,
                         (uint32_t)n.query_start, (uint32_t)n.query_end, (uint32_t)n.matching_bases,
                         (uint32_t)n.anchors.size(), n.score, n.is_revcomp ? 1u : 0u};
    }
    return 0;
}

}  // extern "C"
