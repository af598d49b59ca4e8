// Oracle (test infrastructure only): C entry points used by the tests through
// ctypes to compare stage outputs (randstrobes, index arrays, NAMs, alignments)
// with the GPU library.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <thread>

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

// The same from contigs in memory (ASCII bases), built on `threads` threads;
// *seconds = the index build time.
void* ora_index_from_buffers(size_t n, const char* const* names, const char* const* seqs, const size_t* lens,
                             size_t read_length, int32_t bits, double filter_fraction, uint32_t threads,
                             double* seconds) {
    auto* o = new OraIndex();
    o->refs.resize(n);
    std::atomic<size_t> next{0};
    std::vector<std::thread> th;
    for (uint32_t t = 0; t < std::max<uint32_t>(threads, 1); t++)
        th.emplace_back([&] {
            for (size_t i; (i = next.fetch_add(1)) < n;) {
                o->refs[i].name = names[i];
                o->refs[i].seq.data.reserve(lens[i] / 32 + 1);
                for (size_t j = 0; j < lens[i]; j++) o->refs[i].seq.push((uint8_t)seqs[i][j]);
            }
        });
    for (auto& t : th) t.join();
    SeedingParameters p = SeedingParameters::from_read_length(read_length);
    uint8_t b = bits < 0 ? pick_bits(o->refs, p) : (uint8_t)bits;
    auto t0 = std::chrono::steady_clock::now();
    o->index = make_index(o->refs, p, b, filter_fraction, std::max<uint32_t>(threads, 1));
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return o;
}

struct ora_read_batch {
    size_t n;
    const char* seq;
    const uint64_t* seq_offsets;
    const char* qual;  // NULL: no qualities
    const char* names;
    const uint64_t* name_offsets;
};

struct ora_map_opts {
    uint32_t mode;  // 0 SAM, 1 PAF, 2 abundances
    uint32_t max_secondary;
    float dropoff;
    uint32_t rescue_distance, max_tries, mcs, output_unmapped, use_ssw, eqx, details;
    uint64_t chunk_size;
    uint32_t threads;
};

static void records_from(const ora_read_batch* b, std::vector<SequenceRecord>& out, uint32_t threads) {
    out.resize(b->n);
    const size_t per = 1 << 14, nb = (b->n + per - 1) / per;
    std::atomic<size_t> next{0};
    std::vector<std::thread> th;
    for (uint32_t t = 0; t < std::max<uint32_t>(threads, 1); t++)
        th.emplace_back([&] {
            for (size_t k; (k = next.fetch_add(1)) < nb;)
                for (size_t i = k * per; i < std::min(b->n, (k + 1) * per); i++) {
                    SequenceRecord& r = out[i];
                    r.name.assign(b->names + b->name_offsets[i], b->name_offsets[i + 1] - b->name_offsets[i]);
                    r.seq.assign(b->seq + b->seq_offsets[i], b->seq_offsets[i + 1] - b->seq_offsets[i]);
                    if (b->qual) {
                        r.qual.assign(b->qual + b->seq_offsets[i], b->seq_offsets[i + 1] - b->seq_offsets[i]);
                        r.has_qual = true;
                    }
                }
        });
    for (auto& t : th) t.join();
}

// The chunk driver (driver.cpp) over records in memory.  *out (malloc'ed, release with
// ora_output_free) receives the records' SAM / PAF bytes without a header, or for mode
// 2 the per-contig abundances (f64, divided by contig length) as raw bytes;
// *seconds = the mapping time (record conversion excluded).
static int32_t map_in_memory(OraIndex* o, const std::vector<SequenceRecord>& a, const std::vector<SequenceRecord>* b,
                             const std::vector<uint8_t>* has_mate, const ora_map_opts* opt, char** out,
                             size_t* out_len, double* seconds);

int32_t ora_map_batch(void* h, const ora_read_batch* r1, const ora_read_batch* r2, const ora_map_opts* opt,
                      char** out, size_t* out_len, double* seconds) {
    std::vector<SequenceRecord> a, b;
    records_from(r1, a, opt->threads);
    if (r2) records_from(r2, b, opt->threads);
    return map_in_memory((OraIndex*)h, a, r2 ? &b : nullptr, nullptr, opt, out, out_len, seconds);
}

// As ora_map_batch for one batch of records in file order, paired as --interleaved pairs
// them (src/io/reads.rs:68-113): mixed single-end and paired-end records.
int32_t ora_map_interleaved(void* h, const ora_read_batch* reads, const ora_map_opts* opt, char** out,
                            size_t* out_len, double* seconds) {
    std::vector<SequenceRecord> flat, a, b;
    std::vector<uint8_t> has_mate;
    records_from(reads, flat, opt->threads);
    pair_interleaved(std::move(flat), a, b, has_mate);
    return map_in_memory((OraIndex*)h, a, &b, &has_mate, opt, out, out_len, seconds);
}

static int32_t map_in_memory(OraIndex* o, const std::vector<SequenceRecord>& a, const std::vector<SequenceRecord>* b,
                             const std::vector<uint8_t>* has_mate, const ora_map_opts* opt, char** out,
                             size_t* out_len, double* seconds) {
    Context ctx;
    ctx.refs = &o->refs;
    ctx.index = &o->index;
    ctx.mp.max_secondary = opt->max_secondary;
    ctx.mp.dropoff_threshold = opt->dropoff;
    ctx.mp.rescue_distance = opt->rescue_distance;
    ctx.mp.max_tries = opt->max_tries;
    ctx.mp.mcs = (Mcs)opt->mcs;
    ctx.mp.output_unmapped = opt->output_unmapped != 0;
    ctx.mp.use_ssw = opt->use_ssw != 0;
    ctx.so.eqx = opt->eqx != 0;
    ctx.so.details = opt->details != 0;
    auto t0 = std::chrono::steady_clock::now();
    std::vector<double> ab;
    std::vector<std::string> outs = map_records(ctx, a, b, (MapMode)opt->mode, std::max<uint32_t>(opt->threads, 1),
                                                opt->chunk_size, &ab, has_mate);
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (opt->mode == 2) {
        *out_len = ab.size() * sizeof(double);
        *out = (char*)std::malloc(std::max<size_t>(*out_len, 1));
        for (size_t i = 0; i < ab.size(); i++) ab[i] /= (double)o->refs[i].seq.len;
        std::memcpy(*out, ab.data(), *out_len);
        return 0;
    }
    size_t total = 0;
    std::vector<size_t> at(outs.size() + 1, 0);
    for (size_t i = 0; i < outs.size(); i++) at[i + 1] = at[i] + outs[i].size();
    total = at.back();
    *out = (char*)std::malloc(std::max<size_t>(total, 1));
    *out_len = total;
    std::atomic<size_t> next{0};
    std::vector<std::thread> th;
    for (uint32_t t = 0; t < std::max<uint32_t>(opt->threads, 1); t++)
        th.emplace_back([&] {
            for (size_t i; (i = next.fetch_add(1)) < outs.size();) {
                std::memcpy(*out + at[i], outs[i].data(), outs[i].size());
                std::string().swap(outs[i]);
            }
        });
    for (auto& t : th) t.join();
    return 0;
}

void ora_output_free(char* p) { std::free(p); }

void ora_index_free(void* h) { delete (OraIndex*)h; }

// sizes: [n_randstrobes, bits, filter_cutoff]
void ora_index_info(void* h, uint64_t* out3) {
    auto* o = (OraIndex*)h;
    out3[0] = o->index.randstrobes.size();
    out3[1] = o->index.bits;
    out3[2] = o->index.filter_cutoff;
}

// Pointers to the index arrays (valid until ora_index_free), for comparisons without a copy.
void ora_index_view(void* h, const void** randstrobes, const uint64_t** buckets) {
    auto* o = (OraIndex*)h;
    *randstrobes = o->index.randstrobes.data();
    *buckets = o->index.bucket_starts.data();
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

// ---- unit-vector entry points (the reference's own unit tests, tests/golden/unit_vectors.json)
struct ora_stage {
    int32_t valid, score;
    uint32_t query_start, query_end, ref_start, ref_end, edit_distance, cigar_len;
};

static int32_t put_cigar(const Cigar& c, uint32_t* cigar, size_t cap, ora_stage* o) {
    o->cigar_len = (uint32_t)c.ops.size();
    if (c.ops.size() > cap) return -1;
    for (size_t i = 0; i < c.ops.size(); i++) cigar[i] = c.ops[i];
    return 0;
}

uint64_t ora_xxh64(uint64_t x) { return xxh64(x); }

// SyncmerParameters::pick_bits (src/indexer.rs:294-300) for a FASTA's contigs
uint32_t ora_pick_bits(const char* fasta, uint32_t k, uint32_t s) {
    std::vector<RefSeq> refs;
    std::string err;
    if (!read_fasta(fasta, refs, err)) return 0;
    SeedingParameters p;
    p.k = k;
    p.s = s;
    return pick_bits(refs, p);
}

// kind 0 hamming_align, 1 hamming_align_global (src/aligner.rs:218-291)
int32_t ora_hamming(int32_t kind, const char* q, size_t ql, const char* r, size_t rl, uint8_t match, uint8_t mismatch,
                    uint32_t end_bonus, ora_stage* o, uint32_t* cigar, size_t cap) {
    std::memset(o, 0, sizeof(*o));
    std::string a(q, ql), b(r, rl);
    AlignmentInfo h;
    if (kind == 0) {
        std::optional<AlignmentInfo> x = hamming_align(a, b, match, mismatch, end_bonus);
        if (!x) return 0;
        h = *x;
    } else {
        h = hamming_align_global(a, b, match, mismatch);
    }
    o->valid = 1;
    o->score = (int32_t)h.score;
    o->query_start = (uint32_t)h.query_start;
    o->query_end = (uint32_t)h.query_end;
    o->ref_start = (uint32_t)h.ref_start;
    o->ref_end = (uint32_t)h.ref_end;
    o->edit_distance = (uint32_t)h.edit_distance;
    return put_cigar(h.cigar, cigar, cap, o);
}

// one piecewise DP piece: kind 0 global, 1 xdrop GlobalStartLocalEnd, 2 LocalStartGlobalEnd
int32_t ora_piece(int32_t kind, const char* q, size_t ql, const char* r, size_t rl, uint8_t match, uint8_t mismatch,
                  uint8_t gap_open, uint8_t gap_extend, uint32_t end_bonus, ora_stage* o, uint32_t* cigar,
                  size_t cap) {
    Scores sc;
    sc.match = match;
    sc.mismatch = mismatch;
    sc.gap_open = gap_open;
    sc.gap_extend = gap_extend;
    sc.end_bonus = end_bonus;
    PieceResult p = piecewise_piece(kind, std::string(q, ql), std::string(r, rl), sc);
    std::memset(o, 0, sizeof(*o));
    o->valid = 1;
    o->score = p.score;
    o->query_start = (uint32_t)p.query_start;
    o->query_end = (uint32_t)p.query_end;
    o->ref_start = (uint32_t)p.ref_start;
    o->ref_end = (uint32_t)p.ref_end;
    o->edit_distance = (uint32_t)p.cigar.edit_distance();
    return put_cigar(p.cigar, cigar, cap, o);
}

// remove_spurious_anchors on (query_start, ref_start) pairs in place; returns the count kept
uint32_t ora_remove_spurious_anchors(int32_t* pairs, uint32_t n) {
    std::vector<Anchor> a(n);
    for (uint32_t i = 0; i < n; i++) a[i] = Anchor{0, (size_t)pairs[2 * i + 1], (size_t)pairs[2 * i]};
    remove_spurious_anchors(a);
    for (size_t i = 0; i < a.size(); i++) {
        pairs[2 * i] = (int32_t)a[i].query_start;
        pairs[2 * i + 1] = (int32_t)a[i].ref_start;
    }
    return (uint32_t)a.size();
}

// extend_piecewise with remove_spurious_anchors first, as the mapper runs it
// (src/mapper.rs:586-593); anchors (query_start, ref_start) pairs last to first
int32_t ora_extend_piecewise(const char* q, size_t ql, const char* r, size_t rl, const uint32_t* pairs, uint32_t n,
                             uint32_t k, uint32_t padding, uint8_t match, uint8_t mismatch, uint8_t gap_open,
                             uint8_t gap_extend, uint32_t end_bonus, int32_t xdrop, int32_t prune, ora_stage* o,
                             uint32_t* cigar, size_t cap) {
    Scores sc;
    sc.match = match;
    sc.mismatch = mismatch;
    sc.gap_open = gap_open;
    sc.gap_extend = gap_extend;
    sc.end_bonus = end_bonus;
    std::vector<Anchor> a(n);
    for (uint32_t i = 0; i < n; i++) a[i] = Anchor{0, pairs[2 * i + 1], pairs[2 * i]};
    if (prune) remove_spurious_anchors(a);
    std::memset(o, 0, sizeof(*o));
    std::optional<AlignmentInfo> x = extend_piecewise(std::string(q, ql), std::string(r, rl), a, padding, k, sc, xdrop);
    if (!x) return 0;
    o->valid = 1;
    o->score = (int32_t)x->score;
    o->query_start = (uint32_t)x->query_start;
    o->query_end = (uint32_t)x->query_end;
    o->ref_start = (uint32_t)x->ref_start;
    o->ref_end = (uint32_t)x->ref_end;
    o->edit_distance = (uint32_t)x->edit_distance;
    return put_cigar(x->cigar, cigar, cap, o);
}

// collinear_chaining's best score (src/chainer.rs:85-180) on (ref_id, ref_start,
// query_start) triples with the default chaining parameters
float ora_chain_best_score(const uint64_t* triples, size_t n, uint32_t k, uint64_t max_ref_gap) {
    std::vector<Anchor> a(n);
    for (size_t i = 0; i < n; i++) a[i] = Anchor{triples[3 * i], triples[3 * i + 1], triples[3 * i + 2]};
    ChainingParameters cp;
    std::vector<float> dp;
    std::vector<size_t> pred;
    size_t bi;
    return collinear_chaining(a, k, max_ref_gap, cp, dp, pred, bi);
}

int32_t ora_has_shared_substring(const char* read, size_t rl, const char* ref, size_t fl, uint32_t k) {
    return has_shared_substring(std::string(read, rl), std::string(ref, fl), k) ? 1 : 0;
}

// The index sectors the lookups of get_nams_by_chaining read (32-byte sectors, distinct
// per read; src/index.rs:127-338, src/hit.rs, src/chainer.rs:304-384): out[0] directory
// sectors, out[1] table sectors, out[2] randstrobes probed, summed over the reads.
int32_t ora_lookup_sectors(void* h, const ora_read_batch* b, int32_t mcs, uint32_t rescue_distance, uint64_t* out) {
    auto* o = (OraIndex*)h;
    std::vector<uint64_t> sec;
    const uint64_t dir_lo = (uint64_t)(uintptr_t)o->index.bucket_starts.data() >> 5;
    const uint64_t dir_hi = (uint64_t)(uintptr_t)(o->index.bucket_starts.data() + o->index.bucket_starts.size()) >> 5;
    out[0] = out[1] = out[2] = 0;
    ChainingParameters cp;
    for (size_t i = 0; i < b->n; i++) {
        std::string seq(b->seq + b->seq_offsets[i], b->seq_offsets[i + 1] - b->seq_offsets[i]);
        NamDetails nd;
        sec.clear();
        g_sectors = &sec;
        get_nams_by_chaining(seq, o->index, cp, rescue_distance, (Mcs)mcs, nd);
        g_sectors = nullptr;
        std::sort(sec.begin(), sec.end());
        sec.erase(std::unique(sec.begin(), sec.end()), sec.end());
        for (uint64_t x : sec) (x >= dir_lo && x <= dir_hi ? out[0] : out[1])++;
        out[2] += nd.n_randstrobes;
    }
    return 0;
}

}  // extern "C"
