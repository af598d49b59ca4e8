// C ABI (include/strobealign_gb300.h).  Every entry point converts exceptions into
// status codes; none aborts.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>

#include "host_input.h"
#include "mapper.h"
#include "session.h"
#include "stream.h"

namespace sa {

thread_local std::string g_last_error = "no error";
void set_last_error(const std::string& msg) { g_last_error = msg; }

SeedParams to_seed_params(const sa_seeding_params& p) {
    SeedParams s;
    s.k = p.k;
    s.s = p.s;
    s.t = p.t;
    s.w_min = p.w_min;
    s.w_max = p.w_max;
    s.max_dist = p.max_dist;
    s.pop = p.partial_orientation_pos;
    s.q = p.q;
    s.main_mask = p.main_hash_mask;
    s.fwd_main_mask = p.forward_main_hash_mask;
    return s;
}

void index_extent_gpu(const sa_index& idx, uint32_t& max_pos, uint32_t& max_ref, cudaStream_t st);
void extension_init_tables();

}  // namespace sa

using namespace sa;

#define SA_TRY try {
#define SA_CATCH                                  \
    }                                             \
    catch (const sa::Error& e) {                  \
        set_last_error(e.what());                 \
        return e.code;                            \
    }                                             \
    catch (const std::bad_alloc&) {               \
        set_last_error("host allocation failed"); \
        return SA_ERR_OOM;                        \
    }                                             \
    catch (const std::exception& e) {             \
        set_last_error(e.what());                 \
        return SA_ERR_INVALID;                    \
    }

namespace {

void require(bool cond, const char* msg) {
    if (!cond) throw Error(SA_ERR_INVALID, msg);
}

// src/seeding/parameters.rs:92-221
void params_from_read_length(size_t read_length, sa_seeding_params* p) {
    struct Row { uint32_t profile; size_t thr; uint32_t k, s, wmin, wmax, canonical; };
    static const Row rows[7] = {{1, 70, 18, 14, 1, 4, 50},     {2, 90, 20, 16, 1, 6, 75},    {3, 110, 20, 16, 2, 6, 100},
                                {4, 135, 20, 16, 3, 8, 125},   {5, 175, 20, 16, 5, 11, 150}, {6, 375, 22, 18, 6, 16, 250},
                                {7, SIZE_MAX, 23, 17, 5, 15, 400}};
    const Row* r = &rows[6];
    for (const Row& x : rows)
        if (read_length <= x.thr) { r = &x; break; }
    p->profile = r->profile;
    p->k = r->k;
    p->s = r->s;
    p->t = (r->k - r->s) / 2 + 1;
    p->w_min = r->wmin;
    p->w_max = r->wmax;
    p->q = 255;
    size_t md = r->canonical > 70 ? r->canonical - 70 : 0;
    if (md < r->k) md = r->k;
    if (md > 255) md = 255;
    p->max_dist = (uint32_t)md;
    p->main_hash_mask = ~0ULL << (9 + 17);
    p->partial_orientation_pos = (uint32_t)__builtin_ctzll(p->main_hash_mask) - 1;
    p->forward_main_hash_mask = p->main_hash_mask | (1ULL << p->partial_orientation_pos);
}

void finish_index(sa_index* idx) {
    uint32_t mp = 0, mr = 0;
    index_extent_gpu(*idx, mp, mr, 0);
    idx->max_pos = mp;
    idx->n_refs_seen = idx->n ? mr + 1 : 1;
}

}  // namespace

extern "C" {

const char* sa_last_error(void) { return g_last_error.c_str(); }
const char* sa_version(void) { return "strobealign_gb300 0.1.0 (reference strobealign 0.18.0-alpha)"; }

int32_t sa_seeding_params_from_read_length(size_t read_length, sa_seeding_params* out) {
    SA_TRY
    require(out, "null output");
    params_from_read_length(read_length, out);
    return SA_OK;
    SA_CATCH
}

void sa_chaining_params_default(sa_chaining_params* p) {
    p->max_lookback = 50;
    p->diag_diff_penalty = 0.1f;
    p->gap_length_penalty = 0.05f;
    p->valid_score_threshold = 0.7f;
    p->max_ref_gap = 0;
    p->matches_weight = 0.01f;
    p->max_diagonal_ratio = 10.0f;
}

void sa_mapping_params_default(sa_mapping_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->max_secondary = 0;
    p->dropoff_threshold = 0.5f;
    p->rescue_distance = 100;
    p->max_tries = 20;
    p->mcs_strategy = SA_MCS_ALWAYS;
    p->output_unmapped = 1;
    p->use_ssw = 0;
    p->xdrop = 500;
    p->match = 2;
    p->mismatch = 8;
    p->gap_open = 12;
    p->gap_extend = 1;
    p->end_bonus = 10;
    p->mode = SA_MODE_SAM;
    p->eqx = 0;
    p->details = 0;
    p->fastq_comments = 0;
    p->rg_id = nullptr;
    p->chunk_size = 1000000;
}

int32_t sa_refs_from_fasta(const char* path, sa_refs** out) {
    SA_TRY
    require(path && out, "null argument");
    auto r = std::make_unique<sa_refs>();
    load_fasta(path, r->contigs);
    if (r->contigs.empty()) throw Error(SA_ERR_FORMAT, "No sequences found in the reference FASTA");
    for (auto& c : r->contigs) r->total_len += c.len;
    *out = r.release();
    return SA_OK;
    SA_CATCH
}

int32_t sa_refs_from_buffers(size_t n, const char* const* names, const char* const* seqs, const size_t* lens,
                             sa_refs** out) {
    SA_TRY
    require(out && (n == 0 || (names && seqs && lens)), "null argument");
    auto r = std::make_unique<sa_refs>();
    contigs_from_buffers(n, names, seqs, lens, r->contigs);
    for (auto& c : r->contigs) r->total_len += c.len;
    *out = r.release();
    return SA_OK;
    SA_CATCH
}

size_t sa_refs_count(const sa_refs* refs) { return refs ? refs->contigs.size() : 0; }
size_t sa_refs_total_length(const sa_refs* refs) { return refs ? refs->total_len : 0; }

int32_t sa_refs_contig(const sa_refs* refs, size_t i, const char** name, uint64_t* length) {
    SA_TRY
    require(refs && name && length, "null argument");
    require(i < refs->contigs.size(), "contig index out of range");
    *name = refs->contigs[i].name.c_str();
    *length = refs->contigs[i].len;
    return SA_OK;
    SA_CATCH
}

int32_t sa_refs_decode(const sa_refs* refs, size_t i, uint64_t start, uint64_t end, char* out) {
    SA_TRY
    require(refs && (out || start == end), "null argument");
    require(i < refs->contigs.size(), "contig index out of range");
    const Contig& c = refs->contigs[i];
    require(start <= end && end <= c.len, "range outside the contig");
    static const char kBase[4] = {'A', 'C', 'G', 'T'};
    for (uint64_t p = start; p < end; p++) out[p - start] = kBase[c.bits(p)];
    return SA_OK;
    SA_CATCH
}
uint32_t sa_refs_pick_bits(const sa_refs* refs, const sa_seeding_params* p) {
    return pick_bits(refs->contigs, to_seed_params(*p));
}
void sa_refs_free(sa_refs* refs) { delete refs; }

int32_t sa_index_build(const sa_refs* refs, const sa_seeding_params* p, int32_t bits, double filter_fraction,
                       sa_index** out) {
    SA_TRY
    require(refs && p && out, "null argument");
    require(p->k >= 8 && p->k < 32 && p->s <= p->k && (p->k - p->s) % 2 == 0, "invalid syncmer parameters");
    for (auto& c : refs->contigs)
        require(c.len < (1ULL << 32), "contig longer than 2^32 - 1 nt");
    auto idx = std::make_unique<sa_index>();
    SA_CUDA(cudaGetDevice(&idx->device));
    idx->params = *p;
    idx->sp = to_seed_params(*p);
    uint32_t b = bits < 0 ? pick_bits(refs->contigs, idx->sp) : (uint32_t)bits;
    require(b >= 1 && b <= 32, "bits must be in 1..32");
    build_index_gpu(refs->contigs, idx->sp, b, filter_fraction, *idx, 0);
    finish_index(idx.get());
    *out = idx.release();
    return SA_OK;
    SA_CATCH
}

// .sti version 7 (src/index.rs:345-538); native endianness
int32_t sa_index_write_sti(const sa_index* idx, const char* path) {
    SA_TRY
    require(idx && path, "null argument");
    std::ofstream f(path, std::ios::binary);
    if (!f) throw Error(SA_ERR_IO, std::string("cannot create ") + path);
    auto u32 = [&](uint32_t v) { f.write((const char*)&v, 4); };
    auto u64 = [&](uint64_t v) { f.write((const char*)&v, 8); };
    f.write("STI\x01", 4);
    u32(7);
    u64(8);
    u64(0);
    u32(idx->filter_cutoff);
    u32(idx->bits);
    u32(idx->params.profile);
    u32(idx->params.k);
    u32(idx->params.s);
    u32(idx->params.w_min);
    u32(idx->params.w_max);
    u32((uint32_t)idx->params.q);
    u32(idx->params.max_dist);
    u64(idx->params.main_hash_mask);
    std::vector<RefRandstrobe> rs(idx->n);
    std::vector<uint64_t> bs(((size_t)1 << idx->bits) + 1);
    if (idx->n) SA_CUDA(cudaMemcpy(rs.data(), idx->rs.p, idx->n * 16, cudaMemcpyDeviceToHost));
    SA_CUDA(cudaMemcpy(bs.data(), idx->buckets.p, bs.size() * 8, cudaMemcpyDeviceToHost));
    u64(idx->n);
    f.write((const char*)rs.data(), (std::streamsize)(idx->n * 16));
    u64(bs.size());
    f.write((const char*)bs.data(), (std::streamsize)(bs.size() * 8));
    if (!f) throw Error(SA_ERR_IO, "write failed");
    return SA_OK;
    SA_CATCH
}

int32_t sa_index_read_sti(const char* path, const sa_seeding_params* p, int32_t bits, sa_index** out) {
    SA_TRY
    require(path && p && out, "null argument");
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Error(SA_ERR_IO, std::string("cannot open ") + path);
    auto rd = [&](void* d, size_t n) {
        f.read((char*)d, (std::streamsize)n);
        if (!f) throw Error(SA_ERR_IO, "truncated .sti file");
    };
    char magic[4];
    rd(magic, 4);
    if (std::memcmp(magic, "STI\x01", 4) != 0) throw Error(SA_ERR_STI_MISMATCH, "wrong .sti magic");
    uint32_t ver;
    rd(&ver, 4);
    if (ver != 7) throw Error(SA_ERR_STI_MISMATCH, ".sti file format version is not 7");
    uint64_t reserved;
    rd(&reserved, 8);
    std::vector<char> skip(reserved);
    if (reserved) rd(skip.data(), reserved);
    // filter_cutoff, bits, profile, k, s, w_min, w_max, q, max_dist (src/index.rs:384-402)
    uint32_t v[9];
    rd(v, 4 * 9);
    uint64_t main_mask;
    rd(&main_mask, 8);
    const uint32_t cutoff = v[0], sbits = v[1];
    if (bits >= 0 && sbits != (uint32_t)bits) throw Error(SA_ERR_STI_MISMATCH, "bits differ from the .sti file");
    if (v[2] != p->profile || v[3] != p->k || v[4] != p->s || v[5] != p->w_min || v[6] != p->w_max ||
        (uint64_t)v[7] != p->q || v[8] != p->max_dist || main_mask != p->main_hash_mask)
        throw Error(SA_ERR_STI_MISMATCH, "Index parameters in .sti file and those specified differ");
    uint64_t n;
    rd(&n, 8);
    std::vector<RefRandstrobe> rs(n);
    if (n) rd(rs.data(), n * 16);
    uint64_t nb;
    rd(&nb, 8);
    if (sbits > 32 || nb != ((uint64_t)1 << sbits) + 1)
        throw Error(SA_ERR_STI_MISMATCH, "The randstrobe starts vector has an unexpected size");
    std::vector<uint64_t> bs(nb);
    rd(bs.data(), nb * 8);
    auto idx = std::make_unique<sa_index>();
    SA_CUDA(cudaGetDevice(&idx->device));
    idx->params = *p;
    idx->sp = to_seed_params(*p);
    idx->bits = sbits;
    idx->filter_cutoff = cutoff;
    idx->n = n;
    idx->rs.reserve(n);
    idx->buckets.reserve(nb);
    if (n) SA_CUDA(cudaMemcpy(idx->rs.p, rs.data(), n * 16, cudaMemcpyHostToDevice));
    SA_CUDA(cudaMemcpy(idx->buckets.p, bs.data(), nb * 8, cudaMemcpyHostToDevice));
    finish_index(idx.get());
    *out = idx.release();
    return SA_OK;
    SA_CATCH
}

int32_t sa_index_get_info(const sa_index* idx, sa_index_info* out) {
    SA_TRY
    require(idx && out, "null argument");
    out->bits = idx->bits;
    out->filter_cutoff = idx->filter_cutoff;
    out->n_randstrobes = idx->n;
    out->device_bytes = idx->n * 16 + (((uint64_t)1 << idx->bits) + 1) * 8;
    out->params = idx->params;
    return SA_OK;
    SA_CATCH
}

int32_t sa_index_copy_to_host(const sa_index* idx, void* randstrobes, uint64_t* bucket_starts) {
    SA_TRY
    require(idx, "null index");
    if (randstrobes && idx->n) SA_CUDA(cudaMemcpy(randstrobes, idx->rs.p, idx->n * 16, cudaMemcpyDeviceToHost));
    if (bucket_starts)
        SA_CUDA(cudaMemcpy(bucket_starts, idx->buckets.p, ((((size_t)1) << idx->bits) + 1) * 8, cudaMemcpyDeviceToHost));
    return SA_OK;
    SA_CATCH
}

int32_t sa_index_lookup_batch(const sa_index* idx, const uint64_t* hashes, size_t n, int32_t kind,
                              int64_t* out_position, uint32_t* out_count) {
    SA_TRY
    require(idx && (n == 0 || (hashes && out_position)), "null argument");
    require(kind >= 0 && kind <= 2, "kind must be 0, 1 or 2");
    lookup_batch_gpu(*idx, hashes, n, kind, out_position, out_count, 0);
    return SA_OK;
    SA_CATCH
}

void sa_index_free(sa_index* idx) { delete idx; }

int32_t sa_reads_from_file(const char* path, sa_reads** out) {
    SA_TRY
    require(path && out, "null argument");
    auto r = std::make_unique<sa_reads>();
    load_reads(path, r->store);
    *out = r.release();
    return SA_OK;
    SA_CATCH
}

struct sa_read_file {
    std::unique_ptr<ReadParser> parser;
};

int32_t sa_read_file_open(const char* path, sa_read_file** out) {
    SA_TRY
    require(path && out, "null argument");
    auto f = std::make_unique<sa_read_file>();
    f->parser = std::make_unique<ReadParser>(path);
    *out = f.release();
    return SA_OK;
    SA_CATCH
}

int32_t sa_read_file_next(sa_read_file* f, size_t max_records, sa_reads** out) {
    SA_TRY
    require(f && out, "null argument");
    auto r = std::make_unique<sa_reads>();
    reset_read_store(r->store, !f->parser->fasta());
    f->parser->parse(r->store, max_records);
    *out = r.release();
    return SA_OK;
    SA_CATCH
}

void sa_read_file_close(sa_read_file* f) { delete f; }

int32_t sa_reads_view(const sa_reads* reads, sa_read_batch* v) {
    SA_TRY
    require(reads && v, "null argument");
    const ReadStore& s = reads->store;
    v->n = s.seq_off.size() - 1;
    v->seq = s.seq.data();
    v->seq_offsets = s.seq_off.data();
    v->qual = s.has_qual ? s.qual.data() : nullptr;
    v->names = s.names.data();
    v->name_offsets = s.name_off.data();
    v->comments = s.comments.data();
    v->comment_offsets = s.comment_off.data();
    return SA_OK;
    SA_CATCH
}

void sa_reads_free(sa_reads* reads) { delete reads; }

int32_t sa_estimate_read_length(const char* path, size_t* out) {
    SA_TRY
    require(path && out, "null argument");
    require(std::string(path) != "-", "the read length of standard input cannot be estimated");
    ReadParser parser(path);
    ReadStore rs;
    reset_read_store(rs, !parser.fasta());
    const size_t n = parser.parse(rs, 500);
    *out = n ? (size_t)(rs.seq_off[n] / n) : 0;
    return SA_OK;
    SA_CATCH
}

int32_t sa_reads_pair_interleaved(const sa_read_batch* reads, uint32_t* first_read, size_t capacity,
                                  size_t* n_records) {
    SA_TRY
    require(reads && first_read && n_records, "null argument");
    require(reads->n < UINT32_MAX, "batch too large");
    std::vector<uint32_t> rr;
    pair_records_by_name(*reads, true, rr);
    require(rr.size() <= capacity, "output too small");
    std::copy(rr.begin(), rr.end(), first_read);
    *n_records = rr.size() - 1;
    return SA_OK;
    SA_CATCH
}

int32_t sa_mapper_create(const sa_index* idx, const sa_refs* refs, const sa_chaining_params* cp,
                         const sa_mapping_params* mp, sa_mapper** out) {
    SA_TRY
    require(idx && refs && out, "null argument");
    sa_chaining_params c;
    sa_mapping_params m;
    if (cp) c = *cp;
    else sa_chaining_params_default(&c);
    if (mp) m = *mp;
    else sa_mapping_params_default(&m);
    require(c.max_lookback <= 1024, "max_lookback above 1024 is not supported");
    require(c.max_ref_gap < LOG2_LUT_SIZE, "max_ref_gap too large");
    auto h = std::make_unique<sa_mapper>();
    h->m = new Mapper(idx, refs, c, m);
    *out = h.release();
    return SA_OK;
    SA_CATCH
}

void sa_mapper_free(sa_mapper* m) {
    if (!m) return;
    delete m->m;
    delete m;
}

int32_t sa_map_batch(sa_mapper* m, const sa_read_batch* r1, const sa_read_batch* r2, sa_output* out) {
    SA_TRY
    require(m && r1 && out, "null argument");
    std::memset(out, 0, sizeof(*out));
    m->m->map(r1, r2, out);
    return SA_OK;
    SA_CATCH
}

int32_t sa_map_batch_interleaved(sa_mapper* m, const sa_read_batch* reads, sa_output* out) {
    SA_TRY
    require(m && reads && out, "null argument");
    std::memset(out, 0, sizeof(*out));
    m->m->map_interleaved(reads, out);
    return SA_OK;
    SA_CATCH
}

void sa_output_free(sa_output* out) {
    if (!out) return;
    release_output(out->data);
    out->data = nullptr;
    out->len = 0;
}

int32_t sa_mapper_abundances(const sa_mapper* m, double* out, size_t n) {
    SA_TRY
    require(m && out, "null argument");
    const auto& ab = m->m->abundances();
    const auto& cs = m->m->contig_lengths();
    require(n >= ab.size(), "output too small");
    for (size_t i = 0; i < ab.size(); i++) out[i] = ab[i] / (double)cs[i];
    return SA_OK;
    SA_CATCH
}

int32_t sa_mapper_upload(sa_mapper* m, const sa_read_batch* r1, const sa_read_batch* r2) {
    SA_TRY
    require(m && r1, "null argument");
    m->m->upload(r1, r2);
    return SA_OK;
    SA_CATCH
}

int32_t sa_map_uploaded(sa_mapper* m, sa_output* out) {
    SA_TRY
    require(m && out, "null argument");
    std::memset(out, 0, sizeof(*out));
    m->m->map_uploaded(out);
    return SA_OK;
    SA_CATCH
}

int32_t sa_mapper_set_profiling(sa_mapper* m, int32_t enable) {
    SA_TRY
    require(m, "null argument");
    m->m->set_profiling(enable != 0);
    return SA_OK;
    SA_CATCH
}

int32_t sa_mapper_set_parts(sa_mapper* m, uint32_t parts) {
    SA_TRY
    require(m, "null argument");
    m->m->set_parts(parts);
    return SA_OK;
    SA_CATCH
}

void sa_schedule_params_default(sa_schedule_params* p) {
    if (!p) return;
    p->parts = 8;
    p->overlap = 1;
    p->wave_min_jobs = 32768;
    p->max_wave_jobs = 262144;
}

int32_t sa_mapper_set_schedule(sa_mapper* m, const sa_schedule_params* p) {
    SA_TRY
    require(m && p, "null argument");
    require(p->overlap <= 1, "overlap must be 0 or 1");
    m->m->set_parts(p->parts ? p->parts : 8);
    m->m->set_overlap(p->overlap != 0);
    m->m->set_wave_min_jobs(p->wave_min_jobs ? p->wave_min_jobs : 32768);
    m->m->set_max_wave_jobs(p->max_wave_jobs ? p->max_wave_jobs : 262144);
    return SA_OK;
    SA_CATCH
}

void sa_stream_params_default(sa_stream_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->batch_bases = (uint64_t)1 << 29;
    p->read_ahead = 2;
}

int32_t sa_map_files(sa_mapper* m, const char* reads1, const char* reads2, const char* out_path,
                     const sa_stream_params* p, sa_stream_stats* stats) {
    SA_TRY
    require(m && reads1 && out_path, "null argument");
    StreamConfig cfg;
    if (p) {
        cfg.batch_bases = p->batch_bases;
        cfg.read_ahead = p->read_ahead ? p->read_ahead : 2;
        cfg.append = p->append != 0;
        cfg.header = p->header;
        cfg.header_len = p->header ? p->header_len : 0;
        cfg.interleaved = p->interleaved != 0;
    }
    require(!(cfg.interleaved && reads2), "interleaved input takes one reads file");
    const std::string r2 = reads2 ? reads2 : "";
    const StreamResult r = map_files(*m->m, reads1, reads2 ? &r2 : nullptr, out_path, cfg);
    if (stats) {
        stats->n_reads = r.reads;
        stats->n_records = r.records;
        stats->n_mapped = r.mapped;
        stats->n_batches = r.batches;
        stats->bytes_in = r.bytes_in;
        stats->bytes_out = r.bytes_out;
        stats->seconds_total = r.seconds_total;
        stats->seconds_map = r.seconds_map;
        stats->seconds_wait_input = r.seconds_wait_input;
    }
    return SA_OK;
    SA_CATCH
}

static void tuning_to_c(const Mapper::Tuning& t, sa_tuning* o) {
    o->parts = t.parts;
    o->wave_min_jobs = t.wave_min_jobs;
    o->max_wave_jobs = t.max_wave_jobs;
    o->ssw_wave_max_qlen = t.wave_qmax;
    o->chain_lane_cluster_max = t.chain_lane_max;
    o->l2_fetch_bytes = t.l2_fetch;
}

void sa_tuning_default(sa_tuning* t) {
    if (t) tuning_to_c(Mapper::Tuning(), t);
}

int32_t sa_mapper_set_tuning(sa_mapper* m, const sa_tuning* t) {
    SA_TRY
    require(m && t, "null argument");
    require(t->parts >= 1 && t->max_wave_jobs >= 1 && t->wave_min_jobs >= 1, "tuning values must be positive");
    require(t->ssw_wave_max_qlen >= 1 && t->ssw_wave_max_qlen <= 192, "ssw_wave_max_qlen must be in 1..192");
    require(t->chain_lane_cluster_max >= 1 && t->chain_lane_cluster_max <= 4096,
            "chain_lane_cluster_max must be in 1..4096");
    require(t->l2_fetch_bytes == 0 || t->l2_fetch_bytes == 32 || t->l2_fetch_bytes == 64 || t->l2_fetch_bytes == 128,
            "l2_fetch_bytes must be 0, 32, 64 or 128");
    Mapper::Tuning x;
    x.parts = t->parts;
    x.wave_min_jobs = t->wave_min_jobs;
    x.max_wave_jobs = t->max_wave_jobs;
    x.wave_qmax = t->ssw_wave_max_qlen;
    x.chain_lane_max = t->chain_lane_cluster_max;
    x.l2_fetch = t->l2_fetch_bytes;
    m->m->set_tuning(x);
    return SA_OK;
    SA_CATCH
}

int32_t sa_mapper_get_tuning(const sa_mapper* m, sa_tuning* t) {
    SA_TRY
    require(m && t, "null argument");
    tuning_to_c(m->m->tuning(), t);
    return SA_OK;
    SA_CATCH
}

int32_t sa_mapper_autotune(sa_mapper* m, const sa_read_batch* r1, const sa_read_batch* r2, uint32_t rounds,
                           sa_tune_report* out) {
    SA_TRY
    require(m && r1 && out, "null argument");
    const Mapper::TuneReport rep = m->m->autotune(r1, r2, rounds);
    tuning_to_c(rep.chosen, &out->chosen);
    out->seconds_default = rep.seconds_default;
    out->seconds_tuned = rep.seconds_tuned;
    out->trials = rep.trials;
    return SA_OK;
    SA_CATCH
}

int32_t sa_mapper_get_stats(const sa_mapper* m, sa_mapper_stats* out) {
    SA_TRY
    require(m && out, "null argument");
    *out = m->m->stats();
    return SA_OK;
    SA_CATCH
}

int32_t sa_sam_header(const sa_refs* refs, const char* cmd_line, const char* rg_id, const char* const* rg_fields,
                      size_t n_rg_fields, sa_output* out) {
    SA_TRY
    require(refs && out, "null argument");
    std::string h = "@HD\tVN:1.6\tSO:unsorted\n";
    for (auto& c : refs->contigs) h += "@SQ\tSN:" + c.name + "\tLN:" + std::to_string(c.len) + "\n";
    if (rg_id) {
        h += std::string("@RG\tID:") + rg_id;
        for (size_t i = 0; i < n_rg_fields; i++) h += std::string("\t") + rg_fields[i];
        h += "\n";
    }
    if (cmd_line) h += std::string("@PG\tID:strobealign\tPN:strobealign\tVN:0.18.0-alpha\tCL:") + cmd_line + "\n";
    out->data = (char*)std::malloc(h.size() + 1);
    if (!out->data) throw Error(SA_ERR_OOM, "allocation failed");
    std::memcpy(out->data, h.data(), h.size() + 1);
    out->len = h.size();
    out->n_reads = out->n_mapped = 0;
    out->n_waves = out->n_gpu_launches = 0;
    return SA_OK;
    SA_CATCH
}

// ------------------------------------------------------------------ stage entry points
int32_t sa_randstrobes_batch(const sa_index* idx, const sa_read_batch* reads, sa_query_randstrobe* out,
                             size_t capacity, uint64_t* out_offsets, uint32_t* out_counts) {
    SA_TRY
    require(idx && reads && out_offsets && out_counts, "null argument");
    NamWorkspace ws;
    const uint32_t n = (uint32_t)reads->n;
    uint64_t total = reads->seq_offsets[n] - reads->seq_offsets[0];
    std::vector<uint64_t> off(n + 1);
    for (uint32_t i = 0; i <= n; i++) off[i] = reads->seq_offsets[i] - reads->seq_offsets[0];
    for (uint32_t i = 0; i < n; i++) require(off[i + 1] - off[i] <= MAX_READ_LEN, "read too long");
    ws.seq.reserve(total + 16);
    ws.off.reserve((size_t)n + 1);
    SA_CUDA(cudaMemcpy(ws.seq.p, reads->seq + reads->seq_offsets[0], total, cudaMemcpyHostToDevice));
    SA_CUDA(cudaMemcpy(ws.off.p, off.data(), ((size_t)n + 1) * 8, cudaMemcpyHostToDevice));
    run_seeding(idx->sp, n, total, ws, 0);
    std::vector<uint32_t> cnt(2 * (size_t)n);
    std::vector<uint64_t> h(2 * total), hr(2 * total);
    std::vector<uint32_t> s(2 * total), e(2 * total);
    SA_CUDA(cudaMemcpy(cnt.data(), ws.n_rs.p, cnt.size() * 4, cudaMemcpyDeviceToHost));
    if (total) {
        SA_CUDA(cudaMemcpy(h.data(), ws.qr_hash.p, h.size() * 8, cudaMemcpyDeviceToHost));
        SA_CUDA(cudaMemcpy(hr.data(), ws.qr_hash_rc.p, hr.size() * 8, cudaMemcpyDeviceToHost));
        SA_CUDA(cudaMemcpy(s.data(), ws.qr_start.p, s.size() * 4, cudaMemcpyDeviceToHost));
        SA_CUDA(cudaMemcpy(e.data(), ws.qr_end.p, e.size() * 4, cudaMemcpyDeviceToHost));
    }
    uint64_t w = 0;
    for (uint32_t r = 0; r < n; r++)
        for (int o = 0; o < 2; o++) {
            uint32_t c = cnt[2 * r + o];
            out_offsets[2 * r + o] = w;
            out_counts[2 * r + o] = c;
            if (w + c > capacity) throw Error(SA_ERR_INVALID, "randstrobe output capacity too small");
            for (uint32_t i = 0; i < c; i++) {
                uint64_t src = o * total + off[r] + i;
                out[w + i] = sa_query_randstrobe{h[src], hr[src], s[src], e[src]};
            }
            w += c;
        }
    return SA_OK;
    SA_CATCH
}

// Allocation-free seeding: the checked seeding kernel on caller-owned device
// buffers with the syncmer scratch in a static device array.
int32_t sa_randstrobes_device_noalloc(const sa_index* idx, const uint8_t* d_seq, const uint64_t* d_seq_offsets,
                                      uint32_t n_reads, uint64_t total_bases, uint64_t* d_hash,
                                      uint64_t* d_hash_revcomp, uint32_t* d_start, uint32_t* d_end,
                                      uint32_t* d_counts, void* stream) {
    SA_TRY
    require(idx != nullptr, "null index");
    run_seeding_noalloc(idx->sp, d_seq, d_seq_offsets, n_reads, total_bases, d_hash, d_hash_revcomp, d_start, d_end,
                        d_counts, (cudaStream_t)stream);
    return SA_OK;
    SA_CATCH
}

int32_t sa_nams_batch(const sa_index* idx, const sa_chaining_params* cp, const sa_mapping_params* mp,
                      const sa_read_batch* reads, sa_nam* out, size_t capacity, uint64_t* out_offsets,
                      uint32_t* out_counts, sa_nam_details* out_details) {
    SA_TRY
    require(idx && reads && out_offsets && out_counts, "null argument");
    sa_chaining_params c;
    sa_mapping_params m;
    if (cp) c = *cp;
    else sa_chaining_params_default(&c);
    if (mp) m = *mp;
    else sa_mapping_params_default(&m);
    // the same limits as sa_mapper_create: the chaining log2 table covers gaps below
    // LOG2_LUT_SIZE, and the lookback ring holds 1024 predecessors
    require(c.max_lookback <= 1024, "max_lookback above 1024 is not supported");
    require(c.max_ref_gap < LOG2_LUT_SIZE, "max_ref_gap too large");
    NamWorkspace ws;
    const uint32_t n = (uint32_t)reads->n;
    uint64_t total = reads->seq_offsets[n] - reads->seq_offsets[0];
    std::vector<uint64_t> off(n + 1);
    for (uint32_t i = 0; i <= n; i++) off[i] = reads->seq_offsets[i] - reads->seq_offsets[0];
    for (uint32_t i = 0; i < n; i++) require(off[i + 1] - off[i] <= MAX_READ_LEN, "read too long");
    ws.seq.reserve(total + 16);
    ws.off.reserve((size_t)n + 1);
    SA_CUDA(cudaMemcpy(ws.seq.p, reads->seq + reads->seq_offsets[0], total, cudaMemcpyHostToDevice));
    SA_CUDA(cudaMemcpy(ws.off.p, off.data(), ((size_t)n + 1) * 8, cudaMemcpyHostToDevice));
    NamConfig cfg;
    cfg.cp = ChainParams{c.max_lookback, c.diag_diff_penalty, c.gap_length_penalty, c.valid_score_threshold,
                         c.max_ref_gap, c.matches_weight, c.max_diagonal_ratio};
    cfg.mcs = m.mcs_strategy;
    cfg.rescue_distance = m.rescue_distance;
    DevRefs none{};
    run_nam_pipeline(idx->view(), none, cfg, n, total, idx->max_pos + 512 + idx->params.k, idx->n_refs_seen, ws, 0);
    SA_CUDA(cudaDeviceSynchronize());
    std::vector<uint64_t> noff(n + 1);
    SA_CUDA(cudaMemcpy(noff.data(), ws.nam_off.p, ((size_t)n + 1) * 8, cudaMemcpyDeviceToHost));
    if (noff[n] > capacity) throw Error(SA_ERR_INVALID, "NAM output capacity too small");
    if (noff[n]) SA_CUDA(cudaMemcpy(out, ws.nams.p, noff[n] * sizeof(NamRec), cudaMemcpyDeviceToHost));
    if (out_details) SA_CUDA(cudaMemcpy(out_details, ws.details.p, (size_t)n * sizeof(NamDetailsRec), cudaMemcpyDeviceToHost));
    for (uint32_t r = 0; r < n; r++) {
        out_offsets[r] = noff[r];
        out_counts[r] = (uint32_t)(noff[r + 1] - noff[r]);
    }
    return SA_OK;
    SA_CATCH
}

int32_t sa_align_batch(const sa_mapping_params* mp, size_t n, const char* queries, const uint64_t* qoff,
                       const char* refs, const uint64_t* roff, sa_alignment* out, uint32_t* cigar,
                       size_t cigar_capacity) {
    SA_TRY
    require(n == 0 || (queries && qoff && refs && roff && out), "null argument");
    sa_mapping_params m;
    if (mp) m = *mp;
    else sa_mapping_params_default(&m);
    if (n == 0) return SA_OK;
    uint64_t qtot = qoff[n] - qoff[0], rtot = roff[n] - roff[0];
    std::vector<uint64_t> qo(n + 1), ro(n + 1);
    uint32_t maxq = 1;
    for (size_t i = 0; i <= n; i++) {
        qo[i] = qoff[i] - qoff[0];
        ro[i] = roff[i] - roff[0];
        if (i < n) {
            require(qoff[i + 1] - qoff[i] <= MAX_READ_LEN, "query too long");
            maxq = std::max<uint32_t>(maxq, (uint32_t)(qoff[i + 1] - qoff[i]));
        }
    }
    DevBuf<uint8_t> dq, dr;
    DevBuf<uint64_t> dqo, dro;
    dq.reserve(qtot + 16);
    dr.reserve(rtot + 16);
    dqo.reserve(n + 1);
    dro.reserve(n + 1);
    SA_CUDA(cudaMemcpy(dq.p, queries + qoff[0], qtot, cudaMemcpyHostToDevice));
    SA_CUDA(cudaMemcpy(dr.p, refs + roff[0], rtot, cudaMemcpyHostToDevice));
    SA_CUDA(cudaMemcpy(dqo.p, qo.data(), (n + 1) * 8, cudaMemcpyHostToDevice));
    SA_CUDA(cudaMemcpy(dro.p, ro.data(), (n + 1) * 8, cudaMemcpyHostToDevice));
    ExtWorkspace ws;
    std::vector<ExtJob> jobs(n);
    for (size_t i = 0; i < n; i++) {
        jobs[i] = ExtJob{};
        jobs[i].kind = JOB_ALIGN;
        jobs[i].read = (uint32_t)i;
        jobs[i].ref_id = (uint32_t)i;
        jobs[i].use_ssw = 1;
    }
    ws.jobs.reserve(n);
    SA_CUDA(cudaMemcpy(ws.jobs.p, jobs.data(), n * sizeof(ExtJob), cudaMemcpyHostToDevice));
    AlignScores sc{m.match, m.mismatch, m.gap_open, m.gap_extend, m.end_bonus};
    DevRefs none{};
    run_extension_raw(none, dq.p, dqo.p, dr.p, dro.p, 0, sc, (uint32_t)n, ws, maxq, 0);
    uint64_t w = 0;
    for (size_t i = 0; i < n; i++) {
        const ExtResult& r = ws.h_results[i];
        sa_alignment& a = out[i];
        a.valid = r.valid;
        a.score = r.score;
        a.query_start = r.soft_clip_left;
        a.query_end = (uint32_t)(qo[i + 1] - qo[i]) - r.soft_clip_right;
        a.ref_start = r.ref_start;
        a.ref_end = r.ref_start + r.length;
        a.edit_distance = r.edit_distance;
        a.cigar_offset = (uint32_t)w;
        a.cigar_len = r.valid ? r.cigar_len : 0;
        if (r.valid) {
            if (cigar) {
                if (w + r.cigar_len > cigar_capacity) throw Error(SA_ERR_INVALID, "cigar capacity too small");
                std::memcpy(cigar + w, ws.h_cigar.data() + r.cigar_offset, r.cigar_len * 4);
            }
            w += r.cigar_len;
        }
    }
    return SA_OK;
    SA_CATCH
}

namespace {

void stage_common(const sa_mapping_params* mp, size_t n, const char* q, const uint64_t* qoff, const char* r,
                  const uint64_t* roff, std::vector<uint64_t>& qo, std::vector<uint64_t>& ro, AlignScores& sc) {
    require(n == 0 || (q && qoff && r && roff), "null argument");
    require(n < (1ull << 31), "too many items");
    sa_mapping_params m;
    if (mp) m = *mp;
    else sa_mapping_params_default(&m);
    sc = AlignScores{m.match, m.mismatch, m.gap_open, m.gap_extend, m.end_bonus};
    qo.assign(n + 1, 0);
    ro.assign(n + 1, 0);
    for (size_t i = 0; i <= n; i++) {
        qo[i] = n ? qoff[i] - qoff[0] : 0;
        ro[i] = n ? roff[i] - roff[0] : 0;
        if (i && i <= n) require(qoff[i] >= qoff[i - 1] && roff[i] >= roff[i - 1], "offsets must not decrease");
        if (i < n) require(qoff[i + 1] - qoff[i] <= MAX_READ_LEN, "query too long");
    }
}

}  // namespace

int32_t sa_hamming_batch(const sa_mapping_params* mp, size_t n, const uint32_t* kinds, const char* queries,
                         const uint64_t* query_offsets, const char* refs, const uint64_t* ref_offsets,
                         sa_stage_alignment* out, uint32_t* cigar, size_t cigar_capacity) {
    SA_TRY
    std::vector<uint64_t> qo, ro;
    AlignScores sc;
    stage_common(mp, n, queries, query_offsets, refs, ref_offsets, qo, ro, sc);
    if (n == 0) return SA_OK;
    require(kinds && out && cigar, "null argument");
    for (size_t i = 0; i < n; i++) require(kinds[i] <= 1, "kind must be 0 or 1");
    static_assert(sizeof(sa_stage_alignment) == sizeof(StageAlignment), "stage alignment layout");
    stage_hamming((uint32_t)n, kinds, (const uint8_t*)queries + query_offsets[0], qo.data(),
                  (const uint8_t*)refs + ref_offsets[0], ro.data(), sc, reinterpret_cast<StageAlignment*>(out), cigar,
                  cigar_capacity, 0);
    return SA_OK;
    SA_CATCH
}

int32_t sa_piecewise_pieces(const sa_mapping_params* mp, size_t n, const uint32_t* kinds, const char* queries,
                            const uint64_t* query_offsets, const char* refs, const uint64_t* ref_offsets,
                            sa_stage_alignment* out, uint32_t* cigar, size_t cigar_capacity) {
    SA_TRY
    std::vector<uint64_t> qo, ro;
    AlignScores sc;
    stage_common(mp, n, queries, query_offsets, refs, ref_offsets, qo, ro, sc);
    if (n == 0) return SA_OK;
    require(kinds && out && cigar, "null argument");
    require(sc.gap_open >= sc.gap_extend, "gap_open must be at least gap_extend");
    for (size_t i = 0; i < n; i++) {
        require(kinds[i] <= 2, "kind must be 0, 1 or 2");
        require(ro[i + 1] - ro[i] <= 4 * MAX_READ_LEN, "reference piece too long");
    }
    stage_pieces((uint32_t)n, kinds, (const uint8_t*)queries + query_offsets[0], qo.data(),
                 (const uint8_t*)refs + ref_offsets[0], ro.data(), sc, reinterpret_cast<StageAlignment*>(out), cigar,
                 cigar_capacity, 0);
    return SA_OK;
    SA_CATCH
}

int32_t sa_remove_spurious_anchors(size_t n, int32_t* anchors, const uint64_t* offsets, uint32_t* out_counts) {
    SA_TRY
    if (n == 0) return SA_OK;
    require(anchors && offsets && out_counts, "null argument");
    require(offsets[0] == 0, "offsets must start at 0");
    for (size_t i = 0; i < n; i++) require(offsets[i + 1] >= offsets[i], "offsets must not decrease");
    stage_prune((uint32_t)n, anchors, offsets, out_counts, 0);
    return SA_OK;
    SA_CATCH
}

int32_t sa_piecewise_batch(const sa_mapping_params* mp, uint32_t k, size_t n, const char* queries,
                           const uint64_t* query_offsets, const char* refs, const uint64_t* ref_offsets,
                           const uint32_t* anchors, const uint64_t* anchor_offsets, sa_stage_alignment* out,
                           uint32_t* cigar, size_t cigar_capacity) {
    SA_TRY
    std::vector<uint64_t> qo, ro;
    AlignScores sc;
    stage_common(mp, n, queries, query_offsets, refs, ref_offsets, qo, ro, sc);
    if (n == 0) return SA_OK;
    require(anchors && anchor_offsets && out && cigar, "null argument");
    require(k >= 1 && k <= 32, "k out of range");
    require(sc.gap_open >= sc.gap_extend, "gap_open must be at least gap_extend");
    require(anchor_offsets[0] == 0, "anchor offsets must start at 0");
    for (size_t i = 0; i < n; i++) {
        const uint64_t L = qo[i + 1] - qo[i], W = ro[i + 1] - ro[i];
        require(anchor_offsets[i + 1] > anchor_offsets[i], "every item needs at least one anchor");
        require(W <= 4 * MAX_READ_LEN, "reference window too long");
        for (uint64_t a = anchor_offsets[i]; a < anchor_offsets[i + 1]; a++)
            require(anchors[2 * a] + k <= L && anchors[2 * a + 1] + k <= W, "anchor outside its query or window");
    }
    stage_piecewise((uint32_t)n, (const uint8_t*)queries + query_offsets[0], qo.data(),
                    (const uint8_t*)refs + ref_offsets[0], ro.data(), anchors, anchor_offsets, k, sc,
                    reinterpret_cast<StageAlignment*>(out), cigar, cigar_capacity, 0);
    return SA_OK;
    SA_CATCH
}

}  // extern "C"

// ---------------------------------------------------------------- serving
void sa_session_params_default(sa_session_params* p) {
    if (!p) return;
    p->max_inflight_bases = 0;
    p->max_inflight_requests = 0;
    p->policy_threads = 0;
    p->admission_streams = 2;
    p->borrow_inputs = 0;
    p->device_reserve_bytes = 0;
}

int32_t sa_session_get_info(const sa_session* s, sa_session_info* out) {
    SA_TRY
    require(s && s->s && out, "null argument");
    out->arena_bases = s->s->arena_bases();
    out->device_reserve_bytes = s->s->reserve_bytes();
    out->refused_requests = s->s->refused();
    return SA_OK;
    SA_CATCH
}

int32_t sa_session_create(const sa_index* idx, const sa_refs* refs, const sa_chaining_params* cp,
                          const sa_mapping_params* mp, const sa_session_params* sp, sa_session** out) {
    SA_TRY
    require(idx && refs && out, "null argument");
    sa_chaining_params c;
    sa_mapping_params m;
    if (cp) c = *cp;
    else sa_chaining_params_default(&c);
    if (mp) m = *mp;
    else sa_mapping_params_default(&m);
    require(c.max_lookback <= 1024, "max_lookback above 1024 is not supported");
    require(c.max_ref_gap < LOG2_LUT_SIZE, "max_ref_gap too large");
    SessionConfig sc;
    if (sp) {
        sc.max_inflight_bases = sp->max_inflight_bases;
        sc.max_inflight_requests = sp->max_inflight_requests;
        sc.policy_threads = sp->policy_threads;
        sc.admission_streams = sp->admission_streams ? sp->admission_streams : 2;
        sc.borrow_inputs = sp->borrow_inputs != 0;
        sc.device_reserve_bytes = sp->device_reserve_bytes;
    }
    auto* s = new sa_session{nullptr};
    try {
        s->s = new Session(idx, refs, c, m, sc);
    } catch (...) {
        delete s;
        throw;
    }
    *out = s;
    return SA_OK;
    SA_CATCH
}

int32_t sa_session_submit(sa_session* s, const sa_read_batch* r1, const sa_read_batch* r2, uint64_t* ticket) {
    SA_TRY
    require(s && r1 && ticket, "null argument");
    *ticket = s->s->submit(r1, r2);
    return SA_OK;
    SA_CATCH
}

int32_t sa_session_submit_interleaved(sa_session* s, const sa_read_batch* reads, uint64_t* ticket) {
    SA_TRY
    require(s && reads && ticket, "null argument");
    *ticket = s->s->submit(reads, nullptr, true);
    return SA_OK;
    SA_CATCH
}

int32_t sa_session_poll(sa_session* s, uint64_t ticket, int32_t* done) {
    SA_TRY
    require(s && done, "null argument");
    *done = s->s->poll(ticket);
    return SA_OK;
    SA_CATCH
}

int32_t sa_session_wait(sa_session* s, uint64_t ticket, int64_t timeout_ms, sa_output* out, sa_request_stats* stats,
                        double* abundances, size_t n_abundances) {
    SA_TRY
    require(s && out, "null argument");
    std::unique_ptr<Request> r;
    if (!s->s->wait(ticket, timeout_ms, r)) throw Error(SA_ERR_TIMEOUT, "request not finished within the timeout");
    if (!r->out) throw Error(r->error_code ? r->error_code : SA_ERR_OOM, r->error);
    out->data = r->out;  // ownership passes to the caller (sa_output_free)
    out->len = r->out_len;
    r->out = nullptr;
    out->n_reads = r->n_reads;
    out->n_mapped = r->mapped;
    out->n_waves = r->waves;
    out->n_gpu_launches = 0;
    if (stats) {
        auto sec = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
            return std::chrono::duration<double>(b - a).count();
        };
        stats->seconds_queued = sec(r->t_submit, r->t_admit);
        stats->seconds_service = sec(r->t_admit, r->t_done);
        stats->seconds_total = sec(r->t_submit, r->t_done);
        stats->n_reads = r->n_reads;
        stats->n_waves = r->waves;
        stats->h2d_bytes = r->h2d_bytes;
        stats->d2h_bytes = r->d2h_bytes;
    }
    if (abundances) {
        const auto& cs = s->s->contigs();
        require(n_abundances >= cs.size(), "abundance output too small");
        for (size_t i = 0; i < cs.size(); i++)
            abundances[i] = i < r->abundance.size() ? r->abundance[i] / (double)cs[i].len : 0.0;
    }
    return SA_OK;
    SA_CATCH
}

void sa_session_free(sa_session* s) {
    if (!s) return;
    delete s->s;
    delete s;
}
