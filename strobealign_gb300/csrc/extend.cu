// Base-level extension on the GPU: the reference's extend_seed (src/mapper.rs:532-620),
// rescue_align (src/mapper.rs:1094-1153) and Aligner::align (src/aligner.rs:80-151)
// for a list of jobs.
//
//   k_prepare   thread per job: NAM consistency / orientation repair
//               (src/nam.rs:49-135), projected window, Hamming eligibility
//   k_fill      thread per job: Hamming fast path (src/aligner.rs:166-259) or the
//               SSW task's query and reference bytes
//   k_sw        SSW (ext/ssw/ssw.c:163-596) with the library's striped semantics:
//               one lane per SSE lane, 16 lanes per task in byte mode and 8 in word
//               mode, so 2 resp. 4 tasks per warp; the lazy-F pass leaves E alone
//               and byte mode reruns in word mode once max + bias >= 255
//   k_ssw_wave  the same passes for reads up to 192 nt: eight threads per task, one
//               or two SSE lanes per thread, a wavefront over the reference columns
//   k_band_*    banded_sw (ext/ssw/ssw.c:598-769): band doubling, then the final
//               pass with directions and the traceback, one thread per task
//   k_finalize  M -> =/X (src/cigar.rs:149-187), edit distance and the end-bonus
//               extension of Aligner::align
#include <cub/cub.cuh>

#include <type_traits>

#include "extend.h"

namespace sa {

namespace {

__constant__ uint8_t c_ssw_code[256];   // src/ssw.rs:8-25
__constant__ uint8_t c_comp[256];       // src/revcomp.rs:5-22

constexpr uint32_t FULLM = 0xffffffffu;
// SswTask::raw_off of a task whose banded traceback runs on the per-thread path
constexpr uint64_t RAW_FALLBACK = ~0ull;

__device__ __forceinline__ uint8_t ref_base(const DevRefs& R, uint32_t c, uint64_t i) {
    uint64_t w = __ldg(R.words + R.word_off[c] + (i >> 5));
    return "ACGT"[(w >> ((i & 31) * 2)) & 3];
}

__device__ __forceinline__ uint8_t read_char(const uint8_t* s, uint32_t L, uint32_t i, bool rc) {
    return rc ? c_comp[s[L - 1 - i]] : s[i];
}

// has_shared_substring (src/mapper.rs:1157-1168), warp per rescue job: the
// window's substrings of length 2k/3 go into a shared-memory hash set (2-bit
// codes, the window read straight from the packed reference), then every read
// substring starting at a multiple of k/3 is looked up.  A read substring holding
// anything but A/C/G/T never matches (the window decodes to A/C/G/T only).  Jobs
// without a shared substring are dropped (type 0, nothing to extend).
constexpr uint32_t RESCUE_TAB_MAX = 4096;  // > 2 * (2000 - sub + 1) slots
constexpr unsigned long long RESCUE_EMPTY = ~0ull;

__device__ __forceinline__ uint32_t rescue_slot(uint64_t v, uint32_t bits) {
    return (uint32_t)((v * 0x9E3779B97F4A7C15ull) >> (64 - bits));
}

__global__ void __launch_bounds__(64) k_rescue_filter(const uint32_t* __restrict__ list,
                                                      const uint32_t* __restrict__ n_list,
                                                      const uint8_t* __restrict__ seq, const uint64_t* __restrict__ off,
                                                      DevRefs R, uint32_t k, PrepRec* prep, uint64_t* sz_arena,
                                                      uint64_t* sz_cigar, uint64_t* sz_h) {
    extern __shared__ unsigned long long rescue_tab[];
    const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x & 31, wpb = blockDim.x / 32;
    unsigned long long* tab = rescue_tab + warp * RESCUE_TAB_MAX;
    const uint32_t n = *n_list;
    const uint32_t sub = 2 * k / 3;
    const uint32_t step = k / 3 ? k / 3 : 1;
    const uint64_t mask = (1ull << (2 * sub)) - 1;  // sub <= 21 for k <= 32
    for (uint32_t li = blockIdx.x * wpb + warp; li < n; li += gridDim.x * wpb) {
        const uint32_t t = list[li];
        const PrepRec p = prep[t];
        const uint8_t* s = seq + off[p.read];
        const uint32_t L = p.qlen;
        const uint32_t lim = L > sub ? L - sub : 0;
        bool found;
        if (lim == 0) {
            found = false;
        } else if (sub == 0) {
            found = true;
        } else if (p.wlen < sub) {
            found = false;
        } else {
            const uint32_t entries = p.wlen - sub + 1;
            uint32_t bits = 6;
            while ((1u << bits) < 2 * entries) bits++;
            const uint32_t size = 1u << bits;
            for (uint32_t i = lane; i < size; i += 32) tab[i] = RESCUE_EMPTY;
            __syncwarp();
            const uint64_t* words = R.words + R.word_off[p.ref_id];
            for (uint32_t q = lane; q < entries; q += 32) {
                const uint64_t x = (uint64_t)p.wstart + q;
                const uint64_t w0 = __ldg(words + (x >> 5)), w1 = __ldg(words + (x >> 5) + 1);
                const uint32_t sh = (uint32_t)(x & 31) * 2;
                uint64_t v = sh ? (w0 >> sh) | (w1 << (64 - sh)) : w0;
                v &= mask;
                uint32_t h = rescue_slot(v, bits);
                for (;;) {
                    const unsigned long long prev = atomicCAS(&tab[h], RESCUE_EMPTY, (unsigned long long)v);
                    if (prev == RESCUE_EMPTY || prev == v) break;
                    h = (h + 1) & (size - 1);
                }
            }
            __syncwarp();
            bool hit = false;
            for (uint32_t i = lane * step; i < lim && !hit; i += 32 * step) {
                uint64_t v = 0;
                bool ok = true;
                for (uint32_t j = 0; j < sub; j++) {
                    const uint8_t c = read_char(s, L, i + j, p.rc);
                    const uint32_t code = c == 'A' ? 0 : c == 'C' ? 1 : c == 'G' ? 2 : c == 'T' ? 3 : 4;
                    if (code > 3) { ok = false; break; }
                    v |= (uint64_t)code << (2 * j);
                }
                if (!ok) continue;
                uint32_t h = rescue_slot(v, bits);
                for (;;) {
                    const unsigned long long e = tab[h];
                    if (e == v) { hit = true; break; }
                    if (e == RESCUE_EMPTY) break;
                    h = (h + 1) & (size - 1);
                }
            }
            found = __any_sync(FULLM, hit);
            __syncwarp();
        }
        if (!found && lane == 0) {
            prep[t].type = 0;
            prep[t].cigar_cap = 0;
            sz_arena[t] = 0;
            sz_cigar[t] = 0;
            sz_h[t] = 0;
        }
    }
}

// 2-bit codes of the reference bases [pos, pos + 32) of contig c (pos inside the contig;
// the word after a contig's last is its padding word)
__device__ __forceinline__ uint64_t ref_codes32(const DevRefs& R, uint32_t c, uint64_t pos) {
    const uint64_t* W = R.words + R.word_off[c];
    const uint64_t a = pos >> 5;
    const uint32_t sh = (uint32_t)(pos & 31) * 2;
    const uint64_t w0 = __ldg(W + a);
    return sh ? (w0 >> sh) | (__ldg(W + a + 1) << (64 - sh)) : w0;
}

// "ACGT"[code]
__device__ __forceinline__ uint8_t code_char(uint32_t code) { return (uint8_t)(0x54474341u >> (8 * code)); }

// Mismatches of read positions [qs, qs + cnt) (cnt <= 32) against the reference from pos
__device__ __forceinline__ uint32_t mismatches32(const DevRefs& R, uint32_t c, uint64_t pos, const uint8_t* s,
                                                 uint32_t L, uint32_t qs, uint32_t cnt, bool rc) {
    const uint64_t v = ref_codes32(R, c, pos);
    uint32_t mm = 0;
    for (uint32_t b = 0; b < cnt; b++) mm += read_char(s, L, qs + b, rc) != code_char((uint32_t)(v >> (2 * b)) & 3);
    return mm;
}

// Nam::is_consistent (src/nam.rs:49-69): the k-mers at both ends of the NAM match (k < 32)
__device__ __forceinline__ bool nam_consistent(const DevRefs& R, const uint8_t* s, uint32_t L, uint32_t ref_id,
                                               uint32_t rs, uint32_t re, uint32_t qs, uint32_t qe, bool rc,
                                               uint32_t k) {
    return mismatches32(R, ref_id, rs, s, L, qs, k, rc) == 0 && mismatches32(R, ref_id, re - k, s, L, qe - k, k, rc) == 0;
}

// Mismatches of the read against the reference from ref_start
__device__ __forceinline__ uint32_t hamming_distance(const DevRefs& R, const uint8_t* s, uint32_t L, uint32_t ref_id,
                                                     uint32_t ref_start, bool rc) {
    uint32_t hd = 0;
    for (uint32_t c = 0; c < L; c += 32) hd += mismatches32(R, ref_id, (uint64_t)ref_start + c, s, L, c, L - c < 32 ? L - c : 32, rc);
    return hd;
}

// Thread per job; the reference bases come 32 at a time from the packed words
__global__ void k_prepare(const ExtJob* jobs, uint32_t n, const uint8_t* __restrict__ seq,
                          const uint64_t* __restrict__ off, DevRefs R, uint32_t k, const uint8_t* raw_refs,
                          const uint64_t* raw_off, ExtResult* res, PrepRec* prep, uint64_t* sz_arena,
                          uint64_t* sz_cigar, uint64_t* sz_h, uint32_t* rescue_list, uint32_t* n_rescue,
                          uint32_t* max_pw_window) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        ExtJob jb = jobs[t];
        const uint8_t* s = seq + off[jb.read];
        const uint32_t L = (uint32_t)(off[jb.read + 1] - off[jb.read]);
        ExtResult r{};
        PrepRec p{};
        p.read = jb.read;
        p.qlen = L;
        p.diag = NO_DIAG;
        p.ref_id = jb.ref_id;
        r.valid = 0;
        if (jb.kind == JOB_EXTEND_FAST || jb.kind == JOB_EXTEND_FULL) {
            uint32_t qs = jb.query_start, qe = jb.query_end;
            bool rc = jb.is_revcomp;
            bool cons = nam_consistent(R, s, L, jb.ref_id, jb.ref_start, jb.ref_end, qs, qe, rc, k);
            bool flipped = false;
            if (!cons && jb.kind == JOB_EXTEND_FULL) {
                uint32_t q2s = L - qe, q2e = L - qs;
                if (nam_consistent(R, s, L, jb.ref_id, jb.ref_start, jb.ref_end, q2s, q2e, !rc, k)) {
                    rc = !rc;
                    qs = q2s;
                    qe = q2e;
                    cons = true;
                    flipped = true;
                }
            }
            r.consistent = cons;
            r.flipped = flipped;
            r.nam_query_start = qs;
            r.nam_query_end = qe;
            r.nam_is_revcomp = rc;
            r.is_revcomp = rc;
            p.rc = rc;
            const uint32_t clen = R.len[jb.ref_id];
            uint32_t prs = jb.ref_start > qs ? jb.ref_start - qs : 0;
            uint64_t pre64 = (uint64_t)jb.ref_end + L - qe;
            uint32_t pre = (uint32_t)(pre64 < clen ? pre64 : clen);
            bool hamming = false;
            if ((uint64_t)prs + L == pre && cons) {
                const uint32_t hd = hamming_distance(R, s, L, jb.ref_id, prs, rc);
                if (__fdiv_rn(__uint2float_rn(hd), __uint2float_rn(L)) < 0.05f) hamming = true;
            }
            if (hamming) {
                p.type = 1;
                p.wstart = prs;
                p.wlen = L;
                r.gapped = 0;
            } else {
                r.gapped = 1;
                uint32_t pad = L / 10;
                uint32_t ws = prs > pad ? prs - pad : 0;
                uint64_t we = (uint64_t)pre + pad;
                if (we > clen) we = clen;
                p.wstart = ws;
                p.wlen = (uint32_t)(we - ws);
                p.diag = prs - ws;
                // Aligner::align returns None for reference segments over 2000 (src/aligner.rs:83-86)
                p.type = (jb.use_ssw && p.wlen <= 2000 && L > 0) ? 2 : 0;
                if (!jb.use_ssw) {
                    // extend_piecewise on the NAM's anchors over [ref_start - (L + pad),
                    // ref_end + L + pad) (src/mapper.rs:588-610); single-end only, and only
                    // for consistent NAMs (the policy drops the others)
                    const uint64_t span = (uint64_t)L + pad;
                    const uint32_t ds = jb.ref_start > span ? (uint32_t)(jb.ref_start - span) : 0;
                    uint64_t de = (uint64_t)jb.ref_end + span;
                    if (de > clen) de = clen;
                    p.wstart = ds;
                    p.wlen = de > ds ? (uint32_t)(de - ds) : 0;
                    p.type = (cons && jb.anc_n > 0 && L > 0) ? 3 : 0;
                    if (p.type == 3) atomicMax(max_pw_window, p.wlen);
                }
            }
        } else if (jb.kind == JOB_RESCUE) {
            bool rc = jb.is_revcomp;
            p.rc = rc;
            r.is_revcomp = rc;
            r.gapped = 1;
            p.wstart = jb.ref_start;
            p.wlen = jb.ref_end - jb.ref_start;
            // extended only if has_shared_substring holds (k_rescue_filter)
            p.type = (p.wlen <= 2000 && L > 0) ? 2 : 0;
            if (p.type == 2) rescue_list[atomicAdd(n_rescue, 1u)] = t;
        } else {  // JOB_ALIGN: raw reference bytes
            p.rc = 0;
            p.wstart = 0;
            p.wlen = (uint32_t)(raw_off[jb.ref_id + 1] - raw_off[jb.ref_id]);
            p.type = (p.wlen <= 2000 && L > 0) ? 2 : 0;
        }
        uint64_t ab = 0, cap = 0, hs = 0;
        if (p.type == 1) cap = L + 1;
        if (p.type == 3) {
            ab = (uint64_t)L + p.wlen;
            cap = (uint64_t)L + p.wlen + 8;  // every op consumes a query or reference base
        }
        if (p.type == 2) {
            ab = (uint64_t)L + p.wlen;
            cap = 2ull * L + p.wlen + 4;
            uint64_t len = L > p.wlen ? L : p.wlen;
            hs = 3 * (2 * len + 8);
        }
        p.cigar_cap = (uint32_t)cap;
        res[t] = r;
        prep[t] = p;
        sz_arena[t] = ab;
        sz_cigar[t] = cap;
        sz_h[t] = hs;
    }
}

// run-merging CIGAR writer (Cigar::push, src/cigar.rs:100-110)
// Appends CIGAR ops, merging runs of one op.  The open run stays in a register and is
// stored when the op changes or at finish() (a store and reload per base otherwise).
struct CigarWriter {
    uint32_t* out;
    uint32_t n;
    uint32_t cap;
    bool overflow;
    uint32_t open = 0;  // (len << 4) | op of the run being extended, 0 if none
    __device__ void push(uint32_t op, uint32_t len) {
        if (len == 0) return;
        if (open && (open & 15) == op) {
            open += len << 4;
            return;
        }
        close_run();
        open = (len << 4) | op;
    }
    __device__ void close_run() {
        if (!open) return;
        if (n < cap) out[n++] = open;
        else overflow = true;
        open = 0;
    }
    __device__ void finish() { close_run(); }
};

// highest_scoring_segment (src/aligner.rs:180-216): the best-scoring ungapped segment
// of a query against an equal-length reference (eq(i): base i matches), with the end
// bonus once for each query end the segment reaches.  Returns the score; [bs, be) is
// the segment.
template <class EQ>
__device__ __forceinline__ int32_t highest_scoring_segment(EQ eq, uint32_t L, const AlignScores& sc, uint32_t& bs,
                                                           uint32_t& be) {
    int32_t score = (int32_t)sc.end_bonus, best = 0;
    uint32_t start = 0;
    bs = be = 0;
    for (uint32_t i = 0; i < L; i++) {
        score += eq(i) ? (int32_t)sc.match : -(int32_t)sc.mismatch;
        if (score < 0) { start = i + 1; score = 0; }
        if (score > best) { bs = start; best = score; be = i + 1; }
    }
    if (score + (int32_t)sc.end_bonus > best) {
        best = score + (int32_t)sc.end_bonus;
        be = L;
        bs = start;
    }
    return best;
}

// The =/X CIGAR of [bs, be) (hamming_align, src/aligner.rs:233-248); returns the mismatches.
template <class EQ>
__device__ __forceinline__ uint32_t hamming_cigar(EQ eq, uint32_t bs, uint32_t be, CigarWriter& w) {
    uint32_t mm = 0;
    for (uint32_t i = bs; i < be; i++) {
        const bool e = eq(i);
        mm += !e;
        w.push(e ? 7u : 8u, 1);
    }
    w.finish();
    return mm;
}

// The =/X CIGAR of [bs, be) from a match bit array (hamming_align, src/aligner.rs:233-248),
// a run of equal bits at a time; returns the mismatches.
__device__ __forceinline__ uint32_t hamming_cigar_bits(const uint32_t* bits, uint32_t bs, uint32_t be, CigarWriter& w) {
    uint32_t mm = 0;
    uint32_t i = bs;
    while (i < be) {
        const bool e = (bits[i >> 5] >> (i & 31)) & 1;
        // the end of the run of e starting at i
        uint32_t j = i;
        for (;;) {
            const uint32_t word = e ? ~bits[j >> 5] : bits[j >> 5];
            const uint32_t m = word & (0xffffffffu << (j & 31));
            if (m) {
                j = (j & ~31u) + (uint32_t)(__ffs(m) - 1);
                break;
            }
            j = (j & ~31u) + 32;
            if (j >= be) break;
        }
        if (j > be) j = be;
        const uint32_t len = j - i;
        if (!e) mm += len;
        w.push(e ? 7u : 8u, len);
        i = j;
    }
    w.finish();
    return mm;
}

// A warp takes 32 consecutive jobs, a lane each.  Hamming jobs (hamming_align,
// src/aligner.rs:181-259) run on their lane: the match bits of the read against the
// reference, 32 bases per pair of packed reference words, then the best segment and its
// =/X runs from the bits.  The SSW / piecewise jobs' query and reference window bytes are
// copied into the arena by the whole warp, one job after another.
__global__ void __launch_bounds__(256) k_fill(const ExtJob* jobs, uint32_t n, const uint8_t* __restrict__ seq,
                                              const uint64_t* __restrict__ off, DevRefs R, const uint8_t* raw_refs,
                                              const uint64_t* raw_off, AlignScores sc, PrepRec* prep,
                                              const uint64_t* off_arena, const uint64_t* off_cigar,
                                              const uint64_t* off_h, uint8_t* arena, uint32_t* cigar, ExtResult* res,
                                              SswTask* tasks, uint32_t* counters, uint32_t* pw_list) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nwarps = gridDim.x * (blockDim.x / 32);
    for (uint32_t b0 = (blockIdx.x * blockDim.x + threadIdx.x) / 32 * 32; b0 < n; b0 += nwarps * 32) {
        const uint32_t t = b0 + lane;
        PrepRec p{};
        uint64_t s_off = 0;
        bool align_raw = false;
        if (t < n) {
            p = prep[t];
            p.arena_off = off_arena[t];
            p.cigar_off = off_cigar[t];
            p.h_off = off_h[t];
            prep[t] = p;
            s_off = off[p.read];
            align_raw = p.type == 2 && jobs[t].kind == JOB_ALIGN;
        }
        if (t < n && p.type == 1) {
            const uint8_t* s = seq + s_off;
            const uint32_t L = p.qlen;
            uint32_t bits[MAX_READ_LEN / 32];
            const uint32_t nw = (L + 31) / 32;
            for (uint32_t w = 0; w < nw; w++) {
                const uint64_t v = ref_codes32(R, p.ref_id, (uint64_t)p.wstart + 32 * w);
                const uint32_t cnt = L - 32 * w < 32 ? L - 32 * w : 32;
                uint32_t m = 0;
                for (uint32_t b = 0; b < cnt; b++)
                    m |= (uint32_t)(read_char(s, L, 32 * w + b, p.rc) == code_char((uint32_t)(v >> (2 * b)) & 3)) << b;
                bits[w] = m;
            }
            auto eq = [&](uint32_t i) { return (bool)((bits[i >> 5] >> (i & 31)) & 1); };
            uint32_t bs, be;
            const int32_t best = highest_scoring_segment(eq, L, sc, bs, be);
            CigarWriter cw{cigar + p.cigar_off, 0, p.cigar_cap, false};
            const uint32_t mm = hamming_cigar_bits(bits, bs, be, cw);
            ExtResult r = res[t];
            r.valid = cw.overflow ? 0 : 1;
            r.score = (uint32_t)best;
            r.edit_distance = mm;
            r.ref_start = p.wstart + bs;
            r.length = be - bs;
            r.soft_clip_left = bs;
            r.soft_clip_right = L - be;
            r.cigar_offset = (uint32_t)p.cigar_off;
            r.cigar_len = cw.n;
            res[t] = r;
        }
        // the copies, a job at a time by the whole warp
        uint32_t todo = __ballot_sync(FULLM, t < n && (p.type == 2 || p.type == 3));
        while (todo) {
            const int src = __ffs(todo) - 1;
            todo &= todo - 1;
            const uint32_t jt = b0 + (uint32_t)src;
            const uint64_t aoff = __shfl_sync(FULLM, (unsigned long long)p.arena_off, src);
            const uint64_t so = __shfl_sync(FULLM, (unsigned long long)s_off, src);
            const uint32_t L = __shfl_sync(FULLM, p.qlen, src), rcf = __shfl_sync(FULLM, p.rc, src);
            const uint32_t wlen = __shfl_sync(FULLM, p.wlen, src), wstart = __shfl_sync(FULLM, p.wstart, src);
            const uint32_t ref_id = __shfl_sync(FULLM, p.ref_id, src), type = __shfl_sync(FULLM, p.type, src);
            const bool raw = __shfl_sync(FULLM, align_raw, src);
            const uint8_t* s = seq + so;
            uint8_t* q = arena + aoff;
            for (uint32_t i = lane; i < L; i += 32) q[i] = read_char(s, L, i, rcf);
            uint8_t* w = q + L;
            if (raw) {
                const uint8_t* rr = raw_refs + raw_off[ref_id];
                for (uint32_t i = lane; i < wlen; i += 32) w[i] = rr[i];
            } else {
                for (uint32_t i = lane; i < wlen; i += 32) w[i] = ref_base(R, ref_id, (uint64_t)wstart + i);
            }
            if (lane == (uint32_t)src) {
                if (type == 3) {
                    pw_list[atomicAdd(&counters[19], 1u)] = jt;
                } else {
                    uint32_t ti = atomicAdd(&counters[0], 1u);
                    atomicAdd(reinterpret_cast<unsigned long long*>(counters + 8), (unsigned long long)L * wlen);
                    SswTask tk{};
                    tk.job = jt;
                    tk.raw_off = RAW_FALLBACK;
                    tk.ref_begin1 = -1;
                    tk.read_begin1 = -1;
                    tasks[ti] = tk;
                }
            }
        }
    }
}

// ------------------------------------------------------------------ striped SW
__device__ __forceinline__ int addus8(int a, int b) { int s = a + b; return s > 255 ? 255 : s; }
__device__ __forceinline__ int subus8(int a, int b) { return a > b ? a - b : 0; }
__device__ __forceinline__ int adds16(int a, int b) {
    int s = a + b;
    return s < -32768 ? -32768 : (s > 32767 ? 32767 : s);
}
__device__ __forceinline__ int subus16(int a, int b) {
    unsigned x = (unsigned)a & 0xffffu, y = (unsigned)b & 0xffffu;
    return x > y ? (int)(short)(unsigned short)(x - y) : 0;
}

template <bool WORD>
struct Lanes;
template <>
struct Lanes<false> {
    using T = uint8_t;
    static constexpr int G = 16;
};
template <>
struct Lanes<true> {
    using T = int16_t;
    static constexpr int G = 8;
};

struct EndPos {
    int score, ref, read;
    int cols;  // reference columns processed
};

// One striped pass (sw_sse2_byte / sw_sse2_word).  The G lanes of a group hold one
// SSE register; H, E and the striped query codes live in shared memory.
template <bool WORD>
__device__ EndPos sw_pass(const uint8_t* q, int qlen, bool q_rev, const uint8_t* r, int rlen, bool r_rev,
                          int terminate, const AlignScores& sc, int bias, typename Lanes<WORD>::T* H,
                          typename Lanes<WORD>::T* E, int8_t* qc, unsigned mask, int gl) {
    constexpr int G = Lanes<WORD>::G;
    const int seg = (qlen + G - 1) / G;
    const int gO = sc.gap_open, gE = sc.gap_extend;
    for (int j = 0; j < seg; j++) {
        int pos = gl * seg + j;
        int code = 5;
        if (pos < qlen) code = c_ssw_code[q_rev ? q[qlen - 1 - pos] : q[pos]];
        qc[j * G + gl] = (int8_t)code;
        H[j * G + gl] = 0;
        E[j * G + gl] = 0;
    }
    __syncwarp(mask);
    int max = 0, end_ref = WORD ? 0 : -1, end_read = qlen - 1;
    int vMaxScore = 0, vMaxMark = 0;
    bool overflow = false;
    int cols = 0;
    for (int tt = 0; tt < rlen; tt++) {
        cols = tt + 1;
        const int i = r_rev ? rlen - 1 - tt : tt;
        const int rb = c_ssw_code[r[i]];
        int last = H[(seg - 1) * G + gl];
        int vH = __shfl_up_sync(mask, last, 1, G);
        if (gl == 0) vH = 0;
        int vF = 0, vMaxCol = 0;
        for (int j = 0; j < seg; j++) {
            const int idx = j * G + gl;
            const int code = qc[idx];
            int h;
            if (WORD) {
                int m = code == 5 ? 0 : ((code == rb && rb < 4) ? (int)sc.match : -(int)sc.mismatch);
                h = adds16(vH, m);
            } else {
                int m = code == 5 ? bias : ((code == rb && rb < 4) ? (int)sc.match : -(int)sc.mismatch) + bias;
                h = subus8(addus8(vH, m), bias);
            }
            int e = E[idx];
            h = h > e ? h : e;
            h = h > vF ? h : vF;
            vMaxCol = vMaxCol > h ? vMaxCol : h;
            int hold = H[idx];
            H[idx] = (typename Lanes<WORD>::T)h;
            if (WORD) {
                h = subus16(h, gO);
                e = subus16(e, gE);
                e = e > h ? e : h;
                vF = subus16(vF, gE);
            } else {
                h = subus8(h, gO);
                e = subus8(e, gE);
                e = e > h ? e : h;
                vF = subus8(vF, gE);
            }
            E[idx] = (typename Lanes<WORD>::T)e;
            vF = vF > h ? vF : h;
            vH = hold;
        }
        // lazy-F (ext/ssw/ssw.c:285-299 / :491-502)
        for (int kk = 0; kk < G; kk++) {
            vF = __shfl_up_sync(mask, vF, 1, G);
            if (gl == 0) vF = 0;
            bool done = false;
            for (int j = 0; j < seg; j++) {
                const int idx = j * G + gl;
                int h = H[idx];
                h = h > vF ? h : vF;
                vMaxCol = vMaxCol > h ? vMaxCol : h;
                H[idx] = (typename Lanes<WORD>::T)h;
                bool settled;
                if (WORD) {
                    h = subus16(h, gO);
                    vF = subus16(vF, gE);
                    settled = !(vF > h);
                } else {
                    h = subus8(h, gO);
                    vF = subus8(vF, gE);
                    settled = subus8(vF, h) == 0;
                }
                if (__all_sync(mask, settled)) { done = true; break; }
            }
            if (done) break;
        }
        vMaxScore = vMaxScore > vMaxCol ? vMaxScore : vMaxCol;
        if (__any_sync(mask, vMaxScore != vMaxMark)) {
            vMaxMark = vMaxScore;
            int temp = vMaxScore;
            for (int d = G / 2; d > 0; d >>= 1) {
                int o = __shfl_xor_sync(mask, temp, d, G);
                temp = temp > o ? temp : o;
            }
            if (temp > max) {
                max = temp;
                if (!WORD && max + bias >= 255) { overflow = true; break; }
                end_ref = i;
                int best = 0x7fffffff;
                for (int j = 0; j < seg; j++)
                    if ((int)H[j * G + gl] == max) {
                        int pos = gl * seg + j;
                        best = pos < best ? pos : best;
                    }
                for (int d = G / 2; d > 0; d >>= 1) {
                    int o = __shfl_xor_sync(mask, best, d, G);
                    best = best < o ? best : o;
                }
                end_read = best < qlen - 1 ? best : qlen - 1;
            }
        }
        int cm = vMaxCol;
        for (int d = G / 2; d > 0; d >>= 1) {
            int o = __shfl_xor_sync(mask, cm, d, G);
            cm = cm > o ? cm : o;
        }
        if (cm == terminate) break;
    }
    (void)overflow;
    EndPos res;
    res.cols = cols;
    res.score = WORD ? max : (max + bias >= 255 ? 255 : max);
    res.ref = end_ref;
    res.read = end_read;
    return res;
}

// pass: 0 forward, 1 reverse (start position search)
template <bool WORD>
__global__ void __launch_bounds__(128) k_sw(SswTask* tasks, const uint32_t* list, const uint32_t* n_list_ptr,
                                            uint32_t n_list_host, const PrepRec* prep, const uint8_t* arena,
                                            AlignScores sc, int bias, int pass, int max_seg, uint32_t* counters,
                                            uint32_t* list_word, uint32_t* list_rev_byte, uint32_t* list_rev_word) {
    constexpr int G = Lanes<WORD>::G;
    using T = typename Lanes<WORD>::T;
    extern __shared__ __align__(16) uint8_t smem[];
    const uint32_t n_list = n_list_ptr ? *n_list_ptr : n_list_host;
    const int lane = threadIdx.x & 31;
    const int grp_in_warp = lane / G, gl = lane % G;
    const unsigned mask = (G == 32 ? FULLM : ((1u << G) - 1) << (grp_in_warp * G));
    const int groups_per_block = blockDim.x / G;
    const int grp = threadIdx.x / G;
    const size_t per_group = (size_t)max_seg * G * (2 * sizeof(T) + 1);
    T* H = reinterpret_cast<T*>(smem + grp * per_group);
    T* E = H + max_seg * G;
    int8_t* qc = reinterpret_cast<int8_t*>(E + max_seg * G);
    for (uint32_t base = blockIdx.x * groups_per_block; base < n_list; base += gridDim.x * groups_per_block) {
        const uint32_t li = base + grp;
        if (li >= n_list) continue;  // whole group idles together
        const uint32_t ti = list ? list[li] : li;
        SswTask tk = tasks[ti];
        const PrepRec p = prep[tk.job];
        const uint8_t* q = arena + p.arena_off;
        const uint8_t* r = q + p.qlen;
        if (pass == 0) {
            EndPos e = sw_pass<WORD>(q, (int)p.qlen, false, r, (int)p.wlen, false, WORD ? 65535 : 255, sc, bias, H, E,
                                     qc, mask, gl);
            if (gl == 0) {
                atomicAdd(reinterpret_cast<unsigned long long*>(counters + 8) + 1 + (WORD ? 1 : 0),
                          (unsigned long long)p.qlen * (unsigned long long)e.cols);
                if (!WORD && e.score == 255) {
                    list_word[atomicAdd(&counters[1], 1u)] = ti;
                } else {
                    tk.score1 = e.score;
                    tk.ref_end1 = e.ref;
                    tk.read_end1 = e.read;
                    tk.word = WORD;
                    tasks[ti] = tk;
                    if (WORD) list_rev_word[atomicAdd(&counters[3], 1u)] = ti;
                    else list_rev_byte[atomicAdd(&counters[2], 1u)] = ti;
                }
            }
        } else {
            // reverse pass over read[0..=read_end1] and ref[0..=ref_end1] (ext/ssw/ssw.c:870-888)
            EndPos e;
            if (tk.ref_end1 < 0) {
                e.score = 0;
                e.ref = -1;
                e.read = tk.read_end1;
                e.cols = 0;
            } else {
                e = sw_pass<WORD>(q, tk.read_end1 + 1, true, r, tk.ref_end1 + 1, true, tk.score1, sc, bias, H, E, qc,
                                  mask, gl);
            }
            if (gl == 0) {
                tk.ref_begin1 = e.ref;
                tk.read_begin1 = tk.read_end1 - e.read;
                tk.flag = tk.score1 > e.score ? 2 : 0;
                atomicAdd(reinterpret_cast<unsigned long long*>(counters + 8) + 3 + (WORD ? 1 : 0),
                          (unsigned long long)(tk.read_end1 + 1) * (unsigned long long)e.cols);
                tasks[ti] = tk;
            }
        }
        __syncwarp(mask);
    }
}

// ------------------------------------------------------------------ striped SW, registers
// The same striped passes with each lane's segment column of H and E in registers
// (SEG >= segLen rows per lane, the loops unrolled) and the striped query profile
// (ext/ssw/ssw.c:114-146 qP_byte / qP_word) as signed bytes in shared memory, one
// 32-bit word per four rows.  Scores are plain ints: byte mode without
// saturation equals ssw.c's biased u8 arithmetic until the column max reaches
// 255 - bias, and that column ends the byte pass as an overflow in both forms;
// word scores never reach the i16 limits (|score| <= 2 x 2048 x 127).
template <int G, int SEG>
__device__ EndPos sw_pass_reg(const uint8_t* q, int qlen, bool q_rev, const uint8_t* r, int rlen, bool r_rev,
                              bool check_term, int terminate, const AlignScores& sc, int bias, bool byte_mode,
                              uint32_t* prof, unsigned mask, int gl) {
    constexpr int SEGW = (SEG + 3) / 4;
    const int seg = (qlen + G - 1) / G;
    const int gO = sc.gap_open, gE = sc.gap_extend;
    const int match = sc.match, mism = -(int)sc.mismatch;
    // prof[(b * G + gl) * SEGW + w]: rows gl*seg + 4w .. 4w+3 against reference code b (4 = N)
    for (int b = 0; b < 5; b++) {
        for (int w = 0; w < SEGW; w++) {
            uint32_t word = 0;
            for (int x = 0; x < 4; x++) {
                const int j = 4 * w + x, pos = gl * seg + j;
                int s = 0;
                if (j < seg && pos < qlen) {
                    const int code = c_ssw_code[q_rev ? q[qlen - 1 - pos] : q[pos]];
                    s = (code == b && b < 4) ? match : mism;
                }
                word |= (uint32_t)(uint8_t)(int8_t)s << (8 * x);
            }
            prof[(b * G + gl) * SEGW + w] = word;
        }
    }
    __syncwarp(mask);
    int H[SEG], E[SEG];
#pragma unroll
    for (int j = 0; j < SEG; j++) {
        H[j] = 0;
        E[j] = 0;
    }
    int max = 0, end_ref = byte_mode ? -1 : 0, end_read = qlen - 1;
    int vMaxScore = 0, vMaxMark = 0, cols = 0;
    int rb_next = rlen > 0 ? c_ssw_code[r[r_rev ? rlen - 1 : 0]] : 0;
    for (int tt = 0; tt < rlen; tt++) {
        cols = tt + 1;
        const int i = r_rev ? rlen - 1 - tt : tt;
        const int rb = rb_next;
        if (tt + 1 < rlen) rb_next = c_ssw_code[r[r_rev ? rlen - 2 - tt : tt + 1]];
        uint32_t P[SEGW];
        const uint32_t* pp = prof + (rb * G + gl) * SEGW;
#pragma unroll
        for (int w = 0; w < SEGW; w++) P[w] = pp[w];
        int last = H[0];
#pragma unroll
        for (int j = 1; j < SEG; j++)
            if (j < seg) last = H[j];
        int vH = __shfl_up_sync(mask, last, 1, G);
        if (gl == 0) vH = 0;
        int vF = 0, vMaxCol = 0;
#pragma unroll
        for (int j = 0; j < SEG; j++) {
            if (j >= seg) break;
            const int m = (int)(int8_t)(uint8_t)(P[j >> 2] >> (8 * (j & 3)));
            const int e = E[j];
            int h = vH + m;
            h = h > e ? h : e;
            h = h > vF ? h : vF;
            vMaxCol = vMaxCol > h ? vMaxCol : h;
            vH = H[j];
            H[j] = h;
            int hg = h - gO;
            hg = hg > 0 ? hg : 0;
            const int e2 = e - gE;
            E[j] = e2 > hg ? e2 : hg;
            const int f2 = vF - gE;
            vF = f2 > hg ? f2 : hg;
        }
        // lazy-F (ext/ssw/ssw.c:285-299 / :491-502)
        for (int kk = 0; kk < G; kk++) {
            vF = __shfl_up_sync(mask, vF, 1, G);
            if (gl == 0) vF = 0;
            bool done = false;
#pragma unroll
            for (int j = 0; j < SEG; j++) {
                if (j >= seg) break;
                int h = H[j] > vF ? H[j] : vF;
                vMaxCol = vMaxCol > h ? vMaxCol : h;
                H[j] = h;
                int hg = h - gO;
                hg = hg > 0 ? hg : 0;
                vF = vF - gE > 0 ? vF - gE : 0;
                if (__all_sync(mask, vF <= hg)) {
                    done = true;
                    break;
                }
            }
            if (done) break;
        }
        vMaxScore = vMaxScore > vMaxCol ? vMaxScore : vMaxCol;
        if (__any_sync(mask, vMaxScore != vMaxMark)) {
            vMaxMark = vMaxScore;
            int temp = vMaxScore;
            for (int d = G / 2; d > 0; d >>= 1) {
                const int o = __shfl_xor_sync(mask, temp, d, G);
                temp = temp > o ? temp : o;
            }
            if (temp > max) {
                max = temp;
                if (byte_mode && max + bias >= 255) break;
                end_ref = i;
                int best = 0x7fffffff;
#pragma unroll
                for (int j = 0; j < SEG; j++) {
                    if (j >= seg) break;
                    if (H[j] == max) {
                        const int pos = gl * seg + j;
                        best = pos < best ? pos : best;
                    }
                }
                for (int d = G / 2; d > 0; d >>= 1) {
                    const int o = __shfl_xor_sync(mask, best, d, G);
                    best = best < o ? best : o;
                }
                end_read = best < qlen - 1 ? best : qlen - 1;
            }
        }
        if (check_term) {
            int cm = vMaxCol;
            for (int d = G / 2; d > 0; d >>= 1) {
                const int o = __shfl_xor_sync(mask, cm, d, G);
                cm = cm > o ? cm : o;
            }
            if (cm == terminate) break;
        }
    }
    EndPos res;
    res.cols = cols;
    res.score = !byte_mode ? max : (max + bias >= 255 ? 255 : max);
    res.ref = end_ref;
    res.read = end_read;
    return res;
}

// k_sw with sw_pass_reg: the forward pass never meets its terminate value (byte
// mode stops on overflow first, word scores stay below 65535), so only the reverse
// pass checks it.
template <bool WORD, int SEG>
__global__ void __launch_bounds__(128) k_swr(SswTask* tasks, const uint32_t* list, const uint32_t* n_list_ptr,
                                             uint32_t n_list_host, const PrepRec* prep, const uint8_t* arena,
                                             AlignScores sc, int bias, int pass, uint32_t* counters,
                                             uint32_t* list_word, uint32_t* list_rev_byte, uint32_t* list_rev_word) {
    constexpr int G = Lanes<WORD>::G;
    constexpr int SEGW = (SEG + 3) / 4;
    extern __shared__ __align__(16) uint32_t prof_smem[];
    const uint32_t n_list = n_list_ptr ? *n_list_ptr : n_list_host;
    const int lane = threadIdx.x & 31;
    const int grp_in_warp = lane / G, gl = lane % G;
    const unsigned mask = (G == 32 ? FULLM : ((1u << G) - 1) << (grp_in_warp * G));
    const int groups_per_block = blockDim.x / G;
    const int grp = threadIdx.x / G;
    uint32_t* prof = prof_smem + grp * (5 * G * SEGW);
    for (uint32_t base = blockIdx.x * groups_per_block; base < n_list; base += gridDim.x * groups_per_block) {
        const uint32_t li = base + grp;
        if (li >= n_list) continue;  // whole group idles together
        const uint32_t ti = list ? list[li] : li;
        SswTask tk = tasks[ti];
        const PrepRec p = prep[tk.job];
        const uint8_t* q = arena + p.arena_off;
        const uint8_t* r = q + p.qlen;
        if (pass == 0) {
            EndPos e = sw_pass_reg<G, SEG>(q, (int)p.qlen, false, r, (int)p.wlen, false, false, 0, sc, bias, !WORD,
                                           prof, mask, gl);
            if (gl == 0) {
                atomicAdd(reinterpret_cast<unsigned long long*>(counters + 8) + 1 + (WORD ? 1 : 0),
                          (unsigned long long)p.qlen * (unsigned long long)e.cols);
                if (!WORD && e.score == 255) {
                    list_word[atomicAdd(&counters[1], 1u)] = ti;
                } else {
                    tk.score1 = e.score;
                    tk.ref_end1 = e.ref;
                    tk.read_end1 = e.read;
                    tk.word = WORD;
                    tasks[ti] = tk;
                    if (WORD) list_rev_word[atomicAdd(&counters[3], 1u)] = ti;
                    else list_rev_byte[atomicAdd(&counters[2], 1u)] = ti;
                }
            }
        } else {
            EndPos e;
            if (tk.ref_end1 < 0) {
                e.score = 0;
                e.ref = -1;
                e.read = tk.read_end1;
                e.cols = 0;
            } else {
                e = sw_pass_reg<G, SEG>(q, tk.read_end1 + 1, true, r, tk.ref_end1 + 1, true, true, tk.score1, sc, bias,
                                        !WORD, prof, mask, gl);
            }
            if (gl == 0) {
                tk.ref_begin1 = e.ref;
                tk.read_begin1 = tk.read_end1 - e.read;
                tk.flag = tk.score1 > e.score ? 2 : 0;
                atomicAdd(reinterpret_cast<unsigned long long*>(counters + 8) + 3 + (WORD ? 1 : 0),
                          (unsigned long long)(tk.read_end1 + 1) * (unsigned long long)e.cols);
                tasks[ti] = tk;
            }
        }
        __syncwarp(mask);
    }
}

// ------------------------------------------------------------------ fused SSW, warp per task
// ssw_align's search for both ends (ext/ssw/ssw.c:818-888) for one task per warp,
// in one launch: the byte pass, the word rerun when the byte pass overflows, then
// the reverse pass in the mode that produced the score.
//
// Layout: NL SSE lanes (16 byte, 8 word) of segLen = ceil(L / NL) rows each, as
// in the library.  A lane's rows are split over S = 32 / NL threads in
// consecutive blocks of R = ceil(segLen / S) rows, so thread (l, s) holds rows
// l*segLen + s*R ... in registers and the 32 threads hold the query in order.
//
// Within a column the F recurrence is rewritten as vF' = max(vF - gE, a) with
// a = max(max(vH + m, E) - gO, 0); this equals the library's update whenever
// gap_open >= gap_extend (the term H - gO that vF itself feeds never exceeds
// vF - gE).  It is linear in the max-plus sense, so each thread scans its own rows
// and a max-plus scan over the S threads of a lane supplies the F entering each
// block.  The lazy-F pass has a closed form (below), and the column maximum
// bookkeeping (vMaxScore / vMaxMark) reduces to "the running maximum grew in this
// column".
__device__ __forceinline__ int warp_max32(int v) {
    for (int d = 16; d > 0; d >>= 1) {
        const int o = __shfl_xor_sync(FULLM, v, d);
        v = v > o ? v : o;
    }
    return v;
}
__device__ __forceinline__ int warp_min32(int v) {
    for (int d = 16; d > 0; d >>= 1) {
        const int o = __shfl_xor_sync(FULLM, v, d);
        v = v < o ? v : o;
    }
    return v;
}

template <int NL, int RMAX>
__device__ __noinline__ EndPos ssw_warp_pass(const uint8_t* q, int qlen, bool q_rev, const uint8_t* r, int rlen, bool r_rev,
                                bool check_term, int terminate, const AlignScores& sc, int bias, uint32_t* prof) {
    constexpr int S = 32 / NL;
    constexpr int RW = (RMAX + 3) / 4;
    constexpr bool BYTE = NL == 16;
    if (qlen <= 0) {
        EndPos z;
        z.score = 0;
        z.ref = BYTE ? -1 : 0;
        z.read = qlen - 1;
        z.cols = 0;
        return z;
    }
    const int tau = threadIdx.x & 31, l = tau / S, s = tau % S;
    const int seg = (qlen + NL - 1) / NL;
    const int R = (seg + S - 1) / S;
    const int j0 = s * R;
    int nr = seg - j0;
    nr = nr < 0 ? 0 : (nr > R ? R : nr);
    const int s_last = (seg - 1) / R;
    // owner of the row before this thread's first row (row l*seg + j0 - 1)
    const int pred = s > 0 ? tau - 1 : (l > 0 ? (l - 1) * S + s_last : 0);
    const int gO = sc.gap_open, gE = sc.gap_extend;
    const int match = sc.match, mism = -(int)sc.mismatch;
    // prof[(b * 32 + tau) * RW + w]: this thread's rows j0 + 4w .. 4w+3 against reference code b (4 = N)
    for (int b = 0; b < 5; b++)
        for (int w = 0; w < RW; w++) {
            uint32_t word = 0;
            for (int y = 0; y < 4; y++) {
                const int rr = 4 * w + y, pos = l * seg + j0 + rr;
                int sv = 0;
                if (rr < nr && pos < qlen) {
                    const int code = c_ssw_code[q_rev ? q[qlen - 1 - pos] : q[pos]];
                    sv = (code == b && b < 4) ? match : mism;
                }
                word |= (uint32_t)(uint8_t)(int8_t)sv << (8 * y);
            }
            prof[(b * 32 + tau) * RW + w] = word;
        }
    __syncwarp();
    int H[RMAX], E[RMAX];
#pragma unroll
    for (int rr = 0; rr < RMAX; rr++) {
        H[rr] = 0;
        E[rr] = 0;
    }
    int max = 0, end_ref = BYTE ? -1 : 0, end_read = qlen - 1, cols = 0;
    int rb_next = rlen > 0 ? c_ssw_code[r[r_rev ? rlen - 1 : 0]] : 0;
    for (int tt = 0; tt < rlen; tt++) {
        cols = tt + 1;
        const int i = r_rev ? rlen - 1 - tt : tt;
        const int rb = rb_next;
        if (tt + 1 < rlen) rb_next = c_ssw_code[r[r_rev ? rlen - 2 - tt : tt + 1]];
        uint32_t P[RW];
        const uint32_t* pp = prof + (rb * 32 + tau) * RW;
#pragma unroll
        for (int w = 0; w < RW; w++) P[w] = pp[w];
        int lastH = H[0];
#pragma unroll
        for (int rr = 1; rr < RMAX; rr++)
            if (rr < nr) lastH = H[rr];
        int vH = __shfl_sync(FULLM, lastH, pred);
        if (tau == 0) vH = 0;
        // main pass, part 1: diagonal + E candidates and the local F scan (F entering
        // this thread's first row taken as 0).  max/add pairs are single DPX ops.
        int A[RMAX], F[RMAX];
        int f = 0;
#pragma unroll
        for (int rr = 0; rr < RMAX; rr++) {
            if (rr >= nr) break;
            const int m = (int)(int8_t)(uint8_t)(P[rr >> 2] >> (8 * (rr & 3)));
            const int x = __viaddmax_s32(vH, m, E[rr]);  // max(vH + m, E)
            A[rr] = x;
            vH = H[rr];
            F[rr] = f;
            f = __viaddmax_s32(f, -gE, __viaddmax_s32(x, -gO, 0));  // max(f - gE, max(x - gO, 0))
        }
        // F entering this thread's block: max-plus scan over the lane's threads
        int fin = 0;
        if (S > 1) {
            int D = nr * gE, V = f;
#pragma unroll
            for (int d = 1; d < S; d <<= 1) {
                const int Dp = __shfl_up_sync(FULLM, D, d, S);
                const int Vp = __shfl_up_sync(FULLM, V, d, S);
                if (s >= d) {
                    const int c = Vp - D;
                    V = c > V ? c : V;
                    D += Dp;
                }
            }
            const int pv = __shfl_up_sync(FULLM, V, 1, S);
            fin = s > 0 ? pv : 0;
        }
        // lazy-F (ext/ssw/ssw.c:285-299 / :491-502) in closed form: the loop carries
        // the final F of each lane into the following lanes, decaying by gE per row,
        // and raises H to it; its early exit drops only values that could no longer
        // raise any H.  So H(l, j) = max(H, G(l) - j*gE) with G(l) the maximum over
        // lanes l' < l of Ffinal(l') - (l - 1 - l') * segLen * gE.  G depends only on
        // part 1 and the scan, so the raise joins part 2; E is computed from H before
        // the raise, as in the library (its lazy-F loop leaves E alone).
        int g;
        {
            int fout = fin - nr * gE;
            fout = fout > f ? fout : f;  // F leaving this thread's block
            int Y = __shfl_sync(FULLM, fout, l * S + s_last);
#pragma unroll
            for (int d = 1; d < NL; d <<= 1) {
                const int Yp = __shfl_up_sync(FULLM, Y, d * S);
                const int c = Yp - d * seg * gE;
                if (l >= d) Y = Y > c ? Y : c;
            }
            const int Gp = __shfl_up_sync(FULLM, Y, S);
            g = l > 0 ? Gp - j0 * gE : 0;
        }
        // part 2: H, E with the F entering each row, then the lazy-F raise
        int colmax = 0;
        {
            int fr = fin;
#pragma unroll
            for (int rr = 0; rr < RMAX; rr++) {
                if (rr >= nr) break;
                const int h = __vimax3_s32(A[rr], fr, F[rr]);
                E[rr] = __viaddmax_s32(E[rr], -gE, __viaddmax_s32(h, -gO, 0));  // max(E - gE, max(h - gO, 0))
                H[rr] = h > g ? h : g;
                colmax = __vimax3_s32(colmax, h, g);
                fr -= gE;
                g -= gE;
            }
        }
        if (__any_sync(FULLM, colmax > max)) {
            max = warp_max32(colmax);
            if (BYTE && max + bias >= 255) break;
            end_ref = i;
            int best = 0x7fffffff;
#pragma unroll
            for (int rr = 0; rr < RMAX; rr++) {
                if (rr >= nr) break;
                if (H[rr] == max) {
                    const int pos = l * seg + j0 + rr;
                    best = pos < best ? pos : best;
                }
            }
            best = warp_min32(best);
            end_read = best < qlen - 1 ? best : qlen - 1;
        }
        if (check_term && __any_sync(FULLM, colmax >= terminate) && warp_max32(colmax) == terminate) break;
    }
    EndPos res;
    res.cols = cols;
    res.score = !BYTE ? max : (max + bias >= 255 ? 255 : max);
    res.ref = end_ref;
    res.read = end_read;
    return res;
}

// Tasks are taken in list order through a shared counter, so the longest windows
// (put first by the caller) start first.
// the shortest-read variant fits 5 blocks per SM without spills (96 registers)
template <int RMAX>
__global__ void __launch_bounds__(128, RMAX <= 4 ? 5 : 1) k_ssw(SswTask* tasks, const uint32_t* order, uint32_t n_tasks,
                                             const PrepRec* prep, const uint8_t* arena, AlignScores sc, int bias,
                                             uint32_t* counters, uint32_t* queue, uint32_t qmin) {
    constexpr int RW = (RMAX + 3) / 4;
    extern __shared__ __align__(16) uint32_t ssw_smem[];
    const int lane = threadIdx.x & 31;
    uint32_t* prof = ssw_smem + (threadIdx.x / 32) * (5 * 32 * RW);
    unsigned long long* cells = reinterpret_cast<unsigned long long*>(counters + 8);
    for (;;) {
        uint32_t li = 0;
        if (lane == 0) li = atomicAdd(queue, 1u);
        li = __shfl_sync(FULLM, li, 0);
        if (li >= n_tasks) break;
        const uint32_t ti = order ? order[li] : li;
        SswTask tk = tasks[ti];
        const PrepRec p = prep[tk.job];
        if (p.qlen <= qmin) continue;  // k_ssw_wave's task
        const uint8_t* q = arena + p.arena_off;
        const uint8_t* r = q + p.qlen;
        // forward: byte, word on overflow (ext/ssw/ssw.c:840-862)
        EndPos e = ssw_warp_pass<16, RMAX>(q, (int)p.qlen, false, r, (int)p.wlen, false, false, 0, sc, bias, prof);
        unsigned long long c_fb = (unsigned long long)p.qlen * e.cols, c_fw = 0, c_rb = 0, c_rw = 0;
        bool word = false;
        if (e.score == 255) {
            __syncwarp();
            e = ssw_warp_pass<8, RMAX>(q, (int)p.qlen, false, r, (int)p.wlen, false, false, 0, sc, bias, prof);
            c_fw = (unsigned long long)p.qlen * e.cols;
            word = true;
        }
        tk.score1 = e.score;
        tk.ref_end1 = e.ref;
        tk.read_end1 = e.read;
        tk.word = word;
        // reverse pass over read[0..=read_end1] and ref[0..=ref_end1] (ext/ssw/ssw.c:870-888)
        EndPos b;
        if (tk.ref_end1 < 0) {
            b.score = 0;
            b.ref = -1;
            b.read = tk.read_end1;
            b.cols = 0;
        } else {
            __syncwarp();
            if (word)
                b = ssw_warp_pass<8, RMAX>(q, tk.read_end1 + 1, true, r, tk.ref_end1 + 1, true, true, tk.score1, sc,
                                           bias, prof);
            else
                b = ssw_warp_pass<16, RMAX>(q, tk.read_end1 + 1, true, r, tk.ref_end1 + 1, true, true, tk.score1, sc,
                                            bias, prof);
        }
        (word ? c_rw : c_rb) = (unsigned long long)(tk.read_end1 + 1) * b.cols;
        tk.ref_begin1 = b.ref;
        tk.read_begin1 = tk.read_end1 - b.read;
        tk.flag = tk.score1 > b.score ? 2 : 0;
        if (lane == 0) {
            tasks[ti] = tk;
            atomicAdd(cells + 1, c_fb);
            if (c_fw) atomicAdd(cells + 2, c_fw);
            if (c_rb) atomicAdd(cells + 3, c_rb);
            if (c_rw) atomicAdd(cells + 4, c_rw);
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ SSW, lane wavefront
// ssw_align's passes (ext/ssw/ssw.c:818-888) with eight threads per task, four tasks
// per warp.  Thread t holds the query rows t*N .. t*N + N - 1 in registers: one SSE
// lane of segLen = N rows in word mode (8 lanes), two consecutive lanes of N/2 rows
// in byte mode (16 lanes); rows past the read are the library's padding (score 0).
// Every thread starts at a lane boundary, so its F chain starts at 0 as in the
// library's main loop (ext/ssw/ssw.c:256-283), and the lazy-F pass reduces to a raise
// G that enters each lane: G(l + 1) = max(G(l) - segLen * gE, Ffinal(l)), applied as
// H = max(H, G - j * gE) at row j (E keeps the value before the raise).
//
// The threads form a wavefront over the reference columns: thread t works on column
// s - t at step s and passes to thread t + 1 its last row's H, its final F, its G and
// the column's best (score, row) so far, so the last thread holds each column's
// maximum and the row of its first occurrence, and keeps the running maximum, the
// end positions and the stop conditions (byte overflow, the reverse pass's
// terminate score) in the library's column order.
//
// Scores are ints scaled by 256: the low byte of a packed key holds 255 - row, so a
// single max per cell tracks both the column maximum and its smallest row.  The
// query profile (rows x 5 reference codes) is int16 in shared memory, 8 rows per
// 16-byte word, laid out [code][word][lane] per warp.
constexpr int WV_T = 8;      // threads per task
constexpr int WAVE_NMAX = 24;  // rows per thread: reads up to 8 * 24 = 192 nt
constexpr int WAVE_NMAX_SHORT = 20;  // reads up to 160 nt: fewer registers, five blocks per SM
constexpr int WV_SCALE = 8;  // log2 of the score scale (rows < 256)

struct WaveScores {
    int gO, gE;  // scaled
};
// the default gap penalties (12, 1) as constants: the per-row offsets of the lazy-F
// raise become immediates and the penalties leave the registers
struct DefaultWaveScores {
    static constexpr int gO = 12 << WV_SCALE, gE = 1 << WV_SCALE;
};

template <int N, bool BYTE, class WS>
__device__ __forceinline__ EndPos wave_loop(const uint8_t* r, int rlen, bool r_rev, int qlen, bool check_term,
                                            int terminate, int bias, WS ws, const uint4* prof, int gl,
                                            unsigned m, bool run) {
    constexpr int NW = (N + 7) / 8;
    int H[N], E[N];
#pragma unroll
    for (int j = 0; j < N; j++) {
        H[j] = 0;
        E[j] = 0;
    }
    const int gO = ws.gO, gE = ws.gE;
    const int tb = 255 - gl * N - (N - 1);  // key low byte: 255 - row
    const int gbit = (threadIdx.x & 31) | (WV_T - 1);  // this group's last thread
    int max = 0, end_ref = BYTE ? -1 : 0, end_read = qlen - 1, cols = 0;
    int h_out = 0, f_out = 0, g_out = 0, k_out = -1, b_out = 0, hdiag = 0;
    int rb_next = (run && gl == 0 && rlen > 0) ? c_ssw_code[r[r_rev ? rlen - 1 : 0]] : 0;
    const int steps = run ? rlen + WV_T - 1 : 0;
    bool done = false;
    for (int s = 0;; s++) {
        const bool act = s < steps && !done;
        if (!__any_sync(m, act)) break;
        const int hin = __shfl_up_sync(m, h_out, 1, WV_T);
        const int fin0 = __shfl_up_sync(m, f_out, 1, WV_T);
        const int gin0 = __shfl_up_sync(m, g_out, 1, WV_T);
        const int kin0 = __shfl_up_sync(m, k_out, 1, WV_T);
        int rb = __shfl_up_sync(m, b_out, 1, WV_T);
        const int c = s - gl;
        bool stop = false;
        if (act && gl == 0) {
            rb = rb_next;
            if (s + 1 < rlen) rb_next = c_ssw_code[r[r_rev ? rlen - 2 - s : s + 1]];
        }
        if (act && c >= 0 && c < rlen) {
            const int fin = gl == 0 ? 0 : fin0, gin = gl == 0 ? 0 : gin0, kin = gl == 0 ? -1 : kin0;
            int diag = gl == 0 ? 0 : hdiag;
            // every thread starts a lane: F restarts at 0 and G takes the F leaving the
            // lane above (ext/ssw/ssw.c:285-299); row j of a lane is raised to G - j * gE
            int gb = fin > gin ? fin : gin;
            int F = 0;
            int k0 = -1, k1 = -1;
            uint4 P[NW];
#pragma unroll
            for (int w = 0; w < NW; w++) P[w] = prof[(rb * NW + w) * 32];
#pragma unroll
            for (int j = 0; j < N; j++) {
                constexpr int H2 = BYTE ? N / 2 : N;
                const int jl = BYTE && j >= H2 ? j - H2 : j;  // row within its lane
                const uint32_t pw = (&P[j >> 3].x)[(j >> 1) & 3];
                const int sc = (j & 1) ? ((int)pw >> 16) : (int)(int16_t)(pw & 0xffffu);
                const int A = __viaddmax_s32(diag, sc, E[j]);  // max(H(diag) + score, E)
                const int u = __viaddmax_s32(A, -gO, 0);
                const int Hp = A > F ? A : F;                   // H before the lazy-F raise
                const int t = __viaddmax_s32(F, -gO, u);        // max(Hp - gO, 0)
                E[j] = __viaddmax_s32(E[j], -gE, t);
                // the library's max(F - gE, max(Hp - gO, 0)); F - gO <= F - gE drops out, so
                // the F chain carries one max per row
                F = __viaddmax_s32(F, -gE, u);
                const int gj = gb - jl * gE;
                const int Hr = Hp > gj ? Hp : gj;
                if (j & 1) k1 = __viaddmax_s32(Hr, N - 1 - j, k1);
                else k0 = __viaddmax_s32(Hr, N - 1 - j, k0);
                diag = H[j];
                H[j] = Hr;
                if (BYTE && j == H2 - 1) {
                    // the second lane of this thread starts
                    const int ge = gb - H2 * gE;
                    gb = F > ge ? F : ge;
                    F = 0;
                }
            }
            const int g = gb - (BYTE ? N / 2 : N) * gE;  // G entering the next thread's first row
            int key = k0 > k1 ? k0 : k1;
            key += tb;
            k_out = key > kin ? key : kin;
            h_out = H[N - 1];
            f_out = F;
            g_out = g;
            b_out = rb;
            if (gl == WV_T - 1) {
                // column c complete: the library's per-column bookkeeping
                const int i = r_rev ? rlen - 1 - c : c;
                const int cm = k_out >> WV_SCALE;
                cols = c + 1;
                if (cm > max) {
                    max = cm;
                    if (BYTE && max + bias >= 255) {
                        stop = true;
                    } else {
                        end_ref = i;
                        const int row = 255 - (k_out & 255);
                        end_read = row < qlen - 1 ? row : qlen - 1;
                    }
                }
                if (check_term && cm == terminate) stop = true;
            }
        }
        hdiag = hin;
        if ((__ballot_sync(m, stop) >> gbit) & 1u) done = true;
    }
    EndPos res;
    const int src = WV_T - 1;
    res.cols = __shfl_sync(m, cols, src, WV_T);
    const int mx = __shfl_sync(m, max, src, WV_T);
    res.score = !BYTE ? mx : (mx + bias >= 255 ? 255 : mx);
    res.ref = __shfl_sync(m, end_ref, src, WV_T);
    // the library scans the stored column for the maximum: all rows when it stayed 0
    const int rd = __shfl_sync(m, end_read, src, WV_T);
    res.read = mx == 0 ? 0 : rd;
    return res;
}

// One pass of every group of the warp that runs it (run): this thread's rows of the
// striped profile, then the wavefront with N = 2 * segLen (byte) or segLen (word) rows
// per thread.  All 32 threads enter together.  When the running groups share N, the
// warp runs them in lockstep (full-warp shuffles and votes); otherwise each group runs
// on its own with its own mask.
template <int NMAX, bool BYTE, bool DEF>
__device__ __forceinline__ EndPos wave_pass(bool run, const uint8_t* q, int qlen, bool q_rev, const uint8_t* r, int rlen,
                            bool r_rev, bool check_term, int terminate, const AlignScores& sc, int bias, uint4* prof,
                            int gl, unsigned gm) {
    EndPos z;
    z.score = 0;
    z.ref = BYTE ? -1 : 0;
    z.read = qlen - 1;
    z.cols = 0;
    if (run && qlen <= 0) run = false;
    const int N = !run ? 0 : BYTE ? 2 * ((qlen + 15) / 16) : (qlen + 7) / 8;
    const int nmax = __reduce_max_sync(FULLM, N);
    const int nmin = __reduce_min_sync(FULLM, run ? N : 0x7fffffff);
    if (nmax == 0) return z;  // no group of this warp runs this pass
    const bool uni = nmin == nmax;
    if (!uni && !run) return z;
    const unsigned m = uni ? FULLM : gm;
    const int NN = uni ? nmax : N;
    if (run) {
        const int nw = (NN + 7) / 8;
        const int match = sc.match << WV_SCALE, mism = -((int)sc.mismatch << WV_SCALE);
        for (int b = 0; b < 5; b++)
            for (int w = 0; w < nw; w++) {
                uint32_t v[4];
                for (int x = 0; x < 4; x++) {
                    uint32_t pair = 0;
                    for (int y = 0; y < 2; y++) {
                        const int j = 8 * w + 2 * x + y, pos = gl * NN + j;
                        int sv = 0;
                        if (j < NN && pos < qlen) {
                            const int code = c_ssw_code[q_rev ? q[qlen - 1 - pos] : q[pos]];
                            sv = (code == b && b < 4) ? match : mism;
                        }
                        pair |= (uint32_t)(uint16_t)(int16_t)sv << (16 * y);
                    }
                    v[x] = pair;
                }
                prof[(b * nw + w) * 32] = make_uint4(v[0], v[1], v[2], v[3]);
            }
    }
    using WS = std::conditional_t<DEF, DefaultWaveScores, WaveScores>;
    WS ws{};
    if constexpr (!DEF) ws = WaveScores{(int)sc.gap_open << WV_SCALE, (int)sc.gap_extend << WV_SCALE};
    EndPos res = z;
    // byte mode: N is even, so the odd cases are never taken there
#define SA_WV(K)                                                                                                 \
    case K:                                                                                                      \
        if constexpr (K <= NMAX && (!BYTE || K % 2 == 0))                                                        \
            res = wave_loop<K, BYTE, WS>(r, rlen, r_rev, qlen, check_term, terminate, bias, ws, prof, gl, m, run); \
        break;
    switch (NN) {
        SA_WV(1) SA_WV(2) SA_WV(3) SA_WV(4) SA_WV(5) SA_WV(6) SA_WV(7) SA_WV(8)
        SA_WV(9) SA_WV(10) SA_WV(11) SA_WV(12) SA_WV(13) SA_WV(14) SA_WV(15) SA_WV(16)
        SA_WV(17) SA_WV(18) SA_WV(19) SA_WV(20) SA_WV(21) SA_WV(22) SA_WV(23) SA_WV(24)
        default: break;
    }
#undef SA_WV
    return run ? res : z;
}

// A lower bound of the score ssw.c's striped passes reach (in either striping), from
// the NAM's diagonal: the best local path over diagonals d0 - 4 .. d0 + 3 with at most
// one gap of up to 3 bases, one diagonal per thread of the group (all 32 threads
// enter).  Such a path is a lower bound of the passes' H: every H takes the diagonal
// term; a gap entered from a cell reached diagonally is counted by E (computed from H
// before the lazy-F raise, which already holds the diagonal term) or by F (exact after
// the lazy-F loop); only a path that goes F then E could be missed, and none is used.
// When the bound reaches 255 - bias, the byte pass must overflow, so the task can run
// its word pass directly with the same results.  Returns the group's bound (0 when the
// group does not run).
__device__ __forceinline__ int wave_diag_bound(bool run, const uint8_t* q, int qlen, const uint8_t* r, int rlen,
                                               int d0, const AlignScores& sc, int gl) {
    constexpr int NEG = -(1 << 28);
    const int go = sc.gap_open, ge = sc.gap_extend, mat = sc.match, mis = -(int)sc.mismatch;
    const int rows = __reduce_max_sync(FULLM, run ? qlen : 0);
    const int delta = d0 + gl - 4;
    int A = NEG, B = NEG, best = 0;
    int h1 = NEG, h2 = NEG, h3 = NEG;  // A on this diagonal 1, 2, 3 rows back (h1 = A(i - 1))
    for (int i = 0; i < rows; i++) {
        const bool in = run && i < qlen;
        const int j = i + delta;
        int s = NEG;
        if (in && j >= 0 && j < rlen) {
            const int qc = c_ssw_code[q[i]], rc = c_ssw_code[r[j]];
            s = (qc == rc && qc < 4) ? mat : mis;
        }
        // entries into this diagonal after one gap: deletion from a lower diagonal
        // (lane - g, row i - 1), insertion from a higher one (lane + g, row i - 1 - g)
        const int d1 = __shfl_up_sync(FULLM, h1, 1, WV_T), d2 = __shfl_up_sync(FULLM, h1, 2, WV_T),
                  d3 = __shfl_up_sync(FULLM, h1, 3, WV_T);
        const int i1 = __shfl_down_sync(FULLM, h2, 1, WV_T), i2 = __shfl_down_sync(FULLM, h3, 2, WV_T);
        int x = NEG;
        if (gl >= 1) x = max(x, d1 - go);
        if (gl >= 2) x = max(x, d2 - go - ge);
        if (gl >= 3) x = max(x, d3 - go - 2 * ge);
        if (gl + 1 < WV_T) x = max(x, i1 - go);
        if (gl + 2 < WV_T) x = max(x, i2 - go - ge);
        if (s == NEG) {
            A = NEG;
            B = NEG;
        } else {
            A = max(A, 0) + s;
            B = max(B, x) + s;
            best = max(best, max(A, B));
        }
        h3 = h2;
        h2 = h1;
        h1 = A;
    }
#pragma unroll
    for (int o = WV_T / 2; o; o >>= 1) best = max(best, __shfl_xor_sync(FULLM, best, o, WV_T));
    return run ? best : 0;
}

// ssw_align's end searches with wave_pass for tasks of reads up to 8 * NMAX nt, in
// the longest-first order of k_ssw: each warp takes four consecutive tasks (one per
// group of eight threads) and runs the forward byte pass, the forward word pass of the
// tasks that overflowed, then the reverse passes in each task's mode.
template <int NMAX, bool DEF>
__global__ void __launch_bounds__(128, NMAX <= 20 ? 5 : 4) k_ssw_wave(SswTask* tasks, const uint32_t* order, uint32_t n_tasks,
                                                      const PrepRec* prep, const uint8_t* arena, AlignScores sc,
                                                      int bias, uint32_t* counters, uint32_t qmax) {
    constexpr int NW = (NMAX + 7) / 8;
    extern __shared__ __align__(16) uint4 wv_smem[];
    const int lane = threadIdx.x & 31, gi = lane / WV_T, gl = lane % WV_T;
    const unsigned gm = 0xffu << (WV_T * gi);
    uint4* prof = wv_smem + (threadIdx.x / 32) * (5 * NW * 32) + lane;
    unsigned long long* cells = reinterpret_cast<unsigned long long*>(counters + 8);
    constexpr uint32_t G = 32 / WV_T;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&counters[5], G);
        base = __shfl_sync(FULLM, base, 0);
        if (base >= n_tasks) break;
        const uint32_t li = base + gi;
        uint32_t ti = 0;
        bool have = li < n_tasks;
        if (have) {
            ti = order ? order[li] : li;
            have = prep[tasks[ti].job].qlen <= qmax;  // longer reads: k_ssw's task
        }
        int qlen = 0, wlen = 0;
        const uint8_t* q = arena;
        if (have) {
            const PrepRec& pr = prep[tasks[ti].job];
            qlen = (int)pr.qlen;
            wlen = (int)pr.wlen;
            q = arena + pr.arena_off;
        }
        const uint8_t* r = q + qlen;
        // a byte pass that must overflow is skipped: the word pass alone gives the same
        // results (the task's diagonal bound reaches 255 - bias)
        const uint32_t d0 = have ? prep[tasks[ti].job].diag : NO_DIAG;
        const bool try_bound = have && d0 != NO_DIAG && qlen * (int)sc.match >= 255 - bias;
        bool certain = false;
        if (__any_sync(FULLM, try_bound))
            certain = wave_diag_bound(try_bound, q, qlen, r, wlen, (int)d0, sc, gl) >= 255 - bias;
        // forward: byte, word on overflow (ext/ssw/ssw.c:840-862)
        EndPos e = wave_pass<NMAX, true, DEF>(have && !certain, q, qlen, false, r, wlen, false, false, 0, sc, bias, prof, gl,
                                         gm);
        const bool word = have && (certain || e.score == 255);
        const EndPos ew = wave_pass<NMAX, false, DEF>(word, q, qlen, false, r, wlen, false, false, 0, sc, bias, prof, gl,
                                                 gm);
        unsigned long long c_fb = certain ? 0 : (unsigned long long)qlen * e.cols, c_fw = 0, c_rb = 0, c_rw = 0;
        if (word) {
            e = ew;
            c_fw = (unsigned long long)qlen * e.cols;
        }
        // reverse pass over read[0..=read_end1] and ref[0..=ref_end1] (ext/ssw/ssw.c:870-888)
        const bool rev = have && e.ref >= 0;
        const EndPos bb = wave_pass<NMAX, true, DEF>(rev && !word, q, e.read + 1, true, r, e.ref + 1, true, true, e.score,
                                                sc, bias, prof, gl, gm);
        const EndPos bw = wave_pass<NMAX, false, DEF>(rev && word, q, e.read + 1, true, r, e.ref + 1, true, true, e.score,
                                                 sc, bias, prof, gl, gm);
        EndPos b = word ? bw : bb;
        if (!rev) {
            b.score = 0;
            b.ref = -1;
            b.read = e.read;
            b.cols = 0;
        }
        (word ? c_rw : c_rb) = (unsigned long long)(e.read + 1) * b.cols;
        if (have && gl == 0) {
            SswTask& tk = tasks[ti];
            tk.score1 = e.score;
            tk.ref_end1 = e.ref;
            tk.read_end1 = e.read;
            tk.word = word;
            tk.ref_begin1 = b.ref;
            tk.read_begin1 = e.read - b.read;
            tk.flag = e.score > b.score ? 2 : 0;
            atomicAdd(cells + 1, c_fb);
            if (c_fw) atomicAdd(cells + 2, c_fw);
            if (c_rb) atomicAdd(cells + 3, c_rb);
            if (c_rw) atomicAdd(cells + 4, c_rw);
        }
        __syncwarp();
    }
}

// window length of each task, for the longest-first order of k_ssw
__global__ void k_task_keys(const SswTask* tasks, uint32_t n, const PrepRec* prep, uint32_t* key, uint32_t* idx) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const PrepRec p = prep[tasks[i].job];
        const uint32_t cells = p.wlen * (p.qlen + 1) >> 7;  // < 2^16 for windows <= 2000, queries <= 2048
        key[i] = 0xffffu - (cells < 0xffffu ? cells : 0xffffu);  // ascending: largest first
        idx[i] = i;
    }
}

// ------------------------------------------------------------------ banded_sw
__device__ __forceinline__ int mat_score(int rc, int qc, const AlignScores& sc) {
    return (rc == qc && rc < 4) ? (int)sc.match : -(int)sc.mismatch;
}

// One band pass of banded_sw; with dir == nullptr only the maximum is computed.
__device__ int band_pass(const uint8_t* ref, const uint8_t* read, int ref_len, int read_len, int bw,
                         const AlignScores& sc, int* h_b, int* e_b, int* h_c, uint8_t* dir) {
    const int width = bw * 2 + 3, width_d = bw * 2 + 1;
    const int gO = sc.gap_open, gE = sc.gap_extend;
    int max = 0;
    for (int j = 0; j < width + 1; j++) { h_b[j] = 0; e_b[j] = 0; h_c[j] = 0; }
    for (int i = 0; i < read_len; i++) {
        int beg = i - bw > 0 ? i - bw : 0, end = ref_len - 1 < i + bw ? ref_len - 1 : i + bw;
        int edge = end + 1 < width - 1 ? end + 1 : width - 1;
        int f = 0, u = 0;
        h_b[0] = e_b[0] = h_b[edge] = e_b[edge] = h_c[0] = 0;
        uint8_t* line = dir ? dir + (size_t)width_d * i * 3 : nullptr;
        const int x = i - bw > 0 ? i - bw : 0, xe = i - 1 - bw > 0 ? i - 1 - bw : 0;
        const int qcode = c_ssw_code[read[i]];
        for (int j = beg; j <= end; j++) {
            u = j - x + 1;
            int e = j - xe + 1, b = j - x, d = j - xe;
            int de = (j - x) * 3, df = de + 1, dh = de + 2;
            int t1 = i == 0 ? -gO : h_b[e] - gO;
            int t2 = i == 0 ? -gE : e_b[e] - gE;
            e_b[u] = t1 > t2 ? t1 : t2;
            uint8_t dde = t1 > t2 ? 3 : 2;
            t1 = h_c[b] - gO;
            t2 = f - gE;
            f = t1 > t2 ? t1 : t2;
            uint8_t ddf = t1 > t2 ? 5 : 4;
            int e1 = e_b[u] > 0 ? e_b[u] : 0, f1 = f > 0 ? f : 0;
            t1 = e1 > f1 ? e1 : f1;
            t2 = h_b[d] + mat_score(c_ssw_code[ref[j]], qcode, sc);
            h_c[u] = t1 > t2 ? t1 : t2;
            if (h_c[u] > max) max = h_c[u];
            if (line) {
                line[de] = dde;
                line[df] = ddf;
                line[dh] = t1 <= t2 ? 1 : (e1 > f1 ? dde : ddf);
            }
        }
        for (int j = 1; j <= u; j++) h_b[j] = h_c[j];
    }
    return max;
}

// banded_sw (ext/ssw/ssw.c:598-769), warp per task for bands of up to 31 cells
// (band width <= 15): lane k holds cell x + k of row i (x = max(i - bw, 0)), the
// previous row arrives by shuffles, and the row's F chain
// F(j) = max(H(j-1) - gO, F(j-1) - gE) is a max-plus scan of max(E+, diag) - gO
// over the lanes (exact when gap_open >= gap_extend, as H(j-1) = max(that, F+)).
// Directions are kept as four ballots per row (E opened, F opened, H from the
// diagonal, E over F) in the task's scratch, followed by the CIGAR; the traceback
// reads them with the library's flat-array indexing, so an index that leaves a row
// reads the neighbouring row's entries, or 0 where the pass wrote nothing.
// Tasks whose band outgrows a warp keep raw_off == RAW_FALLBACK for k_band_width.
__device__ int band_pass_warp(const uint8_t* ref, const uint8_t* read, int rl, int ql, int bw, const AlignScores& sc,
                              uint32_t* rowbits) {
    const int lane = threadIdx.x & 31;
    const int gO = sc.gap_open, gE = sc.gap_extend;
    const int width = 2 * bw + 3;
    constexpr int NEG = -(1 << 28);
    int prevH = 0, prevE = 0, mx = 0;
    for (int i = 0; i < ql; i++) {
        const int x = i - bw > 0 ? i - bw : 0, xe = i - 1 - bw > 0 ? i - 1 - bw : 0;
        const int end = rl - 1 < i + bw ? rl - 1 : i + bw;
        const int n = end - x + 1;
        const int edge = end + 1 < width - 1 ? end + 1 : width - 1;
        const int sh = x - xe;
        const bool act = lane < n;
        // previous row: H and E at column j (band index e = lane + sh + 1), H at j - 1
        const int su = lane + sh < 31 ? lane + sh : 31;
        const int sd = lane + sh - 1 > 0 ? lane + sh - 1 : 0;
        int upH = __shfl_sync(FULLM, prevH, su), upE = __shfl_sync(FULLM, prevE, su);
        int dg = __shfl_sync(FULLM, prevH, sd);
        if (lane + sh + 1 == edge) {
            upH = 0;
            upE = 0;
        }
        if (lane + sh == 0) dg = 0;
        const int t1 = i == 0 ? -gO : upH - gO;
        const int t2 = i == 0 ? -gE : upE - gE;
        const int E = t1 > t2 ? t1 : t2;
        const bool dde3 = t1 > t2;
        int D = 0;
        if (act) D = dg + mat_score(c_ssw_code[ref[x + lane]], c_ssw_code[read[i]], sc);
        const int e1 = E > 0 ? E : 0;
        const int B = e1 > D ? e1 : D;
        int T = act ? B - gO : NEG;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int Tp = __shfl_up_sync(FULLM, T, d);
            const int c = Tp - d * gE;
            if (lane >= d && c > T) T = c;
        }
        int Sx = __shfl_up_sync(FULLM, T, 1);
        if (lane == 0) Sx = NEG;
        const int f0 = -(lane + 1) * gE;
        const int f = Sx > f0 ? Sx : f0;
        const int f1 = f > 0 ? f : 0;
        const int H = B > f1 ? B : f1;
        int Hl = __shfl_up_sync(FULLM, H, 1), fl = __shfl_up_sync(FULLM, f, 1);
        if (lane == 0) {
            Hl = 0;
            fl = 0;
        }
        const bool ddf5 = Hl - gO > fl - gE;
        const int tm = e1 > f1 ? e1 : f1;
        if (act && H > mx) mx = H;
        if (rowbits) {
            const unsigned b0 = __ballot_sync(FULLM, act && dde3);
            const unsigned b1 = __ballot_sync(FULLM, act && ddf5);
            const unsigned b2 = __ballot_sync(FULLM, act && tm <= D);
            const unsigned b3 = __ballot_sync(FULLM, act && e1 > f1);
            if (lane == 0) {
                rowbits[4 * i] = b0;
                rowbits[4 * i + 1] = b1;
                rowbits[4 * i + 2] = b2;
                rowbits[4 * i + 3] = b3;
            }
        }
        prevH = act ? H : 0;
        prevE = act ? E : 0;
    }
    for (int d = 16; d > 0; d >>= 1) {
        const int o = __shfl_xor_sync(FULLM, mx, d);
        mx = mx > o ? mx : o;
    }
    return mx;
}

// Cells of one banded pass (the band's cells of every row), warp-collective
__device__ __forceinline__ uint64_t band_cells(int rl, int ql, int bw) {
    const int lane = threadIdx.x & 31;
    uint32_t c = 0;
    for (int i = lane; i < ql; i += 32) {
        const int x = i - bw > 0 ? i - bw : 0;
        const int end = rl - 1 < i + bw ? rl - 1 : i + bw;
        if (end >= x) c += (uint32_t)(end - x + 1);
    }
    for (int d = 16; d > 0; d >>= 1) c += __shfl_xor_sync(FULLM, c, d);
    return c;
}

// banded cells at counters[24..27] (u64): every pass's, and the final pass's
__device__ __forceinline__ void count_band_cells(uint32_t* counters, uint64_t computed, uint64_t canonical) {
    unsigned long long* bc = reinterpret_cast<unsigned long long*>(counters + 24);
    if ((threadIdx.x & 31) == 0) {
        if (computed) atomicAdd(bc, (unsigned long long)computed);
        if (canonical) atomicAdd(bc + 1, (unsigned long long)canonical);
    }
}

// banded_sw's traceback (ext/ssw/ssw.c:680-753) by one thread over the direction bits
// of the last pass: words(row, w0, w1, w2, w3) gives row `row`'s bits for band index k
// (E opened, F opened, H from the diagonal, E over F).  The library walks a flat
// (2bw+1) x 3-byte-per-row array, so an index that leaves a row reads the neighbouring
// row's entries, or 0 where the pass wrote nothing; the walk does the same.  Writes the
// CIGAR (reversed into order) to c; false when the walk fails or c is too small.
template <class Words>
__device__ bool band_trace_thread(Words words, int rl, int ql, int bw, uint32_t* c, uint32_t cap, uint32_t& nc) {
    const int width_d = 2 * bw + 1;
    const int64_t dsize = (int64_t)width_d * ql * 3;
    // the row's four direction words, loaded when the walk enters a row
    int cached = -1;
    uint32_t w0 = 0, w1 = 0, w2 = 0, w3 = 0;
    auto dir_of = [&](int row, int k, int w) -> int {
        const int x = row - bw > 0 ? row - bw : 0;
        const int end = rl - 1 < row + bw ? rl - 1 : row + bw;
        if (k > end - x) return 0;  // not written by the pass
        if (row != cached) {
            words(row, w0, w1, w2, w3);
            cached = row;
        }
        const int dde = (w0 >> k) & 1 ? 3 : 2;
        const int ddf = (w1 >> k) & 1 ? 5 : 4;
        if (w == 0) return dde;
        if (w == 1) return ddf;
        return (w2 >> k) & 1 ? 1 : ((w3 >> k) & 1 ? dde : ddf);
    };
    int i = ql - 1, j = rl - 1, e = 0, which = 2;
    char op = 'M', prev = 'M';
    nc = 0;
    auto enc = [](int l, char o) -> uint32_t { return ((uint32_t)l << 4) | (o == 'M' ? 0u : o == 'I' ? 1u : 2u); };
    while (i >= 0 && j > 0) {
        const int x = i - bw > 0 ? i - bw : 0;
        const int k = j - x;
        int d;
        if (k >= 0 && k < width_d) {
            d = dir_of(i, k, which);  // the flat index falls in row i
        } else {
            // the flat index (row i, band column k) runs into a neighbouring row
            const int64_t at = (int64_t)width_d * i * 3 + (int64_t)k * 3 + which;
            if (at < 0 || at >= dsize) return false;
            const int rem = (int)(at % (3 * width_d));
            d = dir_of((int)(at / (3 * width_d)), rem / 3, rem % 3);
        }
        switch (d) {
            case 1: --i; --j; which = 2; op = 'M'; break;
            case 2: --i; which = 0; op = 'I'; break;
            case 3: --i; which = 2; op = 'I'; break;
            case 4: --j; which = 1; op = 'D'; break;
            case 5: --j; which = 2; op = 'D'; break;
            default: return false;
        }
        if (op == prev) ++e;
        else {
            if (nc >= cap) return false;
            c[nc++] = enc(e, prev);
            prev = op;
            e = 1;
        }
    }
    if (nc + 2 > cap) return false;
    if (op == 'M') c[nc++] = enc(e + 1, op);
    else {
        c[nc++] = enc(e, op);
        c[nc++] = enc(1, 'M');
    }
    for (uint32_t a = 0, b = nc - 1; a < b; a++, b--) {
        const uint32_t tmp = c[a];
        c[a] = c[b];
        c[b] = tmp;
    }
    return true;
}

// banded_sw's pass (ext/ssw/ssw.c:614-676) for band width BW by one thread.  The
// library's h_b, e_b and h_c (indices u = 1 .. 2BW+1 for the band's cells, 0 and the
// edge held at 0) are register arrays: cell j of row i is band index k = j - x
// (x = max(0, i - BW)), u = k + 1, and the previous row's cell j sits at k + 1 + sh
// (sh = 1 once the band has started to slide), so every index is a constant of the
// unrolled loop.  The reference's codes of the band's columns slide along in
// registers.  The row's direction bits go to rows[2i] (bits k: E opened; 16 + k: F
// opened) and rows[2i + 1] (bits k: H from the diagonal; 16 + k: E over F) when rows is
// set.  Returns the maximum; cells counts the band's cells.
template <int BW>
__device__ int band_pass_thread(const uint8_t* ref, const uint8_t* read, int rl, int ql, const AlignScores& sc,
                                uint32_t* rows, uint64_t& cells) {
    constexpr int K = 2 * BW + 1;  // band cells per row
    constexpr int W = K + 2;       // the library's width
    const int gO = sc.gap_open, gE = sc.gap_extend;
    int hb[W], eb[W], hc[W], rc[K];
#pragma unroll
    for (int t = 0; t < W; t++) {
        hb[t] = 0;
        eb[t] = 0;
        hc[t] = 0;
    }
    // codes of columns x .. end of row 0
    const int end0 = rl - 1 < BW ? rl - 1 : BW;
#pragma unroll
    for (int k = 0; k < K; k++) rc[k] = k <= end0 ? c_ssw_code[ref[k]] : 4;
    int mx = 0, prev_end = end0;
    for (int i = 0; i < ql; i++) {
        const int x = i - BW > 0 ? i - BW : 0;
        const int sh = i - BW > 0 ? 1 : 0;  // x - max(0, i - 1 - BW)
        const int end = rl - 1 < i + BW ? rl - 1 : i + BW;
        const int n = end - x + 1;
        if (i > 0) {
            // slide the column codes to this row's band
            if (sh) {
#pragma unroll
                for (int k = 0; k + 1 < K; k++) rc[k] = rc[k + 1];
            }
            if (end > prev_end) {
                const int code = c_ssw_code[ref[end]];
#pragma unroll
                for (int k = 0; k < K; k++)
                    if (k == n - 1) rc[k] = code;
            }
            prev_end = end;
        }
        const int edge = end + 1 < W - 1 ? end + 1 : W - 1;
#pragma unroll
        for (int t = 1; t < W; t++)
            if (t == edge) {
                hb[t] = 0;
                eb[t] = 0;
            }
        hb[0] = eb[0] = hc[0] = 0;
        const int qcode = c_ssw_code[read[i]];
        int f = 0;
        uint32_t d0 = 0, d1 = 0;
#pragma unroll
        for (int k = 0; k < K; k++) {
            if (k < n) {
                const int he = sh ? hb[k + 2 < W ? k + 2 : W - 1] : hb[k + 1];
                const int ee = sh ? eb[k + 2 < W ? k + 2 : W - 1] : eb[k + 1];
                const int hd = sh ? hb[k + 1] : hb[k];
                int t1 = i == 0 ? -gO : he - gO;
                int t2 = i == 0 ? -gE : ee - gE;
                const int E = t1 > t2 ? t1 : t2;
                eb[k + 1] = E;
                d0 |= (uint32_t)(t1 > t2) << k;
                t1 = hc[k] - gO;
                t2 = f - gE;
                f = t1 > t2 ? t1 : t2;
                d0 |= (uint32_t)(t1 > t2) << (16 + k);
                const int e1 = E > 0 ? E : 0, f1 = f > 0 ? f : 0;
                t1 = e1 > f1 ? e1 : f1;
                t2 = hd + mat_score(rc[k], qcode, sc);
                const int H = t1 > t2 ? t1 : t2;
                hc[k + 1] = H;
                if (H > mx) mx = H;
                d1 |= (uint32_t)(t1 <= t2) << k;
                d1 |= (uint32_t)(e1 > f1) << (16 + k);
            }
        }
#pragma unroll
        for (int t = 1; t < W - 1; t++)
            if (t <= n) hb[t] = hc[t];
        cells += (uint64_t)(n > 0 ? n : 0);
        if (rows) {
            rows[2 * i] = d0;
            rows[2 * i + 1] = d1;
        }
    }
    return mx;
}

constexpr int BAND_THREAD_MAX_BW = 5;  // bands up to 11 cells a thread per task

// Tasks by starting band width |rl - ql| + 1: bucket b (1 .. BAND_THREAD_MAX_BW) holds
// its tasks at buckets[b * n_tasks ..] and their count at bucket_n[b]; wider ones go
// straight to k_band_warp's list.  k_band_small then runs the buckets in turn, so the
// threads of a warp share their band width (one template instance per warp).
__global__ void k_band_bucket(const SswTask* tasks, uint32_t n_tasks, uint32_t* buckets, uint32_t* bucket_n,
                              uint32_t* warp_list, uint32_t* counters) {
    for (uint32_t ti = blockIdx.x * blockDim.x + threadIdx.x; ti < n_tasks; ti += gridDim.x * blockDim.x) {
        const SswTask tk = tasks[ti];
        if (tk.ref_begin1 < 0 || tk.read_begin1 < 0) continue;
        const int rl = tk.ref_end1 - tk.ref_begin1 + 1, ql = tk.read_end1 - tk.read_begin1 + 1;
        const int bw = (rl > ql ? rl - ql : ql - rl) + 1;
        if (bw > BAND_THREAD_MAX_BW) warp_list[atomicAdd(&counters[28], 1u)] = ti;
        else buckets[(size_t)bw * n_tasks + atomicAdd(&bucket_n[bw], 1u)] = ti;
    }
}

// banded_sw (ext/ssw/ssw.c:598-769) a thread per task while the band width stays at
// most BAND_THREAD_MAX_BW (the band of an alignment without indels is 3 cells wide, so
// a warp per task left most lanes idle).  A task whose doubling goes past that is left
// for k_band_warp (raw_off stays RAW_FALLBACK), which starts its doubling over.
__global__ void __launch_bounds__(128) k_band_small(SswTask* tasks, uint32_t n_tasks, const PrepRec* prep,
                                                    const uint8_t* arena, int32_t* hscratch, AlignScores sc,
                                                    uint32_t* counters, uint32_t* warp_list, const uint32_t* buckets,
                                                    const uint32_t* bucket_n) {
    uint64_t computed = 0, canonical = 0;
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t bucket = 1, i = blockIdx.x * blockDim.x + threadIdx.x;
    for (;;) {
        // the next task: bucket by bucket, the threads striding through each
        while (bucket <= (uint32_t)BAND_THREAD_MAX_BW && i >= bucket_n[bucket]) {
            i -= bucket_n[bucket];
            bucket++;
        }
        if (bucket > (uint32_t)BAND_THREAD_MAX_BW) break;
        const uint32_t ti = buckets[(size_t)bucket * n_tasks + i];
        i += stride;
        SswTask tk = tasks[ti];
        const PrepRec p = prep[tk.job];
        const uint8_t* q = arena + p.arena_off + tk.read_begin1;
        const uint8_t* r = arena + p.arena_off + p.qlen + tk.ref_begin1;
        const int rl = tk.ref_end1 - tk.ref_begin1 + 1, ql = tk.read_end1 - tk.read_begin1 + 1;
        const int len = rl > ql ? rl : ql;
        int bw = (rl > ql ? rl - ql : ql - rl) + 1;
        // rows in the task's scratch as k_band_warp keeps them, the CIGAR after them
        uint32_t* rows = reinterpret_cast<uint32_t*>(hscratch + p.h_off);
        int mx = 0;
        bool small = true;
        uint64_t cells = 0;
        do {
            if (bw > BAND_THREAD_MAX_BW) {
                small = false;
                break;
            }
            cells = 0;
            switch (bw) {
                case 1: mx = band_pass_thread<1>(r, q, rl, ql, sc, rows, cells); break;
                case 2: mx = band_pass_thread<2>(r, q, rl, ql, sc, rows, cells); break;
                case 3: mx = band_pass_thread<3>(r, q, rl, ql, sc, rows, cells); break;
                case 4: mx = band_pass_thread<4>(r, q, rl, ql, sc, rows, cells); break;
                default: mx = band_pass_thread<5>(r, q, rl, ql, sc, rows, cells); break;
            }
            computed += cells;
            bw *= 2;
        } while (mx < tk.score1 && bw <= len);
        if (!small) {  // raw_off stays RAW_FALLBACK: k_band_warp takes it
            warp_list[atomicAdd(&counters[28], 1u)] = ti;
            continue;
        }
        bw /= 2;
        canonical += cells;
        uint32_t* c = rows + 4 * (size_t)ql;
        uint32_t nc = 0;
        const bool ok = band_trace_thread(
            [&](int row, uint32_t& w0, uint32_t& w1, uint32_t& w2, uint32_t& w3) {
                const uint32_t a = rows[2 * row], b = rows[2 * row + 1];
                w0 = a & 0xffffu;
                w1 = a >> 16;
                w2 = b & 0xffffu;
                w3 = b >> 16;
            },
            rl, ql, bw, c, (uint32_t)(rl + ql + 4), nc);
        tk.band_width = bw;
        if (!ok) {
            tk.flag = 1;
            tk.raw_len = 0;
        } else {
            tk.raw_len = nc;
        }
        tk.raw_off = (uint64_t)p.h_off + 4 * (uint64_t)ql;
        tasks[ti] = tk;
    }
    // the cells of this thread's tasks, one atomic per warp
    unsigned long long cs = computed, cn = canonical;
    for (int d = 16; d > 0; d >>= 1) {
        cs += __shfl_xor_sync(FULLM, cs, d);
        cn += __shfl_xor_sync(FULLM, cn, d);
    }
    count_band_cells(counters, cs, cn);
}

__global__ void __launch_bounds__(128) k_band_warp(SswTask* tasks, const uint32_t* list, const PrepRec* prep,
                                                   const uint8_t* arena, int32_t* hscratch, AlignScores sc,
                                                   uint32_t* counters, uint32_t* wide_list) {
    const int lane = threadIdx.x & 31;
    const uint32_t n_list = counters[28];  // the tasks k_band_small left
    for (;;) {
        uint32_t li = 0;
        if (lane == 0) li = atomicAdd(&counters[6], 1u);
        li = __shfl_sync(FULLM, li, 0);
        if (li >= n_list) break;
        const uint32_t ti = list[li];
        SswTask tk = tasks[ti];
        // skip the tasks k_band_small finished
        if (tk.ref_begin1 < 0 || tk.read_begin1 < 0 || tk.raw_off != RAW_FALLBACK) continue;
        const PrepRec p = prep[tk.job];
        const uint8_t* q = arena + p.arena_off;
        const uint8_t* r = q + p.qlen;
        const int rl = tk.ref_end1 - tk.ref_begin1 + 1, ql = tk.read_end1 - tk.read_begin1 + 1;
        const int len = rl > ql ? rl : ql;
        int bw = (rl > ql ? rl - ql : ql - rl) + 1;
        // band doubling (ext/ssw/ssw.c:626-660).  Every pass records its direction bits:
        // the doubling ends on the width it ran last, so the last pass's bits are the
        // ones the traceback reads and no pass is repeated to record them.
        bool fallback = false;
        int mx = 0;
        uint64_t computed = 0;
        uint32_t* rowbits = reinterpret_cast<uint32_t*>(hscratch + p.h_off);
        do {
            if (bw > 15) {
                fallback = true;
                break;
            }
            mx = band_pass_warp(r + tk.ref_begin1, q + tk.read_begin1, rl, ql, bw, sc, rowbits);
            computed += band_cells(rl, ql, bw);
            bw *= 2;
        } while (mx < tk.score1 && bw <= len);
        if (fallback) {
            count_band_cells(counters, computed, 0);
            if (lane == 0) wide_list[atomicAdd(&counters[29], 1u)] = ti;
            continue;  // raw_off stays RAW_FALLBACK
        }
        bw /= 2;
        count_band_cells(counters, computed, band_cells(rl, ql, bw));
        __syncwarp();
        if (lane == 0) {
            // traceback over the four ballot words per row the passes recorded
            uint32_t* c = rowbits + 4 * (size_t)ql;
            uint32_t nc = 0;
            const bool ok = band_trace_thread(
                [&](int row, uint32_t& w0, uint32_t& w1, uint32_t& w2, uint32_t& w3) {
                    const uint32_t* rb = rowbits + 4 * (size_t)row;
                    w0 = rb[0];
                    w1 = rb[1];
                    w2 = rb[2];
                    w3 = rb[3];
                },
                rl, ql, bw, c, (uint32_t)(rl + ql + 4), nc);
            tk.band_width = bw;
            if (!ok) {
                tk.flag = 1;
                tk.raw_len = 0;
            } else {
                tk.raw_len = nc;
            }
            tk.raw_off = (uint64_t)p.h_off + 4 * (uint64_t)ql;
            tasks[ti] = tk;
        }
        __syncwarp();
    }
}

// The same band pass for any band width: the row's cells in chunks of 32 lanes,
// the previous and current rows in shared memory (two buffers each for H and E),
// and the F scan carried from chunk to chunk.  Directions: four ballots per chunk
// and row, in the task's slice of the direction arena.
__device__ int band_pass_wide(const uint8_t* ref, const uint8_t* read, int rl, int ql, int bw, const AlignScores& sc,
                              int* buf, int maxc, uint32_t* rowbits, int nch) {
    const int lane = threadIdx.x & 31;
    const int gO = sc.gap_open, gE = sc.gap_extend;
    const int width = 2 * bw + 3;
    constexpr int NEG = -(1 << 28);
    int* Hp = buf;
    int* Ep = buf + maxc;
    int* Hc = buf + 2 * maxc;
    int* Ec = buf + 3 * maxc;
    for (int t = lane; t <= width && t < maxc; t += 32) {
        Hp[t] = 0;
        Ep[t] = 0;
    }
    __syncwarp();
    int mx = 0;
    for (int i = 0; i < ql; i++) {
        const int x = i - bw > 0 ? i - bw : 0, xe = i - 1 - bw > 0 ? i - 1 - bw : 0;
        const int end = rl - 1 < i + bw ? rl - 1 : i + bw;
        const int n = end - x + 1;
        const int edge = end + 1 < width - 1 ? end + 1 : width - 1;
        const int sh = x - xe;
        const int rcode = c_ssw_code[read[i]];
        int carryT = NEG, prevH = 0, prevF = 0;
        for (int c = 0; c * 32 < n; c++) {
            const int k = 32 * c + lane;
            const bool act = k < n;
            int upH = 0, upE = 0, dg = 0, D = 0;
            if (act) {
                if (k + sh + 1 != edge) {
                    upH = Hp[k + sh];
                    upE = Ep[k + sh];
                }
                dg = k + sh == 0 ? 0 : Hp[k + sh - 1];
                D = dg + mat_score(c_ssw_code[ref[x + k]], rcode, sc);
            }
            const int t1 = i == 0 ? -gO : upH - gO;
            const int t2 = i == 0 ? -gE : upE - gE;
            const int E = t1 > t2 ? t1 : t2;
            const bool dde3 = t1 > t2;
            const int e1 = E > 0 ? E : 0;
            const int B = e1 > D ? e1 : D;
            int T = act ? B - gO : NEG;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int Tp = __shfl_up_sync(FULLM, T, d);
                const int cc = Tp - d * gE;
                if (lane >= d && cc > T) T = cc;
            }
            {
                const int cc = carryT - (lane + 1) * gE;
                if (cc > T) T = cc;
            }
            int Sx = __shfl_up_sync(FULLM, T, 1);
            if (lane == 0) Sx = carryT;
            const int f0 = -(k + 1) * gE;
            const int f = Sx > f0 ? Sx : f0;
            const int f1 = f > 0 ? f : 0;
            const int H = B > f1 ? B : f1;
            int Hl = __shfl_up_sync(FULLM, H, 1), fl = __shfl_up_sync(FULLM, f, 1);
            if (lane == 0) {
                Hl = prevH;
                fl = prevF;
            }
            const bool ddf5 = Hl - gO > fl - gE;
            const int tm = e1 > f1 ? e1 : f1;
            if (act && H > mx) mx = H;
            if (rowbits) {
                const unsigned b0 = __ballot_sync(FULLM, act && dde3);
                const unsigned b1 = __ballot_sync(FULLM, act && ddf5);
                const unsigned b2 = __ballot_sync(FULLM, act && tm <= D);
                const unsigned b3 = __ballot_sync(FULLM, act && e1 > f1);
                if (lane == 0) {
                    uint32_t* w = rowbits + ((size_t)i * nch + c) * 4;
                    w[0] = b0;
                    w[1] = b1;
                    w[2] = b2;
                    w[3] = b3;
                }
            }
            if (act) {
                Hc[k] = H;
                Ec[k] = E;
            }
            carryT = __shfl_sync(FULLM, T, 31);
            prevH = __shfl_sync(FULLM, H, 31);
            prevF = __shfl_sync(FULLM, f, 31);
        }
        __syncwarp();
        int* t = Hp;
        Hp = Hc;
        Hc = t;
        t = Ep;
        Ep = Ec;
        Ec = t;
    }
    for (int d = 16; d > 0; d >>= 1) {
        const int o = __shfl_xor_sync(FULLM, mx, d);
        mx = mx > o ? mx : o;
    }
    return mx;
}

// traceback (ext/ssw/ssw.c:680-753) over the flat direction array of (2bw+1) x 3
// bytes per row, decoded from the per-chunk ballots; one thread.
__device__ bool band_traceback(const uint32_t* rowbits, int nch, int rl, int ql, int bw, uint32_t* c, uint32_t cap,
                               uint32_t& nc_out) {
    const int width_d = 2 * bw + 1;
    const int64_t dsize = (int64_t)width_d * ql * 3;
    auto dir_at = [&](int64_t at) -> int {
        const int row = (int)(at / (3 * width_d));
        const int rem = (int)(at % (3 * width_d));
        const int k = rem / 3, w = rem % 3;
        const int x = row - bw > 0 ? row - bw : 0;
        const int end = rl - 1 < row + bw ? rl - 1 : row + bw;
        if (k > end - x) return 0;  // not written by the pass
        const uint32_t* rb = rowbits + ((size_t)row * nch + (k >> 5)) * 4;
        const int bit = k & 31;
        const int dde = (rb[0] >> bit) & 1 ? 3 : 2;
        const int ddf = (rb[1] >> bit) & 1 ? 5 : 4;
        if (w == 0) return dde;
        if (w == 1) return ddf;
        return (rb[2] >> bit) & 1 ? 1 : ((rb[3] >> bit) & 1 ? dde : ddf);
    };
    int i = ql - 1, j = rl - 1, e = 0, which = 2;
    int64_t line = (int64_t)width_d * i * 3;
    char op = 'M', prev = 'M';
    uint32_t nc = 0;
    auto enc = [](int l, char o) -> uint32_t { return ((uint32_t)l << 4) | (o == 'M' ? 0u : o == 'I' ? 1u : 2u); };
    while (i >= 0 && j > 0) {
        const int x = i - bw > 0 ? i - bw : 0;
        const int64_t at = line + (int64_t)(j - x) * 3 + which;
        if (at < 0 || at >= dsize) return false;
        switch (dir_at(at)) {
            case 1: --i; --j; which = 2; line -= width_d * 3; op = 'M'; break;
            case 2: --i; which = 0; line -= width_d * 3; op = 'I'; break;
            case 3: --i; which = 2; line -= width_d * 3; op = 'I'; break;
            case 4: --j; which = 1; op = 'D'; break;
            case 5: --j; which = 2; op = 'D'; break;
            default: return false;
        }
        if (op == prev) ++e;
        else {
            if (nc >= cap) return false;
            c[nc++] = enc(e, prev);
            prev = op;
            e = 1;
        }
    }
    if (nc + 2 > cap) return false;
    if (op == 'M') c[nc++] = enc(e + 1, op);
    else {
        c[nc++] = enc(e, op);
        c[nc++] = enc(1, 'M');
    }
    for (uint32_t a = 0, b = nc - 1; a < b; a++, b--) {
        const uint32_t tmp = c[a];
        c[a] = c[b];
        c[b] = tmp;
    }
    nc_out = nc;
    return true;
}

// Band width search of the tasks k_band_warp left (raw_off == RAW_FALLBACK), warp
// per task; sizes their direction (ballot words) and CIGAR slices.
// Over the tasks k_band_warp left (wide_list); dir_size and raw_size are zero for the
// others.
__global__ void __launch_bounds__(32) k_band_width_wide(SswTask* tasks, const uint32_t* n_tasks_ptr,
                                                        const uint32_t* wide_list, const PrepRec* prep,
                                                        const uint8_t* arena, AlignScores sc, int maxc,
                                                        uint64_t* dir_size, uint64_t* raw_size, uint32_t* counters) {
    extern __shared__ int band_smem[];
    const int lane = threadIdx.x & 31;
    const uint32_t n = *n_tasks_ptr;
    for (;;) {
        uint32_t li = 0;
        if (lane == 0) li = atomicAdd(&counters[7], 1u);
        li = __shfl_sync(FULLM, li, 0);
        if (li >= n) break;
        const uint32_t ti = wide_list[li];
        SswTask tk = tasks[ti];
        if (tk.ref_begin1 < 0 || tk.read_begin1 < 0 || tk.raw_off != RAW_FALLBACK) continue;
        const PrepRec p = prep[tk.job];
        const uint8_t* q = arena + p.arena_off;
        const uint8_t* r = q + p.qlen;
        const int rl = tk.ref_end1 - tk.ref_begin1 + 1, ql = tk.read_end1 - tk.read_begin1 + 1;
        const int len = rl > ql ? rl : ql;
        int bw = (rl > ql ? rl - ql : ql - rl) + 1;
        int mx = 0;
        bool fail = false;
        uint64_t computed = 0;
        do {
            if (2 * bw + 4 > maxc) {
                fail = true;
                break;
            }
            mx = band_pass_wide(r + tk.ref_begin1, q + tk.read_begin1, rl, ql, bw, sc, band_smem, maxc, nullptr, 0);
            computed += band_cells(rl, ql, bw);
            bw *= 2;
        } while (mx < tk.score1 && bw <= len);
        bw /= 2;
        count_band_cells(counters, computed, 0);
        if (lane == 0) {
            tk.band_width = bw;
            if (fail) tk.flag = 1;
            tasks[ti] = tk;
            const uint64_t nch = (uint64_t)(2 * bw + 1 + 31) / 32;
            dir_size[ti] = fail ? 0 : (uint64_t)ql * nch * 16;
            raw_size[ti] = fail ? 0 : (uint64_t)rl + ql + 4;
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(32) k_band_trace_wide(SswTask* tasks, const uint32_t* n_tasks_ptr,
                                                        const uint32_t* wide_list, const PrepRec* prep,
                                                        const uint8_t* arena, AlignScores sc, int maxc,
                                                        const uint64_t* dir_off, uint8_t* dir,
                                                        const uint64_t* raw_off, uint32_t* raw, uint32_t* counters) {
    extern __shared__ int band_smem[];
    const int lane = threadIdx.x & 31;
    const uint32_t n = *n_tasks_ptr;
    for (;;) {
        uint32_t li = 0;
        if (lane == 0) li = atomicAdd(&counters[18], 1u);
        li = __shfl_sync(FULLM, li, 0);
        if (li >= n) break;
        const uint32_t ti = wide_list[li];
        SswTask tk = tasks[ti];
        if (tk.ref_begin1 < 0 || tk.read_begin1 < 0 || tk.raw_off != RAW_FALLBACK || tk.flag == 1) continue;
        const PrepRec p = prep[tk.job];
        const uint8_t* q = arena + p.arena_off;
        const uint8_t* r = q + p.qlen;
        const int rl = tk.ref_end1 - tk.ref_begin1 + 1, ql = tk.read_end1 - tk.read_begin1 + 1;
        const int bw = tk.band_width;
        const int nch = (2 * bw + 1 + 31) / 32;
        uint32_t* rowbits = reinterpret_cast<uint32_t*>(dir + dir_off[ti]);
        band_pass_wide(r + tk.ref_begin1, q + tk.read_begin1, rl, ql, bw, sc, band_smem, maxc, rowbits, nch);
        {
            const uint64_t cells = band_cells(rl, ql, bw);
            count_band_cells(counters, cells, cells);
        }
        __syncwarp();
        if (lane == 0) {
            uint32_t nc = 0;
            if (band_traceback(rowbits, nch, rl, ql, bw, raw + raw_off[ti], (uint32_t)(rl + ql + 4), nc)) {
                tk.raw_len = nc;
            } else {
                tk.flag = 1;
                tk.raw_len = 0;
            }
            tasks[ti] = tk;
        }
        __syncwarp();
    }
}

__global__ void k_band_width(SswTask* tasks, const uint32_t* n_tasks_ptr, const PrepRec* prep, const uint8_t* arena,
                             int32_t* hscratch, AlignScores sc, uint64_t* dir_size, uint64_t* raw_size) {
    const uint32_t n = *n_tasks_ptr;
    for (uint32_t ti = blockIdx.x * blockDim.x + threadIdx.x; ti < n; ti += gridDim.x * blockDim.x) {
        SswTask tk = tasks[ti];
        dir_size[ti] = 0;
        raw_size[ti] = 0;
        if (tk.ref_begin1 < 0 || tk.read_begin1 < 0 || tk.raw_off != RAW_FALLBACK) continue;
        const PrepRec p = prep[tk.job];
        const uint8_t* q = arena + p.arena_off;
        const uint8_t* r = q + p.qlen;
        int rl = tk.ref_end1 - tk.ref_begin1 + 1, ql = tk.read_end1 - tk.read_begin1 + 1;
        int bw = (rl > ql ? rl - ql : ql - rl) + 1;
        int len = rl > ql ? rl : ql;
        int* hb = hscratch + p.h_off;
        int cap_w = 2 * len + 8;
        int max = 0;
        do {
            if (bw * 2 + 4 > cap_w) { tk.flag = 1; break; }
            max = band_pass(r + tk.ref_begin1, q + tk.read_begin1, rl, ql, bw, sc, hb, hb + cap_w, hb + 2 * cap_w,
                            nullptr);
            bw *= 2;
        } while (max < tk.score1 && bw <= len);
        bw /= 2;
        tk.band_width = bw;
        tasks[ti] = tk;
        if (tk.flag == 1) continue;
        dir_size[ti] = (uint64_t)(2 * bw + 1) * ql * 3;
        raw_size[ti] = (uint64_t)rl + ql + 4;
    }
}

__global__ void k_band_trace(SswTask* tasks, const uint32_t* n_tasks_ptr, const PrepRec* prep, const uint8_t* arena,
                             int32_t* hscratch, AlignScores sc, const uint64_t* dir_off, uint8_t* dir,
                             const uint64_t* raw_off, uint32_t* raw) {
    const uint32_t n = *n_tasks_ptr;
    for (uint32_t ti = blockIdx.x * blockDim.x + threadIdx.x; ti < n; ti += gridDim.x * blockDim.x) {
        SswTask tk = tasks[ti];
        if (tk.ref_begin1 < 0 || tk.read_begin1 < 0 || tk.flag == 1 || tk.raw_off != RAW_FALLBACK) continue;
        const PrepRec p = prep[tk.job];
        const uint8_t* q = arena + p.arena_off;
        const uint8_t* r = q + p.qlen;
        const int rl = tk.ref_end1 - tk.ref_begin1 + 1, ql = tk.read_end1 - tk.read_begin1 + 1;
        const int len = rl > ql ? rl : ql;
        const int cap_w = 2 * len + 8;
        const int bw = tk.band_width;
        int* hb = hscratch + p.h_off;
        uint8_t* D = dir + dir_off[ti];
        band_pass(r + tk.ref_begin1, q + tk.read_begin1, rl, ql, bw, sc, hb, hb + cap_w, hb + 2 * cap_w, D);
        // traceback (ext/ssw/ssw.c:680-753); cells the last pass did not write read as 0
        const int width_d = 2 * bw + 1;
        const int64_t dsize = (int64_t)width_d * ql * 3;
        int i = ql - 1, j = rl - 1, e = 0, which = 2;
        int64_t line = (int64_t)width_d * i * 3;
        char op = 'M', prev = 'M';
        uint32_t* c = raw + raw_off[ti];
        uint32_t nc = 0;
        const uint32_t cap = (uint32_t)(rl + ql + 4);
        bool fail = false;
        auto enc = [](int l, char o) -> uint32_t { return ((uint32_t)l << 4) | (o == 'M' ? 0u : o == 'I' ? 1u : 2u); };
        while (i >= 0 && j > 0) {
            int x = i - bw > 0 ? i - bw : 0;
            int64_t at = line + (int64_t)(j - x) * 3 + which;
            if (at < 0 || at >= dsize) { fail = true; break; }
            switch (D[at]) {
                case 1: --i; --j; which = 2; line -= width_d * 3; op = 'M'; break;
                case 2: --i; which = 0; line -= width_d * 3; op = 'I'; break;
                case 3: --i; which = 2; line -= width_d * 3; op = 'I'; break;
                case 4: --j; which = 1; op = 'D'; break;
                case 5: --j; which = 2; op = 'D'; break;
                default: fail = true;
            }
            if (fail) break;
            if (op == prev) ++e;
            else {
                if (nc >= cap) { fail = true; break; }
                c[nc++] = enc(e, prev);
                prev = op;
                e = 1;
            }
        }
        if (!fail) {
            if (nc + 2 > cap) fail = true;
            else if (op == 'M') c[nc++] = enc(e + 1, op);
            else {
                c[nc++] = enc(e, op);
                c[nc++] = enc(1, 'M');
            }
        }
        if (fail) {
            tk.flag = 1;
            tk.raw_len = 0;
        } else {
            for (uint32_t a = 0, b = nc - 1; a < b; a++, b--) {
                uint32_t tmp = c[a];
                c[a] = c[b];
                c[b] = tmp;
            }
            tk.raw_len = nc;
        }
        tasks[ti] = tk;
    }
}

// SswAligner::align (src/ssw.rs:156-188) + Aligner::align end bonus (src/aligner.rs:92-148)
// A warp per task: the base comparisons of the front and back extensions and of the
// CIGAR's M runs are made 32 at a time by ballot; lane 0 turns each mask into =/X runs.
// Mismatches among the first cnt positions from (qa, ra), by the warp
__device__ __forceinline__ uint32_t warp_mismatches(const uint8_t* q, const uint8_t* rf, uint32_t qa, uint32_t ra,
                                                    uint32_t cnt, int step) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t mm = 0;
    for (uint32_t c = 0; c < cnt; c += 32) {
        const uint32_t t = c + lane;
        const bool x = t < cnt && q[(int64_t)qa + step * (int64_t)t] != rf[(int64_t)ra + step * (int64_t)t];
        mm += __popc(__ballot_sync(FULLM, x));
    }
    return mm;
}

// =/X runs of q[qa, qa + len) against rf[ra, ...) pushed by lane 0; returns the mismatches
__device__ __forceinline__ uint32_t warp_eq_runs(const uint8_t* q, const uint8_t* rf, uint32_t qa, uint32_t ra,
                                                 uint32_t len, CigarWriter& w) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t mm = 0;
    for (uint32_t c = 0; c < len; c += 32) {
        const uint32_t t = c + lane;
        const uint32_t m = __ballot_sync(FULLM, t < len && q[qa + t] == rf[ra + t]);
        const uint32_t cnt = len - c < 32 ? len - c : 32;
        const uint32_t valid = cnt == 32 ? 0xffffffffu : ((1u << cnt) - 1);
        mm += __popc(~m & valid);
        if (lane == 0) {
            uint32_t pos = 0;
            while (pos < cnt) {
                const bool e = (m >> pos) & 1;
                const uint32_t x = (e ? ~m : m) & valid & (0xffffffffu << pos);
                const uint32_t stop = x ? (uint32_t)(__ffs(x) - 1) : cnt;
                w.push(e ? 7u : 8u, stop - pos);
                pos = stop;
            }
        }
    }
    return mm;
}

__global__ void __launch_bounds__(128) k_finalize(const SswTask* tasks, const uint32_t* n_tasks_ptr,
                                                  const PrepRec* prep, const uint8_t* arena, const uint64_t* raw_off,
                                                  const uint32_t* raw, const int32_t* hscratch, AlignScores sc,
                                                  uint32_t* cigar, ExtResult* res) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t n = *n_tasks_ptr;
    const uint32_t nwarps = gridDim.x * (blockDim.x / 32);
    for (uint32_t ti = (blockIdx.x * blockDim.x + threadIdx.x) / 32; ti < n; ti += nwarps) {
        const SswTask tk = tasks[ti];
        const PrepRec p = prep[tk.job];
        ExtResult r = res[tk.job];
        r.valid = 0;
        if (tk.ref_begin1 < 0 || tk.read_begin1 < 0 || tk.flag != 0) {
            if (lane == 0) res[tk.job] = r;
            continue;
        }
        const uint8_t* q = arena + p.arena_off;
        const uint8_t* rf = q + p.qlen;
        const uint32_t qlen = p.qlen, rlen = p.wlen;
        uint32_t qs = tk.read_begin1, qe = tk.read_end1 + 1, rs = tk.ref_begin1, re = tk.ref_end1 + 1;
        int32_t score = tk.score1;
        // M -> =/X over the aligned segments; reject walks past them (the reference panics there)
        const uint32_t* rw = tk.raw_off == RAW_FALLBACK ? raw + raw_off[ti]
                                                        : reinterpret_cast<const uint32_t*>(hscratch) + tk.raw_off;
        bool bad = false;
        {
            uint32_t qi = qs, ri = rs;
            for (uint32_t a = 0; a < tk.raw_len && !bad; a++) {
                uint32_t op = rw[a] & 15, l = rw[a] >> 4;
                if (op == 0) {
                    if (qi + l > qe || ri + l > re) bad = true;
                    qi += l;
                    ri += l;
                } else if (op == 1) qi += l;
                else ri += l;
            }
        }
        if (bad) {
            if (lane == 0) res[tk.job] = r;
            continue;
        }
        // front extension (src/aligner.rs:92-118): ungapped to the left while both
        // sequences last
        const uint32_t fm = qs < rs ? qs : rs;
        const uint32_t fed = warp_mismatches(q, rf, qs - 1, rs - 1, fm, -1);
        const uint32_t fq = qs - fm, fr = rs - fm;
        const int32_t fscore = score + (int32_t)sc.match * (int32_t)(fm - fed) - (int32_t)sc.mismatch * (int32_t)fed;
        const bool take_front = fq == 0 && fscore + (int32_t)sc.end_bonus > score;
        CigarWriter w{cigar + p.cigar_off, 0, p.cigar_cap, false};
        if (take_front && qs > 0) warp_eq_runs(q, rf, fq, fr, qs - fq, w);
        uint32_t ed = 0;
        {
            uint32_t qi = qs, ri = rs;
            for (uint32_t a = 0; a < tk.raw_len; a++) {
                uint32_t op = rw[a] & 15, l = rw[a] >> 4;
                if (op == 0) {
                    ed += warp_eq_runs(q, rf, qi, ri, l, w);
                    qi += l;
                    ri += l;
                } else if (op == 1) {
                    if (lane == 0) w.push(1, l);
                    ed += l;
                    qi += l;
                } else {
                    if (lane == 0) w.push(2, l);
                    ed += l;
                    ri += l;
                }
            }
        }
        uint32_t a_qs = qs, a_rs = rs;
        uint32_t edits = ed;
        if (take_front) {
            a_qs = 0;
            a_rs = fr;
            score = fscore + (int32_t)sc.end_bonus;
            edits = ed + fed;
        }
        // back extension (src/aligner.rs:120-148)
        const uint32_t bm = qlen - qe < rlen - re ? qlen - qe : rlen - re;
        const uint32_t bmm = warp_mismatches(q, rf, qe, re, bm, 1);
        const uint32_t bq = qe + bm, br = re + bm;
        const int32_t bscore = score + (int32_t)sc.match * (int32_t)(bm - bmm) - (int32_t)sc.mismatch * (int32_t)bmm;
        const uint32_t bed = edits + bmm;
        uint32_t a_qe = qe, a_re = re;
        if (bq == qlen && bscore + (int32_t)sc.end_bonus > score) {
            if (qe < qlen) warp_eq_runs(q, rf, qe, re, bq - qe, w);
            a_qe = qlen;
            a_re = br;
            score = bscore + (int32_t)sc.end_bonus;
            edits = bed;
        }
        if (lane == 0) {
            w.finish();
            r.valid = w.overflow ? 0 : 1;
            r.score = (uint32_t)score;
            r.edit_distance = edits;
            r.ref_start = p.wstart + a_rs;
            r.length = a_re - a_rs;
            r.soft_clip_left = a_qs;
            r.soft_clip_right = qlen - a_qe;
            r.cigar_offset = (uint32_t)p.cigar_off;
            r.cigar_len = w.n;
            res[tk.job] = r;
        }
    }
}

// ------------------------------------------------------------------ piecewise (single end)
// extend_piecewise (src/piecewisealigner.rs:396-510) with remove_spurious_anchors
// (:596-719), warp per job.  The reference runs its DP pieces with the block-aligner
// crate; they are computed here as full affine-gap DPs whose traceback takes a
// deletion, then an insertion, before the diagonal on ties -- the order the reference's
// piecewise unit vectors agree with.  Beyond those vectors and the goldens this path is
// parity-unpinned.
//
// A piece's DP runs row by row on the warp, the columns in chunks of 32 lanes: F and
// the diagonal come from the previous row (shared memory), and the row's E chain
// E(j) = max(H(j-1) - gO, E(j-1) - gE) is a max-plus scan of max(diag, F) - gO over the
// lanes (exact for gap_open >= gap_extend, since H(j-1) = max(that, E(j-1))).  Each cell
// keeps four direction bits for the traceback.
constexpr int PW_NEG = -(1 << 28);
constexpr uint8_t PW_DIAG = 1, PW_FROM_E = 2, PW_EEXT = 4, PW_FEXT = 8, PW_FROM_F = 16;

struct PwPiece {
    int score;
    int bi, bj;  // end cell
    int nops;    // traceback ops, last op first (OP codes of src/cigar.rs)
};

// q: n query bytes, r: m reference bytes (REV: both read backwards).  LOCAL: best cell
// (strict >, row-major, from 0) with the end bonus on the last query row; otherwise the
// end is (n, m).  ops receives the traceback from the end cell back to (0, 0).
template <bool LOCAL, bool REV>
__device__ PwPiece pw_dp(const uint8_t* q, int n, const uint8_t* r, int m, const AlignScores& sc, int* rowbuf,
                         uint8_t* dirs, uint8_t* ops) {
    const int lane = threadIdx.x & 31;
    const int go = sc.gap_open, ge = sc.gap_extend, match = sc.match, mism = sc.mismatch;
    const int W = m + 1;
    int* Hp = rowbuf;
    int* Fp = rowbuf + W;
    int* Hc = rowbuf + 2 * W;
    int* Fc = rowbuf + 3 * W;
    auto qv = [&](int i) { return REV ? q[n - 1 - i] : q[i]; };
    auto rv = [&](int j) { return REV ? r[m - 1 - j] : r[j]; };
    for (int j = lane; j <= m; j += 32) {
        Hp[j] = j == 0 ? 0 : -go - (j - 1) * ge;
        Fp[j] = PW_NEG;
        uint8_t d = 0;
        if (j >= 1) {
            d |= PW_FROM_E;                        // H(0, j) = E(0, j)
            if (j >= 2 && go != ge) d |= PW_EEXT;  // E(0, j) extends E(0, j-1), not opened from H
        }
        dirs[j] = d;
    }
    __syncwarp();
    int best = 0, bi = 0, bj = 0;
    for (int i = 1; i <= n; i++) {
        const int hcol0 = -go - (i - 1) * ge;  // H(i, 0) = F(i, 0)
        if (lane == 0) {
            Hc[0] = hcol0;
            Fc[0] = hcol0;
            dirs[(size_t)i * W] = (i >= 2 && go != ge) ? PW_FEXT : 0;
        }
        const int qc = qv(i - 1);
        const int bonus = (LOCAL && i == n) ? (int)sc.end_bonus : 0;
        int carryT = hcol0 - go, carryE = PW_NEG, carryH = hcol0;
        for (int c = 0; c * 32 < m; c++) {
            const int j = 1 + 32 * c + lane;
            const bool act = j <= m;
            int F = PW_NEG, D = PW_NEG, B = PW_NEG;
            bool fext = false;
            if (act) {
                const int hu = Hp[j], fu = Fp[j];
                const int f1 = hu - go, f2 = fu - ge;
                F = f1 > f2 ? f1 : f2;
                fext = F == fu - ge && F != hu - go;
                D = Hp[j - 1] + (qc == rv(j - 1) ? match : -mism) + bonus;
                B = D > F ? D : F;
            }
            int T = act ? B - go : PW_NEG;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int Tp = __shfl_up_sync(FULLM, T, d);
                const int cc = Tp - d * ge;
                if (lane >= d && cc > T) T = cc;
            }
            {
                const int cc = carryT - (lane + 1) * ge;
                if (cc > T) T = cc;
            }
            int E = __shfl_up_sync(FULLM, T, 1);
            if (lane == 0) E = carryT;
            const int H = B > E ? B : E;
            int El = __shfl_up_sync(FULLM, E, 1), Hl = __shfl_up_sync(FULLM, H, 1);
            if (lane == 0) {
                El = carryE;
                Hl = carryH;
            }
            const bool eext = E == El - ge && E != Hl - go;
            if (act) {
                uint8_t d = 0;
                if (H == D) d |= PW_DIAG;
                if (H == E) d |= PW_FROM_E;
                if (H == F) d |= PW_FROM_F;
                if (eext) d |= PW_EEXT;
                if (fext) d |= PW_FEXT;
                dirs[(size_t)i * W + j] = d;
                Hc[j] = H;
                Fc[j] = F;
            }
            if (LOCAL) {
                int v = act ? H : PW_NEG;
                for (int d = 16; d > 0; d >>= 1) {
                    const int o = __shfl_xor_sync(FULLM, v, d);
                    v = v > o ? v : o;
                }
                if (v > best) {
                    const unsigned at = __ballot_sync(FULLM, act && H == v);
                    best = v;
                    bi = i;
                    bj = 1 + 32 * c + (__ffs(at) - 1);
                }
            }
            carryT = __shfl_sync(FULLM, T, 31);
            carryE = __shfl_sync(FULLM, E, 31);
            carryH = __shfl_sync(FULLM, H, 31);
        }
        __syncwarp();
        int* t = Hp;
        Hp = Hc;
        Hc = t;
        t = Fp;
        Fp = Fc;
        Fc = t;
    }
    if (!LOCAL) {
        best = Hp[m];
        bi = n;
        bj = m;
    }
    __syncwarp();
    PwPiece res;
    res.score = best;
    res.bi = bi;
    res.bj = bj;
    res.nops = 0;
    if (lane == 0) {
        int i = bi, j = bj, state = 0, nops = 0;
        const int limit = 2 * (n + m) + 4;
        for (int it = 0; (i > 0 || j > 0) && it < limit; it++) {
            const uint8_t d = dirs[(size_t)i * W + j];
            if (state == 0) {
                // a deletion, then an insertion, before the diagonal on ties: a gap
                // that ties with matches goes to the end of the run (the reference's
                // extend_piecewise_complex vector, src/piecewisealigner.rs:1672-1710)
                if (j > 0 && (d & PW_FROM_E)) {
                    state = 1;
                } else if (i > 0 && (j == 0 || (d & PW_FROM_F))) {
                    state = 2;
                } else {
                    ops[nops++] = qv(i - 1) == rv(j - 1) ? 7 : 8;  // = / X
                    i--;
                    j--;
                }
            } else if (state == 1) {
                ops[nops++] = 2;  // D
                const bool ext = j > 1 && (d & PW_EEXT);
                j--;
                state = ext ? 1 : 0;
                if (i == 0 && j > 0) state = 1;
            } else {
                ops[nops++] = 1;  // I
                const bool ext = i > 1 && (d & PW_FEXT);
                i--;
                state = ext ? 2 : 0;
                if (j == 0 && i > 0) state = 2;
            }
        }
        res.nops = nops;
    }
    res.nops = __shfl_sync(FULLM, res.nops, 0);
    __syncwarp();
    return res;
}

// remove_spurious_anchors (src/piecewisealigner.rs:596-719) on anchors held as
// (query start, reference start) int pairs, in place; na is updated.  Serial (one
// thread): the first pass erases the anchors between two cancelling indels, the second
// the chain ends (up to ceil(20%) of the anchors on each side) up to an indel.
__device__ void prune_spurious_anchors(int* anc, int& na) {
    auto erase = [&](int from, int to) {  // [from, to)
        for (int x = to; x < na; x++) {
            anc[2 * (x - (to - from))] = anc[2 * x];
            anc[2 * (x - (to - from)) + 1] = anc[2 * x + 1];
        }
        na -= to - from;
    };
    if (na < 2) return;
    const long long tol = 5;
    long long tracked = 0;
    bool has_dev = false;
    int dev = 0, i = 1;
    while (i < na) {
        const long long qd = (long long)anc[2 * (i - 1)] - anc[2 * i];
        const long long rd = (long long)anc[2 * (i - 1) + 1] - anc[2 * i + 1];
        const long long indel = qd - rd;
        if ((indel < 0 ? -indel : indel) > tol) {
            const long long tt = tracked + indel;
            if (has_dev && (tt < 0 ? -tt : tt) <= tol) {
                erase(dev, i);
                i = dev;
                has_dev = false;
                tracked = 0;
                continue;
            }
            has_dev = true;
            dev = i;
            tracked = indel;
        }
        i++;
    }
    const int max_prune = (int)ceilf(__fmul_rn((float)na, 0.20f));
    const int lim = na < max_prune ? na : max_prune;
    for (int x = 1; x < lim; x++) {
        const long long qd = (long long)anc[2 * x] - anc[2 * (x - 1)];
        const long long rd = (long long)anc[2 * x + 1] - anc[2 * (x - 1) + 1];
        if (qd - rd != 0) {
            erase(0, x);
            break;
        }
    }
    const int lo = (na > max_prune ? na - max_prune : 0) + 1;
    for (int x = na; x-- > lo;) {
        const long long qd = (long long)anc[2 * x] - anc[2 * (x - 1)];
        const long long rd = (long long)anc[2 * x + 1] - anc[2 * (x - 1) + 1];
        if (qd - rd != 0) {
            erase(x, na);
            break;
        }
    }
}

// hamming_align_global's score (src/aligner.rs:261-291): matches minus mismatches over
// equal-length pieces, floored at 0.
__device__ __forceinline__ int hamming_global_score(const uint8_t* q, const uint8_t* r, int n, const AlignScores& sc) {
    int hs = 0;
    for (int x = 0; x < n; x++) hs += q[x] == r[x] ? (int)sc.match : -(int)sc.mismatch;
    return hs > 0 ? hs : 0;
}

// The DP rows of a piece live in shared memory when the piece is at most smem_w - 1
// columns wide (PW_SMEM_W: small enough that 32 single-warp blocks fit on an SM), else in
// the block's slice of global scratch.
constexpr uint32_t PW_SMEM_W = 256;
__global__ void __launch_bounds__(32) k_piecewise(const uint32_t* __restrict__ list, const uint32_t* n_list_ptr,
                                                  const ExtJob* jobs, const PrepRec* prep, const uint8_t* arena,
                                                  const uint32_t* __restrict__ anchors, AlignScores sc, uint32_t k,
                                                  uint8_t* scratch, uint64_t cells_bytes, uint64_t ops_bytes,
                                                  uint64_t rows_bytes, uint32_t smem_w, uint32_t* cigar,
                                                  ExtResult* res, uint32_t* counters) {
    extern __shared__ int pw_rows[];
    const int lane = threadIdx.x & 31;
    const uint32_t n_list = *n_list_ptr;
    uint8_t* dirs = scratch + (size_t)blockIdx.x * (cells_bytes + ops_bytes + rows_bytes);
    uint8_t* ops = dirs + cells_bytes;
    int* grows = reinterpret_cast<int*>(ops + ops_bytes);
    auto rows_for = [&](int m) { return (uint32_t)m + 1 <= smem_w ? pw_rows : grows; };
    for (;;) {
        uint32_t li = 0;
        if (lane == 0) li = atomicAdd(&counters[22], 1u);
        li = __shfl_sync(FULLM, li, 0);
        if (li >= n_list) break;
        const uint32_t t = list[li];
        const ExtJob jb = jobs[t];
        const PrepRec p = prep[t];
        const uint8_t* q = arena + p.arena_off;
        const uint8_t* dref = q + p.qlen;
        const int L = (int)p.qlen, RL = (int)p.wlen;
        const int padding = L / 10;
        // anchors (last to first) as (query start, reference start in dref); the
        // pruning below rewrites them in this task's slice of the ops scratch
        int* anc = reinterpret_cast<int*>(ops + (((size_t)L + RL + 8 + 15) & ~(size_t)15));
        const int na0 = (int)jb.anc_n;
        for (int a = lane; a < na0; a += 32) {
            anc[2 * a] = (int)anchors[2 * ((size_t)jb.anc_off + a)];
            anc[2 * a + 1] = (int)anchors[2 * ((size_t)jb.anc_off + a) + 1] - (int)p.wstart;
        }
        __syncwarp();
        int na = na0;
        if (lane == 0) prune_spurious_anchors(anc, na);
        na = __shfl_sync(FULLM, na, 0);
        __syncwarp();
        CigarWriter w{cigar + p.cigar_off, 0, p.cigar_cap, false};
        auto push = [&](uint32_t op, int len) {
            if (lane == 0 && len > 0) w.push(op, (uint32_t)len);
        };
        const int K = (int)k;
        // before the first anchor
        const int fqs = anc[2 * (na - 1)], frs = anc[2 * (na - 1) + 1];
        int pre_qs, pre_rs, score;
        if (fqs > 0 && frs > 0) {
            const int rs = frs > fqs + padding ? frs - (fqs + padding) : 0;
            const PwPiece pc = pw_dp<true, true>(q, fqs, dref + rs, frs - rs, sc, rows_for(frs - rs), dirs, ops);
            if (pc.score == 0) {
                pre_qs = fqs;
                pre_rs = frs;
                score = 0;
            } else {
                pre_qs = fqs - pc.bi;
                pre_rs = rs + (frs - rs) - pc.bj;
                score = pc.score;
                for (int x = 0; x < pc.nops; x++) push(ops[x], 1);
            }
        } else {
            pre_qs = fqs;
            pre_rs = frs;
            score = fqs == 0 ? (int)sc.end_bonus : 0;
        }
        score += K * (int)sc.match;
        push(7, K);
        for (int i = na - 1; i >= 1; i--) {
            const int cqs = anc[2 * (i - 1)], crs = anc[2 * (i - 1) + 1];
            const int pqe = anc[2 * i] + K, prre = anc[2 * i + 1] + K;
            const int qd = cqs - pqe, rd = crs - prre;
            if (rd > 0 && qd > 0) {
                if (rd == qd) {
                    // hamming_align_global, taken if it scores above 85% of all matches;
                    // the comparisons 32 at a time by ballot
                    const int gmm = (int)warp_mismatches(q, dref, (uint32_t)pqe, (uint32_t)prre, (uint32_t)qd, 1);
                    const int hraw = (int)sc.match * (qd - gmm) - (int)sc.mismatch * gmm;
                    const int hsc = hraw > 0 ? hraw : 0;
                    const uint32_t thr = (uint32_t)ceilf(__fmul_rn((float)qd, 0.85f));
                    if (hsc > 0 && (uint32_t)hsc > (uint32_t)sc.match * thr) {
                        score += hsc;
                        warp_eq_runs(q, dref, (uint32_t)pqe, (uint32_t)prre, (uint32_t)qd, w);
                        score += K * (int)sc.match;
                        push(7, K);
                        continue;
                    }
                }
                const PwPiece pc = pw_dp<false, false>(q + pqe, qd, dref + prre, rd, sc, rows_for(rd), dirs, ops);
                score += pc.score;
                for (int x = pc.nops; x-- > 0;) push(ops[x], 1);
                score += K * (int)sc.match;
                push(7, K);
            } else if (rd < qd) {
                const int ins = qd - rd;
                score += -(int)sc.gap_open + (ins - 1) * -(int)sc.gap_extend;
                push(1, ins);
                const int mp = K + rd;
                score += mp * (int)sc.match;
                push(7, mp);
            } else if (rd > qd) {
                const int del = rd - qd;
                score += -(int)sc.gap_open + (del - 1) * -(int)sc.gap_extend;
                push(2, del);
                const int mp = K + qd;
                score += mp * (int)sc.match;
                push(7, mp);
            } else {
                const int mp = K + qd;
                score += mp * (int)sc.match;
                push(7, mp);
            }
        }
        // after the last anchor
        const int lqe = anc[0] + K, lre = anc[1] + K;
        int post_qe, post_re;
        if (lqe < L && lre < RL) {
            const int qlen2 = L - lqe;
            const int re = lre + qlen2 + padding < RL ? lre + qlen2 + padding : RL;
            const PwPiece pc = pw_dp<true, false>(q + lqe, qlen2, dref + lre, re - lre, sc, rows_for(re - lre), dirs,
                                                  ops);
            if (pc.score == 0) {
                post_qe = lqe;
                post_re = lre;
            } else {
                post_qe = lqe + pc.bi;
                post_re = lre + pc.bj;
                for (int x = pc.nops; x-- > 0;) push(ops[x], 1);
            }
            score += pc.score;
        } else {
            post_qe = lqe;
            post_re = lre;
            score += lqe == L ? (int)sc.end_bonus : 0;
        }
        if (lane == 0) w.finish();
        if (lane == 0) {
            ExtResult r = res[t];
            r.valid = 0;
            if (score > 0 && !w.overflow) {
                uint32_t ed = 0;
                for (uint32_t x = 0; x < w.n; x++) {
                    const uint32_t op = w.out[x] & 15;
                    if (op == 8 || op == 1 || op == 2) ed += w.out[x] >> 4;
                }
                r.valid = 1;
                r.score = (uint32_t)score;
                r.edit_distance = ed;
                r.ref_start = p.wstart + (uint32_t)pre_rs;
                r.length = (uint32_t)(post_re - pre_rs);
                r.soft_clip_left = (uint32_t)pre_qs;
                r.soft_clip_right = (uint32_t)(L - post_qe);
                r.cigar_offset = (uint32_t)p.cigar_off;
                r.cigar_len = w.n;
                r.gapped = 1;
            }
            res[t] = r;
        }
        __syncwarp();
    }
}

__global__ void k_cigar_used(const ExtResult* res, uint32_t n, uint64_t* used) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
        used[t] = res[t].valid ? res[t].cigar_len : 0;
}

// copy each valid job's CIGAR into a compact array and point the result at it
__global__ void k_cigar_gather(ExtResult* res, uint32_t n, const uint32_t* cigar, const uint64_t* off,
                               uint32_t* compact) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        ExtResult r = res[t];
        if (!r.valid) continue;
        const uint64_t o = off[t];
        for (uint32_t i = 0; i < r.cigar_len; i++) compact[o + i] = cigar[r.cigar_offset + i];
        r.cigar_offset = (uint32_t)o;
        res[t] = r;
    }
}

inline unsigned grid1(uint64_t n, unsigned block = 256) {
    uint64_t g = (n + block - 1) / block;
    if (g > sm_count() * 16) g = sm_count() * 16;
    return (unsigned)(g ? g : 1);
}

template <class T>
void excl_sum(ExtWorkspace& ws, const T* in, T* out, uint64_t n, cudaStream_t st) {
    size_t tmp = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tmp, in, out, (int64_t)n, st);
    ws.cub_tmp.reserve(tmp);
    cub::DeviceScan::ExclusiveSum(ws.cub_tmp.p, tmp, in, out, (int64_t)n, st);
}

bool g_tables_ready = false;

void init_tables() {
    if (g_tables_ready) return;
    uint8_t code[256], comp[256];
    for (int i = 0; i < 256; i++) { code[i] = 4; comp[i] = 'N'; }
    code['A'] = code['a'] = code['U'] = code['u'] = 0;
    code['C'] = code['c'] = 1;
    code['G'] = code['g'] = 2;
    code['T'] = code['t'] = 3;
    comp['A'] = comp['a'] = 'T';
    comp['C'] = comp['c'] = 'G';
    comp['G'] = comp['g'] = 'C';
    comp['T'] = comp['t'] = comp['U'] = comp['u'] = 'A';
    SA_CUDA(cudaMemcpyToSymbol(c_ssw_code, code, 256));
    SA_CUDA(cudaMemcpyToSymbol(c_comp, comp, 256));
    g_tables_ready = true;
}

// ------------------------------------------------------------------ stage entry points
// Kernels behind sa_hamming_batch, sa_piecewise_pieces, sa_remove_spurious_anchors and
// sa_piecewise_batch: the device functions of the extension path on caller-given
// (query, reference) bytes, for parity tests against the reference's unit vectors.

// Thread per pair: kind 0 hamming_align (src/aligner.rs:218-259; None unless the lengths
// agree), kind 1 hamming_align_global (:261-291).
__global__ void k_stage_hamming(uint32_t n, const uint32_t* kinds, const uint8_t* q, const uint64_t* qo,
                                const uint8_t* r, const uint64_t* ro, AlignScores sc, StageAlignment* out,
                                uint32_t* cigar, const uint64_t* cig_off) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const uint8_t* a = q + qo[t];
        const uint8_t* b = r + ro[t];
        const uint32_t L = (uint32_t)(qo[t + 1] - qo[t]), RL = (uint32_t)(ro[t + 1] - ro[t]);
        StageAlignment o{};
        CigarWriter w{cigar + cig_off[t], 0, (uint32_t)(cig_off[t + 1] - cig_off[t]), false};
        auto eq = [&](uint32_t i) { return a[i] == b[i]; };
        if (kinds[t] == 0) {
            if (L == RL) {
                uint32_t bs, be;
                o.score = highest_scoring_segment(eq, L, sc, bs, be);
                o.edit_distance = hamming_cigar(eq, bs, be, w);
                o.query_start = o.ref_start = bs;
                o.query_end = o.ref_end = be;
                o.valid = !w.overflow;
            }
        } else {
            const uint32_t m = L < RL ? L : RL;
            o.score = hamming_global_score(a, b, (int)m, sc);
            o.edit_distance = hamming_cigar(eq, 0, m, w);
            o.query_end = o.ref_end = L;
            o.valid = !w.overflow;
        }
        o.cigar_offset = (uint32_t)cig_off[t];
        o.cigar_len = w.n;
        out[t] = o;
    }
}

// Warp per piece: kind 0 global_alignment (src/piecewisealigner.rs:68-130), 1 the
// x-drop piece after the last anchor (GlobalStartLocalEnd), 2 the one before the first
// anchor (LocalStartGlobalEnd) (:132-240), as k_piecewise runs them.
__global__ void __launch_bounds__(32) k_stage_pieces(uint32_t n, const uint32_t* kinds, const uint8_t* q,
                                                     const uint64_t* qo, const uint8_t* r, const uint64_t* ro,
                                                     AlignScores sc, uint8_t* scratch, const uint64_t* scr_off,
                                                     StageAlignment* out, uint32_t* cigar, const uint64_t* cig_off) {
    extern __shared__ int pw_rows[];
    const int lane = threadIdx.x & 31;
    for (uint32_t t = blockIdx.x; t < n; t += gridDim.x) {
        const uint8_t* a = q + qo[t];
        const uint8_t* b = r + ro[t];
        const int L = (int)(qo[t + 1] - qo[t]), RL = (int)(ro[t + 1] - ro[t]);
        uint8_t* dirs = scratch + scr_off[t];
        uint8_t* ops = dirs + (size_t)(L + 1) * (RL + 1);
        PwPiece pc;
        if (kinds[t] == 0) pc = pw_dp<false, false>(a, L, b, RL, sc, pw_rows, dirs, ops);
        else if (kinds[t] == 1) pc = pw_dp<true, false>(a, L, b, RL, sc, pw_rows, dirs, ops);
        else pc = pw_dp<true, true>(a, L, b, RL, sc, pw_rows, dirs, ops);
        if (lane == 0) {
            StageAlignment o{};
            CigarWriter w{cigar + cig_off[t], 0, (uint32_t)(cig_off[t + 1] - cig_off[t]), false};
            if (kinds[t] == 2) {
                for (int x = 0; x < pc.nops; x++) w.push(ops[x], 1);
                o.query_start = (uint32_t)(L - pc.bi);
                o.ref_start = (uint32_t)(RL - pc.bj);
                o.query_end = (uint32_t)L;
                o.ref_end = (uint32_t)RL;
            } else {
                for (int x = pc.nops; x-- > 0;) w.push(ops[x], 1);
                o.query_end = (uint32_t)pc.bi;
                o.ref_end = (uint32_t)pc.bj;
            }
            w.finish();
            uint32_t ed = 0;
            for (uint32_t x = 0; x < w.n; x++) {
                const uint32_t op = w.out[x] & 15;
                if (op == 8 || op == 1 || op == 2) ed += w.out[x] >> 4;
            }
            o.valid = !w.overflow;
            o.score = pc.score;
            o.edit_distance = ed;
            o.cigar_offset = (uint32_t)cig_off[t];
            o.cigar_len = w.n;
            out[t] = o;
        }
        __syncwarp();
    }
}

// Thread per chain: remove_spurious_anchors in place on (query start, reference start)
// pairs.
__global__ void k_stage_prune(uint32_t n, int* anc, const uint64_t* off, uint32_t* counts) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int na = (int)(off[t + 1] - off[t]);
        prune_spurious_anchors(anc + 2 * off[t], na);
        counts[t] = (uint32_t)na;
    }
}

}  // namespace

void extension_init_tables() { init_tables(); }

uint32_t run_extension_raw(const DevRefs& refs, const uint8_t* seq, const uint64_t* off, const uint8_t* raw_refs,
                           const uint64_t* raw_off, uint32_t k, const AlignScores& sc, uint32_t n, ExtWorkspace& ws,
                           uint32_t max_qlen, cudaStream_t st, KernelTimers* kt, const uint32_t* anchors,
                           uint32_t max_anchors) {
    init_tables();
    KernelTimers none;
    if (!kt) kt = &none;
    uint32_t launches = 0;
    ws.results.reserve(n);
    ws.prep.reserve(n);
    ws.sizes.reserve(3 * ((size_t)n + 1));
    ws.offs.reserve(3 * ((size_t)n + 1));
    ws.counters.reserve(32);
    if (n == 0) {
        ws.h_results.clear();
        ws.h_cigar.clear();
        return 0;
    }
    uint64_t* sz[3] = {ws.sizes.p, ws.sizes.p + n + 1, ws.sizes.p + 2 * ((size_t)n + 1)};
    uint64_t* of[3] = {ws.offs.p, ws.offs.p + n + 1, ws.offs.p + 2 * ((size_t)n + 1)};
    SA_CUDA(cudaMemsetAsync(ws.counters.p, 0, 32 * sizeof(uint32_t), st));
    kt->begin(KS_PREPARE, st);
    ws.rescue_list.reserve(n);
    k_prepare<<<grid1(n), 256, 0, st>>>(ws.jobs.p, n, seq, off, refs, k, raw_refs, raw_off, ws.results.p, ws.prep.p,
                                        sz[0], sz[1], sz[2], ws.rescue_list.p, ws.counters.p + 4,
                                        ws.counters.p + 20);
    {
        static bool attr = false;
        const size_t smem = 2 * RESCUE_TAB_MAX * sizeof(unsigned long long);
        if (!attr) {
            SA_CUDA(cudaFuncSetAttribute(k_rescue_filter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            attr = true;
        }
        uint64_t blocks = ((uint64_t)n + 1) / 2;
        if (blocks > sm_count() * 3) blocks = sm_count() * 3;
        k_rescue_filter<<<(unsigned)(blocks ? blocks : 1), 64, smem, st>>>(ws.rescue_list.p, ws.counters.p + 4, seq,
                                                                           off, refs, k, ws.prep.p, sz[0], sz[1],
                                                                           sz[2]);
    }
    kt->end(st);
    launches += 2;
    // exclusive scans of arena bytes, CIGAR capacity and banded-DP scratch per job
    uint64_t tot[3];
    for (int c = 0; c < 3; c++) {
        SA_CUDA(cudaMemsetAsync(sz[c] + n, 0, 8, st));
        excl_sum(ws, sz[c], of[c], (uint64_t)n + 1, st);
        SA_CUDA(cudaMemcpyAsync(&tot[c], of[c] + n, 8, cudaMemcpyDeviceToHost, st));
    }
    uint32_t max_pw_window = 0;
    SA_CUDA(cudaMemcpyAsync(&max_pw_window, ws.counters.p + 20, 4, cudaMemcpyDeviceToHost, st));
    launches += 3;
    SA_CUDA(cudaStreamSynchronize(st));
    ws.arena.reserve(tot[0] + 16);
    ws.cigar.reserve(tot[1] + 1);
    ws.hscratch.reserve(tot[2] + 1);
    ws.tasks.reserve(n);
    ws.list_word.reserve(n);
    ws.list_rev_byte.reserve(n);
    ws.list_rev_word.reserve(n);
    kt->begin(KS_FILL, st);
    ws.pw_list.reserve(n);
    k_fill<<<grid1(n), 256, 0, st>>>(
        ws.jobs.p, n, seq, off, refs, raw_refs, raw_off, sc, ws.prep.p, of[0], of[1],
                                     of[2], ws.arena.p, ws.cigar.p, ws.results.p, ws.tasks.p, ws.counters.p,
                                     ws.pw_list.p);
    kt->end(st);
    launches++;
    if (max_pw_window) {
        // single-end piecewise jobs: a warp per job, each warp with its own DP scratch
        if (!anchors) throw Error(SA_ERR_INVALID, "internal: piecewise jobs without anchors");
        auto a16 = [](uint64_t x) { return (x + 15) & ~(uint64_t)15; };
        const uint64_t cells = a16(((uint64_t)max_qlen + 1) * ((uint64_t)max_pw_window + 1));
        const uint64_t opsb = a16((uint64_t)max_qlen + max_pw_window + 8) + a16(8ull * (max_anchors + 1));
        // single-warp blocks, 28 per SM (the registers of 28 fit): the per-job work is
        // mostly serial (anchor pruning, gap checks, traceback pushes, a row at a time), so
        // more resident warps hide its latency; the rows of wide pieces go to global
        // scratch so that the shared rows stay small
        const unsigned blocks = (unsigned)std::min<uint64_t>(n, sm_count() * 28);
        const uint64_t rowsb = a16(16ull * ((uint64_t)max_pw_window + 2));
        ws.pw_scratch.reserve((cells + opsb + rowsb) * blocks);
        const uint32_t smem_w = (uint32_t)std::min<uint64_t>((uint64_t)max_pw_window + 2, PW_SMEM_W);
        const size_t smem = 16 * (size_t)smem_w;
        static size_t attr = 0;
        if (smem > attr) {
            SA_CUDA(cudaFuncSetAttribute(k_piecewise, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            attr = smem;
        }
        kt->begin(KS_EXT_OTHER, st);
        k_piecewise<<<blocks, 32, smem, st>>>(ws.pw_list.p, ws.counters.p + 19, ws.jobs.p, ws.prep.p, ws.arena.p,
                                              anchors, sc, k, ws.pw_scratch.p, cells, opsb, rowsb, smem_w,
                                              ws.cigar.p, ws.results.p, ws.counters.p);
        kt->end(st);
        launches++;
    }
    uint32_t cnt[4];
    SA_CUDA(cudaMemcpyAsync(cnt, ws.counters.p, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaStreamSynchronize(st));
    const uint32_t n_tasks = cnt[0];
    const int bias = sc.mismatch;  // |min(matrix)| for the match/mismatch matrix (ext/ssw/ssw.c:802-806)
    if (n_tasks) {
        const int seg_b = ((int)max_qlen + 15) / 16, seg_w = ((int)max_qlen + 7) / 8;
        const int tpb = 128;
        size_t smem_b = (size_t)(tpb / 16) * seg_b * 16 * (2 * 1 + 1);
        size_t smem_w = (size_t)(tpb / 8) * seg_w * 8 * (2 * 2 + 1);
        static bool attr = false;
        if (!attr) {
            SA_CUDA(cudaFuncSetAttribute(k_sw<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
            SA_CUDA(cudaFuncSetAttribute(k_sw<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
            attr = true;
        }
        auto blocks_for = [](uint32_t items, int per_block) {
            uint64_t b = (items + per_block - 1) / per_block;
            if (b > sm_count() * 16) b = sm_count() * 16;
            return (unsigned)(b ? b : 1);
        };
        // register kernels while the profile fits in int8 and a lane's rows in SEG
        const bool reg_ok = sc.match <= 127 && sc.mismatch <= 128;
        const int segr_b = !reg_ok ? 0 : seg_b <= 8 ? 8 : seg_b <= 16 ? 16 : seg_b <= 32 ? 32 : 0;
        const int segr_w = !reg_ok ? 0 : seg_w <= 8 ? 8 : seg_w <= 20 ? 20 : seg_w <= 32 ? 32 : 0;
        // one striped pass over a task list: byte or word, forward (pass 0) or reverse (pass 1)
        auto sw_launch = [&](bool word, const uint32_t* list, const uint32_t* n_ptr, uint32_t n_host, int pass) {
            const int G = word ? 8 : 16;
            const unsigned grid = blocks_for(n_tasks, tpb / G);
            const int segr = word ? segr_w : segr_b;
            const size_t smem_r = (size_t)(tpb / G) * 5 * G * ((segr + 3) / 4) * 4;
#define SA_SWR(W, S)                                                                                              \
    k_swr<W, S><<<grid, tpb, smem_r, st>>>(ws.tasks.p, list, n_ptr, n_host, ws.prep.p, ws.arena.p, sc, bias, pass, \
                                           ws.counters.p, ws.list_word.p, ws.list_rev_byte.p, ws.list_rev_word.p)
            if (!word && segr == 8) SA_SWR(false, 8);
            else if (!word && segr == 16) SA_SWR(false, 16);
            else if (!word && segr == 32) SA_SWR(false, 32);
            else if (word && segr == 8) SA_SWR(true, 8);
            else if (word && segr == 20) SA_SWR(true, 20);
            else if (word && segr == 32) SA_SWR(true, 32);
            else if (!word)
                k_sw<false><<<grid, tpb, smem_b, st>>>(ws.tasks.p, list, n_ptr, n_host, ws.prep.p, ws.arena.p, sc,
                                                       bias, pass, seg_b, ws.counters.p, ws.list_word.p,
                                                       ws.list_rev_byte.p, ws.list_rev_word.p);
            else
                k_sw<true><<<grid, tpb, smem_w, st>>>(ws.tasks.p, list, n_ptr, n_host, ws.prep.p, ws.arena.p, sc,
                                                      bias, pass, seg_w, ws.counters.p, ws.list_word.p,
                                                      ws.list_rev_byte.p, ws.list_rev_word.p);
#undef SA_SWR
        };
        // rows per thread of the warp-per-task kernel: ceil(segLen / S) in both modes
        const int rows = std::max((seg_b + 1) / 2, (seg_w + 3) / 4);
        const int rmax = rows <= 4 ? 4 : rows <= 8 ? 8 : rows <= 16 ? 16 : 0;
        // the closed-form lazy-F pass needs gap_open > gap_extend: with equal penalties the
        // library's lazy-F loop stops after the first row of each lane
        const bool fused = reg_ok && sc.gap_open > sc.gap_extend && rmax;
        if (fused) {
            // one launch for every pass, longest windows first
            ws.order.reserve(n_tasks);
            kt->begin(KS_SW_BYTE, st);
            k_task_keys<<<grid1(n_tasks), 256, 0, st>>>(ws.tasks.p, n_tasks, ws.prep.p, ws.list_word.p,
                                                        ws.list_rev_word.p);
            size_t tmp = 0;
            cub::DeviceRadixSort::SortPairs(nullptr, tmp, ws.list_word.p, ws.list_rev_byte.p, ws.list_rev_word.p,
                                            ws.order.p, (int)n_tasks, 0, 16, st);
            ws.cub_tmp.reserve(tmp);
            cub::DeviceRadixSort::SortPairs(ws.cub_tmp.p, tmp, ws.list_word.p, ws.list_rev_byte.p,
                                            ws.list_rev_word.p, ws.order.p, (int)n_tasks, 0, 16, st);
            const int wpb = tpb / 32;
            uint64_t blocks = ((uint64_t)n_tasks + wpb - 1) / wpb;
            if (blocks > sm_count() * 16) blocks = sm_count() * 16;
#define SA_SSW(RM)                                                                                              \
    k_ssw<RM><<<(unsigned)blocks, tpb, (size_t)wpb * 5 * 32 * ((RM + 3) / 4) * 4, st>>>(                       \
        ws.tasks.p, ws.order.p, n_tasks, ws.prep.p, ws.arena.p, sc, bias, ws.counters.p, ws.counters.p + 21, \
        wave_qmax)
            // tasks of reads up to wave_qmax (at most 192) nt: eight threads per task; the
            // longer ones of a batch of mixed lengths a warp per task, in a launch before
            const uint32_t wave_qmax = std::min<uint32_t>(ws.wave_qmax, 8 * WAVE_NMAX);
            if (max_qlen > wave_qmax) {
                if (rmax == 4) SA_SSW(4);
                else if (rmax == 8) SA_SSW(8);
                else SA_SSW(16);
                launches++;
            }
            {
                const uint64_t per_block = (uint64_t)wpb * (32 / WV_T);  // tasks per block and round
                uint64_t wblocks = ((uint64_t)n_tasks + per_block - 1) / per_block;
                if (wblocks > sm_count() * 16) wblocks = sm_count() * 16;
                // the kernel's row arrays sized for the longest read it takes
                const bool short_reads = std::min<uint32_t>(max_qlen, wave_qmax) <= 8 * WAVE_NMAX_SHORT;
                const int nmax = short_reads ? WAVE_NMAX_SHORT : WAVE_NMAX;
                const size_t smem = (size_t)wpb * 5 * ((nmax + 7) / 8) * 32 * sizeof(uint4);
                const bool def_gaps = sc.gap_open == 12 && sc.gap_extend == 1;
#define SA_SSWW(NM, DF)                                                                                      \
    k_ssw_wave<NM, DF><<<(unsigned)wblocks, tpb, smem, st>>>(ws.tasks.p, ws.order.p, n_tasks, ws.prep.p,   \
                                                             ws.arena.p, sc, bias, ws.counters.p, wave_qmax)
                if (short_reads && def_gaps) SA_SSWW(WAVE_NMAX_SHORT, true);
                else if (short_reads) SA_SSWW(WAVE_NMAX_SHORT, false);
                else if (def_gaps) SA_SSWW(WAVE_NMAX, true);
                else SA_SSWW(WAVE_NMAX, false);
#undef SA_SSWW
            }
#undef SA_SSW
            kt->end(st);
            launches += 3;
        } else {
        // forward byte pass over all tasks
        kt->begin(KS_SW_BYTE, st);
        sw_launch(false, nullptr, nullptr, n_tasks, 0);
        kt->end(st);
        // forward word pass over the overflowed tasks
        kt->begin(KS_SW_WORD, st);
        sw_launch(true, ws.list_word.p, ws.counters.p + 1, 0, 0);
        kt->end(st);
        // reverse passes
        kt->begin(KS_SW_BYTE, st);
        sw_launch(false, ws.list_rev_byte.p, ws.counters.p + 2, 0, 1);
        kt->end(st);
        kt->begin(KS_SW_WORD, st);
        sw_launch(true, ws.list_rev_word.p, ws.counters.p + 3, 0, 1);
        kt->end(st);
        launches += 4;
        }
        if (sc.gap_open >= sc.gap_extend) {
            kt->begin(KS_BAND, st);
            uint64_t blocks = ((uint64_t)n_tasks + 3) / 4;
            if (blocks > sm_count() * 16) blocks = sm_count() * 16;
            uint64_t tblocks = ((uint64_t)n_tasks + 127) / 128;
            if (tblocks > sm_count() * 16) tblocks = sm_count() * 16;
            ws.band_list.reserve(n_tasks);
            ws.wide_list.reserve(n_tasks);
            ws.band_buckets.reserve((size_t)(BAND_THREAD_MAX_BW + 1) * n_tasks + 8);
            uint32_t* bucket_n = ws.band_buckets.p + (size_t)(BAND_THREAD_MAX_BW + 1) * n_tasks;
            SA_CUDA(cudaMemsetAsync(bucket_n, 0, 8 * sizeof(uint32_t), st));
            k_band_bucket<<<grid1(n_tasks), 256, 0, st>>>(ws.tasks.p, n_tasks, ws.band_buckets.p, bucket_n,
                                                          ws.band_list.p, ws.counters.p);
            k_band_small<<<(unsigned)tblocks, 128, 0, st>>>(ws.tasks.p, n_tasks, ws.prep.p, ws.arena.p,
                                                             ws.hscratch.p, sc, ws.counters.p, ws.band_list.p,
                                                             ws.band_buckets.p, bucket_n);
            k_band_warp<<<(unsigned)blocks, 128, 0, st>>>(ws.tasks.p, ws.band_list.p, ws.prep.p, ws.arena.p,
                                                          ws.hscratch.p, sc, ws.counters.p, ws.wide_list.p);
            kt->end(st);
            launches++;
        }
        ws.dir_size.reserve((size_t)n_tasks + 1);
        ws.dir_off.reserve((size_t)n_tasks + 1);
        ws.raw_size.reserve((size_t)n_tasks + 1);
        ws.raw_off.reserve((size_t)n_tasks + 1);
        const bool wide = sc.gap_open >= sc.gap_extend;
        const int maxc = 2 * (int)std::max<uint32_t>(2048, max_qlen) + 8;
        const size_t band_smem = (size_t)4 * maxc * sizeof(int);
        unsigned band_blocks = (unsigned)std::min<uint64_t>(n_tasks, sm_count() * 3);
        if (!band_blocks) band_blocks = 1;
        kt->begin(KS_BAND, st);
        if (wide) {
            static int attr_smem = 0;
            if ((int)band_smem > attr_smem) {
                SA_CUDA(cudaFuncSetAttribute(k_band_width_wide, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)band_smem));
                SA_CUDA(cudaFuncSetAttribute(k_band_trace_wide, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)band_smem));
                attr_smem = (int)band_smem;
            }
            SA_CUDA(cudaMemsetAsync(ws.dir_size.p, 0, (size_t)n_tasks * 8, st));
            SA_CUDA(cudaMemsetAsync(ws.raw_size.p, 0, (size_t)n_tasks * 8, st));
            k_band_width_wide<<<band_blocks, 32, band_smem, st>>>(ws.tasks.p, ws.counters.p + 29, ws.wide_list.p,
                                                                 ws.prep.p, ws.arena.p, sc, maxc, ws.dir_size.p,
                                                                 ws.raw_size.p, ws.counters.p);
        } else {
            k_band_width<<<grid1(n_tasks, 128), 128, 0, st>>>(ws.tasks.p, ws.counters.p, ws.prep.p, ws.arena.p,
                                                              ws.hscratch.p, sc, ws.dir_size.p, ws.raw_size.p);
        }
        kt->end(st);
        launches++;
        SA_CUDA(cudaMemsetAsync(ws.dir_size.p + n_tasks, 0, 8, st));
        SA_CUDA(cudaMemsetAsync(ws.raw_size.p + n_tasks, 0, 8, st));
        excl_sum(ws, ws.dir_size.p, ws.dir_off.p, (uint64_t)n_tasks + 1, st);
        excl_sum(ws, ws.raw_size.p, ws.raw_off.p, (uint64_t)n_tasks + 1, st);
        launches += 2;
        uint64_t dtot = 0, rtot = 0;
        SA_CUDA(cudaMemcpyAsync(&dtot, ws.dir_off.p + n_tasks, 8, cudaMemcpyDeviceToHost, st));
        SA_CUDA(cudaMemcpyAsync(&rtot, ws.raw_off.p + n_tasks, 8, cudaMemcpyDeviceToHost, st));
        SA_CUDA(cudaStreamSynchronize(st));
        ws.dir.reserve(dtot + 16);
        ws.raw.reserve(rtot + 1);
        SA_CUDA(cudaMemsetAsync(ws.dir.p, 0, dtot + 16, st));
        kt->begin(KS_BAND, st);
        if (wide)
            k_band_trace_wide<<<band_blocks, 32, band_smem, st>>>(ws.tasks.p, ws.counters.p + 29, ws.wide_list.p,
                                                                 ws.prep.p, ws.arena.p, sc, maxc, ws.dir_off.p,
                                                                 ws.dir.p, ws.raw_off.p, ws.raw.p, ws.counters.p);
        else
            k_band_trace<<<grid1(n_tasks, 128), 128, 0, st>>>(ws.tasks.p, ws.counters.p, ws.prep.p, ws.arena.p,
                                                              ws.hscratch.p, sc, ws.dir_off.p, ws.dir.p, ws.raw_off.p,
                                                              ws.raw.p);
        kt->end(st);
        kt->begin(KS_FINALIZE, st);
        // a warp per task
        k_finalize<<<grid1((uint64_t)n_tasks * 32, 128), 128, 0, st>>>(ws.tasks.p, ws.counters.p, ws.prep.p, ws.arena.p,
                                                        ws.raw_off.p, ws.raw.p, ws.hscratch.p, sc, ws.cigar.p,
                                                        ws.results.p);
        kt->end(st);
        launches += 2;
    }
    // compact the CIGARs that were written and copy back results + used ops only
    k_cigar_used<<<grid1(n), 256, 0, st>>>(ws.results.p, n, sz[0]);
    SA_CUDA(cudaMemsetAsync(sz[0] + n, 0, 8, st));
    excl_sum(ws, sz[0], of[0], (uint64_t)n + 1, st);
    uint64_t used = 0;
    SA_CUDA(cudaMemcpyAsync(&used, of[0] + n, 8, cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaStreamSynchronize(st));
    ws.raw.reserve(std::max<uint64_t>(used, 1));  // reused as the compact CIGAR buffer
    k_cigar_gather<<<grid1(n), 256, 0, st>>>(ws.results.p, n, ws.cigar.p, of[0], ws.raw.p);
    launches += 3;
    SA_CUDA(cudaGetLastError());
    ws.h_results.resize(n);
    ws.h_cigar.resize(used);
    SA_CUDA(cudaMemcpyAsync(ws.h_results.data(), ws.results.p, (size_t)n * sizeof(ExtResult), cudaMemcpyDeviceToHost,
                            st));
    if (used) SA_CUDA(cudaMemcpyAsync(ws.h_cigar.data(), ws.raw.p, used * 4, cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaMemcpyAsync(ws.cells, ws.counters.p + 8, 5 * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaMemcpyAsync(ws.cells + 5, ws.counters.p + 24, 2 * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaStreamSynchronize(st));
    tot[1] = used;
    ws.total_cigar = tot[1];
    return launches;
}

uint32_t run_extension(const DevRefs& refs, const NamWorkspace& nws, uint32_t k, const AlignScores& sc, uint32_t n,
                       ExtWorkspace& ws, uint32_t max_qlen, cudaStream_t st, KernelTimers* kt, const uint32_t* anchors,
                       uint32_t max_anchors) {
    return run_extension_raw(refs, nws.seq.p, nws.off.p, nullptr, nullptr, k, sc, n, ws, max_qlen, st, kt, anchors,
                             max_anchors);
}

// ------------------------------------------------------------------ stage entry points
namespace {

template <class T>
void upload(DevBuf<T>& d, const T* h, size_t n, cudaStream_t st) {
    d.reserve(std::max<size_t>(n, 1));
    if (n) SA_CUDA(cudaMemcpyAsync(d.p, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
}

struct StageInputs {
    DevBuf<uint32_t> kinds;
    DevBuf<uint8_t> q, r;
    DevBuf<uint64_t> qo, ro, co;
    DevBuf<StageAlignment> out;
    DevBuf<uint32_t> cigar;
    std::vector<uint64_t> cig_off;
    void load(uint32_t n, const uint32_t* k, const uint8_t* hq, const uint64_t* hqo, const uint8_t* hr,
              const uint64_t* hro, cudaStream_t st) {
        cig_off.assign((size_t)n + 1, 0);
        for (uint32_t i = 0; i < n; i++) cig_off[i + 1] = cig_off[i] + (hqo[i + 1] - hqo[i]) + (hro[i + 1] - hro[i]) + 4;
        upload(kinds, k, n, st);
        upload(q, hq, hqo[n], st);
        upload(r, hr, hro[n], st);
        upload(qo, hqo, (size_t)n + 1, st);
        upload(ro, hro, (size_t)n + 1, st);
        upload(co, cig_off.data(), (size_t)n + 1, st);
        out.reserve(std::max<uint32_t>(n, 1));
        cigar.reserve(cig_off[n] + 1);
    }
    void fetch(uint32_t n, StageAlignment* hout, uint32_t* hcig, size_t cap, cudaStream_t st) {
        if (cig_off[n] > cap) throw Error(SA_ERR_INVALID, "cigar capacity too small");
        if (n) SA_CUDA(cudaMemcpyAsync(hout, out.p, (size_t)n * sizeof(StageAlignment), cudaMemcpyDeviceToHost, st));
        if (cig_off[n]) SA_CUDA(cudaMemcpyAsync(hcig, cigar.p, cig_off[n] * 4, cudaMemcpyDeviceToHost, st));
        SA_CUDA(cudaStreamSynchronize(st));
    }
};

}  // namespace

void stage_hamming(uint32_t n, const uint32_t* kinds, const uint8_t* q, const uint64_t* qo, const uint8_t* r,
                   const uint64_t* ro, const AlignScores& sc, StageAlignment* out, uint32_t* cigar, size_t cap,
                   cudaStream_t st) {
    StageInputs in;
    in.load(n, kinds, q, qo, r, ro, st);
    if (n)
        k_stage_hamming<<<grid1(n), 256, 0, st>>>(n, in.kinds.p, in.q.p, in.qo.p, in.r.p, in.ro.p, sc, in.out.p,
                                                  in.cigar.p, in.co.p);
    SA_CUDA(cudaGetLastError());
    in.fetch(n, out, cigar, cap, st);
}

void stage_pieces(uint32_t n, const uint32_t* kinds, const uint8_t* q, const uint64_t* qo, const uint8_t* r,
                  const uint64_t* ro, const AlignScores& sc, StageAlignment* out, uint32_t* cigar, size_t cap,
                  cudaStream_t st) {
    StageInputs in;
    in.load(n, kinds, q, qo, r, ro, st);
    std::vector<uint64_t> so((size_t)n + 1, 0);
    uint64_t max_r = 0;
    for (uint32_t i = 0; i < n; i++) {
        const uint64_t L = qo[i + 1] - qo[i], R = ro[i + 1] - ro[i];
        so[i + 1] = so[i] + (((L + 1) * (R + 1) + L + R + 8 + 15) & ~15ull);
        max_r = std::max(max_r, R);
    }
    DevBuf<uint8_t> scratch;
    DevBuf<uint64_t> d_so;
    scratch.reserve(so[n] + 16);
    upload(d_so, so.data(), so.size(), st);
    const size_t smem = 16 * ((size_t)max_r + 2);
    if (smem > 48 * 1024)
        SA_CUDA(cudaFuncSetAttribute(k_stage_pieces, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (n)
        k_stage_pieces<<<(unsigned)std::min<uint32_t>(n, 4096), 32, smem, st>>>(
            n, in.kinds.p, in.q.p, in.qo.p, in.r.p, in.ro.p, sc, scratch.p, d_so.p, in.out.p, in.cigar.p, in.co.p);
    SA_CUDA(cudaGetLastError());
    in.fetch(n, out, cigar, cap, st);
}

void stage_prune(uint32_t n, int32_t* anchors, const uint64_t* off, uint32_t* counts, cudaStream_t st) {
    DevBuf<int> d_anc;
    DevBuf<uint64_t> d_off;
    DevBuf<uint32_t> d_cnt;
    upload(d_anc, anchors, 2 * off[n], st);
    upload(d_off, off, (size_t)n + 1, st);
    d_cnt.reserve(std::max<uint32_t>(n, 1));
    if (n) k_stage_prune<<<grid1(n), 128, 0, st>>>(n, d_anc.p, d_off.p, d_cnt.p);
    SA_CUDA(cudaGetLastError());
    if (off[n]) SA_CUDA(cudaMemcpyAsync(anchors, d_anc.p, 2 * off[n] * sizeof(int), cudaMemcpyDeviceToHost, st));
    if (n) SA_CUDA(cudaMemcpyAsync(counts, d_cnt.p, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaStreamSynchronize(st));
}

void stage_piecewise(uint32_t n, const uint8_t* q, const uint64_t* qo, const uint8_t* r, const uint64_t* ro,
                     const uint32_t* anchors, const uint64_t* anc_off, uint32_t k, const AlignScores& sc,
                     StageAlignment* out, uint32_t* cigar, size_t cap, cudaStream_t st) {
    init_tables();
    // one job per (query, window): the arena holds the query then the window, the
    // anchors their (query start, window start) pairs last to first, as a wave of
    // piecewise jobs has them
    std::vector<ExtJob> jobs(std::max<uint32_t>(n, 1));
    std::vector<PrepRec> prep(std::max<uint32_t>(n, 1));
    std::vector<uint8_t> arena;
    std::vector<uint32_t> list(std::max<uint32_t>(n, 1));
    uint64_t cig = 0, max_q = 0, max_w = 0, max_a = 0;
    for (uint32_t i = 0; i < n; i++) {
        const uint64_t L = qo[i + 1] - qo[i], W = ro[i + 1] - ro[i], A = anc_off[i + 1] - anc_off[i];
        if (A == 0) throw Error(SA_ERR_INVALID, "piecewise job without anchors");
        ExtJob j{};
        j.anc_off = (uint32_t)anc_off[i];
        j.anc_n = (uint32_t)A;
        jobs[i] = j;
        PrepRec p{};
        p.type = 3;
        p.qlen = (uint32_t)L;
        p.wlen = (uint32_t)W;
        p.arena_off = arena.size();
        p.cigar_off = cig;
        p.cigar_cap = (uint32_t)(2 * L + W + 4);
        cig += p.cigar_cap;
        arena.insert(arena.end(), q + qo[i], q + qo[i + 1]);
        arena.insert(arena.end(), r + ro[i], r + ro[i + 1]);
        prep[i] = p;
        list[i] = i;
        max_q = std::max(max_q, L);
        max_w = std::max(max_w, W);
        max_a = std::max(max_a, A);
    }
    DevBuf<ExtJob> d_jobs;
    DevBuf<PrepRec> d_prep;
    DevBuf<uint8_t> d_arena, d_scratch;
    DevBuf<uint32_t> d_list, d_anc, d_cigar, d_counters;
    DevBuf<ExtResult> d_res;
    upload(d_jobs, jobs.data(), jobs.size(), st);
    upload(d_prep, prep.data(), prep.size(), st);
    upload(d_arena, arena.data(), arena.size(), st);
    upload(d_list, list.data(), list.size(), st);
    upload(d_anc, anchors, 2 * anc_off[n], st);
    d_cigar.reserve(cig + 1);
    d_res.reserve(std::max<uint32_t>(n, 1));
    d_counters.reserve(24);
    SA_CUDA(cudaMemsetAsync(d_counters.p, 0, 24 * 4, st));
    SA_CUDA(cudaMemcpyAsync(d_counters.p + 19, &n, 4, cudaMemcpyHostToDevice, st));
    SA_CUDA(cudaMemsetAsync(d_res.p, 0, std::max<uint32_t>(n, 1) * sizeof(ExtResult), st));
    auto a16 = [](uint64_t x) { return (x + 15) & ~(uint64_t)15; };
    const uint64_t cells = a16((max_q + 1) * (max_w + 1));
    const uint64_t opsb = a16(max_q + max_w + 8) + a16(8ull * (max_a + 1));
    const unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(n, 1024));
    const uint64_t rowsb = a16(16ull * (max_w + 2));
    d_scratch.reserve((cells + opsb + rowsb) * blocks);
    const uint32_t smem_w = (uint32_t)std::min<uint64_t>(max_w + 2, PW_SMEM_W);
    const size_t smem = 16 * (size_t)smem_w;
    if (n)
        k_piecewise<<<blocks, 32, smem, st>>>(d_list.p, d_counters.p + 19, d_jobs.p, d_prep.p, d_arena.p, d_anc.p, sc,
                                              k, d_scratch.p, cells, opsb, rowsb, smem_w, d_cigar.p, d_res.p,
                                              d_counters.p);
    SA_CUDA(cudaGetLastError());
    std::vector<ExtResult> res(std::max<uint32_t>(n, 1));
    std::vector<uint32_t> hc(cig + 1);
    SA_CUDA(cudaMemcpyAsync(res.data(), d_res.p, res.size() * sizeof(ExtResult), cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaMemcpyAsync(hc.data(), d_cigar.p, hc.size() * 4, cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaStreamSynchronize(st));
    size_t w = 0;
    for (uint32_t i = 0; i < n; i++) {
        const ExtResult& x = res[i];
        StageAlignment o{};
        o.valid = x.valid;
        if (x.valid) {
            if (w + x.cigar_len > cap) throw Error(SA_ERR_INVALID, "cigar capacity too small");
            o.score = (int32_t)x.score;
            o.query_start = x.soft_clip_left;
            o.query_end = prep[i].qlen - x.soft_clip_right;
            o.ref_start = x.ref_start;
            o.ref_end = x.ref_start + x.length;
            o.edit_distance = x.edit_distance;
            o.cigar_offset = (uint32_t)w;
            o.cigar_len = x.cigar_len;
            std::memcpy(cigar + w, hc.data() + x.cigar_offset, (size_t)x.cigar_len * 4);
            w += x.cigar_len;
        }
        out[i] = o;
    }
}

}  // namespace sa
