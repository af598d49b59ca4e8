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
//   k_band_*    banded_sw (ext/ssw/ssw.c:598-769): band doubling, then the final
//               pass with directions and the traceback, one thread per task
//   k_finalize  M -> =/X (src/cigar.rs:149-187), edit distance and the end-bonus
//               extension of Aligner::align
#include <cub/cub.cuh>

#include "extend.h"

namespace sa {

namespace {

__constant__ uint8_t c_ssw_code[256];   // src/ssw.rs:8-25
__constant__ uint8_t c_comp[256];       // src/revcomp.rs:5-22

constexpr uint32_t FULLM = 0xffffffffu;

__device__ __forceinline__ uint8_t ref_base(const DevRefs& R, uint32_t c, uint64_t i) {
    uint64_t w = __ldg(R.words + R.word_off[c] + (i >> 5));
    return "ACGT"[(w >> ((i & 31) * 2)) & 3];
}

__device__ __forceinline__ uint8_t read_char(const uint8_t* s, uint32_t L, uint32_t i, bool rc) {
    return rc ? c_comp[s[L - 1 - i]] : s[i];
}

// Nam::is_consistent (src/nam.rs:49-69) for a NAM in the given orientation
__device__ bool nam_consistent(const DevRefs& R, const uint8_t* s, uint32_t L, uint32_t ref_id, uint32_t rs,
                               uint32_t re, uint32_t qs, uint32_t qe, bool rc, uint32_t k) {
    for (uint32_t i = 0; i < k; i++)
        if (ref_base(R, ref_id, rs + i) != read_char(s, L, qs + i, rc)) return false;
    for (uint32_t i = 0; i < k; i++)
        if (ref_base(R, ref_id, re - k + i) != read_char(s, L, qe - k + i, rc)) return false;
    return true;
}

// has_shared_substring (src/mapper.rs:1157-1168)
__device__ bool shared_substring(const DevRefs& R, uint32_t ref_id, uint32_t ws, uint32_t wl, const uint8_t* s,
                                 uint32_t L, bool rc, uint32_t k) {
    uint32_t sub = 2 * k / 3, step = k / 3;
    uint32_t lim = L > sub ? L - sub : 0;
    if (step == 0) step = 1;
    for (uint32_t i = 0; i < lim; i += step) {
        if (sub == 0) return true;
        if (wl < sub) continue;
        for (uint32_t p = 0; p + sub <= wl; p++) {
            uint32_t t = 0;
            while (t < sub && ref_base(R, ref_id, ws + p + t) == read_char(s, L, i + t, rc)) t++;
            if (t == sub) return true;
        }
    }
    return false;
}

__global__ void k_prepare(const ExtJob* jobs, uint32_t n, const uint8_t* __restrict__ seq,
                          const uint64_t* __restrict__ off, DevRefs R, uint32_t k, const uint8_t* raw_refs,
                          const uint64_t* raw_off, ExtResult* res, PrepRec* prep, uint64_t* sz_arena,
                          uint64_t* sz_cigar, uint64_t* sz_h) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        ExtJob jb = jobs[t];
        const uint8_t* s = seq + off[jb.read];
        const uint32_t L = (uint32_t)(off[jb.read + 1] - off[jb.read]);
        ExtResult r{};
        PrepRec p{};
        p.read = jb.read;
        p.qlen = L;
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
                uint32_t hd = 0;
                for (uint32_t i = 0; i < L; i++) hd += ref_base(R, jb.ref_id, prs + i) != read_char(s, L, i, rc);
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
                // Aligner::align returns None for reference segments over 2000 (src/aligner.rs:83-86)
                p.type = (jb.use_ssw && p.wlen <= 2000 && L > 0) ? 2 : 0;
            }
        } else if (jb.kind == JOB_RESCUE) {
            bool rc = jb.is_revcomp;
            p.rc = rc;
            r.is_revcomp = rc;
            r.gapped = 1;
            p.wstart = jb.ref_start;
            p.wlen = jb.ref_end - jb.ref_start;
            p.type = 0;
            if (p.wlen <= 2000 && L > 0 && shared_substring(R, jb.ref_id, p.wstart, p.wlen, s, L, rc, k)) p.type = 2;
        } else {  // JOB_ALIGN: raw reference bytes
            p.rc = 0;
            p.wstart = 0;
            p.wlen = (uint32_t)(raw_off[jb.ref_id + 1] - raw_off[jb.ref_id]);
            p.type = (p.wlen <= 2000 && L > 0) ? 2 : 0;
        }
        uint64_t ab = 0, cap = 0, hs = 0;
        if (p.type == 1) cap = L + 1;
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
struct CigarWriter {
    uint32_t* out;
    uint32_t n;
    uint32_t cap;
    bool overflow;
    __device__ void push(uint32_t op, uint32_t len) {
        if (len == 0) return;
        if (n > 0 && (out[n - 1] & 15) == op) out[n - 1] += len << 4;
        else if (n < cap) out[n++] = (len << 4) | op;
        else overflow = true;
    }
};

__global__ void k_fill(const ExtJob* jobs, uint32_t n, const uint8_t* __restrict__ seq, const uint64_t* __restrict__ off,
                       DevRefs R, const uint8_t* raw_refs, const uint64_t* raw_off, AlignScores sc, PrepRec* prep,
                       const uint64_t* off_arena, const uint64_t* off_cigar, const uint64_t* off_h, uint8_t* arena,
                       uint32_t* cigar, ExtResult* res, SswTask* tasks, uint32_t* counters) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        PrepRec p = prep[t];
        p.arena_off = off_arena[t];
        p.cigar_off = off_cigar[t];
        p.h_off = off_h[t];
        prep[t] = p;
        const uint8_t* s = seq + off[p.read];
        const uint32_t L = p.qlen;
        if (p.type == 1) {
            // hamming_align (src/aligner.rs:181-259)
            int32_t score = (int32_t)sc.end_bonus, best = 0;
            uint32_t start = 0, bs = 0, be = 0;
            for (uint32_t i = 0; i < L; i++) {
                bool eq = read_char(s, L, i, p.rc) == ref_base(R, p.ref_id, p.wstart + i);
                score += eq ? (int32_t)sc.match : -(int32_t)sc.mismatch;
                if (score < 0) { start = i + 1; score = 0; }
                if (score > best) { bs = start; best = score; be = i + 1; }
            }
            if (score + (int32_t)sc.end_bonus > best) {
                best = score + (int32_t)sc.end_bonus;
                be = L;
                bs = start;
            }
            CigarWriter w{cigar + p.cigar_off, 0, p.cigar_cap, false};
            uint32_t mm = 0;
            for (uint32_t i = bs; i < be; i++) {
                bool eq = read_char(s, L, i, p.rc) == ref_base(R, p.ref_id, p.wstart + i);
                mm += !eq;
                w.push(eq ? 7u : 8u, 1);
            }
            ExtResult r = res[t];
            r.valid = w.overflow ? 0 : 1;
            r.score = (uint32_t)best;
            r.edit_distance = mm;
            r.ref_start = p.wstart + bs;
            r.length = be - bs;
            r.soft_clip_left = bs;
            r.soft_clip_right = L - be;
            r.cigar_offset = (uint32_t)p.cigar_off;
            r.cigar_len = w.n;
            res[t] = r;
        } else if (p.type == 2) {
            uint8_t* q = arena + p.arena_off;
            for (uint32_t i = 0; i < L; i++) q[i] = read_char(s, L, i, p.rc);
            uint8_t* w = q + L;
            if (jobs[t].kind == JOB_ALIGN) {
                const uint8_t* rr = raw_refs + raw_off[p.ref_id];
                for (uint32_t i = 0; i < p.wlen; i++) w[i] = rr[i];
            } else {
                for (uint32_t i = 0; i < p.wlen; i++) w[i] = ref_base(R, p.ref_id, p.wstart + i);
            }
            uint32_t ti = atomicAdd(&counters[0], 1u);
            atomicAdd(reinterpret_cast<unsigned long long*>(counters + 8), (unsigned long long)L * p.wlen);
            SswTask tk{};
            tk.job = t;
            tk.ref_begin1 = -1;
            tk.read_begin1 = -1;
            tasks[ti] = tk;
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
    for (int tt = 0; tt < rlen; tt++) {
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
                if (!WORD && e.score == 255) {
                    list_word[atomicAdd(&counters[1], 1u)] = ti;
                    atomicAdd(reinterpret_cast<unsigned long long*>(counters + 8) + 1,
                              (unsigned long long)p.qlen * p.wlen);
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
            } else {
                e = sw_pass<WORD>(q, tk.read_end1 + 1, true, r, tk.ref_end1 + 1, true, tk.score1, sc, bias, H, E, qc,
                                  mask, gl);
            }
            if (gl == 0) {
                tk.ref_begin1 = e.ref;
                tk.read_begin1 = tk.read_end1 - e.read;
                tk.flag = tk.score1 > e.score ? 2 : 0;
                if (tk.ref_end1 >= 0)
                    atomicAdd(reinterpret_cast<unsigned long long*>(counters + 8) + 2 + (WORD ? 1 : 0),
                              (unsigned long long)(tk.read_end1 + 1) * (unsigned long long)(tk.ref_end1 + 1));
                tasks[ti] = tk;
            }
        }
        __syncwarp(mask);
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

__global__ void k_band_width(SswTask* tasks, const uint32_t* n_tasks_ptr, const PrepRec* prep, const uint8_t* arena,
                             int32_t* hscratch, AlignScores sc, uint64_t* dir_size, uint64_t* raw_size) {
    const uint32_t n = *n_tasks_ptr;
    for (uint32_t ti = blockIdx.x * blockDim.x + threadIdx.x; ti < n; ti += gridDim.x * blockDim.x) {
        SswTask tk = tasks[ti];
        dir_size[ti] = 0;
        raw_size[ti] = 0;
        if (tk.ref_begin1 < 0 || tk.read_begin1 < 0) continue;
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
        if (tk.ref_begin1 < 0 || tk.read_begin1 < 0 || tk.flag == 1) continue;
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
__global__ void k_finalize(const SswTask* tasks, const uint32_t* n_tasks_ptr, const PrepRec* prep, const uint8_t* arena,
                           const uint64_t* raw_off, const uint32_t* raw, AlignScores sc, uint32_t* cigar,
                           ExtResult* res) {
    const uint32_t n = *n_tasks_ptr;
    for (uint32_t ti = blockIdx.x * blockDim.x + threadIdx.x; ti < n; ti += gridDim.x * blockDim.x) {
        const SswTask tk = tasks[ti];
        const PrepRec p = prep[tk.job];
        ExtResult r = res[tk.job];
        r.valid = 0;
        if (tk.ref_begin1 < 0 || tk.read_begin1 < 0 || tk.flag != 0) {
            res[tk.job] = r;
            continue;
        }
        const uint8_t* q = arena + p.arena_off;
        const uint8_t* rf = q + p.qlen;
        const uint32_t qlen = p.qlen, rlen = p.wlen;
        uint32_t qs = tk.read_begin1, qe = tk.read_end1 + 1, rs = tk.ref_begin1, re = tk.ref_end1 + 1;
        int32_t score = tk.score1;
        // M -> =/X over the aligned segments; reject walks past them (the reference panics there)
        const uint32_t* rw = raw + raw_off[ti];
        uint32_t ed = 0;
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
            res[tk.job] = r;
            continue;
        }
        // front extension (src/aligner.rs:92-118)
        uint32_t fq = qs, fr = rs;
        int32_t fscore = score;
        uint32_t fed = 0;
        while (fq > 0 && fr > 0) {
            fq--;
            fr--;
            if (q[fq] == rf[fr]) fscore += sc.match;
            else { fscore -= sc.mismatch; fed++; }
        }
        bool take_front = fq == 0 && fscore + (int32_t)sc.end_bonus > score;
        CigarWriter w{cigar + p.cigar_off, 0, p.cigar_cap, false};
        if (take_front && qs > 0) {
            for (uint32_t a = fq; a < qs; a++) w.push(q[a] == rf[fr + (a - fq)] ? 7u : 8u, 1);
        }
        {
            uint32_t qi = qs, ri = rs;
            for (uint32_t a = 0; a < tk.raw_len; a++) {
                uint32_t op = rw[a] & 15, l = rw[a] >> 4;
                if (op == 0) {
                    for (uint32_t b = 0; b < l; b++) {
                        bool eq = q[qi] == rf[ri];
                        ed += !eq;
                        w.push(eq ? 7u : 8u, 1);
                        qi++;
                        ri++;
                    }
                } else if (op == 1) {
                    w.push(1, l);
                    ed += l;
                    qi += l;
                } else {
                    w.push(2, l);
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
        uint32_t bq = qe, br = re;
        int32_t bscore = score;
        uint32_t bed = edits;
        while (bq < qlen && br < rlen) {
            if (q[bq] == rf[br]) bscore += sc.match;
            else { bscore -= sc.mismatch; bed++; }
            bq++;
            br++;
        }
        uint32_t a_qe = qe, a_re = re;
        if (bq == qlen && bscore + (int32_t)sc.end_bonus > score) {
            if (qe < qlen)
                for (uint32_t a = qe; a < bq; a++) w.push(q[a] == rf[re + (a - qe)] ? 7u : 8u, 1);
            a_qe = qlen;
            a_re = br;
            score = bscore + (int32_t)sc.end_bonus;
            edits = bed;
        }
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
    if (g > 152ULL * 16) g = 152ULL * 16;
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

}  // namespace

void extension_init_tables() { init_tables(); }

uint32_t run_extension_raw(const DevRefs& refs, const uint8_t* seq, const uint64_t* off, const uint8_t* raw_refs,
                           const uint64_t* raw_off, uint32_t k, const AlignScores& sc, uint32_t n, ExtWorkspace& ws,
                           uint32_t max_qlen, cudaStream_t st, KernelTimers* kt) {
    init_tables();
    KernelTimers none;
    if (!kt) kt = &none;
    uint32_t launches = 0;
    ws.results.reserve(n);
    ws.prep.reserve(n);
    ws.sizes.reserve(3 * ((size_t)n + 1));
    ws.offs.reserve(3 * ((size_t)n + 1));
    ws.counters.reserve(16);
    if (n == 0) {
        ws.h_results.clear();
        ws.h_cigar.clear();
        return 0;
    }
    uint64_t* sz[3] = {ws.sizes.p, ws.sizes.p + n + 1, ws.sizes.p + 2 * ((size_t)n + 1)};
    uint64_t* of[3] = {ws.offs.p, ws.offs.p + n + 1, ws.offs.p + 2 * ((size_t)n + 1)};
    SA_CUDA(cudaMemsetAsync(ws.counters.p, 0, 16 * sizeof(uint32_t), st));
    kt->begin(KS_PREPARE, st);
    k_prepare<<<grid1(n), 256, 0, st>>>(ws.jobs.p, n, seq, off, refs, k, raw_refs, raw_off, ws.results.p, ws.prep.p,
                                        sz[0], sz[1], sz[2]);
    kt->end(st);
    launches++;
    // exclusive scans of arena bytes, CIGAR capacity and banded-DP scratch per job
    uint64_t tot[3];
    for (int c = 0; c < 3; c++) {
        SA_CUDA(cudaMemsetAsync(sz[c] + n, 0, 8, st));
        excl_sum(ws, sz[c], of[c], (uint64_t)n + 1, st);
        SA_CUDA(cudaMemcpyAsync(&tot[c], of[c] + n, 8, cudaMemcpyDeviceToHost, st));
    }
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
    k_fill<<<grid1(n), 256, 0, st>>>(ws.jobs.p, n, seq, off, refs, raw_refs, raw_off, sc, ws.prep.p, of[0], of[1],
                                     of[2], ws.arena.p, ws.cigar.p, ws.results.p, ws.tasks.p, ws.counters.p);
    kt->end(st);
    launches++;
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
            if (b > 152ULL * 16) b = 152ULL * 16;
            return (unsigned)(b ? b : 1);
        };
        // forward byte pass over all tasks
        kt->begin(KS_SW_BYTE, st);
        k_sw<false><<<blocks_for(n_tasks, tpb / 16), tpb, smem_b, st>>>(
            ws.tasks.p, nullptr, nullptr, n_tasks, ws.prep.p, ws.arena.p, sc, bias, 0, seg_b, ws.counters.p,
            ws.list_word.p, ws.list_rev_byte.p, ws.list_rev_word.p);
        kt->end(st);
        // forward word pass over the overflowed tasks
        kt->begin(KS_SW_WORD, st);
        k_sw<true><<<blocks_for(n_tasks, tpb / 8), tpb, smem_w, st>>>(
            ws.tasks.p, ws.list_word.p, ws.counters.p + 1, 0, ws.prep.p, ws.arena.p, sc, bias, 0, seg_w,
            ws.counters.p, ws.list_word.p, ws.list_rev_byte.p, ws.list_rev_word.p);
        kt->end(st);
        // reverse passes
        kt->begin(KS_SW_BYTE, st);
        k_sw<false><<<blocks_for(n_tasks, tpb / 16), tpb, smem_b, st>>>(
            ws.tasks.p, ws.list_rev_byte.p, ws.counters.p + 2, 0, ws.prep.p, ws.arena.p, sc, bias, 1, seg_b,
            ws.counters.p, ws.list_word.p, ws.list_rev_byte.p, ws.list_rev_word.p);
        kt->end(st);
        kt->begin(KS_SW_WORD, st);
        k_sw<true><<<blocks_for(n_tasks, tpb / 8), tpb, smem_w, st>>>(
            ws.tasks.p, ws.list_rev_word.p, ws.counters.p + 3, 0, ws.prep.p, ws.arena.p, sc, bias, 1, seg_w,
            ws.counters.p, ws.list_word.p, ws.list_rev_byte.p, ws.list_rev_word.p);
        kt->end(st);
        launches += 4;
        ws.dir_size.reserve((size_t)n_tasks + 1);
        ws.dir_off.reserve((size_t)n_tasks + 1);
        ws.raw_size.reserve((size_t)n_tasks + 1);
        ws.raw_off.reserve((size_t)n_tasks + 1);
        kt->begin(KS_BAND, st);
        k_band_width<<<grid1(n_tasks, 128), 128, 0, st>>>(ws.tasks.p, ws.counters.p, ws.prep.p, ws.arena.p,
                                                          ws.hscratch.p, sc, ws.dir_size.p, ws.raw_size.p);
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
        k_band_trace<<<grid1(n_tasks, 128), 128, 0, st>>>(ws.tasks.p, ws.counters.p, ws.prep.p, ws.arena.p,
                                                          ws.hscratch.p, sc, ws.dir_off.p, ws.dir.p, ws.raw_off.p,
                                                          ws.raw.p);
        kt->end(st);
        kt->begin(KS_FINALIZE, st);
        k_finalize<<<grid1(n_tasks, 128), 128, 0, st>>>(ws.tasks.p, ws.counters.p, ws.prep.p, ws.arena.p,
                                                        ws.raw_off.p, ws.raw.p, sc, ws.cigar.p, ws.results.p);
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
    SA_CUDA(cudaMemcpyAsync(ws.cells, ws.counters.p + 8, 4 * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaStreamSynchronize(st));
    tot[1] = used;
    ws.total_cigar = tot[1];
    return launches;
}

uint32_t run_extension(const DevRefs& refs, const NamWorkspace& nws, uint32_t k, const AlignScores& sc, uint32_t n,
                       ExtWorkspace& ws, uint32_t max_qlen, cudaStream_t st, KernelTimers* kt) {
    return run_extension_raw(refs, nws.seq.p, nws.off.p, nullptr, nullptr, k, sc, n, ws, max_qlen, st, kt);
}

}  // namespace sa
