// NAM finding on the GPU: the reference's get_nams_by_chaining (src/nam.rs:138-166)
// for a whole batch of reads, one launch per stage:
//
//   k_seed          warp per read: canonical syncmers + forward / reverse-complement
//                   randstrobes (src/seeding/{syncmers,strobes,mod}.rs)
//   k_hits          warp per read: index probes with the repeat filter, global and
//                   local rescue, orientation choice (src/hit.rs, src/chainer.rs:205-216)
//   k_anchors       warp per read: anchor count, then fill (src/chainer.rs:304-384)
//   segmented sort  (ref_id, ref_start, query_start) packed in a u64 key
//   k_chain4        warp per eight read orientations: anchor sort and dedup, collinear
//                   chaining DP with the reference's early-break rules evaluated as a
//                   prefix max over the candidates (four lanes per orientation), chain
//                   extraction
//                   (src/chainer.rs:85-180, 386-449)
//   k_nam_compact   warp per read: NAM ids in push order, stable sort by score
//                   (src/nam.rs:168-170); reads with more than 32 NAMs through a
//                   segmented stable sort and k_nam_gather
//
// Floating point follows the reference exactly: f32 with explicit round-to-nearest
// intrinsics (no contraction) and log2(d + 1) from a table built with the host's
// log2f, the function the reference calls.
#include <cub/cub.cuh>

#include <cmath>
#include <mutex>
#include <string>

#include "index_device.cuh"
#include "pipeline.h"

namespace sa {

namespace {

constexpr uint32_t FULL = 0xffffffffu;
constexpr int WARPS_PER_BLOCK = 8;

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ uint32_t lanemask_lt() { return (1u << lane_id()) - 1; }

__device__ __forceinline__ uint8_t nt_code(uint8_t c) {
    switch (c) {
        case 'A': case 'a': return 0;
        case 'C': case 'c': return 1;
        case 'G': case 'g': return 2;
        case 'T': case 't': case 'U': case 'u': return 3;
        default: return 4;
    }
}

// ------------------------------------------------------------------ seeding
// A read packed 2 bits per base (base i at bits 2(i % 32) of word i / 32) with one
// N flag bit per base, so that any window of up to 32 bases comes out in O(1).
__device__ __forceinline__ uint64_t spread_bits(uint32_t v) {
    uint64_t x = v;
    x = (x | (x << 16)) & 0x0000FFFF0000FFFFULL;
    x = (x | (x << 8)) & 0x00FF00FF00FF00FFULL;
    x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0FULL;
    x = (x | (x << 2)) & 0x3333333333333333ULL;
    x = (x | (x << 1)) & 0x5555555555555555ULL;
    return x;
}
__device__ __forceinline__ uint64_t window_bits(const uint64_t* packed, uint32_t q) {
    const uint32_t w = q >> 5, sh = 2 * (q & 31);
    const uint64_t lo = packed[w] >> sh;
    return sh ? lo | (packed[w + 1] << (64 - sh)) : lo;
}
__device__ __forceinline__ uint32_t window_n(const uint32_t* nflags, uint32_t q) {
    const uint32_t w = q >> 5;
    return (uint32_t)((((uint64_t)nflags[w + 1] << 32) | nflags[w]) >> (q & 31));
}
__device__ __forceinline__ uint64_t low_mask(uint32_t bits) { return bits >= 64 ? ~0ULL : (1ULL << bits) - 1; }
// the n-base window w (base 0 in the low bits) as the reference encodes it: forward
// with the first base most significant, reverse complement with the first base least
__device__ __forceinline__ void kmer_codes(uint64_t w, uint32_t n, uint64_t& fw, uint64_t& rc) {
    const uint64_t m = low_mask(2 * n);
    w &= m;
    rc = ~w & m;
    uint64_t r = __brevll(w);
    r = ((r >> 1) & 0x5555555555555555ULL) | ((r & 0x5555555555555555ULL) << 1);
    fw = r >> (64 - 2 * n);
}

// src/seeding/syncmers.rs:171-237: a syncmer at p requires an N-free k-mer window
// and the (t-1)-th of its k-s+1 s-mer hashes to equal their minimum.
// CHECKED (offsets supplied by a caller, not built here): a read whose offsets are
// decreasing, end past `total` or span more than MAX_READ_LEN gets the count
// UINT32_MAX in both orientations and is not touched otherwise.
template <bool CHECKED>
__global__ void __launch_bounds__(256) k_seed(const uint8_t* __restrict__ seq, const uint64_t* __restrict__ off,
                                              uint32_t n, SeedParams p, uint64_t* syn_hash, uint32_t* syn_pos,
                                              uint64_t* qr_hash, uint64_t* qr_hash_rc, uint32_t* qr_start,
                                              uint32_t* qr_end, uint64_t total, uint32_t* n_rs) {
    extern __shared__ uint8_t smem[];
    // per warp: packed bases (MAX_READ_LEN / 32 + 2 words) then N flags
    uint64_t* packed = reinterpret_cast<uint64_t*>(smem + (threadIdx.x / 32) * MAX_READ_LEN);
    uint32_t* nflags = reinterpret_cast<uint32_t*>(packed + MAX_READ_LEN / 32 + 2);
    const uint32_t lane = lane_id();
    const uint32_t span = p.k - p.s, step = 32 - span;
    const uint32_t nwarps = gridDim.x * (blockDim.x / 32);
    for (uint32_t r = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; r < n; r += nwarps) {
        const uint64_t o = off[r];
        if (CHECKED) {
            const uint64_t e = off[r + 1];
            if (e < o || e > total || e - o > MAX_READ_LEN) {
                if (lane == 0) {
                    n_rs[2 * r] = UINT32_MAX;
                    n_rs[2 * r + 1] = UINT32_MAX;
                }
                continue;
            }
        }
        const uint32_t L = (uint32_t)(off[r + 1] - o);
        const uint32_t nwords = (L + 31) / 32;
        for (uint32_t w = 0; w <= nwords; w++) {
            const uint32_t i = w * 32 + lane;
            const uint32_t cc = i < L ? nt_code(seq[o + i]) : 0;
            const uint32_t b0 = __ballot_sync(FULL, cc & 1), b1 = __ballot_sync(FULL, (cc >> 1) & 1);
            const uint32_t bn = __ballot_sync(FULL, cc > 3);
            if (lane == 0) {
                packed[w] = spread_bits(b0) | (spread_bits(b1) << 1);
                nflags[w] = bn;
            }
        }
        __syncwarp();
        uint32_t nsyn = 0;
        for (uint32_t c = 0; L >= p.k && c + p.k <= L; c += step) {
            const uint32_t q = c + lane;
            bool v = q + p.s <= L;
            uint64_t fw = 0, rc = 0;
            if (v) {
                v = (window_n(nflags, q) & (uint32_t)low_mask(p.s)) == 0;
                kmer_codes(window_bits(packed, q), p.s, fw, rc);
            }
            uint64_t hs = v ? xxh64_u64(fw < rc ? fw : rc) : 0;
            bool ok = true;
            uint64_t mn = UINT64_MAX, ht = 0;
            for (uint32_t d = 0; d <= span; d++) {
                uint64_t h = __shfl_down_sync(FULL, hs, d);
                bool vv = __shfl_down_sync(FULL, v, d);
                ok = ok && vv;
                mn = h < mn ? h : mn;
                if (d == p.t - 1) ht = h;
            }
            const uint32_t pos = c + lane;
            bool is_syn = lane < step && pos + p.k <= L && ok && ht == mn;
            uint64_t kh = 0;
            uint32_t fwd = 0;
            if (is_syn) {
                uint64_t kf, kr;
                kmer_codes(window_bits(packed, pos), p.k, kf, kr);
                kh = xxh64_u64(kf < kr ? kf : kr);
                fwd = kf <= kr;
            }
            uint32_t bal = __ballot_sync(FULL, is_syn);
            if (is_syn) {
                uint32_t idx = nsyn + __popc(bal & lanemask_lt());
                syn_hash[o + idx] = kh;
                syn_pos[o + idx] = (pos << 1) | fwd;
            }
            nsyn += __popc(bal);
        }
        __syncwarp();
        const uint32_t nr = L < p.w_max ? 0 : nsyn;
        // forward randstrobes (src/seeding/strobes.rs:145-176)
        for (uint32_t i = lane; i < nr; i += 32) {
            uint64_t h1 = syn_hash[o + i];
            uint32_t p1 = syn_pos[o + i];
            uint32_t pos1 = p1 >> 1;
            uint64_t best = UINT64_MAX;
            uint64_t h2 = h1;
            uint32_t p2 = p1;
            for (uint32_t j = i + p.w_min; j <= i + p.w_max && j < nsyn; j++) {
                uint32_t pj = syn_pos[o + j];
                if ((pj >> 1) > pos1 + p.max_dist) break;
                uint64_t hj = syn_hash[o + j];
                uint64_t ones = (uint64_t)__popcll((h1 ^ hj) & p.q);
                if (ones < best) { best = ones; h2 = hj; p2 = pj; }
            }
            uint64_t f1 = p1 & 1, f2 = p2 & 1;
            qr_hash[o + i] = randstrobe_hash(h1, h2, f1, f2, p);
            qr_hash_rc[o + i] = randstrobe_hash(h2, h1, f1 ^ 1, f2 ^ 1, p);
            qr_start[o + i] = pos1;
            qr_end[o + i] = (p2 >> 1) + p.k;
        }
        // reverse-complement randstrobes from the reversed syncmer list (src/seeding/mod.rs:53-73)
        for (uint32_t ir = lane; ir < nr; ir += 32) {
            uint32_t i = nsyn - 1 - ir;
            uint64_t h1 = syn_hash[o + i];
            uint32_t p1 = syn_pos[o + i];
            uint32_t pos1 = L - (p1 >> 1) - p.k;
            uint32_t f1 = (p1 & 1) ^ 1;
            uint64_t best = UINT64_MAX;
            uint64_t h2 = h1;
            uint32_t pos2 = pos1, f2 = f1;
            for (uint32_t d = p.w_min; d <= p.w_max && d <= i; d++) {
                uint32_t j = i - d;
                uint32_t pj = syn_pos[o + j];
                uint32_t posj = L - (pj >> 1) - p.k;
                if (posj > pos1 + p.max_dist) break;
                uint64_t hj = syn_hash[o + j];
                uint64_t ones = (uint64_t)__popcll((h1 ^ hj) & p.q);
                if (ones < best) { best = ones; h2 = hj; pos2 = posj; f2 = (pj & 1) ^ 1; }
            }
            qr_hash[total + o + ir] = randstrobe_hash(h1, h2, f1, f2, p);
            qr_hash_rc[total + o + ir] = randstrobe_hash(h2, h1, f1 ^ 1, f2 ^ 1, p);
            qr_start[total + o + ir] = pos1;
            qr_end[total + o + ir] = pos2 + p.k;
        }
        if (lane == 0) {
            n_rs[2 * r] = nr;
            n_rs[2 * r + 1] = nr;
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ hits
struct HitsCounts {
    uint32_t fnf, ff, ffound, pnf, pf, pfound, rescued;
};

__device__ __forceinline__ uint32_t warp_sum(uint32_t v) {
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(FULL, v, d);
    return v;
}

// count used by rescue_least_frequent (src/hit.rs:96-107), cached per hit
__device__ __forceinline__ uint32_t hit_count(const DevIndex& ix, uint64_t pos, uint32_t info, uint64_t hash_rc) {
    if (info & 2) return idx_get_count(ix, pos, ix.p.main_mask);
    return idx_count_full(ix, pos, hash_rc);
}

// rescue_least_frequent (src/hit.rs:88-125) over hits [s, e) of one read-orientation.
// Whole warp participates; returns the number rescued (valid in all lanes).
__device__ uint32_t warp_rescue_least_frequent(const DevIndex& ix, uint32_t s, uint32_t e, uint32_t to_rescue,
                                               uint32_t threshold, const uint64_t* hit_pos, uint32_t* hit_info,
                                               uint32_t* cache, const uint64_t* rs_hash_rc) {
    for (uint32_t h = s + lane_id(); h < e; h += 32) {
        if (cache[h] == 0xffffffffu) {
            uint32_t info = hit_info[h];
            cache[h] = hit_count(ix, hit_pos[h], info, rs_hash_rc[info >> 3]);
        }
    }
    __syncwarp();
    uint32_t rescued = 0;
    if (lane_id() == 0) {
        // stable ascending sort by count == pick (count, index) in lexicographic order
        uint32_t pc = 0, pi = 0;
        bool have_prev = false;
        for (uint32_t t = 0; t < to_rescue; t++) {
            uint32_t bc = 0xffffffffu, bi = 0xffffffffu;
            for (uint32_t h = s; h < e; h++) {
                uint32_t c = cache[h];
                if (c > threshold) continue;
                if (have_prev && (c < pc || (c == pc && h <= pi))) continue;
                if (c < bc || (c == bc && h < bi)) { bc = c; bi = h; }
            }
            if (bi == 0xffffffffu) break;
            uint32_t info = hit_info[bi];
            rescued += (info >> 2) & 1;
            hit_info[bi] = info & ~4u;
            pc = bc;
            pi = bi;
            have_prev = true;
        }
    }
    __syncwarp();
    return __shfl_sync(FULL, rescued, 0);
}

// Per-randstrobe index probes of find_hits' first pass (src/hit.rs:143-187), ahead of
// k_hits: lanes run over both orientations' randstrobes of a read together, each lane
// one probe with the latency-parallel lookups.  Writes, per randstrobe slot, the table
// position (UINT64_MAX if absent) and PROBE_* flags; k_hits compacts them in place.
constexpr uint32_t PROBE_FULL = 1, PROBE_PARTIAL = 2, PROBE_FILTERED = 4;

__global__ void __launch_bounds__(256) k_probe(DevIndex ix, const uint64_t* __restrict__ off, uint32_t n,
                                               uint64_t total, uint32_t mcs, const uint64_t* __restrict__ qr_hash,
                                               const uint64_t* __restrict__ qr_hash_rc,
                                               const uint32_t* __restrict__ n_rs, uint64_t* __restrict__ hit_pos,
                                               uint32_t* __restrict__ hit_info) {
    const uint32_t lane = lane_id();
    const uint32_t nwarps = gridDim.x * (blockDim.x / 32);
    const uint32_t cutoff = ix.filter_cutoff;
    for (uint32_t r = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; r < n; r += nwarps) {
        const uint64_t o = off[r];
        const uint32_t n0 = n_rs[2 * r], n1 = n_rs[2 * r + 1];
        for (uint32_t j = lane; j < n0 + n1; j += 32) {
            const uint32_t ori = j >= n0;
            const uint64_t slot = ori * total + o + (j - ori * n0);
            const uint64_t h = qr_hash[slot];
            uint64_t pos;
            bool filtered;
            idx_full_probe(ix, h, qr_hash_rc[slot], cutoff, pos, filtered);
            uint32_t flags = 0;
            if (pos != UINT64_MAX) {
                flags = PROBE_FULL | (filtered ? PROBE_FILTERED : 0u);
            } else if (mcs == SA_MCS_ALWAYS) {
                pos = idx_get_masked_from(ix, h, ix.p.main_mask, false, 0);
                if (pos != UINT64_MAX)
                    flags = PROBE_PARTIAL | (idx_too_frequent_partial(ix, pos, cutoff) ? PROBE_FILTERED : 0u);
            }
            hit_pos[slot] = pos;
            hit_info[slot] = flags;
        }
    }
}

// find_hits (src/hit.rs:129-333) for both orientations of each read, then the
// orientation heuristic (src/chainer.rs:205-216, src/hit.rs:76-81).  The first pass
// reads k_probe's per-slot answers.
__global__ void __launch_bounds__(256) k_hits(DevIndex ix, const uint64_t* __restrict__ off, uint32_t n,
                                              uint64_t total, uint32_t mcs, uint32_t rescue_distance,
                                              const uint64_t* qr_hash, const uint64_t* qr_hash_rc,
                                              const uint32_t* qr_start, const uint32_t* qr_end,
                                              const uint32_t* n_rs, uint64_t* hit_pos, uint32_t* hit_info,
                                              uint32_t* cache, uint32_t* n_hits, uint8_t* orient,
                                              NamDetailsRec* details) {
    const uint32_t lane = lane_id();
    const uint32_t nwarps = gridDim.x * (blockDim.x / 32);
    const uint32_t cutoff = ix.filter_cutoff;
    for (uint32_t r = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; r < n; r += nwarps) {
        const uint64_t o = off[r];
        HitsCounts hc[2];
        for (int ori = 0; ori < 2; ori++) {
            const uint64_t b = ori * total + o;
            const uint32_t nr = n_rs[2 * r + ori];
            uint32_t nh = 0;
            uint32_t fnf = 0, ff = 0, ffound = 0, pnf = 0, pf = 0, pfound = 0;
            const bool do_full = mcs != SA_MCS_FIRST_STROBE;
            // pass 1: full lookups (with partial fallback under MCS always), probed by
            // k_probe; compacted in place (a slot is written only after every lane of
            // the round has read its own)
            if (do_full) {
                for (uint32_t c = 0; c < nr; c += 32) {
                    uint32_t i = c + lane;
                    bool is_hit = false, partial = false, filtered = false;
                    uint64_t pos = UINT64_MAX;
                    if (i < nr) {
                        const uint32_t fl = hit_info[b + i];
                        pos = hit_pos[b + i];
                        filtered = fl & PROBE_FILTERED;
                        if (fl & PROBE_FULL) {
                            is_hit = true;
                            if (filtered) ff++;
                            else ffound++;
                        } else {
                            fnf++;
                            if (mcs == SA_MCS_ALWAYS) {
                                if (fl & PROBE_PARTIAL) {
                                    is_hit = partial = true;
                                    if (filtered) pf++;
                                    else pfound++;
                                } else {
                                    pnf++;
                                }
                            }
                        }
                    }
                    uint32_t bal = __ballot_sync(FULL, is_hit);
                    __syncwarp();
                    if (is_hit) {
                        uint32_t idx = nh + __popc(bal & lanemask_lt());
                        hit_pos[b + idx] = pos;
                        hit_info[b + idx] = (i << 3) | (filtered ? 4u : 0u) | (partial ? 2u : 0u) | 1u;
                        cache[b + idx] = 0xffffffffu;
                    }
                    nh += __popc(bal);
                }
            }
            uint32_t full_hits = warp_sum(ff + ffound);
            bool partial_pass = mcs == SA_MCS_FIRST_STROBE || (mcs == SA_MCS_RESCUE && full_hits == 0);
            if (partial_pass) {
                for (uint32_t c = 0; c < nr; c += 32) {
                    uint32_t i = c + lane;
                    bool is_hit = false, filtered = false;
                    uint64_t pos = UINT64_MAX;
                    if (i < nr) {
                        pos = idx_get_masked_from(ix, qr_hash[b + i], ix.p.main_mask, false, 0);
                        if (pos != UINT64_MAX) {
                            is_hit = true;
                            filtered = idx_too_frequent_partial(ix, pos, cutoff);
                            if (filtered) pf++;
                            else pfound++;
                        } else {
                            pnf++;
                        }
                    }
                    uint32_t bal = __ballot_sync(FULL, is_hit);
                    if (is_hit) {
                        uint32_t idx = nh + __popc(bal & lanemask_lt());
                        hit_pos[b + idx] = pos;
                        hit_info[b + idx] = (i << 3) | (filtered ? 4u : 0u) | 2u | 1u;
                        cache[b + idx] = 0xffffffffu;
                    }
                    nh += __popc(bal);
                }
            }
            __syncwarp();
            HitsCounts d;
            d.fnf = warp_sum(fnf);
            d.ff = warp_sum(ff);
            d.ffound = warp_sum(ffound);
            d.pnf = warp_sum(pnf);
            d.pf = warp_sum(pf);
            d.pfound = warp_sum(pfound);
            d.rescued = 0;
            // rescue (src/hit.rs:270-304)
            uint32_t total_hits = d.pf + d.pfound + d.ff + d.ffound;
            uint32_t nonrep = d.ffound + d.pfound;
            float frac = total_hits > 0 ? __fdiv_rn(__uint2float_rn(nonrep), __uint2float_rn(total_hits)) : 1.0f;
            if (rescue_distance > 0) {
                if (frac < 0.7f && nonrep < 5)
                    d.rescued += warp_rescue_least_frequent(ix, 0, nh, 5, 1000, hit_pos + b, hit_info + b, cache + b,
                                                            qr_hash_rc + b);
                // local rescue over filtered stretches (src/hit.rs:232-268); an interval is
                // processed as soon as it is found, which only touches hits already scanned
                uint32_t scan = 0, last_unf = 0, first_f = 0;
                for (;;) {
                    uint32_t is = 0, ie = 0, tr = 0, found = 0;
                    if (lane == 0) {
                        while (scan < nh) {
                            uint32_t h = scan++;
                            uint32_t info = hit_info[b + h];
                            if (info & 4) continue;
                            uint32_t qs = qr_start[b + (info >> 3)];
                            bool iv = qs > last_unf + rescue_distance;
                            if (iv) { is = first_f; ie = h; tr = (qs - last_unf) / rescue_distance; found = 1; }
                            last_unf = qs;
                            first_f = h + 1;
                            if (iv) break;
                        }
                        if (!found && scan == nh && nh > 0 && scan != 0xffffffffu) {
                            uint32_t lq = qr_start[b + (hit_info[b + nh - 1] >> 3)];
                            uint32_t diff = lq - last_unf;
                            if (diff > rescue_distance) { is = first_f; ie = nh; tr = diff / rescue_distance; found = 1; }
                            scan = 0xffffffffu;
                        }
                    }
                    found = __shfl_sync(FULL, found, 0);
                    if (!found) break;
                    is = __shfl_sync(FULL, is, 0);
                    ie = __shfl_sync(FULL, ie, 0);
                    tr = __shfl_sync(FULL, tr, 0);
                    d.rescued += warp_rescue_least_frequent(ix, is, ie, tr, 10000, hit_pos + b, hit_info + b,
                                                            cache + b, qr_hash_rc + b);
                }
            }
            hc[ori] = d;
            if (lane == 0) n_hits[2 * r + ori] = nh;
        }
        if (lane == 0) {
            uint32_t t0 = hc[0].ffound + hc[0].ff, t1 = hc[1].ffound + hc[1].ff;
            bool b0 = t0 >= t1 * 2 && t0 > t1 + 5;
            bool b1 = t1 >= t0 * 2 && t1 > t0 + 5;
            uint8_t m = b0 ? 1 : b1 ? 2 : 3;
            orient[r] = m;
            NamDetailsRec dr;
            dr.full_not_found = hc[0].fnf + hc[1].fnf;
            dr.full_filtered = hc[0].ff + hc[1].ff;
            dr.full_found = hc[0].ffound + hc[1].ffound;
            dr.partial_not_found = hc[0].pnf + hc[1].pnf;
            dr.partial_filtered = hc[0].pf + hc[1].pf;
            dr.partial_found = hc[0].pfound + hc[1].pfound;
            dr.rescued = hc[0].rescued + hc[1].rescued;
            dr.n_randstrobes = n_rs[2 * r] + n_rs[2 * r + 1];
            dr.n_anchors = 0;
            dr.n_nams = 0;
            dr.both_orientations = m == 3;
            details[r] = dr;
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ anchors
// Anchor keys: (ref_id, ref_start, query_start) packed so that integer order is the
// reference's anchor order (src/chainer.rs:228).
struct AnchorPack {
    uint32_t qbits, pbits;
    __device__ __forceinline__ uint64_t key(uint32_t ref_id, uint32_t ref_start, uint32_t qs) const {
        return ((uint64_t)ref_id << (pbits + qbits)) | ((uint64_t)ref_start << qbits) | qs;
    }
};

// add_to_anchors_full / add_to_anchors_partial (src/chainer.rs:304-366) are split into
// run_head (one lane, the first 32 entries of a run) and warp_run_anchors (the rest).
//
// A hit's run of equal-hash table entries: its first entry and hash (full hits:
// the entry found; partial hits: get_masked_from with the forward main mask).  False
// when a partial hit has no entry under that mask.
__device__ __forceinline__ bool hit_run(const DevIndex& ix, uint64_t pos, uint32_t info, uint64_t hash,
                                        uint64_t& start, uint64_t& fh) {
    if (info & 2) {
        start = idx_get_masked_from(ix, hash, ix.p.fwd_main_mask, true, pos);
        if (start == UINT64_MAX) return false;
        fh = load_rs(ix.rs, start).hash_offset & ix.p.fwd_main_mask;
    } else {
        start = pos;
        fh = load_hash(ix.rs, pos);
    }
    return true;
}

// The first 32 entries of a run by one lane (hit_anchors' loop): anchors to out (if
// not null), their count, the running minimum length difference (full hits).  True
// when the run ended within them; otherwise the warp continues from start + 32.
__device__ __forceinline__ bool run_head(const DevIndex& ix, uint64_t start, uint64_t fh, bool partial, uint32_t qs,
                                         uint32_t qe, AnchorPack ap, uint64_t* out, uint32_t& cnt, uint32_t& minld) {
    const uint32_t k = ix.p.k, ql = qe - qs;
    cnt = 0;
    minld = 0xffffffffu;
    const uint64_t end = start + 32 < ix.n ? start + 32 : ix.n;
    for (uint64_t i = start; i < end; i++) {
        const RefRandstrobe rr = load_rs(ix.rs, i);
        if (partial) {
            if ((rr.hash_offset & ix.p.fwd_main_mask) != fh) return true;
            if (out) out[cnt] = ap.key(rr.ref_index, rr.position, qs);
            cnt++;
        } else {
            if (rs_hash(rr) != fh) return true;
            const uint32_t rl = (uint32_t)(rr.hash_offset & 0xff) + k;
            const uint32_t ld = ql > rl ? ql - rl : rl - ql;
            if (ld <= minld) {
                if (out) {
                    out[cnt] = ap.key(rr.ref_index, rr.position, qs);
                    out[cnt + 1] = ap.key(rr.ref_index, rr.position + rl - k, qe - k);
                }
                cnt += 2;
                minld = ld;
            }
        }
    }
    return end == ix.n;
}

// hit_anchors for one run by the whole warp (arguments uniform across the warp): lanes
// take consecutive entries; the running-minimum length filter of full hits becomes a
// prefix minimum over the lanes carried between 32-entry slices.
__device__ uint32_t warp_run_anchors(const DevIndex& ix, uint64_t start, uint64_t fh, bool partial, uint32_t qs,
                                     uint32_t qe, AnchorPack ap, uint64_t* out, uint32_t carry) {
    const uint32_t lane = lane_id(), k = ix.p.k, ql = qe - qs;
    uint32_t cnt = 0;
    for (uint64_t c = start;; c += 32) {
        const uint64_t i = c + lane;
        bool valid = false;
        RefRandstrobe rr{};
        if (i < ix.n) {
            rr = load_rs(ix.rs, i);
            valid = partial ? (rr.hash_offset & ix.p.fwd_main_mask) == fh : rs_hash(rr) == fh;
        }
        // the table is sorted: the run's entries are a prefix of the lanes
        const uint32_t vb = __ballot_sync(FULL, valid);
        if (partial) {
            if (valid && out) out[cnt + lane] = ap.key(rr.ref_index, rr.position, qs);
            cnt += __popc(vb);
        } else {
            const uint32_t rl = valid ? (uint32_t)(rr.hash_offset & 0xff) + k : 0;
            const uint32_t ld = valid ? (ql > rl ? ql - rl : rl - ql) : 0xffffffffu;
            uint32_t incl = ld;
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL, incl, d);
                if (lane >= (uint32_t)d) incl = min(incl, y);
            }
            uint32_t excl = __shfl_up_sync(FULL, incl, 1);
            if (lane == 0) excl = 0xffffffffu;
            const bool o = valid && ld <= min(carry, excl);
            const uint32_t ob = __ballot_sync(FULL, o);
            if (o && out) {
                const uint32_t p = cnt + 2 * __popc(ob & lanemask_lt());
                out[p] = ap.key(rr.ref_index, rr.position, qs);
                out[p + 1] = ap.key(rr.ref_index, rr.position + rl - k, qe - k);
            }
            cnt += 2 * __popc(ob);
            carry = min(carry, __shfl_sync(FULL, incl, 31));
        }
        if (vb != FULL) break;
    }
    return cnt;
}

__device__ __forceinline__ uint32_t warp_excl_scan(uint32_t v, uint32_t& total) {
    uint32_t x = v;
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(FULL, x, d);
        if (lane_id() >= (uint32_t)d) x += y;
    }
    total = __shfl_sync(FULL, x, 31);
    return x - v;
}

template <bool FILL>
__global__ void __launch_bounds__(256) k_anchors(DevIndex ix, const uint64_t* __restrict__ off, uint32_t n,
                                                 uint64_t total, const uint64_t* qr_hash, const uint32_t* qr_start,
                                                 const uint32_t* qr_end, const uint64_t* hit_pos,
                                                 const uint32_t* hit_info, const uint32_t* n_hits,
                                                 const uint8_t* orient, uint32_t* hit_anchors_n, uint64_t* seg_count,
                                                 const uint64_t* seg_off, uint64_t* anchors, AnchorPack ap,
                                                 NamDetailsRec* details) {
    const uint32_t lane = lane_id();
    const uint32_t nwarps = gridDim.x * (blockDim.x / 32);
    for (uint32_t r = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; r < n; r += nwarps) {
        const uint64_t o = off[r];
        const uint8_t m = orient[r];
        uint32_t read_total = 0;
        for (int ori = 0; ori < 2; ori++) {
            const uint64_t b = ori * total + o;
            const uint32_t nh = (m >> ori) & 1 ? n_hits[2 * r + ori] : 0;
            uint64_t acc = FILL ? seg_off[2 * r + ori] : 0;
            AnchorPack aps = ap;
            uint32_t sum = 0;
            for (uint32_t c = 0; c < nh; c += 32) {
                uint32_t h = c + lane;
                uint32_t cnt = 0, head = 0, minld = 0xffffffffu;
                uint32_t info = 0, qs = 0, qe = 0;
                uint64_t start = 0, fh = 0;
                bool has_run = false, is_long = false;
                if (h < nh) {
                    info = hit_info[b + h];
                    if (!(info & 4)) {
                        const uint32_t ri = info >> 3;
                        qs = qr_start[b + ri];
                        qe = (info & 2) ? qs + ix.p.k : qr_end[b + ri];
                        has_run = hit_run(ix, hit_pos[b + h], info, qr_hash[b + ri], start, fh);
                        if (FILL) cnt = hit_anchors_n[b + h];
                    }
                }
                uint32_t tot = 0, ex = 0;
                if (FILL) ex = warp_excl_scan(cnt, tot);
                // each lane its run's first 32 entries; longer runs continue with the
                // whole warp, one hit at a time
                if (has_run)
                    is_long = !run_head(ix, start, fh, info & 2, qs, qe, aps, FILL ? anchors + acc + ex : nullptr, head,
                                        minld);
                const uint32_t lm = __ballot_sync(FULL, is_long);
                for (uint32_t m = lm; m; m &= m - 1) {
                    const int L = __ffs(m) - 1;
                    const uint32_t hL = __shfl_sync(FULL, head, L);
                    const uint32_t rest = warp_run_anchors(
                        ix, __shfl_sync(FULL, start, L) + 32, __shfl_sync(FULL, fh, L), __shfl_sync(FULL, info, L) & 2,
                        __shfl_sync(FULL, qs, L), __shfl_sync(FULL, qe, L), aps,
                        FILL ? anchors + acc + __shfl_sync(FULL, ex, L) + hL : nullptr, __shfl_sync(FULL, minld, L));
                    if (lane == (uint32_t)L) head += rest;
                }
                if (!FILL) {
                    cnt = head;
                    if (h < nh && !(info & 4)) hit_anchors_n[b + h] = cnt;
                    ex = warp_excl_scan(cnt, tot);
                }
                acc += tot;
                sum += tot;
            }
            if (!FILL && lane == 0) seg_count[2 * r + ori] = sum;
            read_total += sum;
        }
        if (!FILL && lane == 0) details[r].n_anchors = read_total;
    }
}

// ------------------------------------------------------------------ chaining
struct ChainCtx {
    ChainParams cp;
    uint32_t k;
    const float* lut;
    // fl(mx / mn) > max_diagonal_ratio without the division, for integers below 2^24
    // (whose float conversions are exact): with R = M * 2^e (M the 24-bit significand),
    // the quotient rounds above R exactly when mx / mn exceeds the midpoint
    // (2M + 1) * 2^(e - 1), or reaches it when M is odd (ties go to even).  That is
    // mx * 2^(1 - e) > mn * (2M + 1) in 64-bit integers.  ratio_exact is false when R
    // does not fit this form; the division is used then.
    bool ratio_exact;
    bool ratio_strict;
    uint32_t ratio_shift;
    uint64_t ratio_num;
};

// fl(mx / mn) > R, as the reference computes it in f32 (0 / 0 is NaN: false)
__device__ __forceinline__ bool ratio_above(uint32_t mx, uint32_t mn, const ChainCtx& c) {
    if (c.ratio_exact) {
        const uint64_t lhs = (uint64_t)mx << c.ratio_shift, rhs = (uint64_t)mn * c.ratio_num;
        return mx != 0 && (c.ratio_strict ? lhs > rhs : lhs >= rhs);
    }
    return __fdiv_rn(__uint2float_rn(mx), __uint2float_rn(mn)) > c.cp.max_diagonal_ratio;
}

// compute_score (src/chainer.rs:286-302)
__device__ __forceinline__ float chain_score(uint32_t dq, uint32_t dr, const ChainCtx& c) {
    uint32_t dd = dr > dq ? dr - dq : dq - dr;
    uint32_t dg = dq < dr ? dq : dr;
    float score = __uint2float_rn(c.k < dg ? c.k : dg);
    uint32_t dg2 = dg > c.k ? dg - c.k : 0;
    float lin = __fadd_rn(__fmul_rn(c.cp.diag_diff_penalty, __uint2float_rn(dd)),
                          __fmul_rn(c.cp.gap_length_penalty, __uint2float_rn(dg2)));
    float lg = dd >= 1 ? __ldg(c.lut + (dd < LOG2_LUT_SIZE ? dd : LOG2_LUT_SIZE - 1)) : 0.0f;
    return __fsub_rn(score, __fadd_rn(lin, __fmul_rn(0.5f, lg)));
}

// Stable LSD radix sort of anchor indices idx[0..m) by score (dp[idx]) descending, by
// one warp: four 8-bit passes over an order-preserving key, each a warp-ordered stable
// counting scatter (rank among equal digits of a 32-slice from __match_any_sync).
// idx and tmp are ping-pong buffers; the sorted order ends in tmp.
__device__ __forceinline__ uint32_t desc_key(float s) {
    const uint32_t b = __float_as_uint(s == 0.0f ? 0.0f : s);
    return ~((b & 0x80000000u) ? ~b : (b | 0x80000000u));  // ascending key = descending score
}

__device__ void warp_radix_sort_desc(uint32_t* idx, uint32_t* tmp, uint32_t m, const float* dp, uint32_t* hist) {
    const uint32_t lane = lane_id();
    uint32_t* src = idx;
    uint32_t* dst = tmp;
    for (int pass = 0; pass < 4; pass++) {
        const int sh = 8 * pass;
        for (uint32_t t = lane; t < 256; t += 32) hist[t] = 0;
        __syncwarp();
        for (uint32_t c = lane; c < m; c += 32) atomicAdd(&hist[(desc_key(dp[src[c]]) >> sh) & 255], 1u);
        __syncwarp();
        // exclusive scan of the 256 counters, 8 per lane
        uint32_t v[8], sum = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            v[k] = hist[lane * 8 + k];
            sum += v[k];
        }
        uint32_t incl = sum;
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, d);
            if (lane >= (uint32_t)d) incl += y;
        }
        uint32_t run = incl - sum;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            hist[lane * 8 + k] = run;
            run += v[k];
        }
        __syncwarp();
        for (uint32_t c0 = 0; c0 < m; c0 += 32) {
            const uint32_t c = c0 + lane;
            const bool in = c < m;
            const uint32_t x = in ? src[c] : 0;
            const uint32_t dg = in ? (desc_key(dp[x]) >> sh) & 255 : 256 + lane;
            const uint32_t peers = __match_any_sync(FULL, dg);
            const uint32_t base = in ? hist[dg] : 0;
            __syncwarp();
            if (in) {
                dst[base + __popc(peers & lanemask_lt())] = x;
                // the highest lane of each digit group advances the digit's offset
                if ((peers >> lane) == 1u) hist[dg] = base + __popc(peers);
            }
            __syncwarp();
        }
        uint32_t* t = src;
        src = dst;
        dst = t;
    }
    // four passes: the result is back in idx; copy it to tmp for the caller
    for (uint32_t c = lane; c < m; c += 32) tmp[c] = idx[c];
}

// extract_chains (src/chainer.rs:386-449) for one read orientation (segment sg, anchors
// b .. b + N of the deduplicated list) by the whole warp; best_score is the segment's
// best chain score.  hist: this warp's 256 shared counters.
__device__ void chain_extract(const uint64_t* dedup, const float* dp, const uint32_t* pred, uint32_t* aux,
                              uint64_t total_anchors, uint64_t b, uint32_t N, uint32_t sg, float best_score,
                              const AnchorPack& ap, const ChainCtx& cc, NamRec* nam_out, uint32_t* nam_seg_count,
                              uint64_t* anc_out, uint64_t* anc_start, uint32_t* hist) {
    const uint32_t lane = lane_id();
    const uint64_t qmask = (1ULL << ap.qbits) - 1, pmask = (1ULL << ap.pbits) - 1;
    const float valid_score = __fmul_rn(best_score, cc.cp.valid_score_threshold);
    uint32_t* cand = aux + b;
    uint32_t* sorted_c = aux + total_anchors + b;
    uint32_t* used = aux + 2 * total_anchors + b;
    uint32_t M = 0;
    for (uint32_t c = 0; c < N; c += 32) {
        uint32_t i = c + lane;
        bool take = i < N && dp[b + i] >= valid_score;
        uint32_t bal = __ballot_sync(FULL, take);
        if (take) cand[M + __popc(bal & lanemask_lt())] = i;
        if (i < N) used[i] = 0;
        M += __popc(bal);
    }
    __syncwarp();
    // candidates by score, descending, ties in anchor order (a stable sort)
    if (M <= 32) {
        const uint32_t ci = lane < M ? cand[lane] : 0;
        const float s = lane < M ? dp[b + ci] : 0.0f;
        uint32_t rank = 0;
        for (uint32_t u = 0; u < M; u++) {
            const float su = __shfl_sync(FULL, s, u);
            rank += (su > s) || (su == s && u < lane);
        }
        if (lane < M) sorted_c[rank] = ci;
    } else {
        warp_radix_sort_desc(cand, sorted_c, M, dp + b, hist);
    }
    __syncwarp();
    // the walk's used flags: a bit each in the warp's shared counters (free after the
    // sort) when they fit, else the global array
    const bool bits = N <= 32 * 256;
    if (bits)
        for (uint32_t w = lane; w < (N + 31) / 32; w += 32) hist[w] = 0;
    __syncwarp();
    auto is_used = [&](uint32_t j) -> bool { return bits ? (hist[j >> 5] >> (j & 31)) & 1 : used[j] != 0; };
    auto set_used = [&](uint32_t j) {
        if (bits) hist[j >> 5] |= 1u << (j & 31);
        else used[j] = 1;
    };
    if (lane == 0) {
        uint32_t nn = 0;
        NamRec* outp = nam_out + b;
        // a kept chain holds its end anchor (never marked used) and used
        // predecessors, so kept chains list each anchor at most twice; a dropped
        // chain's anchors are overwritten: 3 slots per anchor suffice
        uint64_t* ao = anc_out ? anc_out + 3 * b : nullptr;
        uint32_t acur = 0;
        for (uint32_t c = 0; c < M; c++) {
            uint32_t i = sorted_c[c];
            if (is_used(i)) continue;
            uint32_t j = i;
            bool overlaps = false;
            uint32_t nanch = 1;
            const uint64_t ki = dedup[b + i];
            if (ao) ao[acur] = ki;
            uint32_t matching = cc.k;
            uint32_t cov = (uint32_t)((ki >> ap.qbits) & pmask);
            while (pred[b + j] != 0xffffffffu) {
                j = pred[b + j];
                if (is_used(j)) { overlaps = true; break; }
                if (ao) ao[acur + nanch] = dedup[b + j];
                nanch++;
                set_used(j);
                uint32_t rsj = (uint32_t)((dedup[b + j] >> ap.qbits) & pmask);
                uint32_t d = cov > rsj ? cov - rsj : 0;
                matching += d < cc.k ? d : cc.k;
                cov = rsj;
            }
            if (overlaps) continue;
            const uint64_t kf2 = dedup[b + j];
            NamRec nr;
            nr.nam_id = nn;
            nr.query_start = (uint32_t)(kf2 & qmask);
            nr.query_end = (uint32_t)(ki & qmask) + cc.k;
            nr.ref_start = (uint32_t)((kf2 >> ap.qbits) & pmask);
            nr.ref_end = (uint32_t)((ki >> ap.qbits) & pmask) + cc.k;
            nr.matching_bases = matching;
            nr.ref_id = (uint32_t)(ki >> (ap.pbits + ap.qbits));
            nr.score = __fadd_rn(dp[b + i], __fmul_rn(__uint2float_rn(nanch), cc.cp.matches_weight));
            nr.is_revcomp = sg & 1;
            nr.n_anchors = nanch;
            if (anc_start) anc_start[b + nn] = 3 * b + acur;
            acur += nanch;
            outp[nn++] = nr;
        }
        nam_seg_count[sg] = nn;
    }
    __syncwarp();
}

// extract_chains (src/chainer.rs:386-449) for the eight orientations of a grouped warp at
// once: group g (lanes 4g .. 4g+3) collects its orientation's candidates, and its first
// lane orders them (insertion into the sorted list: a stable sort by score, descending)
// and walks the chains, so the eight walks' dependent loads overlap instead of running
// one orientation after another.  nmax bounds every group's anchor count; sg == ~0u
// marks a group without an orientation.
__device__ void group_chain_extract(const uint64_t* dedup, const float* dp, const uint32_t* pred, uint32_t* aux,
                                    uint64_t total_anchors, uint64_t b, uint32_t N, uint32_t nmax, uint32_t sg,
                                    float best_score, const AnchorPack& ap, const ChainCtx& cc, NamRec* nam_out,
                                    uint32_t* nam_seg_count, uint64_t* anc_out, uint64_t* anc_start) {
    const uint32_t lane = lane_id(), gl = lane % 4, gsh = lane - gl;
    const uint64_t qmask = (1ULL << ap.qbits) - 1, pmask = (1ULL << ap.pbits) - 1;
    const bool has = sg != 0xffffffffu && N > 0;
    const float valid_score = __fmul_rn(best_score, cc.cp.valid_score_threshold);
    uint32_t* cand = aux + b;
    uint32_t* sorted_c = aux + total_anchors + b;
    uint32_t M = 0;
    for (uint32_t c = 0; c < nmax; c += 4) {
        const uint32_t i = c + gl;
        const bool in = has && i < N;
        const bool take = in && dp[b + i] >= valid_score;
        const uint32_t bal = (__ballot_sync(FULL, take) >> gsh) & 15u;
        if (take) cand[M + __popc(bal & ((1u << gl) - 1))] = i;
        M += __popc(bal);
    }
    __syncwarp();
    // used flags of the group's anchors (at most CHAIN_GROUP_MAX = 96) in three words
    uint32_t u0 = 0, u1 = 0, u2 = 0;
    auto is_used = [&](uint32_t j) -> bool {
        const uint32_t w = j < 32 ? u0 : j < 64 ? u1 : u2;
        return (w >> (j & 31)) & 1;
    };
    auto set_used = [&](uint32_t j) {
        const uint32_t m = 1u << (j & 31);
        if (j < 32) u0 |= m;
        else if (j < 64) u1 |= m;
        else u2 |= m;
    };
    if (has && gl == 0) {
        // candidates arrive in anchor order; each goes after every entry scoring at least
        // as much, so equal scores keep anchor order
        for (uint32_t t = 0; t < M; t++) {
            const uint32_t ci = cand[t];
            const float sc = dp[b + ci];
            uint32_t pos = t;
            while (pos > 0 && dp[b + sorted_c[pos - 1]] < sc) {
                sorted_c[pos] = sorted_c[pos - 1];
                pos--;
            }
            sorted_c[pos] = ci;
        }
        uint32_t nn = 0;
        NamRec* outp = nam_out + b;
        uint64_t* ao = anc_out ? anc_out + 3 * b : nullptr;
        uint32_t acur = 0;
        for (uint32_t c = 0; c < M; c++) {
            const uint32_t i = sorted_c[c];
            if (is_used(i)) continue;
            uint32_t j = i;
            bool overlaps = false;
            uint32_t nanch = 1;
            const uint64_t ki = dedup[b + i];
            if (ao) ao[acur] = ki;
            uint32_t matching = cc.k;
            uint32_t cov = (uint32_t)((ki >> ap.qbits) & pmask);
            while (pred[b + j] != 0xffffffffu) {
                j = pred[b + j];
                if (is_used(j)) {
                    overlaps = true;
                    break;
                }
                const uint64_t kj = dedup[b + j];
                if (ao) ao[acur + nanch] = kj;
                nanch++;
                set_used(j);
                const uint32_t rsj = (uint32_t)((kj >> ap.qbits) & pmask);
                const uint32_t d = cov > rsj ? cov - rsj : 0;
                matching += d < cc.k ? d : cc.k;
                cov = rsj;
            }
            if (overlaps) continue;
            const uint64_t kf2 = dedup[b + j];
            NamRec nr;
            nr.nam_id = nn;
            nr.query_start = (uint32_t)(kf2 & qmask);
            nr.query_end = (uint32_t)(ki & qmask) + cc.k;
            nr.ref_start = (uint32_t)((kf2 >> ap.qbits) & pmask);
            nr.ref_end = (uint32_t)((ki >> ap.qbits) & pmask) + cc.k;
            nr.matching_bases = matching;
            nr.ref_id = (uint32_t)(ki >> (ap.pbits + ap.qbits));
            nr.score = __fadd_rn(dp[b + i], __fmul_rn(__uint2float_rn(nanch), cc.cp.matches_weight));
            nr.is_revcomp = sg & 1;
            nr.n_anchors = nanch;
            if (anc_start) anc_start[b + nn] = 3 * b + acur;
            acur += nanch;
            outp[nn++] = nr;
        }
        nam_seg_count[sg] = nn;
    }
    if (sg != 0xffffffffu && N == 0 && gl == 0) nam_seg_count[sg] = 0;
    __syncwarp();
}

// The read orientations that have anchors (only the better orientation of a read gets
// anchors, src/chainer.rs:205-216, so about half are empty), for k_chain4: those with
// at most CHAIN_GROUP_MAX anchors in `list`, taken eight per warp, the others in
// `long_list`, one per warp; key / long_key receive their anchor counts (the lists
// are then ordered by them).  The ranges of those with
// more than CHAIN_SORT_SMALL anchors go to sort_begin / sort_end for a segmented sort;
// k_chain4 sorts the others itself.  n_list: [0] listed, [1] sort ranges, [2] long.
constexpr uint32_t CHAIN_SORT_SMALL = 256;
constexpr uint32_t CHAIN_GROUP_MAX = 96;

__global__ void k_seg_list(const uint64_t* seg_count, const uint64_t* seg_off, uint32_t nseg, uint32_t* list,
                           uint32_t* long_list, uint32_t* n_list, uint64_t* sort_begin, uint64_t* sort_end,
                           uint32_t* key, uint32_t* long_key) {
    const uint32_t lane = lane_id();
    const uint32_t step = gridDim.x * blockDim.x;
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < nseg; base += step) {
        const uint32_t sg = base + lane;
        const uint64_t cnt = sg < nseg ? seg_count[sg] : 0;
        const bool lng = cnt > CHAIN_GROUP_MAX, shrt = cnt > 0 && !lng, big = cnt > CHAIN_SORT_SMALL;
        const uint32_t bs = __ballot_sync(FULL, shrt), bl = __ballot_sync(FULL, lng), bb = __ballot_sync(FULL, big);
        uint32_t as = 0, al = 0, ab = 0;
        if (lane == 0 && bs) as = atomicAdd(n_list, (uint32_t)__popc(bs));
        if (lane == 0 && bb) ab = atomicAdd(n_list + 1, (uint32_t)__popc(bb));
        if (lane == 0 && bl) al = atomicAdd(n_list + 2, (uint32_t)__popc(bl));
        as = __shfl_sync(FULL, as, 0);
        ab = __shfl_sync(FULL, ab, 0);
        al = __shfl_sync(FULL, al, 0);
        if (shrt) {
            list[as + __popc(bs & lanemask_lt())] = sg;
            key[as + __popc(bs & lanemask_lt())] = (uint32_t)cnt;
        }
        if (lng) {
            long_list[al + __popc(bl & lanemask_lt())] = sg;
            long_key[al + __popc(bl & lanemask_lt())] = cnt < 0xffffffffull ? (uint32_t)cnt : 0xffffffffu;
        }
        if (big) {
            const uint32_t k = ab + __popc(bb & lanemask_lt());
            const uint64_t o = seg_off[sg];
            sort_begin[k] = o;
            sort_end[k] = o + cnt;
        }
    }
}

// Ascending bitonic sort of R * 32 keys held R per lane (element r * 32 + lane in v[r]).
template <int R>
__device__ __forceinline__ void warp_bitonic_sort(uint64_t (&v)[R]) {
    const uint32_t lane = lane_id();
#pragma unroll
    for (uint32_t k = 2; k <= 32 * R; k <<= 1) {
#pragma unroll
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
                // partners in two registers of one lane; the direction depends on r only
                const int jr = (int)(j >> 5);
#pragma unroll
                for (int r = 0; r < R; r++) {
                    if (r & jr) continue;
                    const int r2 = r | jr;
                    const bool asc = ((32u * r) & k) == 0;
                    const uint64_t lo = v[r] < v[r2] ? v[r] : v[r2], hi = v[r] < v[r2] ? v[r2] : v[r];
                    v[r] = asc ? lo : hi;
                    v[r2] = asc ? hi : lo;
                }
            } else {
                const bool lower = (lane & j) == 0;
#pragma unroll
                for (int r = 0; r < R; r++) {
                    const uint64_t p = __shfl_xor_sync(FULL, v[r], j);
                    const bool asc = ((32 * r + lane) & k) == 0;
                    const bool take_min = lower == asc;
                    v[r] = take_min ? (p < v[r] ? p : v[r]) : (p > v[r] ? p : v[r]);
                }
            }
        }
    }
}

// Sort the cnt <= 32 * R keys at keys[0..cnt) (one read orientation's anchors, in the
// order k_anchors wrote them) and write the distinct ones back in order; returns their
// number (src/chainer.rs:228-229).
template <int R>
__device__ __forceinline__ uint32_t warp_sort_dedup(uint64_t* keys, uint32_t cnt) {
    const uint32_t lane = lane_id();
    uint64_t v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = 32 * r + lane < cnt ? keys[32 * r + lane] : ~0ULL;
    warp_bitonic_sort<R>(v);
    uint32_t bal[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        uint64_t prev = __shfl_up_sync(FULL, v[r], 1);
        if (r > 0) {
            const uint64_t last = __shfl_sync(FULL, v[r > 0 ? r - 1 : 0], 31);
            if (lane == 0) prev = last;
        }
        const uint32_t e = 32 * r + lane;
        bal[r] = __ballot_sync(FULL, e < cnt && (e == 0 || prev != v[r]));
    }
    __syncwarp();
    uint32_t n = 0;
#pragma unroll
    for (int r = 0; r < R; r++) {
        if ((bal[r] >> lane) & 1u) keys[n + __popc(bal[r] & lanemask_lt())] = v[r];
        n += __popc(bal[r]);
    }
    return n;
}

// Chaining (src/chainer.rs:128-176 and 386-449) for NG = 8 read orientations per warp.
// The anchor sort, the deduplication and the extraction run over the whole warp, one
// orientation after the other.  The DP is serial over a read orientation's anchors;
// the candidates j of anchor i (back to max_lookback) are scored in parallel and an
// exclusive prefix max over them reproduces the reference's downward scan with its
// ">=" updates and its stops (a different reference or a gap >= max_ref_gap ends the
// scan; an update on the same diagonal ends it after that candidate).  The DP runs for
// the NG orientations at once, one group of CG = 4 lanes each, four candidates at a
// time (most anchors stop at the first candidate: the one before on the same
// diagonal).  Orientations with more than CHAIN_GROUP_MAX anchors get a warp each and
// run the DP with all 32 lanes, 32 candidates at a time.  The orientations come from
// k_seg_list (those with anchors); nam_seg_count of the others is zeroed before the
// launch.
//
// RING: max_lookback < 64, so the predecessors of anchor i (and their scores) come
// from a 64-entry ring in shared memory per orientation, written as anchors are
// scored, instead of global memory (this takes the store-to-load round trip out of
// each serial step).
constexpr uint32_t CG = 4;                   // lanes per orientation in the grouped DP
constexpr uint32_t NG = 32 / CG;             // orientations per warp
constexpr uint32_t GMASK = (1u << CG) - 1;  // one group's ballot bits
constexpr uint32_t CHAIN_WARPS = 4;          // warps per block (shared rings: 28 KB per block)

template <bool RING>
__device__ __forceinline__ void chain_candidates(uint32_t j, bool in, const uint64_t* dedup, const float* dp,
                                                 uint64_t b, const uint64_t* ring_key, const float* ring_dp,
                                                 uint32_t ri, uint32_t rsi, uint32_t qi, uint32_t max_ref_gap,
                                                 const ChainCtx& cc, const AnchorPack& ap, bool& hard, bool& valid,
                                                 bool& diag, float& val) {
    const uint64_t qmask = (1ULL << ap.qbits) - 1, pmask = (1ULL << ap.pbits) - 1;
    hard = valid = diag = false;
    val = 0.0f;
    if (!in) return;
    const uint64_t kj = RING ? ring_key[j & 63] : dedup[b + j];
    const uint32_t rj = (uint32_t)(kj >> (ap.pbits + ap.qbits)), rsj = (uint32_t)((kj >> ap.qbits) & pmask),
                   qj = (uint32_t)(kj & qmask);
    if (rj != ri) {
        hard = true;
    } else if (qi >= qj) {
        const uint32_t dq = qi - qj, dr = rsi - rsj;
        if (dr >= max_ref_gap) {
            hard = true;
        } else {
            const uint32_t mx = dq > dr ? dq : dr, mn = dq < dr ? dq : dr;
            if (!ratio_above(mx, mn, cc)) {
                valid = true;
                diag = dq == dr;
                val = __fadd_rn(RING ? ring_dp[j & 63] : dp[b + j], chain_score(dq, dr, cc));
            }
        }
    }
}

// The lookback DP of collinear_chaining (src/chainer.rs:85-180) over anchors [c0, c1)
// of one read orientation (its anchors at dedup[b ..]) by the whole warp: 32
// predecessors per step, the early-break rules as a prefix max over the lanes.
// Predecessors never go below c0 (earlier anchors lie max_ref_gap or more behind, or
// on another reference, and end the reference's scan without contributing).  With
// recheck, (best_score, best_index, best_key) is the running best over all anchors
// before c0 and is updated as the reference updates it (strict >); without, the
// best-index re-check (:150-165) is left out.
template <bool RING>
__device__ void warp_chain_range(const uint64_t* dedup, float* dp, uint32_t* pred, uint64_t b, uint32_t c0, uint32_t c1,
                                 uint32_t floor, uint32_t max_ref_gap, const ChainCtx& cc, const AnchorPack& ap,
                                 uint64_t* ring_key, float* ring_dp, bool recheck, float& best_score,
                                 uint32_t& best_index, uint64_t& best_key) {
    const uint32_t lane = lane_id();
    const uint64_t qmask = (1ULL << ap.qbits) - 1, pmask = (1ULL << ap.pbits) - 1;
    const float kf = __uint2float_rn(cc.k);
    if (RING && c0 > floor) {
        // resuming inside a cluster: the ring takes the anchors before c0 from memory
        for (uint32_t j = (c0 - floor > 64 ? c0 - 64 : floor) + lane; j < c0; j += 32) {
            ring_key[j & 63] = dedup[b + j];
            ring_dp[j & 63] = dp[b + j];
        }
        __syncwarp();
    }
    uint64_t next_key = c0 < c1 ? dedup[b + c0] : 0;
    for (uint32_t i = c0; i < c1; i++) {
        const uint64_t ki = next_key;
        if (i + 1 < c1) next_key = dedup[b + i + 1];
        const uint32_t ri = (uint32_t)(ki >> (ap.pbits + ap.qbits)), rsi = (uint32_t)((ki >> ap.qbits) & pmask),
                       qi = (uint32_t)(ki & qmask);
        uint32_t lookup_end = i > cc.cp.max_lookback ? i - cc.cp.max_lookback : 0;
        if (lookup_end < floor) lookup_end = floor;
        float cur = kf;
        uint32_t cur_pred = 0xffffffffu;
        bool stop = false;
        for (uint32_t base = 0; !stop && base < i - lookup_end; base += 32) {
            const uint32_t t = base + lane;
            const bool in = t < i - lookup_end;
            const uint32_t j = i - 1 - t;
            bool hard, valid, diag;
            float val;
            chain_candidates<RING>(j, in, dedup, dp, b, ring_key, ring_dp, ri, rsi, qi, max_ref_gap, cc, ap, hard,
                                   valid, diag, val);
            // the common case: the first candidate updates and lies on the same diagonal,
            // which ends the scan (the prefix max below would find the same)
            if (__ballot_sync(FULL, lane == 0 && valid && diag && val >= cur)) {
                cur = __shfl_sync(FULL, val, 0);
                cur_pred = i - 1 - base;
                break;
            }
            const uint32_t hb = __ballot_sync(FULL, hard);
            const uint32_t lim = hb ? (uint32_t)(__ffs(hb) - 1) : 32;
            if (lane >= lim) valid = false;
            float incl = valid ? val : -INFINITY;
            for (int d = 1; d < 32; d <<= 1) {
                const float y = __shfl_up_sync(FULL, incl, d);
                if (lane >= (uint32_t)d) incl = fmaxf(incl, y);
            }
            float excl = __shfl_up_sync(FULL, incl, 1);
            if (lane == 0) excl = -INFINITY;
            const bool upd = valid && val >= fmaxf(cur, excl);
            const uint32_t ub = __ballot_sync(FULL, upd);
            const uint32_t sb = __ballot_sync(FULL, upd && diag);
            uint32_t reach = lim;
            if (sb) {
                reach = (uint32_t)__ffs(sb);
                stop = true;
            }
            if (hb) stop = true;
            const uint32_t um = ub & (reach >= 32 ? FULL : ((1u << reach) - 1));
            if (um) {
                const uint32_t last = 31 - __clz(um);
                cur = __shfl_sync(FULL, val, last);
                cur_pred = i - 1 - (base + last);
            }
        }
        if (recheck && best_index != 0xffffffffu) {
            const uint64_t kb = best_key;
            const uint32_t rb = (uint32_t)(kb >> (ap.pbits + ap.qbits)), rsb = (uint32_t)((kb >> ap.qbits) & pmask),
                           qb = (uint32_t)(kb & qmask);
            if (rb == ri && qi > qb) {
                const uint32_t dq = qi - qb, dr = rsi - rsb;
                const uint32_t mx = dq > dr ? dq : dr, mn = dq < dr ? dq : dr;
                if (dr < max_ref_gap && dr > 0 && !ratio_above(mx, mn, cc)) {
                    const float ns = __fadd_rn(best_score, chain_score(dq, dr, cc));
                    if (ns > cur) {
                        cur = ns;
                        cur_pred = best_index;
                    }
                }
            }
        }
        if (lane == 0) {
            dp[b + i] = cur;
            pred[b + i] = cur_pred;
            if (RING) {
                ring_key[i & 63] = ki;
                ring_dp[i & 63] = cur;
            }
        }
        if (recheck && cur > best_score) {
            best_score = cur;
            best_index = i;
            best_key = ki;
        }
        if (!recheck && cur > best_score) best_score = cur;  // the range's maximum
        __syncwarp();
    }
}

// The first anchor of [lo, hi) (one cluster) where the best-index re-check
// (src/chainer.rs:150-165) would change the DP values dp holds from scoring the cluster
// without it; hi when there is none.  Up to that anchor both scorings agree, so the
// running best (best_score / best_index / best_key, strict > updates as the reference
// makes them) is a prefix maximum, taken 32 anchors at a time by a shuffle scan; the
// re-check's test runs on every anchor at once.  On return the running best is the one
// before the returned anchor.
__device__ uint32_t recheck_first_fire(const uint64_t* dedup, const float* dp, uint64_t b, uint32_t lo, uint32_t hi,
                                       uint32_t max_ref_gap, const ChainCtx& cc, const AnchorPack& ap,
                                       float& best_score, uint32_t& best_index, uint64_t& best_key) {
    const uint32_t lane = lane_id();
    const uint64_t qmask = (1ULL << ap.qbits) - 1, pmask = (1ULL << ap.pbits) - 1;
    for (uint32_t c = lo; c < hi; c += 32) {
        const uint32_t i = c + lane;
        const bool in = i < hi;
        const float d = in ? dp[b + i] : -INFINITY;
        const uint64_t k = in ? dedup[b + i] : 0;
        // inclusive prefix (maximum, first index reaching it) over the lanes
        float pv = d;
        uint32_t pi = i;
        for (uint32_t s = 1; s < 32; s <<= 1) {
            const float v2 = __shfl_up_sync(FULL, pv, s);
            const uint32_t i2 = __shfl_up_sync(FULL, pi, s);
            if (lane >= s && v2 >= pv) {
                pv = v2;
                pi = i2;
            }
        }
        // the running best before anchor i: the carry, then lanes < lane
        float ev = __shfl_up_sync(FULL, pv, 1);
        uint32_t ei = __shfl_up_sync(FULL, pi, 1);
        if (lane == 0) ev = -INFINITY;
        float bs = best_score;
        uint32_t bi = best_index;
        bool from_chunk = false;
        if (ev > bs) {
            bs = ev;
            bi = ei;
            from_chunk = true;
        }
        const uint64_t kc = __shfl_sync(FULL, k, from_chunk ? ei - c : 0);
        const uint64_t bk = from_chunk ? kc : best_key;
        bool fire = false;
        if (in && bi != 0xffffffffu) {
            const uint32_t ri = (uint32_t)(k >> (ap.pbits + ap.qbits)), rsi = (uint32_t)((k >> ap.qbits) & pmask),
                           qi = (uint32_t)(k & qmask);
            const uint32_t rb = (uint32_t)(bk >> (ap.pbits + ap.qbits)), rsb = (uint32_t)((bk >> ap.qbits) & pmask),
                           qb = (uint32_t)(bk & qmask);
            if (rb == ri && qi > qb) {
                const uint32_t dq = qi - qb, dr = rsi - rsb;
                const uint32_t mx = dq > dr ? dq : dr, mn = dq < dr ? dq : dr;
                if (dr < max_ref_gap && dr > 0 && !ratio_above(mx, mn, cc))
                    fire = __fadd_rn(bs, chain_score(dq, dr, cc)) > d;
            }
        }
        const uint32_t fb = __ballot_sync(FULL, fire);
        if (fb) {
            const int f = __ffs(fb) - 1;
            best_score = __shfl_sync(FULL, bs, f);
            best_index = __shfl_sync(FULL, bi, f);
            best_key = __shfl_sync(FULL, bk, f);
            return c + (uint32_t)f;
        }
        // the whole chunk: carry its maximum on
        const float v31 = __shfl_sync(FULL, pv, 31);
        const uint32_t i31 = __shfl_sync(FULL, pi, 31);
        const uint64_t k31 = __shfl_sync(FULL, k, (i31 - c) & 31);
        if (v31 > best_score) {
            best_score = v31;
            best_index = i31;
            best_key = k31;
        }
    }
    return hi;
}

// The same for a small cluster [c0, c1) by one thread, without the re-check; returns
// the cluster's maximum.
__device__ float lane_chain_range(const uint64_t* dedup, float* dp, uint32_t* pred, uint64_t b, uint32_t c0,
                                  uint32_t c1, uint32_t max_ref_gap, const ChainCtx& cc, const AnchorPack& ap) {
    const uint64_t qmask = (1ULL << ap.qbits) - 1, pmask = (1ULL << ap.pbits) - 1;
    const float kf = __uint2float_rn(cc.k);
    float mx = 0.0f;
    for (uint32_t i = c0; i < c1; i++) {
        const uint64_t ki = dedup[b + i];
        const uint32_t rsi = (uint32_t)((ki >> ap.qbits) & pmask), qi = (uint32_t)(ki & qmask);
        uint32_t lookup_end = i > cc.cp.max_lookback ? i - cc.cp.max_lookback : 0;
        if (lookup_end < c0) lookup_end = c0;
        float cur = kf;
        uint32_t cur_pred = 0xffffffffu;
        for (uint32_t j = i; j-- > lookup_end;) {
            // one reference within a cluster: the reference's ref_id break cannot fire
            const uint64_t kj = dedup[b + j];
            const uint32_t rsj = (uint32_t)((kj >> ap.qbits) & pmask), qj = (uint32_t)(kj & qmask);
            if (qi < qj) continue;
            const uint32_t dq = qi - qj, dr = rsi - rsj;
            if (dr >= max_ref_gap) break;
            const uint32_t a = dq > dr ? dq : dr, m = dq < dr ? dq : dr;
            if (ratio_above(a, m, cc)) continue;
            const float ns = __fadd_rn(dp[b + j], chain_score(dq, dr, cc));
            if (ns >= cur) {
                cur = ns;
                cur_pred = j;
                if (dq == dr) break;
            }
        }
        dp[b + i] = cur;
        pred[b + i] = cur_pred;
        if (cur > mx) mx = cur;
    }
    return mx;
}


// Sort (orientations up to CHAIN_SORT_SMALL anchors, whose keys are still unsorted in
// the dedup buffer) or take the segmented sort's output, and deduplicate
// (src/chainer.rs:228-229) the anchors [b, e) of one read orientation into
// dedup[b ..]; returns the count.  The whole warp.
__device__ __forceinline__ uint32_t orientation_dedup(const uint64_t* sorted, uint64_t* dedup, uint64_t b, uint64_t e) {
    const uint32_t lane = lane_id();
    const uint32_t cnt = (uint32_t)(e - b);
    if (cnt <= CHAIN_SORT_SMALL) {
        if (cnt <= 32) return warp_sort_dedup<1>(dedup + b, cnt);
        if (cnt <= 64) return warp_sort_dedup<2>(dedup + b, cnt);
        if (cnt <= 128) return warp_sort_dedup<4>(dedup + b, cnt);
        return warp_sort_dedup<8>(dedup + b, cnt);
    }
    uint32_t N = 0;
    for (uint64_t c = b; c < e; c += 32) {
        const uint64_t i = c + lane;
        bool keep = false;
        uint64_t key = 0;
        if (i < e) {
            key = sorted[i];
            keep = i == b || sorted[i - 1] != key;
        }
        const uint32_t bal = __ballot_sync(FULL, keep);
        if (keep) dedup[b + N + __popc(bal & lanemask_lt())] = key;
        N += __popc(bal);
    }
    return N;
}

// Long read orientations (more than CHAIN_GROUP_MAX anchors), before k_chain4.  Anchors
// sorted by (reference, position) fall into clusters: a new one starts where the
// reference changes or the position jumps by max_ref_gap or more.  A predecessor scan
// never crosses into an earlier cluster (the reference's scan breaks there or skips
// without contributing), so a cluster's DP depends on the others only through the
// best-index re-check (src/chainer.rs:150-165), which can fire only once the cluster
// holds the running best, a strict maximum over all earlier anchors.  So the clusters
// are scored at once without the re-check, here, and k_chain4 then takes, in order, each
// cluster whose maximum beats the running best of the clusters before it, finds the
// first anchor where the re-check fires and scores again from there (carrying the
// running best on); the others are final.
//
// k_chain_long_prep: a warp per long orientation u: the dedup, the cluster starts
// (aux[b ..]), and the clusters of up to lane_max anchors scored a thread each (maxima
// at aux[T + b ..] as floats); the larger ones are queued as (u, cluster) items for
// k_chain_big, a warp each.  long_n[u] / long_c[u]: anchors after dedup, clusters.
// k_chain4 then checks each record cluster for the first anchor where the re-check
// fires (recheck_first_fire) and scores again from there only.
__global__ void __launch_bounds__(128) k_chain_long_prep(const uint64_t* __restrict__ off, const uint64_t* seg_off,
                                                         const uint64_t* sorted, uint64_t* dedup, float* dp,
                                                         uint32_t* pred, uint32_t* aux, uint64_t total_anchors,
                                                         AnchorPack ap, ChainCtx cc, const uint32_t* long_list,
                                                         uint32_t n_long, uint32_t* long_n, uint32_t* long_c,
                                                         uint32_t* big_items, uint32_t* n_big, uint32_t lane_max) {
    const uint32_t lane = lane_id();
    const uint64_t pmask = (1ULL << ap.pbits) - 1;
    const uint32_t nwarps = gridDim.x * (blockDim.x / 32);
    for (uint32_t u = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; u < n_long; u += nwarps) {
        const uint32_t sg = long_list[u];
        const uint64_t b = seg_off[sg], e = seg_off[sg + 1];
        const uint32_t N = orientation_dedup(sorted, dedup, b, e);
        __syncwarp();
        const uint32_t read_len = (uint32_t)(off[(sg >> 1) + 1] - off[sg >> 1]);
        const uint32_t max_ref_gap = cc.cp.max_ref_gap ? cc.cp.max_ref_gap : read_len;
        uint32_t* cstart = aux + b;
        float* cmax = reinterpret_cast<float*>(aux + total_anchors + b);
        uint32_t C = 0;
        for (uint32_t c = 0; c < N; c += 32) {
            const uint32_t i = c + lane;
            bool st = false;
            if (i < N) {
                if (i == 0) {
                    st = true;
                } else {
                    const uint64_t ki = dedup[b + i], kp = dedup[b + i - 1];
                    st = (ki >> (ap.pbits + ap.qbits)) != (kp >> (ap.pbits + ap.qbits)) ||
                         (uint32_t)((ki >> ap.qbits) & pmask) - (uint32_t)((kp >> ap.qbits) & pmask) >= max_ref_gap;
                }
            }
            const uint32_t bal = __ballot_sync(FULL, st);
            if (st) cstart[C + __popc(bal & lanemask_lt())] = i;
            C += __popc(bal);
        }
        __syncwarp();
        for (uint32_t c0 = 0; c0 < C; c0 += 32) {
            const uint32_t c = c0 + lane;
            bool big = false;
            if (c < C) {
                const uint32_t lo = cstart[c], hi = c + 1 < C ? cstart[c + 1] : N;
                big = hi - lo > lane_max;
                if (!big) cmax[c] = lane_chain_range(dedup, dp, pred, b, lo, hi, max_ref_gap, cc, ap);
            }
            const uint32_t bal = __ballot_sync(FULL, big);
            uint32_t at = 0;
            if (lane == 0 && bal) at = atomicAdd(n_big, (uint32_t)__popc(bal));
            at = __shfl_sync(FULL, at, 0);
            if (big) {
                const uint32_t x = at + __popc(bal & lanemask_lt());
                big_items[2 * x] = u;
                big_items[2 * x + 1] = c;
            }
        }
        if (lane == 0) {
            long_n[u] = N;
            long_c[u] = C;
        }
        __syncwarp();
    }
}

// The queued large clusters, a warp each, without the re-check (their maxima into
// aux[T + b + cluster]).
template <bool RING>
__global__ void __launch_bounds__(128) k_chain_big(const uint64_t* __restrict__ off, const uint64_t* seg_off,
                                                   const uint64_t* dedup, float* dp, uint32_t* pred, uint32_t* aux,
                                                   uint64_t total_anchors, AnchorPack ap, ChainCtx cc,
                                                   const uint32_t* long_list, const uint32_t* long_n,
                                                   const uint32_t* long_c, const uint32_t* big_items,
                                                   const uint32_t* n_big) {
    __shared__ uint64_t ring_key_s[RING ? 4 * 64 : 1];
    __shared__ float ring_dp_s[RING ? 4 * 64 : 1];
    const uint32_t lane = lane_id(), wib = threadIdx.x / 32;
    const uint32_t nwarps = gridDim.x * (blockDim.x / 32);
    const uint32_t nb = *n_big;
    for (uint32_t x = blockIdx.x * (blockDim.x / 32) + wib; x < nb; x += nwarps) {
        const uint32_t u = big_items[2 * x], c = big_items[2 * x + 1];
        const uint32_t sg = long_list[u], N = long_n[u], C = long_c[u];
        const uint64_t b = seg_off[sg];
        const uint32_t* cstart = aux + b;
        const uint32_t lo = cstart[c], hi = c + 1 < C ? cstart[c + 1] : N;
        const uint32_t read_len = (uint32_t)(off[(sg >> 1) + 1] - off[sg >> 1]);
        const uint32_t max_ref_gap = cc.cp.max_ref_gap ? cc.cp.max_ref_gap : read_len;
        float mx = 0.0f;
        uint32_t bi = 0xffffffffu;
        uint64_t bk = 0;
        warp_chain_range<RING>(dedup, dp, pred, b, lo, hi, lo, max_ref_gap, cc, ap,
                               ring_key_s + (RING ? wib * 64 : 0), ring_dp_s + (RING ? wib * 64 : 0), false, mx, bi,
                               bk);
        if (lane == 0) reinterpret_cast<float*>(aux + total_anchors + b)[c] = mx;
        __syncwarp();
    }
}

template <bool RING>
__global__ void __launch_bounds__(32 * CHAIN_WARPS, 8) k_chain4(const uint64_t* __restrict__ off, uint32_t n, const uint64_t* seg_off,
                                                const uint64_t* sorted, uint64_t* dedup, float* dp, uint32_t* pred,
                                                uint32_t* aux, uint64_t total_anchors, AnchorPack ap, ChainCtx cc,
                                                NamRec* nam_out, uint32_t* nam_seg_count, uint64_t* anc_out,
                                                uint64_t* anc_start, const uint32_t* seg_list, uint32_t n_list,
                                                const uint32_t* long_list, uint32_t n_long, const uint32_t* long_n,
                                                const uint32_t* long_c) {
    __shared__ uint32_t hist[CHAIN_WARPS * 256];
    __shared__ uint64_t ring_key_s[RING ? CHAIN_WARPS * NG * 64 : 1];
    __shared__ float ring_dp_s[RING ? CHAIN_WARPS * NG * 64 : 1];
    const uint32_t lane = lane_id(), g = lane / CG, gl = lane % CG, gsh = CG * g;
    const uint32_t wib = threadIdx.x / 32;
    const uint32_t nwarps = gridDim.x * (blockDim.x / 32);
    const uint64_t qmask = (1ULL << ap.qbits) - 1, pmask = (1ULL << ap.pbits) - 1;
    const float kf = __uint2float_rn(cc.k);
    constexpr uint32_t NONE = 0xffffffffu;
    // units: the long orientations first (one per warp, so they start first), then the
    // short ones NG at a time.  Lane q holds the q-th orientation's segment, anchor count
    // after dedup, first anchor and best score.
    const uint32_t n_units = n_long + (n_list + NG - 1) / NG;
    for (uint32_t u = blockIdx.x * (blockDim.x / 32) + wib; u < n_units; u += nwarps) {
        uint32_t my_sg = NONE;
        if (u < n_long) {
            if (lane == 0) my_sg = long_list[u];
        } else {
            const uint32_t l = NG * (u - n_long) + lane;
            if (lane < NG && l < n_list) my_sg = seg_list[l];
        }
        // dedup (src/chainer.rs:228-229), one orientation after the other; the long
        // orientations were deduplicated by k_chain_long_prep
        uint32_t my_n = 0;
        uint64_t my_b = 0;
        for (uint32_t q = 0; q < NG; q++) {
            const uint32_t sg = __shfl_sync(FULL, my_sg, q);
            if (sg == NONE) continue;
            const uint64_t b = seg_off[sg], e = seg_off[sg + 1];
            const uint32_t N = u < n_long ? long_n[u] : orientation_dedup(sorted, dedup, b, e);
            if (lane == q) {
                my_n = N;
                my_b = b;
            }
        }
        __syncwarp();
        const uint32_t nmax = __reduce_max_sync(FULL, my_n);
        float my_best = 0.0f;
        if (u >= n_long && nmax <= CHAIN_GROUP_MAX) {
            // grouped DP: group g scores the g-th orientation
            const uint32_t sg = __shfl_sync(FULL, my_sg, g);
            const uint32_t N = __shfl_sync(FULL, my_n, g);
            const uint64_t b = __shfl_sync(FULL, my_b, g);
            uint64_t* ring_key = ring_key_s + (RING ? (wib * NG + g) * 64 : 0);
            float* ring_dp = ring_dp_s + (RING ? (wib * NG + g) * 64 : 0);
            const uint32_t read_len = sg != NONE ? (uint32_t)(off[(sg >> 1) + 1] - off[sg >> 1]) : 0;
            const uint32_t max_ref_gap = cc.cp.max_ref_gap ? cc.cp.max_ref_gap : read_len;
            float best_score = 0.0f;
            uint32_t best_index = 0xffffffffu;
            uint64_t best_key = 0;
            uint64_t next_key = N ? dedup[b] : 0;
            for (uint32_t i = 0; i < nmax; i++) {
                const bool act = i < N;
                const uint64_t ki = next_key;
                if (act && i + 1 < N) next_key = dedup[b + i + 1];
                const uint32_t ri = (uint32_t)(ki >> (ap.pbits + ap.qbits)), rsi = (uint32_t)((ki >> ap.qbits) & pmask),
                               qi = (uint32_t)(ki & qmask);
                const uint32_t lookup_end = i > cc.cp.max_lookback ? i - cc.cp.max_lookback : 0;
                const uint32_t span = act ? i - lookup_end : 0;  // candidates j = i-1 .. lookup_end
                float cur = kf;
                uint32_t cur_pred = 0xffffffffu;
                bool more = span > 0;
                for (uint32_t base = 0; __any_sync(FULL, more); base += CG) {
                    const uint32_t t = base + gl;
                    const bool in = more && t < span;
                    const uint32_t j = i - 1 - t;
                    bool hard, valid, diag;
                    float val;
                    chain_candidates<RING>(j, in, dedup, dp, b, ring_key, ring_dp, ri, rsi, qi, max_ref_gap, cc, ap,
                                           hard, valid, diag, val);
                    const uint32_t hb = (__ballot_sync(FULL, hard) >> gsh) & GMASK;
                    const uint32_t lim = hb ? (uint32_t)(__ffs(hb) - 1) : CG;  // lanes >= lim are not reached
                    if (gl >= lim) valid = false;
                    // exclusive prefix max of val over valid lanes in scan order
                    float incl = valid ? val : -INFINITY;
                    for (uint32_t d = 1; d < CG; d <<= 1) {
                        const float y = __shfl_up_sync(FULL, incl, d, CG);
                        if (gl >= d) incl = fmaxf(incl, y);
                    }
                    float excl = __shfl_up_sync(FULL, incl, 1, CG);
                    if (gl == 0) excl = -INFINITY;
                    const bool upd = valid && val >= fmaxf(cur, excl);
                    const uint32_t ub = (__ballot_sync(FULL, upd) >> gsh) & GMASK;
                    const uint32_t sb = (__ballot_sync(FULL, upd && diag) >> gsh) & GMASK;
                    uint32_t reach = lim;
                    bool stop = hb != 0;
                    if (sb) {
                        reach = (uint32_t)__ffs(sb);
                        stop = true;
                    }
                    const uint32_t um = ub & (reach >= CG ? GMASK : ((1u << reach) - 1));
                    const uint32_t last = um ? 31 - __clz(um) : 0;
                    const float lv = __shfl_sync(FULL, val, last, CG);
                    if (more && um) {
                        cur = lv;
                        cur_pred = i - 1 - (base + last);
                    }
                    if (stop || base + CG >= span) more = false;
                }
                // re-check of the best chain end (src/chainer.rs:150-165)
                if (act && best_index != 0xffffffffu) {
                    const uint64_t kb = best_key;
                    const uint32_t rb = (uint32_t)(kb >> (ap.pbits + ap.qbits)),
                                   rsb = (uint32_t)((kb >> ap.qbits) & pmask), qb = (uint32_t)(kb & qmask);
                    if (rb == ri && qi > qb) {
                        const uint32_t dq = qi - qb, dr = rsi - rsb;
                        const uint32_t mx = dq > dr ? dq : dr, mn = dq < dr ? dq : dr;
                        if (dr < max_ref_gap && dr > 0 && !ratio_above(mx, mn, cc)) {
                            const float ns = __fadd_rn(best_score, chain_score(dq, dr, cc));
                            if (ns > cur) {
                                cur = ns;
                                cur_pred = best_index;
                            }
                        }
                    }
                }
                if (act && gl == 0) {
                    dp[b + i] = cur;
                    pred[b + i] = cur_pred;
                    if (RING) {
                        ring_key[i & 63] = ki;
                        ring_dp[i & 63] = cur;
                    }
                }
                if (act && cur > best_score) {
                    best_score = cur;
                    best_index = i;
                    best_key = ki;
                }
                __syncwarp();
            }
            const float bs = __shfl_sync(FULL, best_score, (lane % NG) * CG);
            if (lane < NG) my_best = bs;
            // the eight extractions side by side, a group each
            __syncwarp();
            group_chain_extract(dedup, dp, pred, aux, total_anchors, b, N, nmax, sg, best_score, ap, cc, nam_out,
                                nam_seg_count, anc_out, anc_start);
            continue;
        } else {
            // a long orientation (k_chain_long_prep and k_chain_big scored its clusters
            // without the re-check): the clusters whose maximum beats the running best,
            // in order, again with the re-check
            uint64_t* ring_key = ring_key_s + (RING ? wib * NG * 64 : 0);
            float* ring_dp = ring_dp_s + (RING ? wib * NG * 64 : 0);
            for (uint32_t q = 0; q < NG; q++) {
                const uint32_t sg = __shfl_sync(FULL, my_sg, q), N = __shfl_sync(FULL, my_n, q);
                const uint64_t b = __shfl_sync(FULL, my_b, q);
                if (sg == NONE || N == 0) continue;
                const uint32_t read_len = (uint32_t)(off[(sg >> 1) + 1] - off[sg >> 1]);
                const uint32_t max_ref_gap = cc.cp.max_ref_gap ? cc.cp.max_ref_gap : read_len;
                const uint32_t* cstart = aux + b;
                const float* cmax = reinterpret_cast<const float*>(aux + total_anchors + b);
                const uint32_t C = long_c[u];
                // in order: clusters whose maximum beats the running best, scored again
                float best_score = 0.0f;
                uint32_t best_index = 0xffffffffu;
                uint64_t best_key = 0;
                for (uint32_t c0 = 0; c0 < C; c0 += 32) {
                    const uint32_t c = c0 + lane;
                    const float m = c < C && c > 0 ? cmax[c] : -INFINITY;
                    uint32_t from = 0;
                    for (;;) {
                        const bool rec = c < C && lane >= from && (best_index == 0xffffffffu || m > best_score);
                        const uint32_t bal = __ballot_sync(FULL, rec);
                        if (!bal) break;
                        const uint32_t l = __ffs(bal) - 1, cc0 = c0 + l;
                        const uint32_t lo = cstart[cc0], hi = cc0 + 1 < C ? cstart[cc0 + 1] : N;
                        // the values scored without the re-check stand up to the first
                        // anchor where it would fire; only the rest is scored again
                        const uint32_t i0 = recheck_first_fire(dedup, dp, b, lo, hi, max_ref_gap, cc, ap, best_score,
                                                               best_index, best_key);
                        if (i0 < hi)
                            warp_chain_range<RING>(dedup, dp, pred, b, i0, hi, lo, max_ref_gap, cc, ap, ring_key,
                                                   ring_dp, true, best_score, best_index, best_key);
                        from = l + 1;
                    }
                }
                if (lane == q) my_best = best_score;
                __syncwarp();
            }
        }
        __syncwarp();
        for (uint32_t q = 0; q < NG; q++) {
            const uint32_t sg = __shfl_sync(FULL, my_sg, q), N = __shfl_sync(FULL, my_n, q);
            const uint64_t b = __shfl_sync(FULL, my_b, q);
            const float best = __shfl_sync(FULL, my_best, q);
            if (sg == NONE) continue;
            if (N == 0) {
                if (lane == 0) nam_seg_count[sg] = 0;
                continue;
            }
            chain_extract(dedup, dp, pred, aux, total_anchors, b, N, sg, best, ap, cc, nam_out,
                          nam_seg_count, anc_out, anc_start, hist + wib * 256);
        }
    }
}

// NAM ids in push order (forward chains first), then a stable sort by score,
// descending (src/nam.rs:168-170; the tie shuffle is applied by the host policy)
// Order-preserving u32 key of a NAM score; -0 and +0 map to one key, as they compare
// equal in the reference's sort.
__device__ __forceinline__ uint32_t score_key(float s) {
    const uint32_t b = __float_as_uint(s == 0.0f ? 0.0f : s);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__device__ __forceinline__ uint64_t nam_anchor_src(const uint64_t* anc_start, const uint64_t* seg_off, uint32_t r,
                                                   uint32_t c0, uint32_t t) {
    return t < c0 ? anc_start[seg_off[2 * r] + t] : anc_start[seg_off[2 * r + 1] + t - c0];
}

// NAM ids in push order (forward chains, then reverse) and the stable sort by score,
// descending (src/nam.rs:168-170), warp per read.  Up to 32 NAMs: ranks from the
// warp's scores by shuffles.  More: the NAMs go to tmp in push order with sort keys,
// and the read is listed for the segmented stable sort and k_nam_gather.
__global__ void __launch_bounds__(256) k_nam_compact(uint32_t n, const uint64_t* seg_off, const NamRec* scratch,
                                                     const uint32_t* nam_seg_count, const uint64_t* nam_off,
                                                     NamRec* out, NamDetailsRec* details,
                                                     const uint64_t* anc_start, uint64_t* anc_src,
                                                     uint64_t* anc_count, NamRec* tmp, uint32_t* keys,
                                                     uint32_t* vals, uint32_t* long_reads, uint64_t* long_begin,
                                                     uint64_t* long_end, uint32_t* n_long) {
    const uint32_t lane = lane_id();
    const uint32_t nwarps = gridDim.x * (blockDim.x / 32);
    for (uint32_t r = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; r < n; r += nwarps) {
        const uint32_t c0 = nam_seg_count[2 * r], c1 = nam_seg_count[2 * r + 1], c = c0 + c1;
        const NamRec* s0 = scratch + seg_off[2 * r];
        const NamRec* s1 = scratch + seg_off[2 * r + 1];
        const uint64_t ob = nam_off[r];
        if (lane == 0) details[r].n_nams = c;
        if (c <= 32) {
            NamRec nr{};
            float s = 0.0f;
            if (lane < c) {
                nr = lane < c0 ? s0[lane] : s1[lane - c0];
                s = nr.score;
            }
            uint32_t rank = 0;
            for (uint32_t u = 0; u < c; u++) {
                const float su = __shfl_sync(FULL, s, u);
                rank += (su > s) || (su == s && u < lane);
            }
            if (lane < c) {
                nr.nam_id = lane;
                out[ob + rank] = nr;
                if (anc_src) {
                    anc_src[ob + rank] = nam_anchor_src(anc_start, seg_off, r, c0, lane);
                    anc_count[ob + rank] = nr.n_anchors;
                }
            }
        } else {
            for (uint32_t t = lane; t < c; t += 32) {
                NamRec nr = t < c0 ? s0[t] : s1[t - c0];
                nr.nam_id = t;
                tmp[ob + t] = nr;
                keys[ob + t] = score_key(nr.score);
                vals[ob + t] = t;
            }
            if (lane == 0) {
                const uint32_t i = atomicAdd(n_long, 1u);
                long_reads[i] = r;
                long_begin[i] = ob;
                long_end[i] = ob + c;
            }
        }
    }
}

// the sorted order of each listed read applied: out[ob + rank] = tmp[ob + perm[rank]]
__global__ void __launch_bounds__(256) k_nam_gather(uint32_t n_long, const uint32_t* long_reads,
                                                    const uint64_t* seg_off, const uint32_t* nam_seg_count,
                                                    const uint64_t* nam_off, const NamRec* tmp, const uint32_t* perm,
                                                    NamRec* out, const uint64_t* anc_start, uint64_t* anc_src,
                                                    uint64_t* anc_count) {
    const uint32_t lane = lane_id();
    const uint32_t nwarps = gridDim.x * (blockDim.x / 32);
    for (uint32_t i = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; i < n_long; i += nwarps) {
        const uint32_t r = long_reads[i];
        const uint32_t c0 = nam_seg_count[2 * r], c = c0 + nam_seg_count[2 * r + 1];
        const uint64_t ob = nam_off[r];
        for (uint32_t k = lane; k < c; k += 32) {
            const uint32_t t = perm[ob + k];
            const NamRec nr = tmp[ob + t];
            out[ob + k] = nr;
            if (anc_src) {
                anc_src[ob + k] = nam_anchor_src(anc_start, seg_off, r, c0, t);
                anc_count[ob + k] = nr.n_anchors;
            }
        }
    }
}

__global__ void k_nam_counts(uint32_t n, const uint32_t* nam_seg_count, uint64_t* nam_count) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
        nam_count[r] = (uint64_t)nam_seg_count[2 * r] + nam_seg_count[2 * r + 1];
}

// each NAM's anchors, from the chaining scratch into one array in NAM output order
__global__ void k_nam_anchor_gather(uint64_t total_nams, const uint64_t* src, const uint64_t* dst_off,
                                    const uint64_t* sparse, uint64_t* dense) {
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total_nams;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t s = src[t], d = dst_off[t], c = dst_off[t + 1] - d;
        for (uint64_t u = 0; u < c; u++) dense[d + u] = sparse[s + u];
    }
}

inline unsigned warps_grid(uint64_t items) {
    uint64_t blocks = (items + WARPS_PER_BLOCK - 1) / WARPS_PER_BLOCK;
    if (blocks > sm_count() * 32) blocks = sm_count() * 32;
    return (unsigned)(blocks ? blocks : 1);
}

uint32_t ceil_log2(uint64_t v) {
    uint32_t b = 0;
    while ((1ULL << b) < v) b++;
    return b;
}

template <class T>
void cub_excl_sum(NamWorkspace& ws, const T* in, T* out, uint64_t n, cudaStream_t st) {
    size_t tmp = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tmp, in, out, (int64_t)n, st);
    ws.cub_tmp.reserve(tmp);
    cub::DeviceScan::ExclusiveSum(ws.cub_tmp.p, tmp, in, out, (int64_t)n, st);
}

}  // namespace

uint32_t run_seeding(const SeedParams& sp, uint32_t n, uint64_t total, NamWorkspace& ws, cudaStream_t st,
                     KernelTimers* kt) {
    KernelTimers none;
    if (!kt) kt = &none;
    ws.syn_hash.reserve(total);
    ws.syn_pos.reserve(total);
    ws.qr_hash.reserve(2 * total);
    ws.qr_hash_rc.reserve(2 * total);
    ws.qr_start.reserve(2 * total);
    ws.qr_end.reserve(2 * total);
    ws.n_rs.reserve(2 * (size_t)n);
    size_t smem = WARPS_PER_BLOCK * MAX_READ_LEN;
    kt->begin(KS_SEED, st);
    k_seed<false><<<warps_grid(n), 32 * WARPS_PER_BLOCK, smem, st>>>(ws.seq.p, ws.off.p, n, sp, ws.syn_hash.p,
                                                                     ws.syn_pos.p, ws.qr_hash.p, ws.qr_hash_rc.p,
                                                                     ws.qr_start.p, ws.qr_end.p, total, ws.n_rs.p);
    kt->end(st);
    SA_CUDA(cudaGetLastError());
    return 1;
}

// Syncmer scratch of the allocation-free seeding entry point: hashes (8 bytes per
// base) then positions (4 bytes per base) for at most
// SA_RANDSTROBES_NOALLOC_MAX_BASES bases.  One copy per device, shared by every
// call on that device.  Nothing in it needs to start at zero: each read writes
// its own syncmer slots before reading them.
static __device__ __align__(256) uint8_t g_seed_scratch[(size_t)SA_RANDSTROBES_NOALLOC_MAX_BASES * 12];

void run_seeding_noalloc(const SeedParams& sp, const uint8_t* seq, const uint64_t* off, uint32_t n, uint64_t total,
                         uint64_t* qr_hash, uint64_t* qr_hash_rc, uint32_t* qr_start, uint32_t* qr_end,
                         uint32_t* counts, cudaStream_t st) {
    if (total > SA_RANDSTROBES_NOALLOC_MAX_BASES)
        throw Error(SA_ERR_INVALID, "batch has " + std::to_string(total) + " bases; the allocation-free seeding "
                                    "entry point takes at most " +
                                        std::to_string((uint64_t)SA_RANDSTROBES_NOALLOC_MAX_BASES));
    // scratch address per device and CUDA context, looked up by the first call on that
    // device in that context (a context created anew, e.g. after cudaDeviceReset,
    // looks it up again instead of using a stale address)
    constexpr int MAX_DEVICES = 64;
    using CtxGetCurrent = int (*)(void**);  // cuCtxGetCurrent(CUcontext*)
    static std::mutex mu;
    static CtxGetCurrent ctx_current = nullptr;
    static void* scratch_ctx[MAX_DEVICES] = {};
    static uint8_t* scratch[MAX_DEVICES] = {};
    int dev = 0;
    SA_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES) throw Error(SA_ERR_CUDA, "device ordinal out of range");
    uint8_t* base;
    {
        std::lock_guard<std::mutex> g(mu);
        if (!ctx_current) {
            cudaDriverEntryPointQueryResult q{};
            SA_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", reinterpret_cast<void**>(&ctx_current), 12000,
                                                     cudaEnableDefault, &q));
            if (q != cudaDriverEntryPointSuccess || !ctx_current)
                throw Error(SA_ERR_CUDA, "cuCtxGetCurrent is not available");
        }
        void* ctx = nullptr;
        if (ctx_current(&ctx) != 0) throw Error(SA_ERR_CUDA, "cuCtxGetCurrent failed");
        if (!ctx || !scratch[dev] || scratch_ctx[dev] != ctx) {
            // binds (or creates) the device's primary context and loads the kernel, so
            // that later calls only launch
            cudaFuncAttributes fa;
            SA_CUDA(cudaFuncGetAttributes(&fa, k_seed<true>));
            if (ctx_current(&ctx) != 0 || !ctx) throw Error(SA_ERR_CUDA, "no current CUDA context");
        }
        if (!scratch[dev] || scratch_ctx[dev] != ctx) {
            uint8_t* p = nullptr;
            SA_CUDA(cudaGetSymbolAddress((void**)&p, g_seed_scratch));
            scratch[dev] = p;
            scratch_ctx[dev] = ctx;
        }
        base = scratch[dev];
    }
    if (!n) return;
    if (!off || !counts || (total && (!seq || !qr_hash || !qr_hash_rc || !qr_start || !qr_end)))
        throw Error(SA_ERR_INVALID, "null device pointer");
    uint64_t* syn_hash = reinterpret_cast<uint64_t*>(base);
    uint32_t* syn_pos = reinterpret_cast<uint32_t*>(base + (size_t)SA_RANDSTROBES_NOALLOC_MAX_BASES * 8);
    const size_t smem = WARPS_PER_BLOCK * MAX_READ_LEN;
    k_seed<true><<<warps_grid(n), 32 * WARPS_PER_BLOCK, smem, st>>>(seq, off, n, sp, syn_hash, syn_pos, qr_hash,
                                                                    qr_hash_rc, qr_start, qr_end, total, counts);
    SA_CUDA(cudaGetLastError());
}

uint32_t run_nam_pipeline(const DevIndex& ix, const DevRefs& refs, const NamConfig& cfg, uint32_t n, uint64_t total,
                          uint32_t max_contig_len, uint32_t n_contigs, NamWorkspace& ws, cudaStream_t st,
                          KernelTimers* kt) {
    (void)refs;
    KernelTimers none;
    if (!kt) kt = &none;
    uint32_t launches = 0;
    if (!ws.log2_lut.p) {
        std::vector<float> lut(LOG2_LUT_SIZE);
        for (uint32_t d = 0; d < LOG2_LUT_SIZE; d++) lut[d] = std::log2((float)d + 1.0f);
        ws.log2_lut.reserve(LOG2_LUT_SIZE);
        SA_CUDA(cudaMemcpy(ws.log2_lut.p, lut.data(), LOG2_LUT_SIZE * sizeof(float), cudaMemcpyHostToDevice));
    }
    AnchorPack ap;
    ap.qbits = ceil_log2((uint64_t)MAX_READ_LEN + 1);
    ap.pbits = ceil_log2((uint64_t)max_contig_len + 1);
    uint32_t rbits = ceil_log2((uint64_t)n_contigs);
    if (ap.qbits + ap.pbits + rbits > 64) throw Error(SA_ERR_INVALID, "contig count/length too large for anchor keys");
    launches += run_seeding(ix.p, n, total, ws, st, kt);
    ws.hit_pos.reserve(2 * total);
    ws.hit_info.reserve(2 * total);
    ws.hit_count_cache.reserve(2 * total);
    ws.n_hits.reserve(2 * (size_t)n);
    ws.orient.reserve(n);
    ws.details.reserve(n);
    kt->begin(KS_HITS, st);
    if (cfg.mcs != SA_MCS_FIRST_STROBE) {
        k_probe<<<warps_grid(n), 32 * WARPS_PER_BLOCK, 0, st>>>(ix, ws.off.p, n, total, cfg.mcs, ws.qr_hash.p,
                                                                ws.qr_hash_rc.p, ws.n_rs.p, ws.hit_pos.p,
                                                                ws.hit_info.p);
        launches++;
    }
    k_hits<<<warps_grid(n), 32 * WARPS_PER_BLOCK, 0, st>>>(
        ix, ws.off.p, n, total, cfg.mcs, cfg.rescue_distance, ws.qr_hash.p, ws.qr_hash_rc.p, ws.qr_start.p,
        ws.qr_end.p, ws.n_rs.p, ws.hit_pos.p, ws.hit_info.p, ws.hit_count_cache.p, ws.n_hits.p, ws.orient.p,
        ws.details.p);
    kt->end(st);
    launches++;
    ws.hit_anchors.reserve(2 * total);
    ws.seg_count.reserve(2 * (size_t)n + 1);
    ws.seg_off.reserve(2 * (size_t)n + 1);
    kt->begin(KS_ANCHORS, st);
    k_anchors<false><<<warps_grid(n), 32 * WARPS_PER_BLOCK, 0, st>>>(
        ix, ws.off.p, n, total, ws.qr_hash.p, ws.qr_start.p, ws.qr_end.p, ws.hit_pos.p, ws.hit_info.p, ws.n_hits.p,
        ws.orient.p, ws.hit_anchors.p, ws.seg_count.p, nullptr, nullptr, ap, ws.details.p);
    kt->end(st);
    launches++;
    SA_CUDA(cudaMemsetAsync(ws.seg_count.p + 2 * (size_t)n, 0, 8, st));
    cub_excl_sum(ws, ws.seg_count.p, ws.seg_off.p, 2 * (uint64_t)n + 1, st);
    launches++;
    // seg_list: short list [0, 2n), long list [2n, 4n), counts at 4n
    ws.seg_list.reserve(4 * (size_t)n + 4);
    ws.sort_begin.reserve(2 * (size_t)n);
    ws.sort_end.reserve(2 * (size_t)n);
    uint32_t* const long_list = ws.seg_list.p + 2 * (size_t)n;
    uint32_t* const list_counts = ws.seg_list.p + 4 * (size_t)n;
    ws.seg_key.reserve(4 * (size_t)n);
    ws.seg_key_alt.reserve(4 * (size_t)n);
    ws.seg_sorted.reserve(4 * (size_t)n);
    SA_CUDA(cudaMemsetAsync(list_counts, 0, 12, st));
    k_seg_list<<<warps_grid((2 * (uint64_t)n + 31) / 32), 32 * WARPS_PER_BLOCK, 0, st>>>(
        ws.seg_count.p, ws.seg_off.p, 2 * n, ws.seg_list.p, long_list, list_counts, ws.sort_begin.p, ws.sort_end.p,
        ws.seg_key.p, ws.seg_key.p + 2 * (size_t)n);
    launches++;
    uint64_t total_anchors = 0;
    uint32_t n_list[3] = {0, 0, 0};
    SA_CUDA(cudaMemcpyAsync(&total_anchors, ws.seg_off.p + 2 * (size_t)n, 8, cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaMemcpyAsync(n_list, list_counts, 12, cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaStreamSynchronize(st));
    ws.anchors.reserve(total_anchors);
    ws.anchors_sorted.reserve(total_anchors);
    kt->begin(KS_ANCHORS, st);
    k_anchors<true><<<warps_grid(n), 32 * WARPS_PER_BLOCK, 0, st>>>(
        ix, ws.off.p, n, total, ws.qr_hash.p, ws.qr_start.p, ws.qr_end.p, ws.hit_pos.p, ws.hit_info.p, ws.n_hits.p,
        ws.orient.p, ws.hit_anchors.p, nullptr, ws.seg_off.p, ws.anchors.p, ap, ws.details.p);
    kt->end(st);
    launches++;
    if (n_list[1]) {
        // orientations with more than CHAIN_SORT_SMALL anchors; k_chain4 sorts the rest
        size_t tmp = 0;
        kt->begin(KS_SORT, st);
        cub::DeviceSegmentedSort::SortKeys(nullptr, tmp, ws.anchors.p, ws.anchors_sorted.p, (int64_t)total_anchors,
                                           (int64_t)n_list[1], ws.sort_begin.p, ws.sort_end.p, st);
        ws.cub_tmp.reserve(tmp);
        cub::DeviceSegmentedSort::SortKeys(ws.cub_tmp.p, tmp, ws.anchors.p, ws.anchors_sorted.p,
                                           (int64_t)total_anchors, (int64_t)n_list[1], ws.sort_begin.p, ws.sort_end.p,
                                           st);
        kt->end(st);
        launches++;
    }
    // read orientations by anchor count, largest first: the eight orientations of a
    // grouped warp then have similar counts (the warp runs as many steps as its largest
    // one), and the long orientations start first
    const uint32_t* short_list = ws.seg_list.p;
    const uint32_t* long_sorted = long_list;
    {
        size_t tmp = 0, t2 = 0;
        if (n_list[0] > 1)
            cub::DeviceRadixSort::SortPairsDescending(nullptr, tmp, ws.seg_key.p, ws.seg_key_alt.p, ws.seg_list.p,
                                                      ws.seg_sorted.p, (int64_t)n_list[0], 0, 8, st);
        if (n_list[2] > 1)
            cub::DeviceRadixSort::SortPairsDescending(nullptr, t2, ws.seg_key.p, ws.seg_key_alt.p, ws.seg_list.p,
                                                      ws.seg_sorted.p, (int64_t)n_list[2], 0, 32, st);
        ws.cub_tmp.reserve(std::max(tmp, t2));
        kt->begin(KS_NAMS_OTHER, st);
        if (n_list[0] > 1) {
            cub::DeviceRadixSort::SortPairsDescending(ws.cub_tmp.p, tmp, ws.seg_key.p, ws.seg_key_alt.p,
                                                      ws.seg_list.p, ws.seg_sorted.p, (int64_t)n_list[0], 0, 8, st);
            short_list = ws.seg_sorted.p;
            launches++;
        }
        if (n_list[2] > 1) {
            const size_t o = 2 * (size_t)n;
            cub::DeviceRadixSort::SortPairsDescending(ws.cub_tmp.p, t2, ws.seg_key.p + o, ws.seg_key_alt.p + o,
                                                      long_list, ws.seg_sorted.p + o, (int64_t)n_list[2], 0, 32, st);
            long_sorted = ws.seg_sorted.p + o;
            launches++;
        }
        kt->end(st);
    }
    ws.dp.reserve(total_anchors);
    ws.pred.reserve(total_anchors);
    ws.aux.reserve(3 * total_anchors);
    ws.nam_scratch.reserve(total_anchors);
    ws.nam_seg_count.reserve(2 * (size_t)n);
    ChainCtx cc{cfg.cp, ix.p.k, ws.log2_lut.p, false, true, 0, 0};
    {
        // R = M * 2^e with M the 24-bit significand of a normal positive float
        const float R = cfg.cp.max_diagonal_ratio;
        int ex = 0;
        const float fr = std::frexp(R, &ex);  // R = fr * 2^ex, fr in [0.5, 1)
        if (std::isfinite(R) && R > 0.0f && fr != 0.0f) {
            const uint64_t M = (uint64_t)std::ldexp((double)fr, 24);  // exact: 24 significant bits
            const int e = ex - 24;
            const int shift = 1 - e;
            if (M >= (1u << 23) && M < (1u << 24) && shift >= 0 && shift <= 30) {
                cc.ratio_exact = true;
                cc.ratio_strict = (M & 1) == 0;
                cc.ratio_shift = (uint32_t)shift;
                cc.ratio_num = 2 * M + 1;
            }
        }
    }
    kt->begin(KS_CHAIN, st);
    SA_CUDA(cudaMemsetAsync(ws.nam_seg_count.p, 0, 2 * (size_t)n * sizeof(uint32_t), st));
    const uint64_t chain_units = (uint64_t)n_list[2] + ((uint64_t)n_list[0] + NG - 1) / NG;
    const unsigned chain_grid = (unsigned)std::max<uint64_t>(
        1, std::min<uint64_t>((chain_units + CHAIN_WARPS - 1) / CHAIN_WARPS, sm_count() * 64));
    if (cfg.nam_anchors) {
        ws.anc_sparse.reserve(3 * total_anchors + 1);
        ws.anc_start.reserve(total_anchors + 1);
    }
    // long orientations: dedup, clusters and their first scoring, before k_chain4
    uint32_t* const long_n = ws.seg_key_alt.p;
    uint32_t* const long_c = ws.seg_key_alt.p + 2 * (size_t)n;
    if (n_list[2]) {
        const uint32_t lane_max = std::max<uint32_t>(1, cfg.chain_lane_max);
        const uint64_t cap = total_anchors / (lane_max + 1) + 1;
        ws.chain_big.reserve(2 * cap + 2);
        SA_CUDA(cudaMemsetAsync(ws.chain_big.p, 0, 4, st));
        const unsigned pgrid = (unsigned)std::min<uint64_t>(((uint64_t)n_list[2] + 3) / 4, sm_count() * 16);
        k_chain_long_prep<<<pgrid, 128, 0, st>>>(ws.off.p, ws.seg_off.p, ws.anchors_sorted.p, ws.anchors.p, ws.dp.p,
                                                 ws.pred.p, ws.aux.p, total_anchors, ap, cc, long_sorted, n_list[2],
                                                 long_n, long_c, ws.chain_big.p + 2, ws.chain_big.p, lane_max);
        const unsigned bgrid = (unsigned)(sm_count() * 8);
        if (cfg.cp.max_lookback < 64)
            k_chain_big<true><<<bgrid, 128, 0, st>>>(ws.off.p, ws.seg_off.p, ws.anchors.p, ws.dp.p, ws.pred.p,
                                                     ws.aux.p, total_anchors, ap, cc, long_sorted, long_n, long_c,
                                                     ws.chain_big.p + 2, ws.chain_big.p);
        else
            k_chain_big<false><<<bgrid, 128, 0, st>>>(ws.off.p, ws.seg_off.p, ws.anchors.p, ws.dp.p, ws.pred.p,
                                                      ws.aux.p, total_anchors, ap, cc, long_sorted, long_n, long_c,
                                                      ws.chain_big.p + 2, ws.chain_big.p);
        launches += 2;
    }
    if (cfg.cp.max_lookback < 64)
        k_chain4<true><<<chain_grid, 32 * CHAIN_WARPS, 0, st>>>(
            ws.off.p, n, ws.seg_off.p, ws.anchors_sorted.p, ws.anchors.p, ws.dp.p, ws.pred.p, ws.aux.p,
            total_anchors, ap, cc, ws.nam_scratch.p, ws.nam_seg_count.p, cfg.nam_anchors ? ws.anc_sparse.p : nullptr,
            cfg.nam_anchors ? ws.anc_start.p : nullptr, short_list, n_list[0], long_sorted, n_list[2], long_n, long_c);
    else
        k_chain4<false><<<chain_grid, 32 * CHAIN_WARPS, 0, st>>>(
            ws.off.p, n, ws.seg_off.p, ws.anchors_sorted.p, ws.anchors.p, ws.dp.p, ws.pred.p, ws.aux.p,
            total_anchors, ap, cc, ws.nam_scratch.p, ws.nam_seg_count.p, cfg.nam_anchors ? ws.anc_sparse.p : nullptr,
            cfg.nam_anchors ? ws.anc_start.p : nullptr, short_list, n_list[0], long_sorted, n_list[2], long_n, long_c);
    kt->end(st);
    launches++;
    ws.nam_count.reserve((size_t)n + 1);
    ws.nam_off.reserve((size_t)n + 1);
    kt->begin(KS_NAMS_OTHER, st);
    k_nam_counts<<<(n + 255) / 256 + 1, 256, 0, st>>>(n, ws.nam_seg_count.p, ws.nam_count.p);
    SA_CUDA(cudaMemsetAsync(ws.nam_count.p + n, 0, 8, st));
    cub_excl_sum(ws, ws.nam_count.p, ws.nam_off.p, (uint64_t)n + 1, st);
    kt->end(st);
    launches += 2;
    uint64_t total_nams = 0;
    SA_CUDA(cudaMemcpyAsync(&total_nams, ws.nam_off.p + n, 8, cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaStreamSynchronize(st));
    ws.nams.reserve(total_nams);
    if (cfg.nam_anchors) {
        ws.nam_anc_src.reserve(total_nams + 1);
        ws.nam_anc_off.reserve(total_nams + 1);
    }
    ws.nam_tmp.reserve(total_nams);
    ws.nam_keys.reserve(2 * total_nams);
    ws.nam_vals.reserve(2 * total_nams);
    ws.long_reads.reserve((size_t)n + 1);
    ws.long_begin.reserve((size_t)n);
    ws.long_end.reserve((size_t)n);
    kt->begin(KS_NAMS_OTHER, st);
    SA_CUDA(cudaMemsetAsync(ws.long_reads.p + n, 0, 4, st));
    k_nam_compact<<<warps_grid(n), 32 * WARPS_PER_BLOCK, 0, st>>>(
        n, ws.seg_off.p, ws.nam_scratch.p, ws.nam_seg_count.p, ws.nam_off.p, ws.nams.p, ws.details.p,
        cfg.nam_anchors ? ws.anc_start.p : nullptr, cfg.nam_anchors ? ws.nam_anc_src.p : nullptr,
        cfg.nam_anchors ? ws.nam_anc_off.p : nullptr, ws.nam_tmp.p, ws.nam_keys.p, ws.nam_vals.p,
        ws.long_reads.p, ws.long_begin.p, ws.long_end.p, ws.long_reads.p + n);
    launches++;
    uint32_t n_long = 0;
    SA_CUDA(cudaMemcpyAsync(&n_long, ws.long_reads.p + n, 4, cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaStreamSynchronize(st));
    if (n_long) {
        uint32_t* keys_out = ws.nam_keys.p + total_nams;
        uint32_t* perm = ws.nam_vals.p + total_nams;
        size_t tmp = 0;
        cub::DeviceSegmentedSort::StableSortPairsDescending(nullptr, tmp, ws.nam_keys.p, keys_out, ws.nam_vals.p,
                                                            perm, (int64_t)total_nams, (int64_t)n_long,
                                                            ws.long_begin.p, ws.long_end.p, st);
        ws.cub_tmp.reserve(tmp);
        cub::DeviceSegmentedSort::StableSortPairsDescending(ws.cub_tmp.p, tmp, ws.nam_keys.p, keys_out,
                                                            ws.nam_vals.p, perm, (int64_t)total_nams,
                                                            (int64_t)n_long, ws.long_begin.p, ws.long_end.p, st);
        k_nam_gather<<<warps_grid(n_long), 32 * WARPS_PER_BLOCK, 0, st>>>(
            n_long, ws.long_reads.p, ws.seg_off.p, ws.nam_seg_count.p, ws.nam_off.p, ws.nam_tmp.p, perm, ws.nams.p,
            cfg.nam_anchors ? ws.anc_start.p : nullptr, cfg.nam_anchors ? ws.nam_anc_src.p : nullptr,
            cfg.nam_anchors ? ws.nam_anc_off.p : nullptr);
        launches += 2;
    }
    kt->end(st);
    ws.anchor_qbits = ap.qbits;
    ws.anchor_pbits = ap.pbits;
    ws.last_total_nam_anchors = 0;
    if (cfg.nam_anchors) {
        // counts -> offsets in place, then the gather
        SA_CUDA(cudaMemsetAsync(ws.nam_anc_off.p + total_nams, 0, 8, st));
        ws.nam_count.reserve(total_nams + 1);
        SA_CUDA(cudaMemcpyAsync(ws.nam_count.p, ws.nam_anc_off.p, (total_nams + 1) * 8, cudaMemcpyDeviceToDevice, st));
        cub_excl_sum(ws, ws.nam_count.p, ws.nam_anc_off.p, total_nams + 1, st);
        uint64_t tot = 0;
        SA_CUDA(cudaMemcpyAsync(&tot, ws.nam_anc_off.p + total_nams, 8, cudaMemcpyDeviceToHost, st));
        SA_CUDA(cudaStreamSynchronize(st));
        ws.nam_anc.reserve(tot + 1);
        if (total_nams)
            k_nam_anchor_gather<<<(unsigned)std::min<uint64_t>((total_nams + 255) / 256, sm_count() * 16), 256, 0, st>>>(
                total_nams, ws.nam_anc_src.p, ws.nam_anc_off.p, ws.anc_sparse.p, ws.nam_anc.p);
        launches += 3;
        ws.last_total_nam_anchors = tot;
    }
    SA_CUDA(cudaGetLastError());
    ws.last_total_nams = total_nams;
    return launches;
}

}  // namespace sa
