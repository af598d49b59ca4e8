// Device-side StrobemerIndex probes (src/index.rs:127-338, src/partition.rs).
// All lookups are functions of the sorted table only, so any lower-bound search
// returns the reference's partition point.
#pragma once
#include "sa_internal.h"

namespace sa {

__device__ __forceinline__ uint64_t rs_hash(const RefRandstrobe& r) { return r.hash_offset & HASH_MASK; }

// 16-byte vectorised load of one table entry
__device__ __forceinline__ RefRandstrobe load_rs(const RefRandstrobe* rs, uint64_t i) {
    ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(rs) + i);
    RefRandstrobe r;
    r.hash_offset = v.x;
    r.position = (uint32_t)v.y;
    r.ref_index = (uint32_t)(v.y >> 32);
    return r;
}

__device__ __forceinline__ uint64_t load_hash(const RefRandstrobe* rs, uint64_t i) {
    return __ldg(reinterpret_cast<const unsigned long long*>(rs) + 2 * i) & HASH_MASK;
}

// get_masked_from (src/index.rs:159-197); returns UINT64_MAX when absent
__device__ __forceinline__ uint64_t idx_get_masked_from(const DevIndex& ix, uint64_t hash, uint64_t mask,
                                                        bool has_start, uint64_t start) {
    const uint64_t masked = hash & mask;
    const uint64_t top = hash >> (64 - ix.bits);
    ulonglong2 b;
    if ((top & 1) == 0) {
        b = __ldg(reinterpret_cast<const ulonglong2*>(ix.buckets + top));
    } else {
        b.x = __ldg(reinterpret_cast<const unsigned long long*>(ix.buckets) + top);
        b.y = __ldg(reinterpret_cast<const unsigned long long*>(ix.buckets) + top + 1);
    }
    uint64_t ps = has_start ? start : b.x, pe = b.y;
    if (ps >= pe) return UINT64_MAX;
    uint64_t len = pe - ps;
    if (len < 4) {
        for (uint64_t i = 0; i < len; i++) {
            uint64_t h = load_hash(ix.rs, ps + i) & mask;
            if (h == masked) return ps + i;
            if (h > masked) return UINT64_MAX;
        }
        return UINT64_MAX;
    }
    uint64_t lo = 0, hi = len;
    while (lo < hi) {
        uint64_t mid = lo + (hi - lo) / 2;
        if ((load_hash(ix.rs, ps + mid) & mask) < masked) lo = mid + 1;
        else hi = mid;
    }
    if (lo < len && (load_hash(ix.rs, ps + lo) & mask) == masked) return ps + lo;
    return UINT64_MAX;
}

// get_count (src/index.rs:272-295)
__device__ __forceinline__ uint32_t idx_get_count(const DevIndex& ix, uint64_t position, uint64_t mask) {
    uint64_t key = load_hash(ix.rs, position);
    uint64_t masked = key & mask;
    uint64_t top = key >> (64 - ix.bits);
    uint64_t pe = __ldg(reinterpret_cast<const unsigned long long*>(ix.buckets) + top + 1);
    if (pe - position < 8) {
        uint32_t c = 1;
        for (uint64_t p = position + 1; p < pe; p++) {
            if ((load_hash(ix.rs, p) & mask) == masked) c++;
            else break;
        }
        return c;
    }
    uint64_t lo = 0, hi = pe - position;
    while (lo < hi) {
        uint64_t mid = lo + (hi - lo) / 2;
        if ((load_hash(ix.rs, position + mid) & mask) <= masked) lo = mid + 1;
        else hi = mid;
    }
    return (uint32_t)lo;
}

__device__ __forceinline__ uint64_t idx_full_forward(const DevIndex& ix, uint64_t h) {
    return idx_get_masked_from(ix, h, HASH_MASK, false, 0);
}

// is_too_frequent_forward (src/index.rs:298-307): guarded by the index's own cutoff
__device__ __forceinline__ bool idx_too_frequent_forward(const DevIndex& ix, uint64_t pos, uint32_t cutoff) {
    if (pos + ix.filter_cutoff < ix.n) return load_hash(ix.rs, pos) == load_hash(ix.rs, pos + cutoff);
    return false;
}

// is_too_frequent (src/index.rs:309-323)
__device__ __forceinline__ bool idx_too_frequent(const DevIndex& ix, uint64_t pos, uint32_t cutoff, uint64_t hash_rc) {
    if (idx_too_frequent_forward(ix, pos, cutoff)) return true;
    uint64_t rc = idx_full_forward(ix, hash_rc);
    if (rc != UINT64_MAX) {
        if (idx_too_frequent_forward(ix, rc, cutoff)) return true;
        uint64_t c = (uint64_t)idx_get_count(ix, pos, HASH_MASK) + idx_get_count(ix, rc, HASH_MASK);
        return c > cutoff;
    }
    return false;
}

// is_too_frequent_partial (src/index.rs:325-337)
__device__ __forceinline__ bool idx_too_frequent_partial(const DevIndex& ix, uint64_t pos, uint32_t cutoff) {
    if (pos + cutoff < ix.n)
        return (load_hash(ix.rs, pos) & ix.p.main_mask) == (load_hash(ix.rs, pos + cutoff) & ix.p.main_mask);
    return false;
}

// get_count_full (src/index.rs:254-263)
__device__ __forceinline__ uint32_t idx_count_full(const DevIndex& ix, uint64_t pos, uint64_t hash_rc) {
    uint64_t rc = idx_full_forward(ix, hash_rc);
    uint32_t r = rc == UINT64_MAX ? 0 : idx_get_count(ix, rc, HASH_MASK);
    return r + idx_get_count(ix, pos, HASH_MASK);
}

// ------------------------------------------------------------------ latency-parallel probes
// The same answers as idx_full_forward / idx_too_frequent above, with the dependent
// memory rounds cut down: both orientations' lookups proceed side by side, a bucket of
// up to 8 entries is scanned with independent loads instead of a binary search (the
// lower bound is the number of smaller keys), larger buckets narrow 8-ary, and the
// repeat test loads the entries at pos + cutoff and pos + 1 of both hits at once.

// bucket range [ps, pe) of a full hash (same directory reads as idx_get_masked_from)
__device__ __forceinline__ void idx_bucket(const DevIndex& ix, uint64_t hash, uint64_t& ps, uint64_t& pe) {
    const uint64_t top = hash >> (64 - ix.bits);
    if ((top & 1) == 0) {
        ulonglong2 b = __ldg(reinterpret_cast<const ulonglong2*>(ix.buckets + top));
        ps = b.x;
        pe = b.y;
    } else {
        ps = __ldg(reinterpret_cast<const unsigned long long*>(ix.buckets) + top);
        pe = __ldg(reinterpret_cast<const unsigned long long*>(ix.buckets) + top + 1);
    }
}

// narrow [lo, hi) to at most 8 entries around the lower bound of key, 8-ary
__device__ __forceinline__ void idx_narrow(const DevIndex& ix, uint64_t key, uint64_t& lo, uint64_t& hi) {
    while (hi - lo > 8) {
        const uint64_t len = hi - lo;
        uint64_t piv[7];
        uint64_t hv[7];
#pragma unroll
        for (int t = 0; t < 7; t++) {
            piv[t] = lo + len * (uint64_t)(t + 1) / 8;
            hv[t] = load_hash(ix.rs, piv[t]);
        }
        uint64_t nlo = lo, nhi = hi;
#pragma unroll
        for (int t = 0; t < 7; t++) {
            if (hv[t] < key) nlo = piv[t] + 1;
        }
#pragma unroll
        for (int t = 6; t >= 0; t--) {
            if (hv[t] >= key) nhi = piv[t];
        }
        // the lower bound lies in [nlo, nhi]; keep one entry past the range so that an
        // equal key at nhi is seen
        lo = nlo;
        hi = nhi < hi ? nhi + 1 : hi;
    }
}

// lower bound of key in [lo, hi) (hi - lo <= 8) and whether the key is present
__device__ __forceinline__ uint64_t idx_scan8(const DevIndex& ix, uint64_t key, uint64_t lo, uint64_t hi) {
    const uint32_t len = (uint32_t)(hi - lo);
    uint64_t hv[8];
#pragma unroll
    for (int t = 0; t < 8; t++) hv[t] = (uint32_t)t < len ? load_hash(ix.rs, lo + t) : UINT64_MAX;
    uint32_t lt = 0;
    bool eq = false;
#pragma unroll
    for (int t = 0; t < 8; t++) {
        lt += hv[t] < key;
        eq |= (uint32_t)t < len && hv[t] == key;
    }
    return eq ? lo + lt : UINT64_MAX;
}

// count of the run of hash at pos (get_count with the full mask), given the bucket
// end and the preloaded hash at pos + 1
__device__ __forceinline__ uint32_t idx_count_at(const DevIndex& ix, uint64_t pos, uint64_t bucket_end,
                                                 uint64_t h_pos, uint64_t h_next) {
    if (pos + 1 >= bucket_end || h_next != h_pos) return 1;
    return idx_get_count(ix, pos, HASH_MASK);
}

// full lookup of h (forward) with is_too_frequent (src/index.rs:309-323) using the
// reverse-complement hash hrc; pos = UINT64_MAX when absent
__device__ __forceinline__ void idx_full_probe(const DevIndex& ix, uint64_t h, uint64_t hrc, uint32_t cutoff,
                                               uint64_t& pos, bool& filtered) {
    const uint64_t ka = h & HASH_MASK, kb = hrc & HASH_MASK;
    uint64_t sa, ea, sb, eb;
    idx_bucket(ix, h, sa, ea);
    idx_bucket(ix, hrc, sb, eb);
    filtered = false;
    uint64_t la = sa, ha = sa < ea ? ea : sa, lb = sb, hb = sb < eb ? eb : sb;
    if (ha - la > 8) idx_narrow(ix, ka, la, ha);
    if (hb - lb > 8) idx_narrow(ix, kb, lb, hb);
    const uint64_t pa = idx_scan8(ix, ka, la, ha);
    pos = pa;
    if (pa == UINT64_MAX) return;
    const uint64_t pb = idx_scan8(ix, kb, lb, hb);
    // everything the repeat test can read, at once
    const bool ga = pa + ix.filter_cutoff < ix.n, gb = pb != UINT64_MAX && pb + ix.filter_cutoff < ix.n;
    const uint64_t a_cut = ga ? load_hash(ix.rs, pa + cutoff) : 0;
    const uint64_t a_next = pa + 1 < ix.n ? load_hash(ix.rs, pa + 1) : 0;
    const uint64_t b_cut = gb ? load_hash(ix.rs, pb + cutoff) : 0;
    const uint64_t b_next = pb != UINT64_MAX && pb + 1 < ix.n ? load_hash(ix.rs, pb + 1) : 0;
    if (ga && a_cut == ka) {
        filtered = true;
        return;
    }
    if (pb == UINT64_MAX) return;
    if (gb && b_cut == kb) {
        filtered = true;
        return;
    }
    const uint64_t c = (uint64_t)idx_count_at(ix, pa, ea, ka, a_next) + idx_count_at(ix, pb, eb, kb, b_next);
    filtered = c > cutoff;
}

}  // namespace sa
