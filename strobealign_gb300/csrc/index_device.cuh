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

}  // namespace sa
