// GPU construction of the StrobemerIndex (src/indexer.rs:18-253) and batched
// lookups (src/index.rs:127-338).
//
// Build: (1) one thread per reference position tests the canonical open-syncmer
// condition on the 2-bit reference (the reference never holds N: wildcards are
// pseudo-random bases, src/packed_seq.rs:50-59, so a syncmer is a pure function of
// its k-mer window); (2) the flagged positions are compacted in order; (3) one
// thread per syncmer picks its partner among the next w_min..w_max syncmers of the
// same contig within max_dist (src/seeding/strobes.rs:145-176); (4) a radix sort on
// the full 128-bit (hash_offset, position, ref_index) key reproduces the reference's
// sorted order exactly; (5) the bucket directory and the repeat cutoff are derived
// from the sorted table.
#include <cub/cub.cuh>
#include <cuda/std/tuple>
#include <thrust/iterator/counting_iterator.h>

#include "host_state.h"
#include "index_device.cuh"

namespace sa {

namespace {

// 2-bit base i of a contig (LSB-first packing)
__device__ __forceinline__ uint64_t bases_le(const uint64_t* w, uint64_t i, uint32_t nb) {
    // nb <= 32 bases starting at i, packed little-endian (base i in bits 0..1)
    uint64_t wi = i >> 5;
    uint32_t sh = (uint32_t)(i & 31) * 2;
    uint64_t v = w[wi] >> sh;
    if (sh + 2 * nb > 64) v |= w[wi + 1] << (64 - sh);
    return nb == 32 ? v : (v & ((1ULL << (2 * nb)) - 1));
}

// reverse the order of the 2-bit groups of a 64-bit word
__device__ __forceinline__ uint64_t rev2(uint64_t x) {
    x = __brevll(x);
    return ((x >> 1) & 0x5555555555555555ULL) | ((x & 0x5555555555555555ULL) << 1);
}

// canonical value of the nb-mer at i: min(forward, reverse complement)
// (src/seeding/syncmers.rs:186-199, 217-221)
__device__ __forceinline__ uint64_t canonical(const uint64_t* w, uint64_t i, uint32_t nb, bool* is_fwd) {
    uint64_t le = bases_le(w, i, nb);
    uint64_t fwd = rev2(le) >> (64 - 2 * nb);
    uint64_t mask = nb == 32 ? ~0ULL : ((1ULL << (2 * nb)) - 1);
    uint64_t rc = (~le) & mask;
    if (is_fwd) *is_fwd = fwd <= rc;
    return fwd < rc ? fwd : rc;
}

__device__ __forceinline__ uint32_t find_contig(const uint64_t* cstart, uint32_t n, uint64_t g) {
    uint32_t lo = 0, hi = n;  // last c with cstart[c] <= g
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) / 2;
        if (cstart[mid] <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void k_syncmer_flags(const uint64_t* words, const uint64_t* word_off, const uint32_t* clen,
                                const uint64_t* cstart, uint32_t ncontig, uint64_t total, SeedParams p,
                                uint8_t* flags) {
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < total;
         g += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t c = find_contig(cstart, ncontig, g);
        uint64_t pos = g - cstart[c];
        uint8_t f = 0;
        if (pos + p.k <= clen[c]) {
            const uint64_t* w = words + word_off[c];
            uint64_t mn = UINT64_MAX, ht = 0;
            for (uint32_t q = 0; q <= p.k - p.s; q++) {
                uint64_t h = xxh64_u64(canonical(w, pos + q, p.s, nullptr));
                mn = h < mn ? h : mn;
                if (q == p.t - 1) ht = h;
            }
            f = ht == mn;
        }
        flags[g] = f;
    }
}

struct SyncmerRec {
    uint64_t hash;
    uint32_t pos;
    uint32_t contig_fwd;  // contig << 1 | is_forward
};

__global__ void k_syncmer_info(const uint64_t* words, const uint64_t* word_off, const uint64_t* cstart,
                               uint32_t ncontig, const uint64_t* gpos, const uint64_t* count, SeedParams p,
                               SyncmerRec* out) {
    uint64_t n = *count;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t g = gpos[i];
        uint32_t c = find_contig(cstart, ncontig, g);
        uint64_t pos = g - cstart[c];
        bool fwd;
        uint64_t v = canonical(words + word_off[c], pos, p.k, &fwd);
        out[i] = SyncmerRec{xxh64_u64(v), (uint32_t)pos, (c << 1) | (fwd ? 1u : 0u)};
    }
}

// src/seeding/strobes.rs:145-176 + src/indexer.rs:239-250
__global__ void k_ref_randstrobes(const SyncmerRec* sy, const uint64_t* count, SeedParams p, RefRandstrobe* out) {
    uint64_t n = *count;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        SyncmerRec s1 = sy[i];
        uint32_t c = s1.contig_fwd >> 1;
        uint64_t maxpos = (uint64_t)s1.pos + p.max_dist;
        uint64_t best = UINT64_MAX;
        SyncmerRec s2 = s1;
        for (uint64_t j = i + p.w_min; j <= i + p.w_max && j < n; j++) {
            SyncmerRec cj = sy[j];
            if ((cj.contig_fwd >> 1) != c) break;
            if (cj.pos > maxpos) break;
            uint64_t ones = (uint64_t)__popcll((s1.hash ^ cj.hash) & p.q);
            if (ones < best) {
                best = ones;
                s2 = cj;
            }
        }
        uint64_t h = randstrobe_hash(s1.hash, s2.hash, s1.contig_fwd & 1, s2.contig_fwd & 1, p);
        uint64_t off = (uint8_t)(s2.pos - s1.pos);
        out[i] = RefRandstrobe{(h & HASH_MASK) | off, s1.pos, c};
    }
}

struct RsDecomposer {
    __host__ __device__ ::cuda::std::tuple<uint64_t&, uint32_t&, uint32_t&> operator()(RefRandstrobe& r) const {
        return {r.hash_offset, r.position, r.ref_index};
    }
};

// Bucket directory exactly as src/indexer.rs:82-124 fills it: bucket_starts[0] = 0,
// and for x >= 1 the first position p >= 1 that starts a new hash with top bits
// >= x (N if none).  Entry 0 only ever starts bucket 0, so when the smallest hash
// has top bits t > 0, buckets 1..t begin at the end of its run.
__global__ void k_buckets(const RefRandstrobe* rs, uint64_t n, uint32_t bits, uint64_t* buckets) {
    const uint64_t nb = (1ULL << bits) + 1;
    const uint64_t h0 = n ? rs_hash(rs[0]) : 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i <= n; i += (uint64_t)gridDim.x * blockDim.x) {
        int64_t lo, hi;
        if (i == 0) {
            lo = -1;
            hi = n == 0 ? (int64_t)nb - 1 : 0;
        } else {
            uint64_t hp = rs_hash(rs[i - 1]);
            if (i < n && rs_hash(rs[i]) == hp) continue;  // not the start of a new hash
            lo = hp == h0 ? 0 : (int64_t)(hp >> (64 - bits));
            hi = i == n ? (int64_t)nb - 1 : (int64_t)(rs_hash(rs[i]) >> (64 - bits));
        }
        for (int64_t x = lo + 1; x <= hi; x++) buckets[x] = i;
    }
}

// run lengths of equal hashes -> histogram of counts (capped at 101) + number of
// distinct hashes (src/indexer.rs:82-137)
__global__ void k_run_hist(const RefRandstrobe* rs, uint64_t n, unsigned long long* hist, unsigned long long* unique) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t h = rs_hash(rs[i]);
        if (i > 0 && rs_hash(rs[i - 1]) == h) continue;
        atomicAdd(unique, 1ULL);
        uint64_t e = i + 1;
        while (e < n && rs_hash(rs[e]) == h) e++;
        uint64_t c = e - i;
        atomicAdd(&hist[c > 101 ? 101 : c], 1ULL);
    }
}

__global__ void k_lookup(DevIndex ix, const uint64_t* hashes, uint64_t n, int kind, int64_t* out_pos,
                         uint32_t* out_count) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t mask = kind == 0 ? HASH_MASK : kind == 1 ? ix.p.main_mask : ix.p.fwd_main_mask;
        uint64_t pos = idx_get_masked_from(ix, hashes[i], mask, false, 0);
        out_pos[i] = pos == UINT64_MAX ? -1 : (int64_t)pos;
        if (out_count) out_count[i] = pos == UINT64_MAX ? 0 : idx_get_count(ix, pos, mask);
    }
}

__global__ void k_extent(const RefRandstrobe* rs, uint64_t n, unsigned int* out) {
    unsigned int mp = 0, mr = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        mp = max(mp, rs[i].position);
        mr = max(mr, rs[i].ref_index);
    }
    atomicMax(out, mp);
    atomicMax(out + 1, mr);
}

inline unsigned grid_for(uint64_t n, unsigned block) {
    uint64_t g = (n + block - 1) / block;
    if (g > sm_count() * 64) g = sm_count() * 64;
    return (unsigned)(g == 0 ? 1 : g);
}

}  // namespace

void build_index_gpu(const std::vector<Contig>& contigs, const SeedParams& sp, uint32_t bits, double filter_fraction,
                     sa_index& idx, cudaStream_t st) {
    const uint32_t nc = (uint32_t)contigs.size();
    std::vector<uint64_t> word_off(nc), cstart(nc + 1, 0);
    std::vector<uint32_t> clen(nc);
    uint64_t nwords = 0;
    for (uint32_t c = 0; c < nc; c++) {
        word_off[c] = nwords;
        nwords += contigs[c].words.size() + 1;  // one guard word per contig
        clen[c] = (uint32_t)contigs[c].len;
        cstart[c + 1] = cstart[c] + contigs[c].len;
    }
    const uint64_t total = cstart[nc];
    DevBuf<uint64_t> d_words, d_woff, d_cstart;
    DevBuf<uint32_t> d_clen;
    d_words.reserve(nwords);
    d_woff.reserve(nc);
    d_cstart.reserve(nc + 1);
    d_clen.reserve(nc);
    {
        std::vector<uint64_t> hw(nwords, 0);
        for (uint32_t c = 0; c < nc; c++)
            std::copy(contigs[c].words.begin(), contigs[c].words.end(), hw.begin() + word_off[c]);
        SA_CUDA(cudaMemcpyAsync(d_words.p, hw.data(), nwords * 8, cudaMemcpyHostToDevice, st));
        SA_CUDA(cudaMemcpyAsync(d_woff.p, word_off.data(), nc * 8, cudaMemcpyHostToDevice, st));
        SA_CUDA(cudaMemcpyAsync(d_cstart.p, cstart.data(), (nc + 1) * 8, cudaMemcpyHostToDevice, st));
        SA_CUDA(cudaMemcpyAsync(d_clen.p, clen.data(), nc * 4, cudaMemcpyHostToDevice, st));
        SA_CUDA(cudaStreamSynchronize(st));
    }
    // (1) syncmer flags
    DevBuf<uint8_t> d_flags;
    d_flags.reserve(total);
    if (total)
        k_syncmer_flags<<<grid_for(total, 256), 256, 0, st>>>(d_words.p, d_woff.p, d_clen.p, d_cstart.p, nc, total, sp,
                                                             d_flags.p);
    // (2) compaction in position order
    DevBuf<uint64_t> d_gpos, d_count;
    d_gpos.reserve(total + 1);
    d_count.reserve(1);
    SA_CUDA(cudaMemsetAsync(d_count.p, 0, 8, st));
    if (total) {
        size_t tmp = 0;
        thrust::counting_iterator<uint64_t> it(0);
        cub::DeviceSelect::Flagged(nullptr, tmp, it, d_flags.p, d_gpos.p, d_count.p, (int64_t)total, st);
        DevBuf<uint8_t> d_tmp;
        d_tmp.reserve(tmp);
        cub::DeviceSelect::Flagged(d_tmp.p, tmp, it, d_flags.p, d_gpos.p, d_count.p, (int64_t)total, st);
    }
    uint64_t nsy = 0;
    SA_CUDA(cudaMemcpyAsync(&nsy, d_count.p, 8, cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaStreamSynchronize(st));
    d_flags.release();
    // (3) syncmers -> randstrobes (one per syncmer, src/seeding/strobes.rs:216-238)
    DevBuf<SyncmerRec> d_sy;
    d_sy.reserve(nsy);
    if (nsy) k_syncmer_info<<<grid_for(nsy, 256), 256, 0, st>>>(d_words.p, d_woff.p, d_cstart.p, nc, d_gpos.p, d_count.p, sp, d_sy.p);
    d_gpos.release();
    DevBuf<RefRandstrobe> d_unsorted;
    d_unsorted.reserve(nsy);
    if (nsy) k_ref_randstrobes<<<grid_for(nsy, 256), 256, 0, st>>>(d_sy.p, d_count.p, sp, d_unsorted.p);
    SA_CUDA(cudaStreamSynchronize(st));
    SA_CUDA(cudaGetLastError());
    d_sy.release();
    // (4) sort on (hash_offset, position, ref_index)
    idx.rs.reserve(nsy);
    if (nsy) {
        size_t tmp = 0;
        cub::DeviceRadixSort::SortKeys(nullptr, tmp, d_unsorted.p, idx.rs.p, (int64_t)nsy, RsDecomposer{}, 0, 128, st);
        DevBuf<uint8_t> d_tmp;
        d_tmp.reserve(tmp);
        cub::DeviceRadixSort::SortKeys(d_tmp.p, tmp, d_unsorted.p, idx.rs.p, (int64_t)nsy, RsDecomposer{}, 0, 128, st);
        SA_CUDA(cudaStreamSynchronize(st));
    }
    d_unsorted.release();
    // (5) bucket directory and filter cutoff
    uint64_t nb = (1ULL << bits) + 1;
    idx.buckets.reserve(nb);
    k_buckets<<<grid_for(nsy + 1, 256), 256, 0, st>>>(idx.rs.p, nsy, bits, idx.buckets.p);
    DevBuf<unsigned long long> d_hist;
    d_hist.reserve(103);
    SA_CUDA(cudaMemsetAsync(d_hist.p, 0, 103 * 8, st));
    if (nsy) k_run_hist<<<grid_for(nsy, 256), 256, 0, st>>>(idx.rs.p, nsy, d_hist.p, d_hist.p + 102);
    unsigned long long hist[103];
    SA_CUDA(cudaMemcpyAsync(hist, d_hist.p, sizeof(hist), cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaStreamSynchronize(st));
    SA_CUDA(cudaGetLastError());
    uint64_t unique = hist[102];
    // counts of repeated hashes sorted descending; the entry at index_cutoff, clamped
    uint64_t n_rep = 0;
    for (int c = 2; c <= 101; c++) n_rep += hist[c];
    uint64_t index_cutoff = (uint64_t)((double)unique * filter_fraction);
    uint64_t cutoff;
    if (index_cutoff < n_rep) {
        // value v with (#counts >= v) > index_cutoff >= (#counts > v); bin 101 stands for >= 101
        uint64_t above = 0;
        cutoff = 2;
        for (int c = 101; c >= 2; c--) {
            above += hist[c];
            if (above > index_cutoff) { cutoff = (uint64_t)c; break; }
        }
    } else if (n_rep > 0) {
        cutoff = 101;
        for (int c = 2; c <= 101; c++)
            if (hist[c]) { cutoff = (uint64_t)c; break; }
    } else {
        cutoff = 30;
    }
    if (cutoff < 30) cutoff = 30;
    if (cutoff > 100) cutoff = 100;
    idx.filter_cutoff = (uint32_t)cutoff;
    idx.bits = bits;
    idx.n = nsy;
    idx.sp = sp;
}

void index_extent_gpu(const sa_index& idx, uint32_t& max_pos, uint32_t& max_ref, cudaStream_t st) {
    DevBuf<unsigned int> d;
    d.reserve(2);
    SA_CUDA(cudaMemsetAsync(d.p, 0, 8, st));
    if (idx.n) k_extent<<<grid_for(idx.n, 256), 256, 0, st>>>(idx.rs.p, idx.n, d.p);
    unsigned int h[2];
    SA_CUDA(cudaMemcpyAsync(h, d.p, 8, cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaStreamSynchronize(st));
    max_pos = h[0];
    max_ref = h[1];
}

void lookup_batch_gpu(const sa_index& idx, const uint64_t* hashes, size_t n, int kind, int64_t* out_pos,
                      uint32_t* out_count, cudaStream_t st) {
    if (n == 0) return;
    DevBuf<uint64_t> d_h;
    DevBuf<int64_t> d_p;
    DevBuf<uint32_t> d_c;
    d_h.reserve(n);
    d_p.reserve(n);
    if (out_count) d_c.reserve(n);
    SA_CUDA(cudaMemcpyAsync(d_h.p, hashes, n * 8, cudaMemcpyHostToDevice, st));
    k_lookup<<<grid_for(n, 256), 256, 0, st>>>(idx.view(), d_h.p, n, kind, d_p.p, out_count ? d_c.p : nullptr);
    SA_CUDA(cudaGetLastError());
    SA_CUDA(cudaMemcpyAsync(out_pos, d_p.p, n * 8, cudaMemcpyDeviceToHost, st));
    if (out_count) SA_CUDA(cudaMemcpyAsync(out_count, d_c.p, n * 4, cudaMemcpyDeviceToHost, st));
    SA_CUDA(cudaStreamSynchronize(st));
}

}  // namespace sa
