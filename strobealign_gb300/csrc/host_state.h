// Host-side state behind the C-ABI handles.
#pragma once
#include <algorithm>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "sa_internal.h"

namespace sa {

#define SA_CUDA(call)                                                                              \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            throw ::sa::Error(e_ == cudaErrorMemoryAllocation ? SA_ERR_OOM : SA_ERR_CUDA,          \
                              std::string(#call) + ": " + cudaGetErrorString(e_));                 \
    } while (0)

// One contig in PackedSeq form (src/packed_seq.rs:11-126).
struct Contig {
    std::string name;
    std::vector<uint64_t> words;
    size_t len = 0;
    void push(uint8_t c);
    uint8_t bits(size_t i) const { return (uint8_t)((words[i >> 5] >> ((i & 31) * 2)) & 3); }
};

void load_fasta(const std::string& path, std::vector<Contig>& out);
void contigs_from_buffers(size_t n, const char* const* names, const char* const* seqs, const size_t* lens,
                          std::vector<Contig>& out);
uint32_t pick_bits(const std::vector<Contig>& cs, const SeedParams& p);

// Owned read records (concatenated buffers with offsets).
struct ReadStore {
    std::string seq, qual, names, comments;
    std::vector<uint64_t> seq_off, name_off, comment_off;
    std::vector<uint8_t> has_comment;
    bool has_qual = false;
    uint64_t qual_off_unused = 0;
};
void load_reads(const std::string& path, ReadStore& rs);

// Streaming multiprocessors of the calling thread's current device; grid sizes are
// capped at multiples of it (queried once per device and thread).
inline uint64_t sm_count() {
    static thread_local int cached_dev = -1;
    static thread_local uint64_t cached = 1;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return cached;
    if (dev != cached_dev) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0) cached = (uint64_t)v;
        cached_dev = dev;
    }
    return cached;
}

// Device buffer with RAII release.
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    // grow-only reallocation; contents are not preserved
    void reserve(size_t count) {
        if (count <= n && p) return;
        release();
        size_t c = std::max<size_t>(count, 1);
        cudaError_t e = cudaMalloc(&p, c * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            throw Error(SA_ERR_OOM, "cudaMalloc of " + std::to_string(c * sizeof(T)) + " bytes failed");
        }
        n = c;
    }
};

// Pinned host buffer, grow-only.
template <class T>
struct PinnedBuf {
    T* p = nullptr;
    size_t n = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() { if (p) cudaFreeHost(p); }
    void reserve(size_t count) {
        if (count <= n && p) return;
        if (p) cudaFreeHost(p);
        p = nullptr;
        size_t c = std::max<size_t>(count, 1);
        if (cudaMallocHost(&p, c * sizeof(T)) != cudaSuccess) {
            p = nullptr;
            throw Error(SA_ERR_OOM, "pinned allocation failed");
        }
        n = c;
    }
};

}  // namespace sa

struct sa_refs {
    std::vector<sa::Contig> contigs;
    size_t total_len = 0;
};

struct sa_reads {
    sa::ReadStore store;
};

struct sa_index {
    sa_seeding_params params;
    sa::SeedParams sp;
    uint32_t bits = 0;
    uint32_t filter_cutoff = 0;
    uint64_t n = 0;
    int device = 0;
    uint32_t max_pos = 0;      // largest strobe-1 position in the table
    uint32_t n_refs_seen = 1;  // largest reference index + 1
    sa::DevBuf<sa::RefRandstrobe> rs;
    sa::DevBuf<uint64_t> buckets;
    sa::DevIndex view() const {
        sa::DevIndex v;
        v.rs = rs.p;
        v.n = n;
        v.buckets = buckets.p;
        v.bits = bits;
        v.filter_cutoff = filter_cutoff;
        v.p = sp;
        return v;
    }
};

namespace sa {
// index.cu
void build_index_gpu(const std::vector<Contig>& contigs, const SeedParams& sp, uint32_t bits, double filter_fraction,
                     sa_index& idx, cudaStream_t stream);
void lookup_batch_gpu(const sa_index& idx, const uint64_t* hashes, size_t n, int kind, int64_t* out_pos,
                      uint32_t* out_count, cudaStream_t stream);
}  // namespace sa
