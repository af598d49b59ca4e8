// Small host-side helpers shared by the batch driver and the session engine.
#pragma once
#include <sys/mman.h>

#include <algorithm>
#include <cstdlib>
#include <memory>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace sa {

// Array of trivially constructible elements allocated without initialisation (a
// vector resize value-initialises what is then overwritten anyway); resize drops the
// contents
template <class T>
struct PodArray {
    std::unique_ptr<T[]> p;
    size_t n = 0, cap = 0;
    void resize(size_t k) {
        if (k > cap) {
            p.reset(new T[k]);
            cap = k;
        }
        n = k;
    }
    T* data() { return p.get(); }
    const T* data() const { return p.get(); }
    size_t size() const { return n; }
    T& operator[](size_t i) { return p[i]; }
    const T& operator[](size_t i) const { return p[i]; }
    T* begin() { return p.get(); }
    T* end() { return p.get() + n; }
};
using RawBytes = PodArray<char>;

// Output buffer for the caller (released with free()): large ones 2 MiB aligned and
// advised to use huge pages, so that the first touch of hundreds of MB faults in few
// pages.
inline char* alloc_output(size_t bytes) {
    if (bytes < (64u << 20)) return (char*)std::malloc(bytes);
    void* p = nullptr;
    if (posix_memalign(&p, 2u << 20, bytes) != 0) return nullptr;
#ifdef MADV_HUGEPAGE
    madvise(p, bytes, MADV_HUGEPAGE);
#endif
    return (char*)p;
}

// fn(begin, end) over [0, n) split into `threads` contiguous ranges on their own threads
template <class F>
inline void parallel_ranges(uint64_t n, unsigned threads, F fn) {
    threads = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(threads, n / 4096 + 1));
    if (threads == 1) {
        fn((uint64_t)0, n);
        return;
    }
    std::vector<std::thread> th;
    for (unsigned t = 0; t < threads; t++) th.emplace_back(fn, n * t / threads, n * (t + 1) / threads);
    for (auto& x : th) x.join();
}

// memcpy split over threads for large copies
inline void parallel_memcpy(void* dst, const void* src, size_t bytes, unsigned threads) {
    const size_t per = (size_t)4 << 20;
    threads = (unsigned)std::max<size_t>(1, std::min<size_t>(threads, bytes / per + 1));
    if (threads == 1) {
        if (bytes) std::memcpy(dst, src, bytes);
        return;
    }
    std::vector<std::thread> th;
    for (unsigned t = 0; t < threads; t++) {
        const size_t a = bytes * t / threads, b = bytes * (t + 1) / threads;
        th.emplace_back([=] { std::memcpy((char*)dst + a, (const char*)src + a, b - a); });
    }
    for (auto& x : th) x.join();
}

// One copy of every chunk's output pieces into dst with up to `threads` threads,
// each copying a run of consecutive pieces of about equal total size.
template <class Chunk>
inline void gather_chunk_outputs(const std::vector<Chunk>& chunks, char* dst, unsigned threads) {
    struct Seg {
        const char* src;
        size_t len;
    };
    std::vector<Seg> segs;
    for (const auto& c : chunks)
        for (const auto& p : c.pieces) segs.push_back(Seg{(p.spec ? c.spec_out.data() : c.out.data()) + p.off, p.len});
    std::vector<size_t> start(segs.size() + 1, 0);
    for (size_t i = 0; i < segs.size(); i++) start[i + 1] = start[i] + segs[i].len;
    const size_t total = start.back();
    threads = std::max(1u, std::min<unsigned>(threads, (unsigned)std::max<size_t>(segs.size(), 1)));
    if (threads == 1 || total < (8u << 20)) {
        for (size_t i = 0; i < segs.size(); i++) std::memcpy(dst + start[i], segs[i].src, segs[i].len);
        return;
    }
    std::vector<std::thread> th;
    size_t first = 0;
    for (unsigned t = 0; t < threads && first < segs.size(); t++) {
        const size_t goal = total * (t + 1) / threads;
        size_t last = first;
        while (last < segs.size() && (start[last + 1] <= goal || last == first)) last++;
        if (t + 1 == threads) last = segs.size();
        th.emplace_back([&, first, last] {
            for (size_t i = first; i < last; i++) std::memcpy(dst + start[i], segs[i].src, segs[i].len);
        });
        first = last;
    }
    for (auto& x : th) x.join();
}

}  // namespace sa
