// Small host-side helpers shared by the batch driver and the session engine.
#pragma once
#include <sys/mman.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace sa {

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
