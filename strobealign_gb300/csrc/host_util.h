// Small host-side helpers shared by the batch driver and the session engine.
#pragma once
#include <algorithm>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace sa {

// Concatenates parts into dst with up to `threads` threads, each copying a run of
// consecutive parts of about equal total size.
inline void parallel_concat(const std::vector<const std::string*>& parts, char* dst, unsigned threads) {
    size_t total = 0;
    for (auto* p : parts) total += p->size();
    threads = std::max(1u, std::min<unsigned>(threads, (unsigned)parts.size()));
    if (threads == 1 || total < (8u << 20)) {
        size_t o = 0;
        for (auto* p : parts) {
            std::memcpy(dst + o, p->data(), p->size());
            o += p->size();
        }
        return;
    }
    std::vector<size_t> start(parts.size() + 1, 0);
    for (size_t i = 0; i < parts.size(); i++) start[i + 1] = start[i] + parts[i]->size();
    std::vector<std::thread> th;
    size_t first = 0;
    for (unsigned t = 0; t < threads && first < parts.size(); t++) {
        const size_t goal = total * (t + 1) / threads;
        size_t last = first;
        while (last < parts.size() && (start[last + 1] <= goal || last == first)) last++;
        if (t + 1 == threads) last = parts.size();
        th.emplace_back([&, first, last] {
            for (size_t i = first; i < last; i++) std::memcpy(dst + start[i], parts[i]->data(), parts[i]->size());
        });
        first = last;
    }
    for (auto& x : th) x.join();
}

}  // namespace sa
