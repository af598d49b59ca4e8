// Small host-side helpers shared by the batch driver and the session engine.
#pragma once
#include <sys/mman.h>

#include <algorithm>
#include <cstdlib>
#include <memory>
#include <mutex>
#include <unordered_map>
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
    void clear() { n = 0; }
    T& operator[](size_t i) { return p[i]; }
    const T& operator[](size_t i) const { return p[i]; }
    T* begin() { return p.get(); }
    T* end() { return p.get() + n; }
};
using RawBytes = PodArray<char>;

// Growable byte buffer for formatted output.  Unlike std::string it grows without
// zero-filling: tail(bound) hands out room for a write of at most bound bytes and
// commit(end) keeps what was written, so a record is formatted in place.
class OutBuf {
  public:
    size_t size() const { return n_; }
    bool empty() const { return n_ == 0; }
    const char* data() const { return p_.get(); }
    char* data() { return p_.get(); }
    void clear() { n_ = 0; }
    void reserve(size_t k) {
        if (k > cap_) grow(k);
    }
    void resize(size_t k) {  // bytes past the old size are not initialised
        if (k > cap_) grow(k);
        n_ = k;
    }
    char* tail(size_t bound) {
        if (n_ + bound > cap_) grow(n_ + bound);
        return p_.get() + n_;
    }
    void commit(const char* end) { n_ = (size_t)(end - p_.get()); }
    void append(const char* s, size_t k) {
        if (k) std::memcpy(tail(k), s, k);
        n_ += k;
    }
    void push_back(char c) {
        *tail(1) = c;
        n_++;
    }
    OutBuf& operator+=(const std::string& s) {
        append(s.data(), s.size());
        return *this;
    }
    OutBuf& operator+=(const char* s) {
        append(s, std::strlen(s));
        return *this;
    }

  private:
    void grow(size_t need) {
        size_t c = cap_ * 2 > need ? cap_ * 2 : need;
        if (c < 4096) c = 4096;
        std::unique_ptr<char[]> q(new char[c]);
        if (n_) std::memcpy(q.get(), p_.get(), n_);
        p_ = std::move(q);
        cap_ = c;
    }
    std::unique_ptr<char[]> p_;
    size_t n_ = 0, cap_ = 0;
};

// Output buffers handed to the caller (released with release_output, which
// sa_output_free calls).  Large ones are 2 MiB aligned and advised to use huge pages,
// and a few released ones are kept for reuse: a stream of batches then writes its SAM
// into memory that is already paged in instead of faulting in hundreds of MB each time.
class OutputPool {
  public:
    static constexpr size_t LARGE = (size_t)64 << 20;
    char* alloc(size_t bytes) {
        if (bytes < LARGE) return (char*)std::malloc(bytes);
        std::lock_guard<std::mutex> g(mu_);
        size_t best = free_.size();
        for (size_t i = 0; i < free_.size(); i++)
            if (free_[i].second >= bytes && (best == free_.size() || free_[i].second < free_[best].second)) best = i;
        if (best < free_.size()) {
            const auto it = free_[best];
            free_.erase(free_.begin() + (ptrdiff_t)best);
            kept_ -= it.second;
            caps_[it.first] = it.second;
            return it.first;
        }
        void* p = nullptr;
        if (posix_memalign(&p, (size_t)2 << 20, bytes) != 0) return nullptr;
#ifdef MADV_HUGEPAGE
        madvise(p, bytes, MADV_HUGEPAGE);
#endif
        caps_[(char*)p] = bytes;
        return (char*)p;
    }
    void release(char* p) {
        if (!p) return;
        std::lock_guard<std::mutex> g(mu_);
        const auto it = caps_.find(p);
        if (it == caps_.end()) {
            std::free(p);
            return;
        }
        const size_t cap = it->second;
        caps_.erase(it);
        if (free_.size() < 4 && kept_ + cap <= ((size_t)8 << 30)) {
            free_.emplace_back(p, cap);
            kept_ += cap;
        } else {
            std::free(p);
        }
    }

  private:
    std::mutex mu_;
    std::unordered_map<char*, size_t> caps_;        // large buffers handed out
    std::vector<std::pair<char*, size_t>> free_;    // released, kept for reuse
    size_t kept_ = 0;
};

inline OutputPool& output_pool() {
    static OutputPool pool;
    return pool;
}
inline char* alloc_output(size_t bytes) { return output_pool().alloc(bytes); }
inline void release_output(char* p) { output_pool().release(p); }

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

// A chunk's output pieces, in order, into dst (one thread).
template <class Chunk>
inline void copy_chunk_output(const Chunk& c, char* dst) {
    for (const auto& p : c.pieces) {
        std::memcpy(dst, (p.spec ? c.spec_out.data() : c.out.data()) + p.off, p.len);
        dst += p.len;
    }
}

// One copy of the output pieces of chunks [chunk0, end) into dst with up to `threads`
// threads, each copying a run of consecutive pieces of about equal total size.
template <class Chunk>
inline void gather_chunk_outputs(const std::vector<Chunk>& chunks, char* dst, unsigned threads, size_t chunk0 = 0) {
    struct Seg {
        const char* src;
        size_t len;
    };
    std::vector<Seg> segs;
    for (size_t ci = chunk0; ci < chunks.size(); ci++) {
        const auto& c = chunks[ci];
        for (const auto& p : c.pieces) segs.push_back(Seg{(p.spec ? c.spec_out.data() : c.out.data()) + p.off, p.len});
    }
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
