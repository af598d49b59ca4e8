// Optional per-kernel timing with CUDA events recorded on the launching stream.
#pragma once
#include <cuda_runtime.h>

#include <vector>

namespace sa {

enum KSlot : int {
    KS_SEED = 0, KS_HITS, KS_ANCHORS, KS_SORT, KS_CHAIN, KS_NAMS_OTHER,
    KS_PREPARE, KS_FILL, KS_SW_BYTE, KS_SW_WORD, KS_BAND, KS_FINALIZE, KS_EXT_OTHER, KS_COUNT
};

struct KernelTimers {
    bool enabled = false;
    double ms[KS_COUNT] = {};
    uint64_t launches[KS_COUNT] = {};
    struct Rec { int slot; cudaEvent_t a, b; };
    std::vector<Rec> open;
    std::vector<cudaEvent_t> pool;
    cudaEvent_t get() {
        if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
    void begin(int slot, cudaStream_t st) {
        if (!enabled) return;
        Rec r{slot, get(), get()};
        cudaEventRecord(r.a, st);
        open.push_back(r);
    }
    void end(cudaStream_t st) {
        if (!enabled || open.empty()) return;
        cudaEventRecord(open.back().b, st);
    }
    void collect() {
        for (auto& r : open) {
            cudaEventSynchronize(r.b);
            float t = 0;
            cudaEventElapsedTime(&t, r.a, r.b);
            ms[r.slot] += t;
            launches[r.slot]++;
            pool.push_back(r.a);
            pool.push_back(r.b);
        }
        open.clear();
    }
    void reset() {
        for (int i = 0; i < KS_COUNT; i++) { ms[i] = 0; launches[i] = 0; }
    }
    ~KernelTimers() {
        for (auto& r : open) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
        for (auto e : pool) cudaEventDestroy(e);
    }
};

}  // namespace sa
