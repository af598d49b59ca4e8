// Integer-ALU throughput of the device, measured: the denominator of the Smith-Waterman
// rooflines.  Every thread runs eight independent chains of the two instruction forms
// the SSW and banded kernels are made of (a fused add-then-max, and a max), so the
// issue rate, not latency, bounds the loop.
#include <cuda_runtime.h>

#include "host_state.h"
#include "strobealign_gb300.h"

namespace sa {
namespace {

constexpr int PROBE_ITERS = 4096;
constexpr int PROBE_CHAINS = 8;

__global__ void __launch_bounds__(256) k_alu_probe(int* out, int seed, int fused) {
    int a[PROBE_CHAINS];
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; c++) a[c] = seed + c + (int)threadIdx.x;
    const int b = seed & 7, lim = seed >> 3;
    if (fused) {
        for (int i = 0; i < PROBE_ITERS; i++) {
#pragma unroll
            for (int c = 0; c < PROBE_CHAINS; c++) a[c] = __viaddmax_s32(a[c], b, lim);
        }
    } else {
        for (int i = 0; i < PROBE_ITERS; i++) {
#pragma unroll
            for (int c = 0; c < PROBE_CHAINS; c++) a[c] = max(a[c], lim + c) ^ b;
        }
    }
    int s = 0;
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; c++) s += a[c];
    if (s == 0x7fffffff) out[0] = s;  // keeps the chains live; never true for these seeds
}

}  // namespace
}  // namespace sa

// Instructions per second of each form, the median of five timed launches over the
// whole device (after one warm-up launch).  out[0]: add-then-max (one instruction),
// out[1]: max plus xor (two instructions, counted as two).
extern "C" int32_t sa_measure_int_alu(double* out) {
    using namespace sa;
    if (!out) return SA_ERR_INVALID;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SA_ERR_CUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return SA_ERR_CUDA;
    int* d = nullptr;
    if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return SA_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const unsigned blocks = (unsigned)sms * 8, threads = 256;
    int32_t rc = SA_OK;
    for (int form = 0; form < 2 && rc == SA_OK; form++) {
        const double ops_per_iter = form == 0 ? 1.0 : 2.0;
        k_alu_probe<<<blocks, threads>>>(d, 1 << 4, form == 0);
        float ms[5];
        for (int r = 0; r < 5; r++) {
            cudaEventRecord(e0);
            k_alu_probe<<<blocks, threads>>>(d, 1 << 4, form == 0);
            cudaEventRecord(e1);
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                rc = SA_ERR_CUDA;
                break;
            }
            cudaEventElapsedTime(&ms[r], e0, e1);
        }
        if (rc != SA_OK) break;
        for (int i = 0; i < 5; i++)
            for (int j = i + 1; j < 5; j++)
                if (ms[j] < ms[i]) {
                    const float t = ms[i];
                    ms[i] = ms[j];
                    ms[j] = t;
                }
        const double ops = (double)blocks * threads * PROBE_ITERS * PROBE_CHAINS * ops_per_iter;
        out[form] = ms[2] > 0 ? ops / (ms[2] * 1e-3) : 0.0;
    }
    if (cudaGetLastError() != cudaSuccess) rc = SA_ERR_CUDA;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    return rc;
}
