// Integer-pipe calibration: measured throughput of the instructions the DP
// cell update is made of, and of the whole per-cell op mix with every operand
// in registers (no shuffles, no loads, full ILP).  The latter is the
// calibrated roofline the pass kernels are compared against; the former shows
// whether the DPX max forms issue at full rate on this GPU.
//
// Each probe thread runs `iters` rounds over 8 independent accumulators;
// clock64() around the timed loop gives cycles per block, and every block of
// the grid is resident at once (grid = SMs x 4 blocks of 256 threads), so
// lane-ops per clock per SM = 4 * 256 * 8 * iters / cycles.
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/gbsw.h"

namespace {

constexpr int kProbeThreads = 256;
constexpr int kProbeBlocksPerSM = 4;

enum Mode {
    M_ADDMAX_RELU = 0,   // __viaddmax_s32_relu
    M_MAX3_RELU,         // __vimax3_s32_relu
    M_PLAIN_ADDMAX,      // max(a + b, c) with plain IADD + IMNMX
    M_ADDMAX_RELU_16X2,  // __viaddmax_s16x2_relu
    M_MAX3_RELU_16X2,    // __vimax3_s16x2_relu
    M_IADD,              // plain add
    M_CELL_DPX,          // whole int32 cell update, DPX forms
    M_CELL_PLAIN,        // whole int32 cell update, plain ops
    M_COUNT
};

// The dual-pair pass's cell block on registers only: 16 columns x 2 pairs
// (int16x2) per application, the exact op sequence of sw_dual.cu's inner loop
// (prmt score, four add-max DPX ops, the serial E chain, row max).
constexpr int kDualCols = 16;
__device__ __forceinline__ unsigned prmt_probe(unsigned a, unsigned b, unsigned sel) {
    unsigned r;
    asm volatile("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(sel));
    return r;
}
__global__ void __launch_bounds__(256) probe_dual(int iters, int seed, int* sink, long long* cycles) {
    unsigned ho[kDualCols], f[kDualCols], pa[kDualCols], pb[kDualCols];
#pragma unroll
    for (int c = 0; c < kDualCols; ++c) {
        ho[c] = 0xfffafffau + (threadIdx.x & 7) * 0x10001u + c;
        f[c] = (unsigned)c;
        pa[c] = 0xfd03fdfdu ^ (unsigned)(c * 0x01010101 * (seed & 1));
        pb[c] = 0x03fdfdfdu;
    }
    const unsigned open2 = 0xfffafffau, ext2 = 0xffffffffu, neg2 = 0x80008000u;
    unsigned e = threadIdx.x, mrow = 0, acc = 0;
    __syncthreads();
    long long t0 = clock64();
    for (int it = 0; it < iters; ++it) {
        const unsigned sel = (unsigned)(it & 3) * 0x11u + (unsigned)((it >> 2) & 3) * 0x1100u + 0xC480u;
        unsigned diag = open2;
        mrow = open2;
#pragma unroll
        for (int c = 0; c < kDualCols; ++c) {
            const unsigned s2 = prmt_probe(pa[c], pb[c], sel);
            const unsigned fv = __viaddmax_s16x2_relu(f[c], ext2, ho[c]);
            const unsigned u2 = __viaddmax_s16x2(diag, s2, neg2);
            const unsigned t = __viaddmax_s16x2(fv, open2, u2);
            const unsigned hov = __viaddmax_s16x2(e, open2, t);
            e = __viaddmax_s16x2_relu(e, ext2, t);
            diag = ho[c];
            ho[c] = hov;
            f[c] = fv;
            if (c & 1) mrow = __vimax3_s16x2(mrow, ho[c - 1], hov);
        }
        acc ^= mrow;
    }
    __syncthreads();
    long long t1 = clock64();
#pragma unroll
    for (int c = 0; c < kDualCols; ++c) acc ^= ho[c] ^ f[c];
    if (acc == 0x7fffffffu) sink[0] = (int)acc;
    if (threadIdx.x == 0) cycles[blockIdx.x] = t1 - t0;
}

// One application per accumulator; a whole DP cell counts as one application.
template <int MODE>
__device__ __forceinline__ void step(int (&a)[8], int (&f)[8], int b, int c) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int nb = a[(k + 1) & 7];
        if constexpr (MODE == M_ADDMAX_RELU) {
            a[k] = __viaddmax_s32_relu(a[k], b, nb);
        } else if constexpr (MODE == M_MAX3_RELU) {
            a[k] = __vimax3_s32_relu(a[k], nb, c);
        } else if constexpr (MODE == M_PLAIN_ADDMAX) {
            a[k] = max(a[k] + b, nb);
        } else if constexpr (MODE == M_ADDMAX_RELU_16X2) {
            a[k] = (int)__viaddmax_s16x2_relu((unsigned)a[k], (unsigned)b, (unsigned)nb);
        } else if constexpr (MODE == M_MAX3_RELU_16X2) {
            a[k] = (int)__vimax3_s16x2_relu((unsigned)a[k], (unsigned)nb, (unsigned)c);
        } else if constexpr (MODE == M_IADD) {
            a[k] = a[k] + nb + b;
        } else {
            // one DP cell: s from a compare, F, E, H, H+open, running max
            constexpr bool D = MODE == M_CELL_DPX;
            int s = ((a[k] & 3) == (b & 3)) ? 5 : -3;
            int fv, ev, h;
            if constexpr (D) {
                fv = __viaddmax_s32_relu(f[k], -1, nb);
                ev = __viaddmax_s32_relu(c, -1, a[k]);
                h = __vimax3_s32_relu(a[k] + s, ev, fv);
            } else {
                fv = max(max(f[k] - 1, nb), 0);
                ev = max(max(c - 1, a[k]), 0);
                h = max(max(a[k] + s, ev), max(fv, 0));
            }
            f[k] = fv;
            a[k] = h - 6;
        }
    }
}

template <int MODE>
__global__ void __launch_bounds__(kProbeThreads) probe(int iters, int seed, int* sink, long long* cycles) {
    int a[8], f[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        a[k] = (int)(threadIdx.x * 7 + k * 13 + seed);
        f[k] = k;
    }
    int b = seed & 7, c = (seed >> 3) & 7;
    __syncthreads();
    long long t0 = clock64();
    for (int it = 0; it < iters; ++it) {
        step<MODE>(a, f, b, c);
        b ^= it;
        c += 1;
    }
    __syncthreads();
    long long t1 = clock64();
    int acc = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) acc ^= a[k] ^ f[k];
    if (acc == 0x7fffffff) sink[0] = acc;  // keeps the loop alive
    if (threadIdx.x == 0) cycles[blockIdx.x] = t1 - t0;
}

typedef void (*ProbeFn)(int, int, int*, long long*);
const ProbeFn kProbes[M_COUNT] = {probe<0>, probe<1>, probe<2>, probe<3>, probe<4>, probe<5>, probe<6>, probe<7>};

}  // namespace

extern "C" int gbsw_calibrate(int device, gbsw_calibration* out) {
    if (!out) return GBSW_EINVAL;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return GBSW_ECUDA;
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return GBSW_ECUDA;
    const int blocks = sms * kProbeBlocksPerSM;
    int* sink = nullptr;
    long long* cyc = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    e = cudaMalloc(&sink, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&cyc, sizeof(long long) * blocks);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    std::vector<long long> h((size_t)blocks);
    const int iters = 1 << 15;
    double rates[M_COUNT] = {};
    double mhz_sum = 0;
    for (int m = 0; e == cudaSuccess && m < M_COUNT; ++m) {
        kProbes[m]<<<blocks, kProbeThreads>>>(64, m, sink, cyc);  // warm-up
        cudaEventRecord(e0);
        kProbes[m]<<<blocks, kProbeThreads>>>(iters, m, sink, cyc);
        cudaEventRecord(e1);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess)
            e = cudaMemcpy(h.data(), cyc, sizeof(long long) * blocks, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) break;
        double avg = 0;
        for (long long v : h) avg += (double)v;
        avg /= blocks;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        rates[m] = (double)kProbeBlocksPerSM * kProbeThreads * 8.0 * iters / avg;
        if (ms > 0) mhz_sum += avg / (ms * 1e3);  // cycles per microsecond = MHz
    }
    if (sink) cudaFree(sink);
    if (cyc) cudaFree(cyc);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e != cudaSuccess) return GBSW_ECUDA;
    out->sms = sms;
    out->addmax_relu_s32 = rates[M_ADDMAX_RELU];
    out->max3_relu_s32 = rates[M_MAX3_RELU];
    out->plain_addmax_s32 = rates[M_PLAIN_ADDMAX];
    out->addmax_relu_s16x2 = rates[M_ADDMAX_RELU_16X2];
    out->max3_relu_s16x2 = rates[M_MAX3_RELU_16X2];
    out->iadd_s32 = rates[M_IADD];
    out->cell_dpx = rates[M_CELL_DPX];
    out->cell_plain = rates[M_CELL_PLAIN];
    out->sm_mhz = mhz_sum / M_COUNT;

    // dual cell block: 2 * kDualCols cells per application
    {
        int* sink2 = nullptr;
        long long* cyc2 = nullptr;
        cudaError_t e2 = cudaMalloc(&sink2, sizeof(int));
        if (e2 == cudaSuccess) e2 = cudaMalloc(&cyc2, sizeof(long long) * blocks);
        const int iters2 = 1 << 12;
        if (e2 == cudaSuccess) {
            probe_dual<<<blocks, kProbeThreads>>>(16, 3, sink2, cyc2);
            probe_dual<<<blocks, kProbeThreads>>>(iters2, 3, sink2, cyc2);
            e2 = cudaGetLastError();
        }
        if (e2 == cudaSuccess) e2 = cudaDeviceSynchronize();
        if (e2 == cudaSuccess) e2 = cudaMemcpy(h.data(), cyc2, sizeof(long long) * blocks, cudaMemcpyDeviceToHost);
        if (sink2) cudaFree(sink2);
        if (cyc2) cudaFree(cyc2);
        if (e2 != cudaSuccess) return GBSW_ECUDA;
        double avg = 0;
        for (long long v : h) avg += (double)v;
        avg /= blocks;
        out->cell_dual = (double)kProbeBlocksPerSM * kProbeThreads * 2.0 * kDualCols * iters2 / avg;
    }
    return GBSW_OK;
}
