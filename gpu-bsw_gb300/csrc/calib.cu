// Integer-pipe calibration: measured throughput of the instructions the DP
// cell update is made of, and of the whole per-cell op mix with every operand
// in registers (no shuffles, no loads, full ILP).  The latter is the
// calibrated roofline the pass kernels are compared against; the former shows
// whether the DPX max forms issue at full rate on this GPU.
//
// Each probe thread runs `iters` rounds over 8 independent accumulators;
// clock64() around the timed loop gives ticks per block, and every block of
// the grid is resident at once (grid = SMs x 4 blocks of 256 threads), so
// lane-ops per tick per SM = 4 * 256 * 8 * iters / ticks.  clock64 does not
// advance at the SM clock on GB300 (ncu's active cycles of the same probe are
// about 1.6x its ticks), so the roofline is the cell probes' throughput timed
// with CUDA events: cells / seconds with every SM busy, after a warm-up that
// brings the SM clock up.
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
    // profile words from memory, so that the compiler cannot fold them into the loop
    const unsigned base = (unsigned)sink[1] & 0x01010101u;
#pragma unroll
    for (int c = 0; c < kDualCols; ++c) {
        ho[c] = 0xfffafffau + (threadIdx.x & 7) * 0x10001u + c;
        f[c] = (unsigned)c;
        pa[c] = 0xfd03fdfdu ^ (unsigned)(c * 0x01010101 * (seed & 1)) ^ base;
        pb[c] = 0x03fdfdfdu ^ (base << 1);
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

// The int32 pass's cell block on registers only: 16 columns per application,
// the op sequence of sw_pass.cuh's inner loop for DNA profiles (sign-extending
// prmt score, F, the diagonal add, T, H + open, the serial E chain, row max).
__global__ void __launch_bounds__(256) probe_int32(int iters, int seed, int* sink, long long* cycles) {
    int ho[kDualCols], f[kDualCols];
    unsigned prof[kDualCols];
#pragma unroll
    for (int c = 0; c < kDualCols; ++c) {
        ho[c] = -6 + (int)(threadIdx.x & 7) + c;
        f[c] = c;
        prof[c] = 0xfdfdfd03u ^ (unsigned)(c * 0x01010101 * (seed & 1)) ^ ((unsigned)sink[1 + c] & 0x01010101u);
    }
    const int open = -6 - (seed & 1), ext = -1, gmax = -1;
    int e = (int)threadIdx.x, mrow = 0;
    unsigned acc = 0;
    __syncthreads();
    long long t0 = clock64();
    for (int it = 0; it < iters; ++it) {
        const unsigned sel = (unsigned)(it & 3) * 0x1111u + 0x8880u;
        int diag = open;
        mrow = open;
#pragma unroll
        for (int c = 0; c < kDualCols; ++c) {
            int sp;
            asm volatile("prmt.b32 %0, %1, 0, %2;" : "=r"(sp) : "r"(prof[c]), "r"(sel));
            const int fv = __viaddmax_s32_relu(f[c], ext, ho[c]);
            const int t = __viaddmax_s32(fv, open, diag + sp);
            const int hov = __viaddmax_s32(e, open, t);
            e = __viaddmax_s32_relu(e, gmax, t);
            diag = ho[c];
            ho[c] = hov;
            f[c] = fv;
            if (c & 1) mrow = __vimax3_s32(mrow, ho[c - 1], hov);
        }
        acc ^= (unsigned)mrow;
    }
    __syncthreads();
    long long t1 = clock64();
#pragma unroll
    for (int c = 0; c < kDualCols; ++c) acc ^= (unsigned)(ho[c] ^ f[c]);
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
    e = cudaMalloc(&sink, sizeof(int) * 32);  // [0]: keeps results alive; [1..16]: zero inputs
    if (e == cudaSuccess) e = cudaMemset(sink, 0, sizeof(int) * 32);
    if (e == cudaSuccess) e = cudaMalloc(&cyc, sizeof(long long) * blocks);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    std::vector<long long> h((size_t)blocks);
    // Times one launch; returns its mean ticks per block and its milliseconds.
    auto timed = [&](auto launch, double* ticks, float* ms) -> cudaError_t {
        cudaEventRecord(e0);
        launch();
        cudaEventRecord(e1);
        cudaError_t r = cudaGetLastError();
        if (r == cudaSuccess) r = cudaEventSynchronize(e1);
        if (r == cudaSuccess) r = cudaMemcpy(h.data(), cyc, sizeof(long long) * blocks, cudaMemcpyDeviceToHost);
        if (r != cudaSuccess) return r;
        double avg = 0;
        for (long long v : h) avg += (double)v;
        *ticks = avg / blocks;
        return cudaEventElapsedTime(ms, e0, e1);
    };
    // warm-up: about 15 ms of the dual probe brings the SM clock up
    if (e == cudaSuccess) {
        probe_dual<<<blocks, kProbeThreads>>>(1 << 14, 3, sink, cyc);
        e = cudaGetLastError();
    }
    const int iters = 1 << 15;
    double rates[M_COUNT] = {};
    double per_s[M_COUNT] = {};  // applications per second, all SMs
    double mhz_sum = 0;
    int mhz_n = 0;
    for (int m = 0; e == cudaSuccess && m < M_COUNT; ++m) {
        kProbes[m]<<<blocks, kProbeThreads>>>(64, m, sink, cyc);
        double ticks = 0;
        float ms = 0;
        e = timed([&] { kProbes[m]<<<blocks, kProbeThreads>>>(iters, m, sink, cyc); }, &ticks, &ms);
        if (e != cudaSuccess || ticks <= 0 || ms <= 0) break;
        rates[m] = (double)kProbeBlocksPerSM * kProbeThreads * 8.0 * iters / ticks;
        per_s[m] = (double)blocks * kProbeThreads * 8.0 * iters / (ms * 1e-3);
        mhz_sum += ticks / (ms * 1e3);  // ticks per microsecond
        ++mhz_n;
    }
    // the int32 pass's cell block: kDualCols cells per application
    double int32_rate = 0, int32_per_s = 0;
    if (e == cudaSuccess) {
        const int iters2 = 1 << 14;
        double ticks = 0;
        float ms = 0;
        e = timed([&] { probe_int32<<<blocks, kProbeThreads>>>(iters2, 3, sink, cyc); }, &ticks, &ms);
        if (e == cudaSuccess && ticks > 0 && ms > 0) {
            const double cells = (double)kProbeThreads * kDualCols * iters2;  // per block
            int32_rate = kProbeBlocksPerSM * cells / ticks;
            int32_per_s = blocks * cells / (ms * 1e-3);
        }
    }
    // the dual cell block: 2 * kDualCols cells per application
    double dual_rate = 0, dual_per_s = 0;
    if (e == cudaSuccess) {
        const int iters2 = 1 << 14;
        double ticks = 0;
        float ms = 0;
        e = timed([&] { probe_dual<<<blocks, kProbeThreads>>>(iters2, 3, sink, cyc); }, &ticks, &ms);
        if (e == cudaSuccess && ticks > 0 && ms > 0) {
            const double cells = (double)kProbeThreads * 2.0 * kDualCols * iters2;  // per block
            dual_rate = kProbeBlocksPerSM * cells / ticks;
            dual_per_s = blocks * cells / (ms * 1e-3);
        }
    }
    if (sink) cudaFree(sink);
    if (cyc) cudaFree(cyc);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e != cudaSuccess || mhz_n < M_COUNT || dual_per_s <= 0 || int32_per_s <= 0) return GBSW_ECUDA;
    out->sms = sms;
    out->sm_mhz = mhz_sum / mhz_n;
    out->addmax_relu_s32 = rates[M_ADDMAX_RELU];
    out->max3_relu_s32 = rates[M_MAX3_RELU];
    out->plain_addmax_s32 = rates[M_PLAIN_ADDMAX];
    out->addmax_relu_s16x2 = rates[M_ADDMAX_RELU_16X2];
    out->max3_relu_s16x2 = rates[M_MAX3_RELU_16X2];
    out->iadd_s32 = rates[M_IADD];
    out->cell_dpx = rates[M_CELL_DPX];
    out->cell_plain = rates[M_CELL_PLAIN];
    out->cell_dual = dual_rate;
    out->cell_dpx_gcups = per_s[M_CELL_DPX] / 1e9;
    out->cell_dual_gcups = dual_per_s / 1e9;
    out->cell_int32 = int32_rate;
    out->cell_int32_gcups = int32_per_s / 1e9;
    return GBSW_OK;
}
