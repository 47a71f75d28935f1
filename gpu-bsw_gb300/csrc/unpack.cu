// Device unpack of gbsw_packed streams into the raw byte buffers the passes
// read.  HBM-bound: each DNA word becomes one 16-byte store, each eight protein
// words three; escape runs are copied over afterwards, one warp per run.
#include <algorithm>

#include "pack.h"

namespace gbsw {
namespace {

constexpr int kUnpackThreads = 256;
// The DNA letters by code: byte c of the word is the letter of code c.
constexpr unsigned kDnaLetters = 'A' | ('C' << 8) | ('T' << 16) | ('G' << 24);

// Four 2-bit codes (x, lowest first) -> their four letters, one per byte.
__device__ __forceinline__ unsigned dna4(unsigned x) {
    const unsigned sel = (x & 3u) | ((x & 0xcu) << 2) | ((x & 0x30u) << 4) | ((x & 0xc0u) << 6);
    return __byte_perm(kDnaLetters, 0, sel);
}

template <bool ALIGNED>
__global__ void __launch_bounds__(kUnpackThreads) unpack_dna(const uint32_t* __restrict__ words, int64_t nsym,
                                                              uint8_t* __restrict__ out) {
    const int64_t nwords = (nsym + GBSW_DNA_PER_WORD - 1) / GBSW_DNA_PER_WORD;
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nwords;
         w += (int64_t)gridDim.x * blockDim.x) {
        const unsigned x = __ldg(words + w);
        const int64_t at = w * GBSW_DNA_PER_WORD;
        if (ALIGNED && at + GBSW_DNA_PER_WORD <= nsym) {
            *reinterpret_cast<uint4*>(out + at) =
                make_uint4(dna4(x & 0xffu), dna4((x >> 8) & 0xffu), dna4((x >> 16) & 0xffu), dna4(x >> 24));
        } else {
            const int64_t left = nsym - at;
            const int m = left < GBSW_DNA_PER_WORD ? (int)left : GBSW_DNA_PER_WORD;
            for (int j = 0; j < m; ++j) out[at + j] = (uint8_t)(kDnaLetters >> (8 * ((x >> (2 * j)) & 3u)));
        }
    }
}

// Eight words (48 residues, three 16-byte stores) per thread.
constexpr int kAaWordsPerThread = 8;
constexpr int kAaSymsPerThread = kAaWordsPerThread * GBSW_PROTEIN_PER_WORD;

template <bool ALIGNED>
__global__ void __launch_bounds__(kUnpackThreads) unpack_protein(const uint32_t* __restrict__ words, int64_t nsym,
                                                                  uint8_t* __restrict__ out) {
    const int64_t ngroups = (nsym + kAaSymsPerThread - 1) / kAaSymsPerThread;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ngroups;
         g += (int64_t)gridDim.x * blockDim.x) {
        const int64_t at = g * kAaSymsPerThread;
        const uint32_t* src = words + g * kAaWordsPerThread;
        if (ALIGNED && at + kAaSymsPerThread <= nsym) {
            unsigned o[kAaSymsPerThread / 4];
#pragma unroll
            for (int k = 0; k < kAaSymsPerThread / 4; ++k) o[k] = 0;
#pragma unroll
            for (int k = 0; k < kAaWordsPerThread; ++k) {
                const unsigned x = __ldg(src + k);
#pragma unroll
                for (int j = 0; j < GBSW_PROTEIN_PER_WORD; ++j) {
                    const int s = k * GBSW_PROTEIN_PER_WORD + j;
                    o[s >> 2] |= (((x >> (5 * j)) & 31u) + 'A') << (8 * (s & 3));
                }
            }
            uint4* dst = reinterpret_cast<uint4*>(out + at);
            dst[0] = make_uint4(o[0], o[1], o[2], o[3]);
            dst[1] = make_uint4(o[4], o[5], o[6], o[7]);
            dst[2] = make_uint4(o[8], o[9], o[10], o[11]);
        } else {
            const int64_t end = at + kAaSymsPerThread < nsym ? at + kAaSymsPerThread : nsym;
            for (int64_t s = at; s < end; ++s) {
                const unsigned x = __ldg(words + s / GBSW_PROTEIN_PER_WORD);
                out[s] = (uint8_t)(((x >> (5 * (int)(s % GBSW_PROTEIN_PER_WORD))) & 31u) + 'A');
            }
        }
    }
}

// Escape runs over the unpacked symbols, one warp per run; writes outside
// out[0 : nsym) are dropped.
__global__ void __launch_bounds__(kUnpackThreads) unpack_escapes(const int64_t* __restrict__ run_at,
                                                                  const int64_t* __restrict__ run_off,
                                                                  const uint8_t* __restrict__ bytes, int64_t nruns,
                                                                  int64_t nsym, uint8_t* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * blockDim.x / 32;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; r < nruns; r += warps) {
        const int64_t at = run_at[r], b = run_off[r], len = run_off[r + 1] - b;
        for (int64_t j = lane; j < len; j += 32) {
            const int64_t pos = at + j;
            if (pos >= 0 && pos < nsym) out[pos] = bytes[b + j];
        }
    }
}

int grid_for(int64_t items, int per_block) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
        sms = 1;
    return (int)std::max<int64_t>(1, std::min<int64_t>((items + per_block - 1) / per_block, (int64_t)sms * 8));
}

}  // namespace

cudaError_t launch_unpack(int kind, const gbsw_packed& p, uint8_t* out, cudaStream_t stream) {
    if (p.nsym <= 0) return cudaSuccess;
    const bool aligned = (reinterpret_cast<uintptr_t>(out) & 15u) == 0;
    if (kind == GBSW_DNA) {
        const int64_t items = (p.nsym + GBSW_DNA_PER_WORD - 1) / GBSW_DNA_PER_WORD;
        const int grid = grid_for(items, kUnpackThreads);
        if (aligned)
            unpack_dna<true><<<grid, kUnpackThreads, 0, stream>>>(p.words, p.nsym, out);
        else
            unpack_dna<false><<<grid, kUnpackThreads, 0, stream>>>(p.words, p.nsym, out);
    } else {
        const int64_t items = (p.nsym + kAaSymsPerThread - 1) / kAaSymsPerThread;
        const int grid = grid_for(items, kUnpackThreads);
        if (aligned)
            unpack_protein<true><<<grid, kUnpackThreads, 0, stream>>>(p.words, p.nsym, out);
        else
            unpack_protein<false><<<grid, kUnpackThreads, 0, stream>>>(p.words, p.nsym, out);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && p.nruns > 0) {
        const int grid = grid_for(p.nruns, kUnpackThreads / 32);
        unpack_escapes<<<grid, kUnpackThreads, 0, stream>>>(p.run_at, p.run_off, p.run_bytes, p.nruns, p.nsym, out);
        e = cudaGetLastError();
    }
    return e;
}

}  // namespace gbsw

extern "C" int gbsw_unpack_device(int kind, const gbsw_packed* packed, uint8_t* out, void* stream) {
    if ((kind != GBSW_DNA && kind != GBSW_PROTEIN) || !packed || packed->nsym < 0 || packed->nruns < 0)
        return GBSW_EINVAL;
    if (packed->nsym == 0) return GBSW_OK;
    if (!out || !packed->words) return GBSW_EINVAL;
    if (packed->nruns > 0 && (!packed->run_at || !packed->run_off || !packed->run_bytes)) return GBSW_EINVAL;
    return gbsw::launch_unpack(kind, *packed, out, static_cast<cudaStream_t>(stream)) == cudaSuccess ? GBSW_OK
                                                                                                    : GBSW_ECUDA;
}
