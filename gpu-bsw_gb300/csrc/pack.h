// Packed sequence streams (the gbsw_packed format of gbsw.h): the host packer
// shared by gbsw_pack and the C++ drop-in's ingest, and the device unpack.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/gbsw.h"

namespace gbsw {

__host__ __device__ constexpr int symbols_per_word(int kind) {
    return kind == GBSW_DNA ? GBSW_DNA_PER_WORD : GBSW_PROTEIN_PER_WORD;
}
__host__ __device__ constexpr int bits_per_symbol(int kind) { return kind == GBSW_DNA ? 2 : 5; }

// Escape runs found while packing, with positions in the packed stream.
struct EscapeRuns {
    std::vector<int64_t> at;     // first raw byte of each run
    std::vector<int64_t> len;    // bytes of each run
    std::vector<uint8_t> bytes;  // the runs' bytes, back to back
    // Appends a run, merging it into the last one when they touch.
    void add(int64_t pos, const char* s, int64_t n) {
        if (n <= 0) return;
        if (!at.empty() && at.back() + len.back() == pos) {
            len.back() += n;
        } else {
            at.push_back(pos);
            len.push_back(n);
        }
        bytes.insert(bytes.end(), s, s + n);
    }
    void append(const EscapeRuns& o) {
        for (size_t r = 0, b = 0; r < o.at.size(); b += (size_t)o.len[r], ++r)
            add(o.at[r], reinterpret_cast<const char*>(o.bytes.data()) + b, o.len[r]);
    }
    void clear() {
        at.clear();
        len.clear();
        bytes.clear();
    }
};

// Packs `len` raw bytes that start at symbol `pos` of a stream, where `pos` is
// a multiple of the symbols per word: writes the ceil(len / per word) words
// from words[0] (the last one zero-filled past the end) and adds the escaped
// bytes' runs, at stream positions, to `esc`.
void pack_span(int kind, const char* s, int64_t len, int64_t pos, uint32_t* words, EscapeRuns* esc);

// Device unpack of a packed stream into out[0 : nsym) (gbsw_unpack_device
// without the argument checks).
cudaError_t launch_unpack(int kind, const gbsw_packed& packed, uint8_t* out, cudaStream_t stream);

}  // namespace gbsw
