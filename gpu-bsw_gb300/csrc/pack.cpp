// Host packer of the gbsw_packed format: 2-bit DNA and 5-bit protein codes in
// 32-bit words, with runs of bytes outside the alphabet kept raw.  The
// reference copies raw bytes (utils.cpp:30-54); the packed form carries the
// same bytes in a quarter (DNA) or 5/8 (protein) of the space, and unpacks to
// exactly the bytes it came from, so every scoring rule of the passes -- raw
// byte compares of DNA (kernel.cpp:366), the protein encoding table
// (driver.cpp:252-258) and its error for symbols outside it -- sees the
// caller's bytes unchanged.
#include "pack.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>

namespace gbsw {
namespace {

// byte -> code; kEscape (code bits 0) for a byte outside the alphabet
constexpr uint8_t kEscape = 0x80;

struct Tables {
    uint8_t t[2][256];
    Tables() {
        std::memset(t, kEscape, sizeof(t));
        const char dna[4] = {'A', 'C', 'T', 'G'};  // (b >> 1) & 3 of each is its index
        for (int c = 0; c < 4; ++c) t[GBSW_DNA][(uint8_t)dna[c]] = (uint8_t)c;
        for (int c = 0; c < 26; ++c) t[GBSW_PROTEIN]['A' + c] = (uint8_t)c;
    }
};
const Tables kTables;

// Adds the escaped bytes of one word's symbols s[0 : m) (stream position pos).
void escapes_of(const uint8_t* T, const char* s, int m, int64_t pos, EscapeRuns* esc) {
    for (int j = 0; j < m;) {
        if (!(T[(uint8_t)s[j]] & kEscape)) {
            ++j;
            continue;
        }
        int e = j + 1;
        while (e < m && (T[(uint8_t)s[e]] & kEscape)) ++e;
        esc->add(pos + j, s + j, e - j);
        j = e;
    }
}

template <int P, int B>
void pack_words(const uint8_t* T, const char* s, int64_t len, int64_t pos, uint32_t* words, EscapeRuns* esc) {
    const int64_t full = len / P;
    for (int64_t w = 0; w < full; ++w) {
        const char* q = s + w * P;
        uint32_t word = 0, flags = 0;
#pragma GCC unroll 16
        for (int j = 0; j < P; ++j) {
            const uint32_t c = T[(uint8_t)q[j]];
            flags |= c;
            word |= (c & 31u) << (B * j);
        }
        words[w] = word;
        if (flags & kEscape) escapes_of(T, q, P, pos + w * P, esc);
    }
    const int rest = (int)(len - full * P);
    if (rest > 0) {
        const char* q = s + full * P;
        uint32_t word = 0, flags = 0;
        for (int j = 0; j < rest; ++j) {
            const uint32_t c = T[(uint8_t)q[j]];
            flags |= c;
            word |= (c & 31u) << (B * j);
        }
        words[full] = word;
        if (flags & kEscape) escapes_of(T, q, rest, pos + full * P, esc);
    }
}

static_assert(__BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__, "the 64-bit DNA packer reads bytes little-endian");

// DNA, eight bytes at a time in one 64-bit word (plain integer operations, the
// same on every host): the codes are (b >> 1) & 3 of each byte; the bytes are
// all A/C/G/T exactly when rebuilding each byte's letter from its code gives
// the bytes back.  With b0, b1 the code's bits, the letter is
// 0x41 + 2 b0 + 0x13 b1 - 0x0f (b0 & b1): A 0x41, C 0x43, T 0x54, G 0x47; no
// byte lane borrows or carries.  Returns the 16 code bits, or -1 when a byte
// is not one of the four letters.
inline int32_t dna8(uint64_t v) {
    constexpr uint64_t kOnes = 0x0101010101010101ull;
    const uint64_t c = (v >> 1) & (3 * kOnes);
    const uint64_t b0 = c & kOnes, b1 = (c >> 1) & kOnes;
    const uint64_t letters = 0x41 * kOnes + 2 * b0 + 0x13 * b1 - 0x0f * (b0 & b1);
    if (letters != v) return -1;
    uint64_t x = (c | (c >> 6)) & 0x000f000f000f000full;  // two codes per 16-bit lane
    x = (x | (x >> 12)) & 0x000000ff000000ffull;          // four per 32-bit lane
    return (int32_t)((x | (x >> 24)) & 0xffffu);
}

void pack_dna(const uint8_t* T, const char* s, int64_t len, int64_t pos, uint32_t* words, EscapeRuns* esc) {
    const int64_t full = len / GBSW_DNA_PER_WORD;
    for (int64_t w = 0; w < full; ++w) {
        const char* q = s + w * GBSW_DNA_PER_WORD;
        uint64_t lo, hi;
        std::memcpy(&lo, q, 8);  // little-endian hosts: byte k is bits 8k..8k+7
        std::memcpy(&hi, q + 8, 8);
        const int32_t a = dna8(lo), b = dna8(hi);
        if (a >= 0 && b >= 0) {
            words[w] = (uint32_t)a | ((uint32_t)b << 16);
        } else {
            pack_words<GBSW_DNA_PER_WORD, 2>(T, q, GBSW_DNA_PER_WORD, pos + w * GBSW_DNA_PER_WORD, words + w, esc);
        }
    }
    const int64_t done = full * GBSW_DNA_PER_WORD;
    if (len > done) pack_words<GBSW_DNA_PER_WORD, 2>(T, s + done, len - done, pos + done, words + full, esc);
}

}  // namespace

void pack_span(int kind, const char* s, int64_t len, int64_t pos, uint32_t* words, EscapeRuns* esc) {
    const uint8_t* T = kTables.t[kind == GBSW_DNA ? GBSW_DNA : GBSW_PROTEIN];
    if (kind == GBSW_DNA)
        pack_dna(T, s, len, pos, words, esc);
    else
        pack_words<GBSW_PROTEIN_PER_WORD, 5>(T, s, len, pos, words, esc);
}

}  // namespace gbsw

extern "C" {

int64_t gbsw_packed_words(int kind, int64_t nsym) {
    if ((kind != GBSW_DNA && kind != GBSW_PROTEIN) || nsym < 0) return -1;
    const int64_t p = gbsw::symbols_per_word(kind);
    return (nsym + p - 1) / p;
}

int gbsw_pack(int kind, const char* raw, int64_t nsym, int threads, uint32_t* words, int64_t run_cap,
              int64_t* run_at, int64_t* run_off, int64_t byte_cap, uint8_t* run_bytes, int64_t* nruns,
              int64_t* nbytes) {
    if ((kind != GBSW_DNA && kind != GBSW_PROTEIN) || nsym < 0 || run_cap < 0 || byte_cap < 0 || !nruns ||
        !nbytes)
        return GBSW_EINVAL;
    if (nsym > 0 && (!raw || !words)) return GBSW_EINVAL;
    if (run_cap > 0 && (!run_at || !run_off)) return GBSW_EINVAL;
    if (byte_cap > 0 && !run_bytes) return GBSW_EINVAL;
    const int64_t per = gbsw::symbols_per_word(kind);
    // chunks of whole words, packed independently; runs that meet at a chunk
    // edge are merged when the chunks' runs are joined
    const int64_t chunk = per * 65536;
    const int64_t nchunks = (nsym + chunk - 1) / chunk;
    std::vector<gbsw::EscapeRuns> esc((size_t)nchunks);
    unsigned hw = std::thread::hardware_concurrency();
    unsigned nthreads = threads > 0 ? (unsigned)threads : std::min(16u, hw ? hw : 1u);
    nthreads = (unsigned)std::max<int64_t>(1, std::min<int64_t>(nthreads, nchunks));
    std::atomic<int64_t> next{0};
    auto worker = [&]() {
        for (int64_t c; (c = next.fetch_add(1)) < nchunks;) {
            const int64_t b = c * chunk, len = std::min(chunk, nsym - b);
            gbsw::pack_span(kind, raw + b, len, b, words + b / per, &esc[(size_t)c]);
        }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nthreads; ++t) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
    gbsw::EscapeRuns all;
    for (const auto& e : esc) all.append(e);
    *nruns = (int64_t)all.at.size();
    *nbytes = (int64_t)all.bytes.size();
    if (run_off) run_off[0] = 0;
    if (*nruns > run_cap || *nbytes > byte_cap) return GBSW_ETOOBIG;
    int64_t off = 0;
    for (int64_t r = 0; r < *nruns; ++r) {
        run_at[r] = all.at[(size_t)r];
        off += all.len[(size_t)r];
        run_off[r + 1] = off;
    }
    if (*nbytes > 0) std::memcpy(run_bytes, all.bytes.data(), (size_t)*nbytes);
    return GBSW_OK;
}

}  // extern "C"
