// gbsw_align_device_noalloc: the device-resident alignment entry for callers
// that must not allocate GPU memory (see include/gbsw.h).
//
// Who needs it: code that runs where cudaMalloc is off limits -- inside a
// host callback or a memory-pool-controlled region of another framework, in a
// process whose allocator is owned by someone else (a caching allocator that
// must see every byte), or after the device has been filled to a fixed budget
// so that a fresh allocation could fail half-way through a pipeline.  Such a
// caller already holds its inputs and outputs on the device and only needs
// the alignment itself.
//
// How: every byte of working memory the passes need (schedule arrays, work-queue
// counters, error flags, the protein tables and the strip-boundary buffer) lives
// in ONE file-scope __device__ array of fixed size, g_noalloc_scratch below.  It
// is part of the library image.  CUDA loads a module lazily by default, and this
// file's module holds no kernel, so the array is committed on a device (in the
// current context) by the first lookup of its address there; from then on that
// device holds it until the process exits.  Host code may not use the array's
// name as a device address (on the host it names a stand-in object), so every
// call looks the address up with cudaGetSymbolAddress on the current device --
// cheap once the module is loaded, and right for whichever context is current
// (a cached pointer could outlive a cudaDeviceReset or belong to another
// context).  A call with n == 0 that passes the argument checks does the lookup
// too, so a caller can commit the array before it fills the device.
#include <cuda_runtime.h>

#include "../../include/gbsw.h"
#include "schedule.h"
#include "sw_kernels.h"

namespace {

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Layout of the scratch array (byte offsets).
constexpr size_t kHistBytes = sizeof(int) * ((size_t)gbsw::kBuckets + 2 * gbsw::kRanges);
constexpr size_t kOffHist = 0;
constexpr size_t kOffMisc = align256(kOffHist + kHistBytes);                    // 8 ints
constexpr size_t kOffMatrix = align256(kOffMisc + 8 * sizeof(int));             // 25 x 25 ints
constexpr size_t kOffEncoding = align256(kOffMatrix + sizeof(int) * gbsw::kAADim * gbsw::kAADim);
constexpr size_t kOffCls = align256(kOffEncoding + 128 * sizeof(int));
constexpr size_t kOffKeys = align256(kOffCls + (size_t)GBSW_NOALLOC_MAX_PAIRS);
constexpr size_t kOffOrder = align256(kOffKeys + sizeof(int) * (size_t)GBSW_NOALLOC_MAX_PAIRS);
constexpr size_t kOffBoundary = align256(kOffOrder + sizeof(int) * (size_t)GBSW_NOALLOC_MAX_PAIRS);
constexpr size_t kBoundaryBytes = (size_t)GBSW_NOALLOC_SCRATCH_BYTES - kOffBoundary;
static_assert(kOffBoundary < (size_t)GBSW_NOALLOC_SCRATCH_BYTES, "scratch layout");

static __device__ __align__(256) unsigned char g_noalloc_scratch[GBSW_NOALLOC_SCRATCH_BYTES];

const char* kAAOrder = "ARNDCQEGHILKMFPSTWYVBZX*";

bool fits_int8(int v) { return v >= -127 && v <= 127; }

int mode_of(const gbsw_scoring* sc, int cls, bool dna_profile_ok, bool aa_profile_ok) {
    if (sc->kind == GBSW_PROTEIN) return aa_profile_ok ? gbsw::kScoreAaProfile : gbsw::kScoreAaWide;
    return (cls == 0 && dna_profile_ok) ? gbsw::kScoreDnaProfile : gbsw::kScoreDnaRaw;
}

}  // namespace

extern "C" int gbsw_align_device_noalloc(const gbsw_scoring* sc, const uint8_t* ref,
                                         const int64_t* ref_off, const uint8_t* query,
                                         const int64_t* query_off, int64_t n, int32_t max_len,
                                         int32_t* top_scores, int32_t* ref_begin, int32_t* ref_end,
                                         int32_t* query_begin, int32_t* query_end, void* stream) {
    if (!sc || (sc->kind != GBSW_DNA && sc->kind != GBSW_PROTEIN)) return GBSW_EINVAL;
    if (sc->gap_open > 0 || sc->gap_extend > 0) return GBSW_EINVAL;
    if (sc->kind == GBSW_PROTEIN && !sc->matrix) return GBSW_EINVAL;
    if (n < 0 || max_len < 0) return GBSW_EINVAL;
    if (n > GBSW_NOALLOC_MAX_PAIRS || max_len > GBSW_NOALLOC_MAX_LEN) return GBSW_ETOOBIG;
    cudaStream_t s = (cudaStream_t)stream;

    // ---- the array's device address in the current context (loads and
    // commits the array on the first call there, n == 0 included) ----
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GBSW_ECUDA;
    void* addr = nullptr;
    if (cudaGetSymbolAddress(&addr, g_noalloc_scratch) != cudaSuccess || !addr) return GBSW_ECUDA;
    unsigned char* base = (unsigned char*)addr;
    if (n == 0) return GBSW_OK;
    if (!ref || !ref_off || !query || !query_off || !top_scores || !ref_begin || !ref_end ||
        !query_begin || !query_end)
        return GBSW_EINVAL;
    int* hist = (int*)(base + kOffHist);
    int* misc = (int*)(base + kOffMisc);
    int* matrix = (int*)(base + kOffMatrix);
    int* encoding = (int*)(base + kOffEncoding);
    int2* boundary = (int2*)(base + kOffBoundary);

    const bool protein = sc->kind == GBSW_PROTEIN;
    const bool dpx = true;
    const bool dna_profile_ok = !protein && fits_int8(sc->match) && fits_int8(sc->mismatch);
    bool aa_profile_ok = protein;
    if (protein)
        for (int k = 0; k < 576; ++k) aa_profile_ok = aa_profile_ok && fits_int8(sc->matrix[k]);
    const int nclasses = protein ? 1 : 2;

    // Grid: as many resident blocks as the boundary buffer has room for, at most
    // the occupancy of the variants used.
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GBSW_ECUDA;
    int bps = 1 << 20;
    for (int cls = 0; cls < nclasses; ++cls)
        for (int rev = 0; rev < 2; ++rev) {
            int b = 0;
            if (gbsw::pass_occupancy(mode_of(sc, cls, dna_profile_ok, aa_profile_ok), rev != 0, dpx, gbsw::kG, &b) !=
                cudaSuccess)
                return GBSW_ECUDA;
            bps = b < bps ? (b > 0 ? b : 1) : bps;
        }
    const int rows = ((max_len > 0 ? max_len : 1) + 1) & ~1;  // even, as the passes need
    const int groups_per_block = gbsw::pass_threads() / gbsw::kG;
    const long long fit_groups = (long long)(kBoundaryBytes / (sizeof(int2) * (size_t)rows));
    long long blocks = fit_groups / groups_per_block;
    if (blocks > (long long)sms * bps) blocks = (long long)sms * bps;
    if (blocks < 1) return GBSW_ETOOBIG;

    // ---- what must start at zero (the array keeps the previous call's contents) ----
    if (cudaMemsetAsync(misc, 0, 8 * sizeof(int), s) != cudaSuccess) return GBSW_ECUDA;
    if (protein) {
        int tab[gbsw::kAADim * gbsw::kAADim + 128];
        for (int r = 0; r < gbsw::kAADim; ++r)
            for (int c = 0; c < gbsw::kAADim; ++c)
                tab[r * gbsw::kAADim + c] = (r < 24 && c < 24) ? (int)sc->matrix[r * 24 + c] : gbsw::kNegBig;
        int* enc = tab + gbsw::kAADim * gbsw::kAADim;
        for (int k = 0; k < 128; ++k) enc[k] = 0;
        for (int k = 0; kAAOrder[k]; ++k) enc[(int)kAAOrder[k]] = k;
        // pageable source: the copy is staged before the call returns
        if (cudaMemcpyAsync(matrix, tab, sizeof(int) * gbsw::kAADim * gbsw::kAADim, cudaMemcpyHostToDevice, s) !=
                cudaSuccess ||
            cudaMemcpyAsync(encoding, enc, sizeof(int) * 91, cudaMemcpyHostToDevice, s) != cudaSuccess)
            return GBSW_ECUDA;
    }

    gbsw::SchedParams sp{};
    sp.ref = ref;
    sp.ref_off = ref_off;
    sp.query = query;
    sp.query_off = query_off;
    sp.n = n;
    sp.protein = protein ? 1 : 0;
    sp.dna_profile_ok = dna_profile_ok ? 1 : 0;
    sp.score = top_scores;
    sp.ref_end = ref_end;
    sp.query_end = query_end;
    sp.cls = base + kOffCls;
    sp.keys = (int*)(base + kOffKeys);
    sp.hist = hist;
    sp.class_range = hist + gbsw::kBuckets;
    sp.order = (int*)(base + kOffOrder);
    sp.error = misc + 2;

    gbsw::PassParams p{};
    p.ref = ref;
    p.ref_off = ref_off;
    p.query = query;
    p.query_off = query_off;
    p.n = n;
    p.open = sc->gap_open;
    p.ext = sc->gap_extend;
    p.match = sc->match;
    p.mismatch = sc->mismatch;
    p.aa_matrix = matrix;
    p.aa_encoding = encoding;
    p.score = top_scores;
    p.ref_begin = ref_begin;
    p.ref_end = ref_end;
    p.query_begin = query_begin;
    p.query_end = query_end;
    p.order = sp.order;
    p.class_range = sp.class_range;
    p.scratch = boundary;
    p.scratch_rows = rows;
    p.error = misc + 2;
    for (int rev = 0; rev < 2; ++rev) {
        if (gbsw::build_schedule(sp, rev != 0, sms, s) != cudaSuccess) return GBSW_ECUDA;
        for (int cls = 0; cls < nclasses; ++cls) {
            p.cls = cls;
            p.queue = misc + (rev ? 4 : 0) + cls;
            if (gbsw::launch_pass(mode_of(sc, cls, dna_profile_ok, aa_profile_ok), rev != 0, dpx, gbsw::kG, p,
                                  (int)blocks, s) != cudaSuccess)
                return GBSW_ECUDA;
        }
    }

    // ---- synchronous: report the batch's device-side checks ----
    int flags = 0;
    if (cudaMemcpyAsync(&flags, misc + 2, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GBSW_ECUDA;
    if (flags & gbsw::kErrSymbol) return GBSW_ESYMBOL;
    if (flags & gbsw::kErrBounds) return GBSW_ELENGTH;
    if (flags & gbsw::kErrNoHit) return GBSW_EINTERNAL;
    return GBSW_OK;
}
