// Process-wide pool of page-locked host blocks (see pinned_pool.h).
#include "pinned_pool.h"

#include <cuda_runtime.h>

#include <map>
#include <mutex>

namespace gbsw {
namespace {

constexpr size_t kMinBlock = size_t(1) << 20;
// Free blocks kept for reuse; larger releases go back to the system.
constexpr size_t kPoolLimit = size_t(4) << 30;

std::mutex g_mu;
std::multimap<size_t, void*>* g_free = nullptr;  // size -> block (never destroyed: freed at exit by the driver)
size_t g_cached = 0;

size_t round_up(size_t bytes) {
    size_t b = kMinBlock;
    while (b < bytes) b <<= 1;
    return b;
}

}  // namespace

void* pinned_acquire(size_t bytes, size_t* got) {
    const size_t want = round_up(bytes ? bytes : 1);
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_free) g_free = new std::multimap<size_t, void*>();
        auto it = g_free->find(want);
        if (it != g_free->end()) {
            void* p = it->second;
            g_free->erase(it);
            g_cached -= want;
            *got = want;
            return p;
        }
    }
    void* p = nullptr;
    if (cudaMallocHost(&p, want) != cudaSuccess) {
        cudaGetLastError();  // leave no error behind for the caller's next cudaGetLastError
        return nullptr;
    }
    *got = want;
    return p;
}

void pinned_release(void* ptr, size_t bytes) {
    if (!ptr) return;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_free) g_free = new std::multimap<size_t, void*>();
        if (g_cached + bytes <= kPoolLimit) {
            g_free->emplace(bytes, ptr);
            g_cached += bytes;
            return;
        }
    }
    cudaFreeHost(ptr);
}

size_t pinned_pool_limit() { return kPoolLimit; }

size_t pinned_pool_cached() {
    std::lock_guard<std::mutex> lock(g_mu);
    return g_cached;
}

}  // namespace gbsw
