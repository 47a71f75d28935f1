// Process-wide pool of page-locked host blocks.  The C++ drop-in's ingest
// staging and the serving loop's batch buffers draw from it, so a process that
// uses both pins one set of buffers rather than two, and a buffer released by
// one is reused by the other without a new cudaMallocHost (which maps and
// locks pages, tens of milliseconds for a few hundred MB).
#pragma once
#include <cstddef>

namespace gbsw {

// A block of at least `bytes` page-locked bytes (sizes are rounded up to a power
// of two from 1 MiB, so blocks are interchangeable); nullptr when cudaMallocHost
// fails.  *got receives the block's size.
void* pinned_acquire(size_t bytes, size_t* got);
// Back to the pool; the pool keeps up to pinned_pool_limit() bytes of free
// blocks and frees the rest.
void pinned_release(void* ptr, size_t bytes);
size_t pinned_pool_limit();
// Free bytes the pool holds now (for tests and reports).
size_t pinned_pool_cached();

// Grow-on-demand typed buffer over the pool (contents are not preserved).
template <typename T>
struct PooledPinned {
    T* ptr = nullptr;
    size_t cap = 0;    // elements
    size_t bytes = 0;  // block size
    bool reserve(size_t n) {
        if (n <= cap) return true;
        release();
        size_t got = 0;
        void* p = pinned_acquire(n * sizeof(T), &got);
        if (!p) return false;
        ptr = static_cast<T*>(p);
        bytes = got;
        cap = got / sizeof(T);
        return true;
    }
    void release() {
        if (ptr) pinned_release(ptr, bytes);
        ptr = nullptr;
        cap = bytes = 0;
    }
    PooledPinned() = default;
    PooledPinned(const PooledPinned&) = delete;
    PooledPinned& operator=(const PooledPinned&) = delete;
    ~PooledPinned() { release(); }
};

}  // namespace gbsw
