// Host-side bulk copies and comparisons split over threads: a single thread
// moves about 10 GB/s on the Grace host, far below what its memory and the
// NVLink-C2C link to the GPU sustain, so the matrix upload stages its values
// through pinned memory chunk by chunk with all host cores, overlapped with
// the host-to-device copies of the previous chunk.
#pragma once

#include <algorithm>
#include <cstring>
#include <thread>
#include <vector>

#include "lss_common.hpp"

namespace lss {

inline int host_threads()
{
    return (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
}

// dst[0..bytes) = src[0..bytes) with up to `threads` threads
inline void parallel_copy(void *dst, const void *src, size_t bytes, int threads)
{
    constexpr size_t MIN_PART = 4u << 20;
    const int t = (int)std::max<size_t>(1, std::min<size_t>(threads, bytes / MIN_PART));
    if (t <= 1) {
        std::memcpy(dst, src, bytes);
        return;
    }
    const size_t part = (bytes + t - 1) / t;
    std::vector<std::thread> pool;
    for (int i = 1; i < t; ++i) {
        const size_t lo = std::min(bytes, i * part), hi = std::min(bytes, lo + part);
        pool.emplace_back([=]() { std::memcpy((char *)dst + lo, (const char *)src + lo, hi - lo); });
    }
    std::memcpy(dst, src, std::min(bytes, part));
    for (auto &th : pool) th.join();
}

// a[0..bytes) == b[0..bytes), compared with up to `threads` threads
inline bool parallel_equal(const void *a, const void *b, size_t bytes, int threads)
{
    constexpr size_t MIN_PART = 4u << 20;
    const int t = (int)std::max<size_t>(1, std::min<size_t>(threads, bytes / MIN_PART));
    if (t <= 1) return std::memcmp(a, b, bytes) == 0;
    const size_t part = (bytes + t - 1) / t;
    std::vector<char> same(t, 1);
    std::vector<std::thread> pool;
    for (int i = 1; i < t; ++i) {
        const size_t lo = std::min(bytes, i * part), hi = std::min(bytes, lo + part);
        pool.emplace_back([=, &same]() { same[i] = std::memcmp((const char *)a + lo, (const char *)b + lo, hi - lo) == 0; });
    }
    same[0] = std::memcmp(a, b, std::min(bytes, part)) == 0;
    for (auto &th : pool) th.join();
    return std::all_of(same.begin(), same.end(), [](char c) { return c != 0; });
}

// Host-to-device upload of `bytes` from pageable `src` through two pinned
// chunks of `chunk` bytes (pin holds 2 * chunk): chunk k is copied into pinned
// memory by all host threads while chunk k-1 is in flight to the device.
// Ordered on stream s; returns when the last chunk has been handed to the
// copy engine (the staging buffer stays busy until s reaches that point).
inline void upload_staged(void *dst, const void *src, size_t bytes, PinnedBuf &pin, cudaEvent_t ev[2],
                          cudaStream_t s, size_t chunk = 64u << 20)
{
    if (bytes == 0) return;
    chunk = std::min(chunk, bytes);
    char *stage = (char *)pin.get(2 * chunk);
    const int threads = host_threads();
    for (size_t off = 0, k = 0; off < bytes; off += chunk, ++k) {
        const size_t len = std::min(chunk, bytes - off);
        char *buf = stage + (k & 1) * chunk;
        if (k >= 2) LSS_CUDA(cudaEventSynchronize(ev[k & 1]));  // the copy that used this half is done
        parallel_copy(buf, (const char *)src + off, len, threads);
        LSS_CUDA(cudaMemcpyAsync((char *)dst + off, buf, len, cudaMemcpyHostToDevice, s));
        LSS_CUDA(cudaEventRecord(ev[k & 1], s));
    }
}

}  // namespace lss
