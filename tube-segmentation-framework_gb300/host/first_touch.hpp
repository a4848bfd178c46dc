// first_touch.hpp -- host loops split over a few threads.
//
// parallel_tasks(n, fn) runs fn(0) .. fn(n-1), each on its own thread but the
// first, which runs on the caller's; a thread that cannot be started runs its
// task on the caller's thread instead, so the call always completes every task.
//
// parallel_fill: a new large allocation is backed by pages the kernel maps and
// zeroes on first touch, one page at a time in the touching thread.  Filling a
// volume-sized buffer (tens to hundreds of MB) from up to 16 threads spreads
// that cost before a device-to-host copy writes into it.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <system_error>
#include <thread>
#include <vector>

namespace tsf_host {

// Threads worth using for `bytes` of streaming work: up to 16, at least 4 MB each.
inline size_t host_threads(size_t bytes) {
    const size_t min_slice = (size_t)4 << 20;
    const unsigned hw = std::thread::hardware_concurrency();
    return std::max<size_t>(1, std::min<size_t>({hw ? (size_t)hw : 1, (size_t)16, bytes / min_slice}));
}

template <typename Fn> void parallel_tasks(size_t n, Fn fn) {
    std::vector<std::thread> pool;
    pool.reserve(n);
    size_t t = 1;
    try {
        for (; t < n; t++) pool.emplace_back(fn, t);
    } catch (const std::system_error &) {
        for (; t < n; t++) fn(t);   // no thread for the rest: run them here
    }
    if (n) fn(0);
    for (auto &th : pool) th.join();
}

inline void parallel_fill(void *p, int value, size_t bytes) {
    const size_t nt = host_threads(bytes);
    char *c = static_cast<char *>(p);
    parallel_tasks(nt, [=](size_t t) {
        const size_t b0 = bytes * t / nt, b1 = bytes * (t + 1) / nt;
        std::memset(c + b0, value, b1 - b0);
    });
}

}  // namespace tsf_host
