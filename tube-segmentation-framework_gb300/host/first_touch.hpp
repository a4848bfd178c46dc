// first_touch.hpp -- fills fresh host buffers from several threads.
//
// A new large allocation is backed by pages the kernel maps and zeroes on
// first touch, one page at a time in the touching thread.  Filling a volume-
// sized buffer (tens to hundreds of MB) from up to 16 threads spreads that
// cost before a device-to-host copy or a rasterisation writes into it.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <thread>
#include <vector>

namespace tsf_host {

inline void parallel_fill(void *p, int value, size_t bytes) {
    const size_t min_slice = (size_t)4 << 20;
    const unsigned hw = std::thread::hardware_concurrency();
    const size_t nt = std::max<size_t>(1, std::min<size_t>({hw ? (size_t)hw : 1, (size_t)16, bytes / min_slice}));
    char *c = static_cast<char *>(p);
    auto work = [=](size_t t) {
        const size_t b0 = bytes * t / nt, b1 = bytes * (t + 1) / nt;
        std::memset(c + b0, value, b1 - b0);
    };
    std::vector<std::thread> pool;
    for (size_t t = 1; t < nt; t++) pool.emplace_back(work, t);
    work(0);
    for (auto &th : pool) th.join();
}

}  // namespace tsf_host
