// Host-side copies of caller arrays into page-locked buffers, split over a
// small process-wide pool of threads: one core copies about 13 GB/s on the
// Grace host, which made the copy of a 2.6 M-point input (41.6 MB) the
// largest part of a host-buffer call after the build.
#pragma once

#include <cstddef>

namespace qdtg {

// Copies bytes from src to dst (not overlapping) using up to the pool's
// threads plus the caller's; returns when the copy is complete. Small
// copies run on the calling thread. Safe to call from several threads.
void parallel_copy(void* dst, const void* src, size_t bytes) noexcept;

struct CopyItem
{
    void*       dst;
    const void* src;
    size_t      bytes;
};

// Copies n independent items (a gather of many small arrays), the items split
// into groups of about equal bytes over the pool; returns when all are done.
void parallel_copy_many(const CopyItem* items, size_t n) noexcept;

}  // namespace qdtg
