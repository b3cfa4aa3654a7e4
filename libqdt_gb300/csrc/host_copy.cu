// A small pool of host threads for large memcpy calls (host_copy.hpp). The
// pool is created on first use and never destroyed (its threads wait on a
// condition variable until the process ends), so no static destructor races
// with a copy in flight.
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "host_copy.hpp"

namespace qdtg {

namespace {

struct Piece
{
    const CopyItem*   items;   // items [i0, i1) of the call
    size_t            i0, i1;
    std::atomic<int>* left;    // pieces of the call not yet done
};

void copy_items(const CopyItem* items, size_t i0, size_t i1)
{
    for (size_t i = i0; i < i1; ++i)
        if (items[i].bytes) std::memcpy(items[i].dst, items[i].src, items[i].bytes);
}

struct Pool
{
    std::mutex              mu;
    std::condition_variable work, done;
    std::deque<Piece>       queue;
    int                     threads = 0;

    explicit Pool(int n)
    {
        for (int i = 0; i < n; ++i)
        {
            try
            {
                std::thread([this] { loop(); }).detach();
                ++threads;
            }
            catch (...)
            {
                break;
            }
        }
    }

    void loop()
    {
        for (;;)
        {
            Piece p;
            {
                std::unique_lock<std::mutex> lk(mu);
                work.wait(lk, [this] { return !queue.empty(); });
                p = queue.front();
                queue.pop_front();
            }
            copy_items(p.items, p.i0, p.i1);
            if (p.left->fetch_sub(1, std::memory_order_acq_rel) == 1)
            {
                std::lock_guard<std::mutex> lk(mu);
                done.notify_all();
            }
        }
    }
};

Pool* pool()
{
    static Pool* p = [] {
        const unsigned hw = std::thread::hardware_concurrency();
        const int      n = (int)std::min<unsigned>(7u, hw > 1 ? hw - 1 : 0u);
        return n > 0 ? new (std::nothrow) Pool(n) : nullptr;
    }();
    return p;
}

constexpr size_t kMinParallel = (size_t)4 << 20;   // below this, one memcpy
constexpr size_t kMinPiece = (size_t)1 << 20;

// Runs the groups [cut[g], cut[g + 1]) of items: group 0 on the calling
// thread, the others on the pool.
void run_groups(Pool* p, const CopyItem* items, const size_t* cut, size_t groups)
{
    std::atomic<int> left((int)(groups - 1));
    if (groups > 1)
    {
        {
            std::lock_guard<std::mutex> lk(p->mu);
            for (size_t g = 1; g < groups; ++g) p->queue.push_back(Piece{ items, cut[g], cut[g + 1], &left });
        }
        if (groups == 2) p->work.notify_one();
        else p->work.notify_all();
    }
    copy_items(items, cut[0], cut[1]);
    if (groups > 1)
    {
        std::unique_lock<std::mutex> lk(p->mu);
        p->done.wait(lk, [&] { return left.load(std::memory_order_acquire) == 0; });
    }
}

constexpr size_t kMaxGroups = 8;

}  // namespace

void parallel_copy(void* dst, const void* src, size_t bytes) noexcept
{
    if (bytes == 0) return;
    Pool* p = bytes >= kMinParallel ? pool() : nullptr;
    if (!p || p->threads == 0)
    {
        std::memcpy(dst, src, bytes);
        return;
    }
    const size_t parts = std::min<size_t>(std::min<size_t>((size_t)p->threads + 1, kMaxGroups), bytes / kMinPiece);
    const size_t step = (bytes / parts + 63) & ~(size_t)63;
    CopyItem     items[kMaxGroups];
    size_t       cut[kMaxGroups + 1];
    size_t       n = 0;
    for (size_t off = 0; off < bytes && n < kMaxGroups; off += step, ++n)
    {
        const size_t len = (n + 1 == kMaxGroups) ? bytes - off : std::min(step, bytes - off);
        items[n] = CopyItem{ static_cast<char*>(dst) + off, static_cast<const char*>(src) + off, len };
        cut[n] = n;
    }
    cut[n] = n;
    run_groups(p, items, cut, n);
}

void parallel_copy_many(const CopyItem* items, size_t n) noexcept
{
    if (n == 0) return;
    size_t total = 0;
    for (size_t i = 0; i < n; ++i) total += items[i].bytes;
    Pool* p = total >= kMinParallel ? pool() : nullptr;
    if (!p || p->threads == 0)
    {
        copy_items(items, 0, n);
        return;
    }
    // contiguous groups of items of about total / groups bytes each
    const size_t groups = std::min<size_t>(std::min<size_t>((size_t)p->threads + 1, kMaxGroups), n);
    const size_t target = total / groups + 1;
    size_t       cut[kMaxGroups + 1];
    size_t       g = 0, acc = 0;
    cut[0] = 0;
    for (size_t i = 0; i < n && g + 1 < groups; ++i)
    {
        acc += items[i].bytes;
        if (acc >= target * (g + 1)) cut[++g] = i + 1;
    }
    cut[++g] = n;
    // drop empty groups (a single large item can close several at once)
    size_t k = 0;
    for (size_t j = 0; j < g; ++j)
        if (cut[j + 1] > cut[j]) cut[k++] = cut[j];
    cut[k] = n;
    run_groups(p, items, cut, k);
}

}  // namespace qdtg
