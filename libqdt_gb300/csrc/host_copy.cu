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
    char*               dst;
    const char*         src;
    size_t              bytes;
    std::atomic<int>*   left;   // pieces of the call not yet done
};

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
            std::memcpy(p.dst, p.src, p.bytes);
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
    const size_t     parts = std::min<size_t>((size_t)p->threads + 1, bytes / kMinPiece);
    const size_t     step = (bytes / parts + 63) & ~(size_t)63;
    std::atomic<int> left(0);
    char*            d = static_cast<char*>(dst);
    const char*      s = static_cast<const char*>(src);
    // pieces 1.. go to the pool, piece 0 stays here
    size_t queued = 0;
    {
        std::lock_guard<std::mutex> lk(p->mu);
        for (size_t off = step; off < bytes; off += step)
        {
            p->queue.push_back(Piece{ d + off, s + off, std::min(step, bytes - off), &left });
            ++queued;
        }
        left.store((int)queued, std::memory_order_relaxed);
    }
    if (queued == 1) p->work.notify_one();
    else if (queued > 1) p->work.notify_all();
    std::memcpy(d, s, std::min(step, bytes));
    if (queued)
    {
        std::unique_lock<std::mutex> lk(p->mu);
        p->done.wait(lk, [&] { return left.load(std::memory_order_acquire) == 0; });
    }
}

}  // namespace qdtg
