// Byte-for-byte check of the host copy pool (tests/test_host_copy.py).
#include "host_copy.hpp"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <thread>
#include <random>
#include <atomic>
using namespace qdtg;
int main()
{
    std::mt19937_64 r(3);
    int bad = 0;
    for (int t = 0; t < 200; ++t) {
        size_t n = (r() % 4 == 0) ? r() % 1000 : (r() % (40u << 20));
        std::vector<unsigned char> a(n), b(n, 0);
        for (size_t i = 0; i < n; i += 4093) a[i] = (unsigned char)(r());
        if (n) a[n - 1] = 7;
        parallel_copy(b.data(), a.data(), n);
        if (a != b) ++bad;
    }
    for (int t = 0; t < 100; ++t) {
        size_t k = 1 + r() % 300;
        std::vector<std::vector<char>> src(k), dst(k);
        std::vector<CopyItem> items(k);
        for (size_t i = 0; i < k; ++i) {
            size_t n = (r() % 10 == 0) ? (r() % (8u << 20)) : r() % 70000;
            src[i].assign(n, (char)(i * 7 + 1)); dst[i].assign(n, 0);
            items[i] = CopyItem{ dst[i].data(), src[i].data(), n };
        }
        parallel_copy_many(items.data(), k);
        for (size_t i = 0; i < k; ++i) if (src[i] != dst[i]) { ++bad; break; }
    }
    // concurrent callers
    std::vector<std::thread> th;
    std::atomic<int> cbad{0};
    for (int c = 0; c < 6; ++c) th.emplace_back([&, c] {
        std::vector<char> a(12 << 20, (char)c), b(12 << 20, 0);
        for (int it = 0; it < 20; ++it) { parallel_copy(b.data(), a.data(), a.size()); if (a != b) cbad++; }
    });
    for (auto& x : th) x.join();
    printf("bad %d concurrent bad %d\n", bad, cbad.load());
    return bad || cbad;
}
