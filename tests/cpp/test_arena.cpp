// Host test of the output-arena allocator used by the serving loop.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>
#include "dmc_arena.h"

#define CHECK(c) do { if (!(c)) { std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c); std::exit(1); } } while (0)

int main()
{
    using dmc::Arena;
    Arena a(1000);                              // rounds down to 960 = 15 granules
    CHECK(a.capacity() == 960);
    uint64_t x = a.alloc(1), y = a.alloc(64), z = a.alloc(65);
    CHECK(x == 0 && y == 64 && z == 128);
    CHECK(a.used() == 256 && a.largest_free() == 704);
    a.release(y, 64);                           // hole in the middle
    CHECK(a.fragments() == 2 && a.largest_free() == 704);
    CHECK(a.alloc(128) == 256);                 // first fit skips the 64-element hole
    CHECK(a.alloc(64) == 64);                   // and fills it exactly
    uint64_t big = a.alloc(10000);
    CHECK(big == Arena::kNone);
    // shrink keeps the head and returns the tail
    uint64_t w = a.alloc(320);
    CHECK(w == 384);
    uint64_t kept = a.shrink(w, 320, 70);
    CHECK(kept == 128 && a.largest_free() == 960 - 384 - 128);
    a.release(w, kept);
    a.release(x, 1); a.release(64, 64); a.release(z, 65); a.release(256, 128);
    CHECK(a.used() == 0 && a.fragments() == 1 && a.largest_free() == 960);
    CHECK(a.peak() >= 704);
    // random churn keeps the books balanced and coalesces back to one range
    std::mt19937_64 rng(7);
    Arena b(1 << 20);
    std::vector<std::pair<uint64_t, uint64_t>> live;
    for (int it = 0; it < 20000; ++it) {
        if (live.empty() || (rng() % 3)) {
            uint64_t n = 1 + rng() % 5000;
            uint64_t o = b.alloc(n);
            if (o != Arena::kNone) {
                for (auto &l : live) CHECK(o + Arena::round(n) <= l.first || l.first + Arena::round(l.second) <= o);
                CHECK(o % Arena::kGranule == 0 && o + Arena::round(n) <= b.capacity());
                live.push_back({o, n});
            }
        } else {
            size_t k = rng() % live.size();
            if (rng() % 2) {
                uint64_t keep = rng() % (live[k].second + 1);
                live[k].second = b.shrink(live[k].first, live[k].second, keep);
            }
            b.release(live[k].first, live[k].second);
            live.erase(live.begin() + k);
        }
    }
    for (auto &l : live) b.release(l.first, l.second);
    CHECK(b.used() == 0 && b.fragments() == 1 && b.largest_free() == b.capacity());
    std::printf("ok\n");
    return 0;
}
