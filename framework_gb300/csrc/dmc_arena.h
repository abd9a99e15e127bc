// Range allocator over a fixed arena of elements (vertices or quads), used
// by the serving loop to hand each batch a slice of the output buffers.
//
// First fit over an ordered free list with coalescing.  Sizes are rounded up
// to kGranule elements so that every slice starts 256-byte aligned for both
// 12-byte vertices and 16-byte quads.  Host-only; no CUDA.
#pragma once
#include <stdint.h>
#include <iterator>
#include <map>

namespace dmc {

class Arena {
public:
    static constexpr uint64_t kGranule = 64;
    static constexpr uint64_t kNone = ~0ull;

    explicit Arena(uint64_t capacity = 0) { reset(capacity); }

    void reset(uint64_t capacity)
    {
        cap_ = capacity / kGranule * kGranule;
        free_.clear();
        if (cap_) free_[0] = cap_;
        used_ = 0;
        peak_ = 0;
    }

    static uint64_t round(uint64_t n) { return (n + kGranule - 1) / kGranule * kGranule; }

    // Offset of a new range of at least n elements, or kNone.
    uint64_t alloc(uint64_t n)
    {
        n = round(n ? n : 1);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            const uint64_t off = it->first, len = it->second;
            free_.erase(it);
            if (len > n) free_[off + n] = len - n;
            used_ += n;
            if (used_ > peak_) peak_ = used_;
            return off;
        }
        return kNone;
    }

    // Returns [off, off + n) (n as given to alloc or shrink) to the free list.
    void release(uint64_t off, uint64_t n)
    {
        n = round(n ? n : 1);
        used_ -= n;
        auto next = free_.lower_bound(off);
        uint64_t start = off, len = n;
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                start = prev->first;
                len += prev->second;
                free_.erase(prev);
            }
        }
        if (next != free_.end() && off + n == next->first) {
            len += next->second;
            free_.erase(next);
        }
        free_[start] = len;
    }

    // Keeps the first keep elements of a range of n and frees the tail;
    // returns the new size to pass to release.
    uint64_t shrink(uint64_t off, uint64_t n, uint64_t keep)
    {
        n = round(n ? n : 1);
        keep = round(keep ? keep : 1);
        if (keep < n) release(off + keep, n - keep);
        return keep < n ? keep : n;
    }

    uint64_t largest_free() const
    {
        uint64_t m = 0;
        for (const auto &f : free_)
            if (f.second > m) m = f.second;
        return m;
    }

    uint64_t capacity() const { return cap_; }
    uint64_t used() const { return used_; }
    uint64_t peak() const { return peak_; }
    size_t fragments() const { return free_.size(); }

private:
    uint64_t cap_ = 0, used_ = 0, peak_ = 0;
    std::map<uint64_t, uint64_t> free_;   // offset -> length
};

}  // namespace dmc
