// fk_firstfit.h -- first-fit bookkeeping of one memory block by offsets, with
// coalescing on release.  Host code only (no CUDA): the request server keeps
// its device block's free and used ranges here, and a CPU test drives it
// directly.
#pragma once
#include <stddef.h>

#include <algorithm>
#include <iterator>
#include <map>

namespace fk {

class FirstFit {
  public:
    static constexpr size_t NONE = ~size_t(0);
    static size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

    // Manage [0, cap) (rounded up to 256 bytes); forgets every earlier range.
    void reset(size_t cap) {
        cap_ = round256(cap);
        free_.clear();
        used_.clear();
        in_use_ = peak_ = 0;
        if (cap_) free_[0] = cap_;
    }
    // Offset of a block of at least `bytes` (rounded up to 256, at least 256):
    // the lowest free range that holds it.  NONE when no free range does.
    size_t alloc(size_t bytes) {
        bytes = round256(std::max<size_t>(bytes, 1));
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            const size_t off = it->first, rest = it->second - bytes;
            free_.erase(it);
            if (rest) free_[off + bytes] = rest;
            used_[off] = bytes;
            in_use_ += bytes;
            peak_ = std::max(peak_, in_use_);
            return off;
        }
        return NONE;
    }
    // Returns the block that starts at `off` to the free ranges, merged with
    // the free ranges right before and after it.  Offsets that are not the
    // start of a used block are ignored.
    void release(size_t off) {
        auto u = used_.find(off);
        if (u == used_.end()) return;
        const size_t bytes = u->second;  // the block's own size (u is invalid after the erase)
        size_t start = off, size = bytes;
        in_use_ -= bytes;
        used_.erase(u);
        auto next = free_.lower_bound(off);
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                start = prev->first;
                size += prev->second;
                free_.erase(prev);
            }
        }
        next = free_.lower_bound(off);
        if (next != free_.end() && next->first == off + bytes) {
            size += next->second;
            free_.erase(next);
        }
        free_[start] = size;
    }
    size_t capacity() const { return cap_; }
    size_t in_use() const { return in_use_; }
    size_t peak() const { return peak_; }
    size_t free_ranges() const { return free_.size(); }
    // Size of the largest free range.
    size_t largest_free() const {
        size_t m = 0;
        for (const auto& f : free_) m = std::max(m, f.second);
        return m;
    }

  private:
    size_t cap_ = 0, in_use_ = 0, peak_ = 0;
    std::map<size_t, size_t> free_, used_;  // offset -> size
};

}  // namespace fk
