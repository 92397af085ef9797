// cf_arena.h — best-fit allocator over one device allocation (the server's
// HBM budget).  Host-side bookkeeping only; 256-byte aligned blocks; adjacent
// free blocks are merged on release.  Free blocks are indexed both by offset
// (for merging) and by (length, offset) (for the best fit), so allocation and
// release are O(log blocks).  Not thread-safe (the server serialises).
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <iterator>
#include <map>
#include <set>
#include <utility>

namespace cfrt {

class Arena {
public:
    void reset(unsigned char* base, size_t bytes)
    {
        base_ = base;
        size_ = bytes;
        used_ = 0;
        free_.clear();
        by_len_.clear();
        live_.clear();
        if (bytes) add_free(0, bytes);
    }

    // Device address of a block of at least `bytes` (the smallest free block
    // that fits, lowest offset among equals), or nullptr when none fits.
    unsigned char* alloc(size_t bytes)
    {
        bytes = (bytes + 255) & ~(size_t)255;
        if (bytes == 0) bytes = 256;
        auto it = by_len_.lower_bound(std::make_pair(bytes, (size_t)0));
        if (it == by_len_.end()) return nullptr;
        const size_t len = it->first, off = it->second;
        by_len_.erase(it);
        free_.erase(off);
        if (len > bytes) add_free(off + bytes, len - bytes);
        live_[off] = bytes;
        used_ += bytes;
        return base_ + off;
    }

    void release(unsigned char* p)
    {
        if (!p) return;
        const size_t off = (size_t)(p - base_);
        auto lit = live_.find(off);
        if (lit == live_.end()) return;
        size_t len = lit->second;
        live_.erase(lit);
        used_ -= len;
        size_t start = off;
        auto next = free_.lower_bound(off);
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                start = prev->first;
                len += prev->second;
                remove_free(prev);
            }
        }
        next = free_.lower_bound(start + len);
        if (next != free_.end() && next->first == start + len) {
            len += next->second;
            remove_free(next);
        }
        add_free(start, len);
    }

    size_t used() const { return used_; }
    size_t size() const { return size_; }
    size_t largest_free() const { return by_len_.empty() ? 0 : by_len_.rbegin()->first; }
    size_t free_blocks() const { return free_.size(); }

private:
    void add_free(size_t off, size_t len)
    {
        free_[off] = len;
        by_len_.emplace(len, off);
    }
    void remove_free(std::map<size_t, size_t>::iterator it)
    {
        by_len_.erase(std::make_pair(it->second, it->first));
        free_.erase(it);
    }

    unsigned char* base_ = nullptr;
    size_t size_ = 0, used_ = 0;
    std::map<size_t, size_t> free_;                 // offset -> length
    std::set<std::pair<size_t, size_t>> by_len_;    // (length, offset) of each free block
    std::map<size_t, size_t> live_;                 // offset -> length
};

}  // namespace cfrt
