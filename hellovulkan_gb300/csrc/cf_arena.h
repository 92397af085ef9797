// cf_arena.h — first-fit allocator over one device allocation (the server's
// HBM budget).  Host-side bookkeeping only; 256-byte aligned blocks; adjacent
// free blocks are merged on release.  Not thread-safe (the server serialises).
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <iterator>
#include <map>

namespace cfrt {

class Arena {
public:
    void reset(unsigned char* base, size_t bytes)
    {
        base_ = base;
        size_ = bytes;
        used_ = 0;
        free_.clear();
        if (bytes) free_[0] = bytes;
    }

    // Device address of a block of at least `bytes`, or nullptr when no free
    // block is large enough.
    unsigned char* alloc(size_t bytes)
    {
        bytes = (bytes + 255) & ~(size_t)255;
        if (bytes == 0) bytes = 256;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            const size_t off = it->first, len = it->second;
            free_.erase(it);
            if (len > bytes) free_[off + bytes] = len - bytes;
            live_[off] = bytes;
            used_ += bytes;
            return base_ + off;
        }
        return nullptr;
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
                free_.erase(prev);
            }
        }
        next = free_.lower_bound(start + len);
        if (next != free_.end() && next->first == start + len) {
            len += next->second;
            free_.erase(next);
        }
        free_[start] = len;
    }

    size_t used() const { return used_; }
    size_t size() const { return size_; }
    size_t largest_free() const
    {
        size_t m = 0;
        for (const auto& kv : free_) m = kv.second > m ? kv.second : m;
        return m;
    }

private:
    unsigned char* base_ = nullptr;
    size_t size_ = 0, used_ = 0;
    std::map<size_t, size_t> free_;  // offset -> length
    std::map<size_t, size_t> live_;  // offset -> length
};

}  // namespace cfrt
