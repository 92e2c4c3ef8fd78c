// arena.h -- first-fit free list over one device arena (host-side bookkeeping only:
// offsets and sizes in bytes, no device calls).
//
// The batch engine carves every admitted shot's planes, snapshot store and inputs out
// of one preallocated device arena.  Free blocks are kept sorted by offset; an
// allocation takes the lowest-offset block that fits (sizes rounded up to the
// alignment), and a free merges the block with both neighbours, so freeing everything
// restores the single block the arena started as.
#pragma once

#include <algorithm>
#include <cstddef>
#include <iterator>
#include <map>

namespace w2d {

class ArenaFreeList {
public:
    explicit ArenaFreeList(size_t align) : align_(align) {}

    // The whole arena free again: one block of `bytes` rounded down to the alignment.
    void reset(size_t bytes)
    {
        blocks_.clear();
        const size_t b = bytes / align_ * align_;
        if (b) blocks_[0] = b;
    }

    size_t round(size_t bytes) const { return (bytes + align_ - 1) / align_ * align_; }

    bool alloc(size_t bytes, size_t* off)
    {
        bytes = round(bytes);
        for (auto it = blocks_.begin(); it != blocks_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes;
                const size_t noff = it->first + bytes;
                blocks_.erase(it);
                if (rest) blocks_[noff] = rest;
                return true;
            }
        }
        return false;
    }

    // `off` and `bytes` as given to (and returned by) alloc.
    void free(size_t off, size_t bytes)
    {
        bytes = round(bytes);
        auto it = blocks_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != blocks_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            blocks_.erase(nx);
        }
        if (it != blocks_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                blocks_.erase(it);
            }
        }
    }

    size_t largest() const
    {
        size_t m = 0;
        for (const auto& kv : blocks_) m = std::max(m, kv.second);
        return m;
    }

    const std::map<size_t, size_t>& blocks() const { return blocks_; }

private:
    size_t align_;
    std::map<size_t, size_t> blocks_;  // offset -> bytes
};

}  // namespace w2d
