// First-fit allocator of index ranges (cells, faces, ... of a batch arena) with coalescing frees.
#pragma once

#include <iterator>
#include <map>

namespace fv2d {

class RangeAlloc {
public:
    void reset(long long cap) { cap_ = cap; free_.clear(); if (cap > 0) free_[0] = cap; used_ = 0; }
    bool alloc(long long n, long long* start) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                *start = it->first;
                const long long rest = it->second - n, at = it->first + n;
                free_.erase(it);
                if (rest > 0) free_[at] = rest;
                used_ += n;
                return true;
            }
        }
        return false;
    }
    void release(long long start, long long n) {
        if (n <= 0) return;
        used_ -= n;
        auto it = free_.emplace(start, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
        }
    }
    long long used() const { return used_; }
    long long cap() const { return cap_; }
private:
    long long cap_ = 0, used_ = 0;
    std::map<long long, long long> free_;
};

}  // namespace fv2d
