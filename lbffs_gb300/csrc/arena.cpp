#include "arena.h"

namespace lbffs {

Arena::Arena(void* base, size_t size) : base_(static_cast<char*>(base)), size_(size)
{
    if (size_ > 0) free_[0] = size_;
}

void* Arena::alloc(size_t bytes)
{
    std::lock_guard<std::mutex> lock(mu_);
    const size_t n = ((bytes ? bytes : 1) + kAlign - 1) / kAlign * kAlign;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
        if (it->second < n) continue;
        const size_t off = it->first, len = it->second;
        free_.erase(it);
        if (len > n) free_[off + n] = len - n;
        used_[off] = n;
        in_use_ += n;
        if (in_use_ > peak_) peak_ = in_use_;
        return base_ + off;
    }
    return nullptr;
}

void Arena::release(void* p)
{
    if (!p) return;
    std::lock_guard<std::mutex> lock(mu_);
    const size_t off = static_cast<size_t>(static_cast<char*>(p) - base_);
    auto u = used_.find(off);
    if (u == used_.end()) return;
    size_t start = off, len = u->second;
    used_.erase(u);
    in_use_ -= len;
    // merge with the free neighbours
    auto next = free_.lower_bound(start);
    if (next != free_.end() && next->first == start + len) {
        len += next->second;
        next = free_.erase(next);
    }
    if (next != free_.begin()) {
        auto prev = std::prev(next);
        if (prev->first + prev->second == start) {
            start = prev->first;
            len += prev->second;
            free_.erase(prev);
        }
    }
    free_[start] = len;
}

bool Arena::owns(const void* p) const
{
    const char* c = static_cast<const char*>(p);
    return c >= base_ && c < base_ + size_;
}

size_t Arena::largest_free() const
{
    std::lock_guard<std::mutex> lock(mu_);
    size_t m = 0;
    for (const auto& kv : free_)
        if (kv.second > m) m = kv.second;
    return m;
}

}  // namespace lbffs
