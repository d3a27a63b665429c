// Device-memory arena for the server: one cudaMalloc of the HBM budget, carved into aligned
// blocks with a first-fit free list that merges neighbours on release.  Admission of a case is
// a transaction over its blocks, so the budget bounds the resident footprint exactly.
#pragma once
#include <cstddef>
#include <map>
#include <mutex>

namespace lbffs {

class Arena {
public:
    // takes ownership of [base, base + size)
    Arena(void* base, size_t size);
    // nullptr when no free block is large enough
    void* alloc(size_t bytes);
    void release(void* p);
    bool owns(const void* p) const;
    size_t in_use() const { return in_use_; }
    size_t peak() const { return peak_; }
    size_t capacity() const { return size_; }
    size_t largest_free() const;
    static constexpr size_t kAlign = 256;

private:
    char* base_;
    size_t size_;
    std::map<size_t, size_t> free_;  // offset -> length
    std::map<size_t, size_t> used_;  // offset -> length
    size_t in_use_ = 0, peak_ = 0;
    mutable std::mutex mu_;
};

}  // namespace lbffs
