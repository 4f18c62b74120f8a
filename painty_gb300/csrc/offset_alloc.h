// offset_alloc.h -- host bookkeeping of a contiguous range carved into allocations: best fit
// over the free ranges, neighbours merged on release. Offsets and lengths are in bytes; the
// caller rounds lengths to its granule. No CUDA: the server's device heap keeps its
// reservation's layout here, and a CPU test drives it directly.
#pragma once

#include <cstddef>
#include <map>
#include <unordered_map>

namespace pg {

class OffsetAllocator {
 public:
  explicit OffsetAllocator(size_t size = 0) { reset(size); }

  void reset(size_t size) {
    free_by_off_.clear();
    free_by_len_.clear();
    used_.clear();
    size_ = size;
    if (size_) insert_free(0, size_);
  }

  // The offset of a new allocation of `len` bytes (best fit: the smallest free range that
  // holds it, its lowest part), or false when no free range is large enough.
  bool alloc(size_t len, size_t* off) {
    if (len == 0) return false;
    auto it = free_by_len_.lower_bound(len);
    if (it == free_by_len_.end()) return false;
    const size_t flen = it->first, foff = it->second;
    erase_free(foff, flen);
    if (flen > len) insert_free(foff + len, flen - len);
    used_.emplace(foff, len);
    *off = foff;
    return true;
  }

  // Releases the allocation at `off`; false when there is none. The range merges with free
  // neighbours on either side.
  bool release(size_t off) {
    auto u = used_.find(off);
    if (u == used_.end()) return false;
    size_t len = u->second;
    used_.erase(u);
    auto next = free_by_off_.find(off + len);
    if (next != free_by_off_.end()) {
      const size_t nl = next->second;
      erase_free(off + len, nl);
      len += nl;
    }
    auto prev = free_by_off_.lower_bound(off);
    if (prev != free_by_off_.begin()) {
      --prev;
      if (prev->first + prev->second == off) {
        const size_t po = prev->first, pl = prev->second;
        erase_free(po, pl);
        off = po;
        len += pl;
      }
    }
    insert_free(off, len);
    return true;
  }

  size_t size() const { return size_; }
  size_t free_ranges() const { return free_by_off_.size(); }
  size_t allocations() const { return used_.size(); }
  size_t largest_free() const { return free_by_len_.empty() ? 0 : free_by_len_.rbegin()->first; }
  size_t free_bytes() const {
    size_t n = 0;
    for (const auto& kv : free_by_off_) n += kv.second;
    return n;
  }

 private:
  size_t size_ = 0;
  std::map<size_t, size_t> free_by_off_;       // offset -> length
  std::multimap<size_t, size_t> free_by_len_;  // length -> offset
  std::unordered_map<size_t, size_t> used_;    // offset -> length

  void insert_free(size_t off, size_t len) {
    free_by_off_.emplace(off, len);
    free_by_len_.emplace(len, off);
  }
  void erase_free(size_t off, size_t len) {
    free_by_off_.erase(off);
    auto r = free_by_len_.equal_range(len);
    for (auto it = r.first; it != r.second; ++it)
      if (it->second == off) {
        free_by_len_.erase(it);
        break;
      }
  }
};

}  // namespace pg
