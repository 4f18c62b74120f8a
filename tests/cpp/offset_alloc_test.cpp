// The server heap's bookkeeping (painty_gb300/csrc/offset_alloc.h) against a byte map of the
// range: random allocations and releases never overlap or leave the range, every allocation is
// a best fit, releases merge neighbours (the free ranges are exactly the maximal free runs of
// the byte map), and releasing everything leaves one free range of the full size. Prints "ok"
// and returns 0, or names the first failure and returns 1.
#include <cstdio>
#include <map>
#include <random>
#include <vector>

#include "offset_alloc.h"

namespace {

int fail(const char* what, long step) {
  std::printf("FAIL at step %ld: %s\n", step, what);
  return 1;
}

// Maximal runs of free bytes in the map, as offset -> length.
std::map<size_t, size_t> free_runs(const std::vector<int>& owner) {
  std::map<size_t, size_t> runs;
  size_t i = 0;
  while (i < owner.size()) {
    if (owner[i] != 0) {
      i++;
      continue;
    }
    size_t j = i;
    while (j < owner.size() && owner[j] == 0) j++;
    runs.emplace(i, j - i);
    i = j;
  }
  return runs;
}

}  // namespace

int main() {
  const size_t kGranule = 256, kGranules = 4096;
  const size_t size = kGranule * kGranules;
  pg::OffsetAllocator heap(size);
  std::vector<int> owner(kGranules, 0);  // 0 free, else allocation id
  std::map<int, std::pair<size_t, size_t>> live;  // id -> (offset, length) in bytes
  std::mt19937_64 rng(7);
  int next_id = 1;
  for (long step = 0; step < 200000; step++) {
    const bool do_alloc = live.empty() || (rng() % 100) < 55;
    if (do_alloc) {
      // lengths from 1 to 64 granules, skewed small
      const size_t g = 1 + (rng() % 64) * (rng() % 64) / 64;
      const size_t len = g * kGranule;
      size_t off = 0;
      const auto runs = free_runs(owner);
      size_t best = 0;
      for (const auto& r : runs)
        if (r.second * kGranule >= len && (best == 0 || r.second * kGranule < best))
          best = r.second * kGranule;
      if (!heap.alloc(len, &off)) {
        if (best != 0) return fail("alloc refused with a free run that fits", step);
        continue;
      }
      if (off % kGranule != 0 || off + len > size) return fail("allocation outside the range", step);
      const size_t g0 = off / kGranule;
      bool in_run_of_best = false;
      for (const auto& r : runs)
        if (g0 >= r.first && g0 + g <= r.first + r.second && r.second * kGranule == best)
          in_run_of_best = true;
      if (!in_run_of_best) return fail("not a best fit", step);
      for (size_t k = g0; k < g0 + g; k++) {
        if (owner[k] != 0) return fail("overlapping allocation", step);
        owner[k] = next_id;
      }
      live.emplace(next_id++, std::make_pair(off, len));
    } else {
      auto it = live.begin();
      std::advance(it, static_cast<long>(rng() % live.size()));
      const size_t off = it->second.first, len = it->second.second;
      if (!heap.release(off)) return fail("release refused", step);
      if (heap.release(off)) return fail("double release accepted", step);
      for (size_t k = off / kGranule; k < (off + len) / kGranule; k++) owner[k] = 0;
      live.erase(it);
    }
    if (step % 97 == 0) {
      const auto runs = free_runs(owner);
      if (heap.free_ranges() != runs.size()) return fail("free ranges not merged", step);
      size_t fb = 0, lf = 0;
      for (const auto& r : runs) {
        fb += r.second * kGranule;
        if (r.second * kGranule > lf) lf = r.second * kGranule;
      }
      if (heap.free_bytes() != fb || heap.largest_free() != lf)
        return fail("free bytes differ from the byte map", step);
    }
  }
  for (const auto& kv : live)
    if (!heap.release(kv.second.first)) return fail("final release refused", -1);
  if (heap.free_ranges() != 1 || heap.free_bytes() != size || heap.allocations() != 0)
    return fail("not one free range of the full size after releasing everything", -1);
  if (heap.release(12345)) return fail("release of an offset never allocated accepted", -1);
  std::printf("ok\n");
  return 0;
}
