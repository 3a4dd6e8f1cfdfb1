// Free list of a server arena: offset -> size of each free range, kept
// coalesced (no two free ranges touch).  First-fit allocation; freeing
// merges with the neighbouring free ranges.  Host code only; checked on
// the CPU by tests/test_freelist.py.
#pragma once
#include <cstdint>
#include <iterator>
#include <map>

// first-fit: offset of a range of `size`, or -1; size <= 0 takes nothing (0)
inline int64_t list_alloc(std::map<int64_t, int64_t>& fl, int64_t size) {
  if (size <= 0) return 0;
  for (auto it = fl.begin(); it != fl.end(); ++it) {
    if (it->second >= size) {
      const int64_t off = it->first;
      const int64_t rest = it->second - size;
      fl.erase(it);
      if (rest > 0) fl[off + size] = rest;
      return off;
    }
  }
  return -1;
}

inline void list_free(std::map<int64_t, int64_t>& fl, int64_t off, int64_t size) {
  if (size <= 0) return;
  auto it = fl.emplace(off, size).first;
  auto next = std::next(it);
  if (next != fl.end() && it->first + it->second == next->first) {
    it->second += next->second;
    fl.erase(next);
  }
  if (it != fl.begin()) {
    auto prev = std::prev(it);
    if (prev->first + prev->second == it->first) {
      prev->second += it->second;
      fl.erase(it);
    }
  }
}
