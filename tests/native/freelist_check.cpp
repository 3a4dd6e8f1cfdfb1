// CPU test harness of the server's arena free list (csrc/freelist.h): a
// free list of `capacity`, driven by a sequence of operations.
#include <cstdint>
#include <map>

#include "../../madsdp.jl_gb300/csrc/freelist.h"

extern "C" {

// ops[i] > 0: allocate ops[i] (result offset or -1 in out[i]);
// ops[i] < 0: free the allocation made by operation -ops[i] - 1 (sizes[i]
// holds its size, offs[i] its offset).  After the run, the free list is
// written to free_off / free_size (at most max_free entries); returns its
// length.
int64_t freelist_run(int64_t capacity, int64_t nops, const int64_t* ops, const int64_t* offs, const int64_t* sizes,
                     int64_t* out, int64_t max_free, int64_t* free_off, int64_t* free_size) {
  std::map<int64_t, int64_t> fl;
  fl[0] = capacity;
  for (int64_t i = 0; i < nops; ++i) {
    if (ops[i] > 0) out[i] = list_alloc(fl, ops[i]);
    else {
      list_free(fl, offs[i], sizes[i]);
      out[i] = 0;
    }
  }
  int64_t k = 0;
  for (const auto& e : fl) {
    if (k < max_free) {
      free_off[k] = e.first;
      free_size[k] = e.second;
    }
    ++k;
  }
  return k;
}

}  // extern "C"
