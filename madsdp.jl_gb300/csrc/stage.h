// Host staging of a batch's problem data into the layout the kernel reads.
//
// For every problem: b, d_lin, C_lin and the norms ||b||, ||d_lin||,
// max ||C_i|| into its data range; for every block: C, the constraint
// entries sorted by (constraint, column, row) with the constraint pointer,
// the same entries by position (row + column * n, in constraint order) with
// the position pointer, ||C||_max and the constraint structure.
//
// Each problem owns one contiguous range of every staging array (its data
// range starts at ProbDesc::bdat and runs to the next problem's; its
// entries and pointers follow its blocks' offsets), so problems are staged
// on several host threads, each zeroing and writing only its own ranges:
// the staging arrays need no initialization.  Host code only (no CUDA),
// compiled into the library and into the CPU tests of the staging.
#pragma once
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <thread>
#include <vector>

#include "layout.h"

struct StageBuffers {
  double* dd;        // data arena [n_dd]
  int64_t n_dd;
  int32_t* erow;     // entries by constraint [n_ent]
  int32_t* ecol;
  double* eval;
  int32_t* pcon;     // entries by position [n_ent]
  double* pval;
  int64_t* ptr;      // per block: constraint pointer (m + 1), position pointer (n * n + 1)
};

// Stages problem p (whose data range ends at dd_end); false if a
// constraint entry is out of range.  idx and fill are scratch.
inline bool stage_problem(const msdp_problem_desc& d, const ProbDesc& pd, BlockDesc* blocks, int64_t dd_end,
                          const StageBuffers& s, std::vector<int64_t>& idx, std::vector<int64_t>& fill) {
  const int64_t m = d.m, ns = d.ns;
  std::fill(s.dd + pd.bdat, s.dd + dd_end, 0.0);
  double* dat = s.dd + pd.bdat;
  double bn = 0.0, dn = 0.0, cmax = 0.0;
  for (int64_t j = 0; j < m; ++j) {
    dat[j] = d.b[j];
    bn = std::max(bn, std::fabs(d.b[j]));
  }
  for (int64_t k = 0; k < ns; ++k) {
    dat[m + k] = d.d_lin[k];
    dn = std::max(dn, std::fabs(d.d_lin[k]));
  }
  for (int64_t k = 0; k < m * ns; ++k) dat[m + ns + k] = d.C_lin[k];
  for (int i = 0; i < d.nblocks; ++i) {
    BlockDesc& bd = blocks[i];
    const int64_t n = bd.n, nn = n * n, nnz = bd.nnz;
    double cn = 0.0;
    double* cdst = s.dd + bd.cdat;
    const double* csrc = d.C[i];
    for (int64_t k = 0; k < nn; ++k) {
      cdst[k] = csrc[k];
      cn = std::max(cn, std::fabs(csrc[k]));
    }
    bd.cnorm = cn;
    cmax = std::max(cmax, cn);
    const int32_t* con = d.A_con[i];
    const int32_t* row = d.A_row[i];
    const int32_t* col = d.A_col[i];
    const double* val = d.A_val[i];
    for (int64_t e = 0; e < nnz; ++e)
      if (con[e] < 0 || con[e] >= m || row[e] < 0 || row[e] >= n || col[e] < 0 || col[e] >= n) return false;
    // entries by (constraint, column, row); data built by the Python and
    // Julia front ends arrive in this order already
    idx.resize(nnz);
    std::iota(idx.begin(), idx.end(), 0);
    auto before = [&](int64_t a, int64_t c2) {
      if (con[a] != con[c2]) return con[a] < con[c2];
      if (col[a] != col[c2]) return col[a] < col[c2];
      return row[a] < row[c2];
    };
    if (!std::is_sorted(idx.begin(), idx.end(), before)) std::sort(idx.begin(), idx.end(), before);
    int64_t* cptr = s.ptr + bd.conptr;
    std::fill(cptr, cptr + m + 1, 0);
    int32_t* erow = s.erow + bd.ent;
    int32_t* ecol = s.ecol + bd.ent;
    double* eval = s.eval + bd.ent;
    for (int64_t e = 0; e < nnz; ++e) {
      const int64_t q = idx[e];
      erow[e] = row[q];
      ecol[e] = col[q];
      eval[e] = val[q];
      cptr[con[q] + 1] += 1;
    }
    for (int64_t j = 0; j < m; ++j) cptr[j + 1] += cptr[j];
    // Hankel 0/1 structure: m = 2n-1 and constraint j holds exactly the
    // entries (a, j-a) with value 1
    bool hankel = (m == 2 * n - 1) && nnz == n * n;
    for (int64_t j = 0; hankel && j < m; ++j) {
      const int64_t lo = std::max<int64_t>(0, j - n + 1), hi = std::min<int64_t>(j, n - 1);
      if (cptr[j + 1] - cptr[j] != hi - lo + 1) {
        hankel = false;
        break;
      }
      int64_t prev_col = -1;
      for (int64_t q = cptr[j]; q < cptr[j + 1]; ++q) {
        if (erow[q] + ecol[q] != j || eval[q] != 1.0 || ecol[q] <= prev_col) {
          hankel = false;
          break;
        }
        prev_col = ecol[q];
      }
    }
    bd.structure = choose_structure(hankel, n, m, nnz);
    // by position (counting sort, stable in constraint order)
    int64_t* pptr = s.ptr + bd.posptr;
    std::fill(pptr, pptr + nn + 1, 0);
    for (int64_t e = 0; e < nnz; ++e) pptr[row[e] + (int64_t)col[e] * n + 1] += 1;
    for (int64_t k = 0; k < nn; ++k) pptr[k + 1] += pptr[k];
    fill.assign(pptr, pptr + nn);
    int32_t* pcon = s.pcon + bd.ent;
    double* pval = s.pval + bd.ent;
    for (int64_t e = 0; e < nnz; ++e) {
      const int64_t q = idx[e];
      const int64_t slot = fill[row[q] + (int64_t)col[q] * n]++;
      pcon[slot] = con[q];
      pval[slot] = val[q];
    }
  }
  dat[m + ns + m * ns + 0] = bn;
  dat[m + ns + m * ns + 1] = dn;
  dat[m + ns + m * ns + 2] = cmax;
  return true;
}

// Stages every problem on up to `threads` host threads (problems taken in
// chunks from a shared counter); false if any problem has an entry out of
// range.  The result does not depend on the thread count.
inline bool stage_batch(const msdp_problem_desc* probs, int32_t nprob, const ProbDesc* hprob, BlockDesc* hblk,
                        const StageBuffers& s, int threads) {
  constexpr int kChunk = 16;
  threads = std::max(1, std::min(threads, (nprob + kChunk - 1) / kChunk));
  std::atomic<int32_t> next{0};
  std::atomic<bool> ok{true};
  auto work = [&]() {
    std::vector<int64_t> idx, fill;
    for (;;) {
      const int32_t p0 = next.fetch_add(kChunk);
      if (p0 >= nprob || !ok.load(std::memory_order_relaxed)) return;
      const int32_t p1 = std::min(nprob, p0 + kChunk);
      for (int32_t p = p0; p < p1; ++p) {
        const int64_t dd_end = p + 1 < nprob ? hprob[p + 1].bdat : s.n_dd;
        if (!stage_problem(probs[p], hprob[p], hblk + hprob[p].blk0, dd_end, s, idx, fill)) {
          ok.store(false);
          return;
        }
      }
    }
  };
  if (threads == 1) {
    work();
  } else {
    std::vector<std::thread> pool;
    pool.reserve(threads - 1);
    try {
      for (int t = 1; t < threads; ++t) pool.emplace_back(work);
    } catch (...) {
      // fewer threads than asked: the ones started and this one do the work
    }
    work();
    for (auto& th : pool) th.join();
  }
  return ok.load();
}
