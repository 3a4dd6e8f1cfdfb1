// CPU test harness of the host staging of a batch (csrc/stage.h): lays the
// problems out the way msdp_batch_create does (each problem's data range
// followed by its blocks', padded to 4 elements; entries and pointers
// block after block) and stages them on a given number of threads.
#define __host__
#define __device__
#include "../../madsdp.jl_gb300/csrc/stage.h"

namespace {
int64_t pad4(int64_t x) { return (x + 3) & ~int64_t(3); }

void layout(const msdp_problem_desc* probs, int32_t nprob, std::vector<ProbDesc>& hp, std::vector<BlockDesc>& hb,
            int64_t* sizes) {
  int64_t o_dd = 0, o_ent = 0, o_ptr = 0;
  hp.assign(nprob, ProbDesc{});
  hb.clear();
  for (int32_t p = 0; p < nprob; ++p) {
    const msdp_problem_desc& d = probs[p];
    hp[p].nblocks = d.nblocks;
    hp[p].m = d.m;
    hp[p].ns = d.ns;
    hp[p].blk0 = (int32_t)hb.size();
    hp[p].bdat = o_dd;
    o_dd = pad4(o_dd + d.m + d.ns + (int64_t)d.m * d.ns + 3);
    for (int i = 0; i < d.nblocks; ++i) {
      BlockDesc bd{};
      bd.n = d.sides[i];
      bd.nnz = d.A_nnz[i];
      bd.cdat = o_dd;
      o_dd = pad4(o_dd + (int64_t)bd.n * bd.n);
      bd.ent = o_ent;
      o_ent += bd.nnz;
      bd.conptr = o_ptr;
      o_ptr += d.m + 1;
      bd.posptr = o_ptr;
      o_ptr += (int64_t)bd.n * bd.n + 1;
      hb.push_back(bd);
    }
  }
  sizes[0] = o_dd;
  sizes[1] = o_ent;
  sizes[2] = o_ptr;
  sizes[3] = (int64_t)hb.size();
}
}  // namespace

extern "C" {

// sizes: [data arena, entries, pointers, blocks]
void stage_sizes(const msdp_problem_desc* probs, int32_t nprob, int64_t* sizes) {
  std::vector<ProbDesc> hp;
  std::vector<BlockDesc> hb;
  layout(probs, nprob, hp, hb, sizes);
}

// Stages into the given arrays; per block writes its offsets
// (cdat, ent, conptr, posptr), structure and ||C||_max.  Returns 1 on
// success, 0 when an entry is out of range.
int stage_run(const msdp_problem_desc* probs, int32_t nprob, int threads, double* dd, int32_t* erow, int32_t* ecol,
              double* eval, int32_t* pcon, double* pval, int64_t* ptr, int64_t* block_offsets, int32_t* structure,
              double* cnorm) {
  std::vector<ProbDesc> hp;
  std::vector<BlockDesc> hb;
  int64_t sizes[4];
  layout(probs, nprob, hp, hb, sizes);
  const StageBuffers sb{dd, sizes[0], erow, ecol, eval, pcon, pval, ptr};
  if (!stage_batch(probs, nprob, hp.data(), hb.data(), sb, threads)) return 0;
  for (size_t k = 0; k < hb.size(); ++k) {
    block_offsets[4 * k + 0] = hb[k].cdat;
    block_offsets[4 * k + 1] = hb[k].ent;
    block_offsets[4 * k + 2] = hb[k].conptr;
    block_offsets[4 * k + 3] = hb[k].posptr;
    structure[k] = hb[k].structure;
    cnorm[k] = hb[k].cnorm;
  }
  return 1;
}

}  // extern "C"
