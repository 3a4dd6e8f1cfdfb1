// msdp_solve_static: a solve of one problem that allocates no memory.
//
// Some callers cannot allocate device memory at all: code that runs where a
// framework owns every byte of the GPU (a serving runtime with a fixed
// memory pool, a plugin host that forbids cudaMalloc), or a control loop
// that must not risk an allocation failure or the synchronization a
// cudaMalloc/cudaFree implies.  For them this entry point runs the same FP64
// interior-point kernel as msdp_batch_solve on one problem, with every
// device-side buffer (descriptors, problem data, workspaces) carved out of
// one file-scope static device array of MSDP_STATIC_SCRATCH_BYTES.  Inputs
// and outputs are the caller's host buffers; only cudaMemcpyAsync,
// cudaMemsetAsync and kernel launches are issued, on the caller's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "../../include/madsdp_gpu.h"
#include "launch.h"

namespace {

constexpr int64_t kScratchBytes = MSDP_STATIC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

// The scratch.  Every device that loads the library holds it until exit.
// In host code `g_static_scratch` is only a stand-in for the symbol; its
// device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

void* g_scratch_addr[kMaxDevices];
bool g_scratch_ready[kMaxDevices];

// Stable counting sorts of the raw coordinate entries of one block into the
// by-constraint and by-position layouts the IPM kernel reads, plus the data
// norms.  One thread does the ordered scatters so the result is
// deterministic.
__global__ void static_prepare_kernel(BatchDev B, const int32_t* raw_con, const int32_t* raw_row,
                                      const int32_t* raw_col, const double* raw_val, int64_t* count_buf) {
  const ProbDesc& pd = B.prob[0];
  const int m = pd.m, ns = pd.ns;
  double* dat = const_cast<double*>(B.dd) + pd.bdat;
  if (threadIdx.x == 0) {
    double bn = 0.0, dn = 0.0, cmax = 0.0;
    for (int j = 0; j < m; ++j) bn = fmax(bn, fabs(dat[j]));
    for (int k = 0; k < ns; ++k) dn = fmax(dn, fabs(dat[m + k]));
    for (int i = 0; i < pd.nblocks; ++i) {
      BlockDesc& bd = const_cast<BlockDesc&>(B.blk[i]);
      const int64_t n = bd.n, nn = n * n, nnz = bd.nnz;
      const double* C = B.dd + bd.cdat;
      double cn = 0.0;
      for (int64_t k = 0; k < nn; ++k) cn = fmax(cn, fabs(C[k]));
      bd.cnorm = cn;
      bd.structure = choose_structure(false, n, m, nnz);
      cmax = fmax(cmax, cn);
      const int32_t* con = raw_con + bd.ent;
      const int32_t* row = raw_row + bd.ent;
      const int32_t* col = raw_col + bd.ent;
      const double* val = raw_val + bd.ent;
      int64_t* cptr = const_cast<int64_t*>(B.ptr) + bd.conptr;
      int64_t* pptr = const_cast<int64_t*>(B.ptr) + bd.posptr;
      for (int64_t j = 0; j <= m; ++j) cptr[j] = 0;
      for (int64_t k = 0; k <= nn; ++k) pptr[k] = 0;
      for (int64_t e = 0; e < nnz; ++e) {
        cptr[con[e] + 1] += 1;
        pptr[row[e] + (int64_t)col[e] * n + 1] += 1;
      }
      for (int64_t j = 0; j < m; ++j) cptr[j + 1] += cptr[j];
      for (int64_t k = 0; k < nn; ++k) pptr[k + 1] += pptr[k];
      int64_t* fill = count_buf;
      for (int64_t j = 0; j < m; ++j) fill[j] = cptr[j];
      int32_t* erow = const_cast<int32_t*>(B.e_row) + bd.ent;
      int32_t* ecol = const_cast<int32_t*>(B.e_col) + bd.ent;
      double* eval = const_cast<double*>(B.e_val) + bd.ent;
      for (int64_t e = 0; e < nnz; ++e) {
        const int64_t q = fill[con[e]]++;
        erow[q] = row[e]; ecol[q] = col[e]; eval[q] = val[e];
      }
      for (int64_t k = 0; k < nn; ++k) fill[k] = pptr[k];
      int32_t* pcon = const_cast<int32_t*>(B.p_con) + bd.ent;
      double* pval = const_cast<double*>(B.p_val) + bd.ent;
      // by position, in constraint order (scan the by-constraint list)
      int j = 0;
      for (int64_t q = 0; q < nnz; ++q) {
        while (j < m && cptr[j + 1] <= q) ++j;
        const int64_t pos = erow[q] + (int64_t)ecol[q] * n;
        const int64_t t = fill[pos]++;
        pcon[t] = j; pval[t] = eval[q];
      }
    }
    dat[m + ns + (int64_t)m * ns + 0] = bn;
    dat[m + ns + (int64_t)m * ns + 1] = dn;
    dat[m + ns + (int64_t)m * ns + 2] = cmax;
  }
}

inline int64_t a32(int64_t bytes) { return (bytes + 255) & ~int64_t(255); }

}  // namespace

extern "C" int msdp_solve_static(const msdp_problem_desc* prob, const msdp_components* comp,
                                 const msdp_options* opt, void* stream_ptr, double* const* X, double* y,
                                 double* x, double* z, msdp_stats* stats) {
  if (!prob || prob->nblocks < 0 || prob->m < 0 || prob->ns < 0 || (prob->nblocks == 0 && prob->ns == 0))
    return MSDP_ERR_INVALID_ARGUMENT;
  const int nb = prob->nblocks, m = prob->m, ns = prob->ns;
  if (nb > MSDP_STATIC_MAX_BLOCKS) return MSDP_ERR_TOO_LARGE;
  msdp_components c;
  msdp_options o;
  if (comp) c = *comp; else msdp_default_components(&c);
  if (opt) o = *opt; else msdp_default_options(&o);
  if (c.algorithm != MSDP_PRIMAL_DUAL || c.schur != MSDP_DENSE_CHOLESKY || c.precision != MSDP_FP64)
    return MSDP_ERR_UNSUPPORTED;
  if (o.max_iter < 0 || o.max_schur_reg < 0 || !(c.shrink > 0.0 && c.shrink < 1.0) ||
      !(c.boundary > 0.0 && c.boundary <= 1.0) || !(c.tau > 0.0) ||
      (c.initial_point == MSDP_DUAL_SHIFT && !(c.initial_shift > 0.0)) ||
      (c.initial_point == MSDP_SCALED_IDENTITY && c.scale != 0.0 && !(std::isfinite(c.scale) && c.scale > 0.0)))
    return MSDP_ERR_INVALID_ARGUMENT;
  if (c.initial_point == MSDP_INITIAL_POINT) return MSDP_ERR_UNSUPPORTED;
  cudaStream_t st = (cudaStream_t)stream_ptr;

  // ---- sizes: every factor of the layout below is bounded first, so the
  // int64 offsets cannot overflow for any int32 side or count
  if (8 * (int64_t)m * m > kScratchBytes || 8 * (int64_t)m * ns > kScratchBytes) return MSDP_ERR_TOO_LARGE;
  int64_t total_nnz = 0, nn_sum = 0;
  for (int i = 0; i < nb; ++i) {
    const int64_t n = prob->sides[i];
    if (n <= 0 || prob->A_nnz[i] < 0) return MSDP_ERR_INVALID_ARGUMENT;
    if (8 * n * n > kScratchBytes || prob->A_nnz[i] > kScratchBytes / 52) return MSDP_ERR_TOO_LARGE;
    total_nnz += prob->A_nnz[i];
    nn_sum += n * n;
  }
  if (total_nnz > kScratchBytes / 52 || 8 * nn_sum > kScratchBytes) return MSDP_ERR_TOO_LARGE;
  // the coordinate lists must be in range: checked before anything is
  // enqueued, so a rejected call leaves the shared array as it was
  for (int i = 0; i < nb; ++i)
    for (int64_t q = 0; q < prob->A_nnz[i]; ++q)
      if (prob->A_con[i][q] < 0 || prob->A_con[i][q] >= m || prob->A_row[i][q] < 0 ||
          prob->A_row[i][q] >= prob->sides[i] || prob->A_col[i][q] < 0 || prob->A_col[i][q] >= prob->sides[i])
        return MSDP_ERR_INVALID_ARGUMENT;

  // ---- layout inside the scratch (byte offsets)
  ProbDesc pd;
  BlockDesc bds[MSDP_STATIC_MAX_BLOCKS];
  std::memset(&pd, 0, sizeof(pd));
  std::memset(bds, 0, sizeof(bds));
  int64_t dd = 0, d64 = 0, ent = 0, ptr = 0;
  pd.nblocks = nb; pd.m = m; pd.ns = ns; pd.blk0 = 0;
  pd.bdat = dd; dd += (int64_t)m + ns + (int64_t)m * ns + 3;
  pd.v64 = d64; d64 += (int64_t)V_MCOUNT * m + (int64_t)S_COUNT * ns + SC_COUNT;
  pd.H64 = d64; d64 += (int64_t)m * m;
  pd.Hf = -1; pd.Lf = -1;
  pd.ntraj = 0;
  pd.qr = -1;
  pd.piv = -1;
  pd.K = 0;
  pd.traj = d64;
  for (int i = 0; i < nb; ++i) {
    const int64_t n = prob->sides[i];
    BlockDesc& bd = bds[i];
    bd.n = (int32_t)n; bd.nnz = prob->A_nnz[i];
    bd.cdat = dd; dd += n * n;
    bd.m64 = d64; d64 += (int64_t)M_COUNT * n * n + BS_COUNT;
    bd.w64 = d64; d64 += (int64_t)W_COUNT * n * n + (int64_t)WV_COUNT * (n + 1);
    bd.w32 = -1;
    bd.ent = ent; ent += bd.nnz;
    bd.conptr = ptr; ptr += m + 1;
    bd.posptr = ptr; ptr += n * n + 1;
  }
  const int64_t cnt_len = std::max<int64_t>((int64_t)m, nn_sum) + 1;
  int64_t off = 0;
  const int64_t o_prob = off; off += a32(sizeof(ProbDesc));
  const int64_t o_blk = off; off += a32(sizeof(BlockDesc) * std::max(nb, 1));
  const int64_t o_order = off; off += a32(sizeof(int32_t));
  const int64_t o_queue = off; off += a32(sizeof(int32_t));
  const int64_t o_dd = off; off += a32(sizeof(double) * dd);
  const int64_t o_d64 = off; off += a32(sizeof(double) * d64);
  const int64_t o_erow = off; off += a32(sizeof(int32_t) * total_nnz);
  const int64_t o_ecol = off; off += a32(sizeof(int32_t) * total_nnz);
  const int64_t o_eval = off; off += a32(sizeof(double) * total_nnz);
  const int64_t o_pcon = off; off += a32(sizeof(int32_t) * total_nnz);
  const int64_t o_pval = off; off += a32(sizeof(double) * total_nnz);
  const int64_t o_rcon = off; off += a32(sizeof(int32_t) * total_nnz);
  const int64_t o_rrow = off; off += a32(sizeof(int32_t) * total_nnz);
  const int64_t o_rcol = off; off += a32(sizeof(int32_t) * total_nnz);
  const int64_t o_rval = off; off += a32(sizeof(double) * total_nnz);
  const int64_t o_ptr = off; off += a32(sizeof(int64_t) * ptr);
  const int64_t o_cnt = off; off += a32(sizeof(int64_t) * cnt_len);
  if (off > kScratchBytes) return MSDP_ERR_TOO_LARGE;

  // ---- device address of the scratch: once per device, that device current
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MSDP_ERR_CUDA;
  if (!g_scratch_ready[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || p == nullptr) return MSDP_ERR_CUDA;
    if (msdp_ipm_setup(0) != cudaSuccess) return MSDP_ERR_CUDA;
    g_scratch_addr[dev] = p;
    g_scratch_ready[dev] = true;
  }
  unsigned char* base = (unsigned char*)g_scratch_addr[dev];

  // ---- upload (copies only) and zero what must start at zero
  cudaError_t e = cudaSuccess;
  // an error return still waits for the copies in flight: their sources
  // (this frame's descriptors, the caller's arrays) may be read until then
  auto bail = [&]() {
    cudaStreamSynchronize(st);
    return MSDP_ERR_CUDA;
  };
  auto up = [&](int64_t dst, const void* src, size_t bytes) {
    if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(base + dst, src, bytes, cudaMemcpyHostToDevice, st);
  };
  const int32_t zero_order = 0;
  if (e == cudaSuccess) e = cudaMemsetAsync(base, 0, (size_t)off, st);
  up(o_prob, &pd, sizeof(ProbDesc));
  up(o_blk, bds, sizeof(BlockDesc) * nb);
  up(o_order, &zero_order, sizeof(int32_t));
  up(o_dd + sizeof(double) * pd.bdat, prob->b, sizeof(double) * m);
  up(o_dd + sizeof(double) * (pd.bdat + m), prob->d_lin, sizeof(double) * ns);
  up(o_dd + sizeof(double) * (pd.bdat + m + ns), prob->C_lin, sizeof(double) * m * ns);
  for (int i = 0; i < nb; ++i) {
    const BlockDesc& bd = bds[i];
    up(o_dd + sizeof(double) * bd.cdat, prob->C[i], sizeof(double) * bd.n * bd.n);
    up(o_rcon + sizeof(int32_t) * bd.ent, prob->A_con[i], sizeof(int32_t) * bd.nnz);
    up(o_rrow + sizeof(int32_t) * bd.ent, prob->A_row[i], sizeof(int32_t) * bd.nnz);
    up(o_rcol + sizeof(int32_t) * bd.ent, prob->A_col[i], sizeof(int32_t) * bd.nnz);
    up(o_rval + sizeof(double) * bd.ent, prob->A_val[i], sizeof(double) * bd.nnz);
  }
  if (e != cudaSuccess) return bail();

  BatchDev B;
  std::memset(&B, 0, sizeof(B));
  B.nprob = 1;
  B.prob = (const ProbDesc*)(base + o_prob);
  B.blk = (const BlockDesc*)(base + o_blk);
  B.order = (const int32_t*)(base + o_order);
  B.dd = (const double*)(base + o_dd);
  B.d64 = (double*)(base + o_d64);
  B.d32 = nullptr;
  B.e_row = (const int32_t*)(base + o_erow);
  B.e_col = (const int32_t*)(base + o_ecol);
  B.e_val = (const double*)(base + o_eval);
  B.p_con = (const int32_t*)(base + o_pcon);
  B.p_val = (const double*)(base + o_pval);
  B.ptr = (const int64_t*)(base + o_ptr);
  B.queue = (int32_t*)(base + o_queue);
  Params& prm = B.prm;
  prm.algorithm = c.algorithm; prm.direction = c.direction; prm.step = c.step; prm.centering = c.centering;
  prm.initial_point = c.initial_point; prm.schur = c.schur; prm.precision = MSDP_FP64;
  prm.centering_max_iter = c.centering_max_iter;
  prm.tau = c.tau; prm.shrink = c.shrink; prm.boundary = c.boundary; prm.sigma_exponent = c.sigma_exponent;
  prm.initial_ratio = c.initial_ratio; prm.ratio = c.ratio; prm.scale = c.scale;
  prm.initial_shift = c.initial_shift; prm.max_shift = c.max_shift;
  prm.dc_beta = c.dc_beta; prm.dc_delta = c.dc_delta; prm.dc_A = c.dc_A;
  prm.tol = o.tol; prm.max_wall_time = o.max_wall_time; prm.mu_min = o.mu_min;
  prm.regularize_schur = o.regularize_schur; prm.switch_tol = o.switch_tol;
  prm.max_iter = o.max_iter; prm.max_schur_reg = o.max_schur_reg;

  static_prepare_kernel<<<1, 32, 0, st>>>(B, (const int32_t*)(base + o_rcon), (const int32_t*)(base + o_rrow),
                                          (const int32_t*)(base + o_rcol), (const double*)(base + o_rval),
                                          (int64_t*)(base + o_cnt));
  if (cudaGetLastError() != cudaSuccess) return bail();
  // initialize!, then iterate to termination (the work queue starts at 0)
  prm.op = OP_INITIALIZE;
  if (msdp_ipm_launch(0, B, 1, st) != cudaSuccess) return bail();
  if (cudaMemsetAsync(base + o_queue, 0, sizeof(int32_t), st) != cudaSuccess) return bail();
  prm.op = OP_ITERATE;
  prm.max_iterations = 0;
  if (msdp_ipm_launch(0, B, 1, st) != cudaSuccess) return bail();

  // ---- outputs
  double sc[SC_COUNT];
  auto down = [&](void* dst, int64_t src, size_t bytes) {
    if (e == cudaSuccess && dst && bytes) e = cudaMemcpyAsync(dst, base + src, bytes, cudaMemcpyDeviceToHost, st);
  };
  const int64_t v = o_d64 + sizeof(double) * pd.v64;
  down(sc, v + sizeof(double) * ((int64_t)V_MCOUNT * m + (int64_t)S_COUNT * ns), sizeof(double) * SC_COUNT);
  down(y, v + sizeof(double) * ((int64_t)V_Y * m), sizeof(double) * m);
  down(x, v + sizeof(double) * ((int64_t)V_MCOUNT * m + (int64_t)S_X * ns), sizeof(double) * ns);
  down(z, v + sizeof(double) * ((int64_t)V_MCOUNT * m + (int64_t)S_Z * ns), sizeof(double) * ns);
  for (int i = 0; i < nb; ++i)
    if (X) down(X[i], o_d64 + sizeof(double) * (bds[i].m64 + (int64_t)M_X * bds[i].n * bds[i].n),
                sizeof(double) * bds[i].n * bds[i].n);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return bail();
  if ((int)sc[SC_STATUS] == MSDP_STATUS_INITIAL_POINT_ERROR) return MSDP_ERR_INITIAL_POINT;
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->status = (int32_t)sc[SC_STATUS];
    stats->iter = (int32_t)sc[SC_ITER];
    stats->iter_fp64 = (int32_t)sc[SC_N64];
    stats->pobj = sc[SC_POBJ]; stats->dobj = sc[SC_DOBJ];
    stats->inf_pr = sc[SC_INFPR]; stats->inf_du = sc[SC_INFDU]; stats->gap = sc[SC_GAP];
    stats->mu = sc[SC_MU]; stats->sigma = sc[SC_SIGMA]; stats->alpha = sc[SC_ALPHA]; stats->beta = sc[SC_BETA];
    stats->solve_ns = sc[SC_SOLVE_NS];
  }
  return MSDP_OK;
}
