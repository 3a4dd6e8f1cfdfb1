// Host side of the C ABI (include/madsdp_gpu.h): batch layout, upload,
// kernel launches and readback.  One context = one device + one stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/madsdp_gpu.h"
#include "launch.h"
#include "stage.h"

struct msdp_context {
  int device = 0;
  int nsm = 0;
  cudaStream_t stream = nullptr;
  std::string err;
};

struct msdp_batch {
  msdp_context* ctx = nullptr;
  int nprob = 0;
  bool mixed = false;
  Params prm{};
  std::vector<ProbDesc> hprob;
  std::vector<BlockDesc> hblk;
  // device arrays
  ProbDesc* dprob = nullptr;
  BlockDesc* dblk = nullptr;
  int32_t* dorder = nullptr;
  double* dd = nullptr;
  double* d64 = nullptr;
  float* d32 = nullptr;
  int32_t *erow = nullptr, *ecol = nullptr, *pcon = nullptr;
  double *eval = nullptr, *pval = nullptr;
  int64_t* ptr = nullptr;
  int32_t* queue = nullptr;
  double* scal = nullptr;  // gathered scalars nprob * SC_COUNT
  int64_t n_dd = 0, n_d64 = 0, n_d32 = 0, n_ent = 0, n_ptr = 0;
  int64_t bytes = 0;
  int64_t launches = 0;
  int64_t upload_bytes = 0;
  int grid = 0;
  // packed download of every solution (built on the first call)
  double* gsol = nullptr;
  void* gseg = nullptr;
  int64_t nseg = 0, sol_size = 0;
};

namespace {

int fail(msdp_context* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? MSDP_ERR_OUT_OF_MEMORY : MSDP_ERR_CUDA, \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                  \
    }                                                                                   \
  } while (0)

inline int64_t align4(int64_t x) { return (x + 3) & ~int64_t(3); }

template <class T>
int dev_alloc(msdp_context* ctx, T** p, int64_t count, int64_t* bytes) {
  *p = nullptr;
  if (count <= 0) count = 1;
  CK(cudaMalloc((void**)p, sizeof(T) * (size_t)count));
  *bytes += sizeof(T) * count;
  return 0;
}

}  // namespace

extern "C" {

void msdp_default_components(msdp_components* c) {
  std::memset(c, 0, sizeof(*c));
  c->algorithm = MSDP_PRIMAL_DUAL;
  c->direction = MSDP_NT;
  c->step = MSDP_EIGEN_STEP;
  c->centering = MSDP_MEHROTRA;
  c->initial_point = MSDP_SCALED_IDENTITY;
  c->schur = MSDP_DENSE_CHOLESKY;
  c->precision = MSDP_FP64;
  c->centering_max_iter = 50;
  c->tau = 0.95;
  c->shrink = 0.8;
  c->boundary = 0.95;
  c->sigma_exponent = 3.0;
  c->initial_ratio = 0.25;
  c->ratio = 0.5;
  c->scale = 0.0;
  c->initial_shift = 1.0;
  c->max_shift = 1e10;
  c->dc_beta = 0.2;
  c->dc_delta = 1.0;
  c->dc_A = 2.0;
}

void msdp_default_options(msdp_options* o) {
  std::memset(o, 0, sizeof(*o));
  o->tol = 1e-7;
  o->max_iter = 100;
  o->max_schur_reg = 8;
  o->max_wall_time = 3600.0;
  o->mu_min = 1e-14;
  o->regularize_schur = 1e-12;
  o->datasparsity = 8;
  o->mixed_refine = 2;
  o->switch_tol = 0.0;
}

int msdp_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}

int msdp_context_create(int device, msdp_context** out) {
  if (!out) return MSDP_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  msdp_context* ctx = new msdp_context();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = msdp_ipm_setup(0);
  if (e == cudaSuccess) e = msdp_ipm_setup(1);
  if (e != cudaSuccess) {
    delete ctx;
    return MSDP_ERR_CUDA;
  }
  *out = ctx;
  return MSDP_OK;
}

int msdp_context_destroy(msdp_context* ctx) {
  if (!ctx) return MSDP_OK;
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return MSDP_OK;
}

const char* msdp_last_error(const msdp_context* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

void* msdp_context_stream(const msdp_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int msdp_batch_destroy(msdp_batch* b) {
  if (!b) return MSDP_OK;
  void* ptrs[] = {b->dprob, b->dblk, b->dorder, b->dd, b->d64, b->d32, b->erow, b->ecol,
                  b->pcon,  b->eval, b->pval,   b->ptr, b->queue, b->scal, b->gsol, b->gseg};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete b;
  return MSDP_OK;
}

int64_t msdp_batch_device_bytes(const msdp_batch* b) { return b ? b->bytes : 0; }
int64_t msdp_batch_launch_count(const msdp_batch* b) { return b ? b->launches : 0; }

int msdp_batch_create(msdp_context* ctx, const msdp_problem_desc* probs, int32_t nprob,
                      const msdp_components* comp, const msdp_options* opt, msdp_batch** out) {
  if (!ctx || !out || !probs || nprob <= 0) return fail(ctx, MSDP_ERR_INVALID_ARGUMENT, "invalid batch arguments");
  *out = nullptr;
  msdp_components c;
  msdp_options o;
  if (comp) c = *comp; else msdp_default_components(&c);
  if (opt) o = *opt; else msdp_default_options(&o);
  // ---- component checks (src/qr_schur.jl:12-22, src/dual_centering.jl:68-76)
  if (c.schur == MSDP_QR_SCHUR && !(c.algorithm == MSDP_PRIMAL_DUAL && c.direction == MSDP_NT))
    return fail(ctx, MSDP_ERR_INVALID_ARGUMENT, "QRSchur requires PrimalDual with the NT direction.");
  if (c.algorithm == MSDP_DUAL_CENTERING) {
    for (int p = 0; p < nprob; ++p) {
      if (probs[p].ns > 0)
        return fail(ctx, MSDP_ERR_INITIAL_POINT, "MadSDP: `DualCentering` does not support scalar (LP) blocks yet.");
      if (probs[p].nblocks == 0)
        return fail(ctx, MSDP_ERR_INITIAL_POINT, "MadSDP: `DualCentering` needs at least one PSD block.");
    }
  } else if (c.algorithm != MSDP_PRIMAL_DUAL) {
    return fail(ctx, MSDP_ERR_INVALID_ARGUMENT, "unknown algorithm");
  }
  if (c.schur == MSDP_QR_SCHUR && c.precision != MSDP_FP64)
    return fail(ctx, MSDP_ERR_INVALID_ARGUMENT, "QRSchur requires Float64 data.");
  if (c.precision != MSDP_FP64 && c.precision != MSDP_MIXED)
    return fail(ctx, MSDP_ERR_UNSUPPORTED, "this precision runs on the whole-GPU solver only");

  if (c.initial_point == MSDP_SCALED_IDENTITY && c.scale != 0.0 && !(std::isfinite(c.scale) && c.scale > 0.0))
    return fail(ctx, MSDP_ERR_INVALID_ARGUMENT, "The identity scale must be finite and positive.");
  if (o.max_iter < 0 || o.max_schur_reg < 0) return fail(ctx, MSDP_ERR_INVALID_ARGUMENT, "invalid options");
  if (!(c.shrink > 0.0 && c.shrink < 1.0) || !(c.boundary > 0.0 && c.boundary <= 1.0) || !(c.tau > 0.0))
    return fail(ctx, MSDP_ERR_INVALID_ARGUMENT, "invalid step-length parameters");
  if (c.initial_point == MSDP_DUAL_SHIFT && !(c.initial_shift > 0.0))
    return fail(ctx, MSDP_ERR_INVALID_ARGUMENT, "DualShift needs a positive initial shift");

  msdp_batch* b = new msdp_batch();
  b->ctx = ctx;
  b->nprob = nprob;
  b->mixed = (c.precision == MSDP_MIXED);
  Params& prm = b->prm;
  prm.algorithm = c.algorithm; prm.direction = c.direction; prm.step = c.step; prm.centering = c.centering;
  prm.initial_point = c.initial_point; prm.schur = c.schur; prm.precision = c.precision;
  prm.centering_max_iter = c.centering_max_iter;
  prm.tau = c.tau; prm.shrink = c.shrink; prm.boundary = c.boundary; prm.sigma_exponent = c.sigma_exponent;
  prm.initial_ratio = c.initial_ratio; prm.ratio = c.ratio; prm.scale = c.scale;
  prm.initial_shift = c.initial_shift; prm.max_shift = c.max_shift;
  prm.dc_beta = c.dc_beta; prm.dc_delta = c.dc_delta; prm.dc_A = c.dc_A;
  prm.tol = o.tol; prm.max_wall_time = o.max_wall_time; prm.mu_min = o.mu_min;
  prm.regularize_schur = o.regularize_schur; prm.switch_tol = o.switch_tol;
  prm.max_iter = o.max_iter; prm.max_schur_reg = o.max_schur_reg;
  prm.mixed_refine = std::max(0, std::min(o.mixed_refine, 8));

  // ---- layout pass
  int64_t nblk_total = 0;
  for (int p = 0; p < nprob; ++p) {
    const msdp_problem_desc& d = probs[p];
    if (d.nblocks < 0 || d.m < 0 || d.ns < 0 || (d.nblocks == 0 && d.ns == 0)) {
      msdp_batch_destroy(b);
      return fail(ctx, MSDP_ERR_INVALID_ARGUMENT, "MadSDP: model has no variables.");
    }
    nblk_total += d.nblocks;
  }
  b->hprob.resize(nprob);
  b->hblk.resize(nblk_total);
  int64_t o_dd = 0, o64 = 0, o32 = 0, o_ent = 0, o_ptr = 0;
  int64_t bi = 0;
  std::vector<double> cost(nprob, 0.0);
  for (int p = 0; p < nprob; ++p) {
    const msdp_problem_desc& d = probs[p];
    ProbDesc& pd = b->hprob[p];
    pd.nblocks = d.nblocks; pd.m = d.m; pd.ns = d.ns; pd.blk0 = (int32_t)bi;
    const int64_t m = d.m, ns = d.ns;
    pd.bdat = o_dd; o_dd = align4(o_dd + m + ns + m * ns + 3);
    pd.v64 = o64; o64 = align4(o64 + V_MCOUNT * m + S_COUNT * ns + SC_COUNT);
    pd.H64 = o64; o64 = align4(o64 + m * m);
    if (b->mixed) {
      pd.Hf = o32; o32 = align4(o32 + m * m);
      pd.Lf = o32; o32 = align4(o32 + m * m);
    } else {
      pd.Hf = -1; pd.Lf = -1;
    }
    pd.ntraj = o.max_iter + 2;
    pd.traj = o64; o64 = align4(o64 + (int64_t)pd.ntraj * TRAJ_FIELDS);
    int64_t K = ns;
    for (int i = 0; i < d.nblocks; ++i) K += (int64_t)d.sides[i] * (d.sides[i] + 1) / 2;
    pd.K = (int32_t)K;
    if (c.schur == MSDP_QR_SCHUR) { pd.qr = o64; o64 = align4(o64 + K * m + 2 * m + 2 * K); }
    else pd.qr = -1;
    if (c.schur == MSDP_MADNLP_SCHUR) { pd.piv = o64; o64 = align4(o64 + m); }
    else pd.piv = -1;
    double nnz_sum = 0.0;
    for (int i = 0; i < d.nblocks; ++i, ++bi) {
      BlockDesc& bd = b->hblk[bi];
      const int64_t n = d.sides[i];
      if (n <= 0) {
        msdp_batch_destroy(b);
        return fail(ctx, MSDP_ERR_INVALID_ARGUMENT, "block sides must be positive");
      }
      bd.n = (int32_t)n;
      bd.nnz = d.A_nnz[i];
      bd.cdat = o_dd; o_dd = align4(o_dd + n * n);
      bd.m64 = o64; o64 = align4(o64 + M_COUNT * n * n + BS_COUNT);
      bd.w64 = o64; o64 = align4(o64 + W_COUNT * n * n + WV_COUNT * (n + 1));
      if (b->mixed) { bd.w32 = o32; o32 = align4(o32 + W_COUNT * n * n + WV_COUNT * (n + 1)); }
      else bd.w32 = -1;
      bd.ent = o_ent; o_ent += bd.nnz;
      bd.conptr = o_ptr; o_ptr += m + 1;
      bd.posptr = o_ptr; o_ptr += n * n + 1;
      nnz_sum += (double)bd.nnz;
      cost[p] += 60.0 * (double)(n * n * n);
    }
    cost[p] += nnz_sum * nnz_sum + (double)(m * m * m) / 3.0;
  }
  b->n_dd = o_dd; b->n_d64 = o64; b->n_d32 = o32; b->n_ent = o_ent; b->n_ptr = o_ptr;

  // ---- host staging (stage.h), on the host threads
  std::unique_ptr<double[]> hdd(new double[std::max<int64_t>(o_dd, 1)]);
  std::unique_ptr<int32_t[]> herow(new int32_t[std::max<int64_t>(o_ent, 1)]);
  std::unique_ptr<int32_t[]> hecol(new int32_t[std::max<int64_t>(o_ent, 1)]);
  std::unique_ptr<int32_t[]> hpcon(new int32_t[std::max<int64_t>(o_ent, 1)]);
  std::unique_ptr<double[]> heval(new double[std::max<int64_t>(o_ent, 1)]);
  std::unique_ptr<double[]> hpval(new double[std::max<int64_t>(o_ent, 1)]);
  std::unique_ptr<int64_t[]> hptr(new int64_t[std::max<int64_t>(o_ptr, 1)]);
  const StageBuffers sb{hdd.get(), o_dd, herow.get(), hecol.get(), heval.get(), hpcon.get(), hpval.get(), hptr.get()};
  if (!stage_batch(probs, nprob, b->hprob.data(), b->hblk.data(), sb, (int)std::thread::hardware_concurrency())) {
    msdp_batch_destroy(b);
    return fail(ctx, MSDP_ERR_INVALID_ARGUMENT, "constraint entry out of range");
  }
  std::vector<int32_t> order(nprob);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c2) { return cost[a] > cost[c2]; });

  // ---- device allocation and upload
  int rc = 0;
  int64_t& by = b->bytes;
  if ((rc = dev_alloc(ctx, &b->dprob, nprob, &by)) || (rc = dev_alloc(ctx, &b->dblk, std::max<int64_t>(nblk_total, 1), &by)) ||
      (rc = dev_alloc(ctx, &b->dorder, nprob, &by)) || (rc = dev_alloc(ctx, &b->dd, o_dd, &by)) ||
      (rc = dev_alloc(ctx, &b->d64, o64, &by)) || (rc = dev_alloc(ctx, &b->d32, o32, &by)) ||
      (rc = dev_alloc(ctx, &b->erow, o_ent, &by)) || (rc = dev_alloc(ctx, &b->ecol, o_ent, &by)) ||
      (rc = dev_alloc(ctx, &b->pcon, o_ent, &by)) || (rc = dev_alloc(ctx, &b->eval, o_ent, &by)) ||
      (rc = dev_alloc(ctx, &b->pval, o_ent, &by)) || (rc = dev_alloc(ctx, &b->ptr, o_ptr, &by)) ||
      (rc = dev_alloc(ctx, &b->queue, 1, &by)) || (rc = dev_alloc(ctx, &b->scal, (int64_t)nprob * SC_COUNT, &by))) {
    msdp_batch_destroy(b);
    return rc;
  }
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaSuccess;
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
  };
  up(b->dprob, b->hprob.data(), sizeof(ProbDesc) * nprob);
  up(b->dblk, b->hblk.data(), sizeof(BlockDesc) * nblk_total);
  up(b->dorder, order.data(), sizeof(int32_t) * nprob);
  up(b->dd, hdd.get(), sizeof(double) * o_dd);
  up(b->erow, herow.get(), sizeof(int32_t) * o_ent);
  up(b->ecol, hecol.get(), sizeof(int32_t) * o_ent);
  up(b->pcon, hpcon.get(), sizeof(int32_t) * o_ent);
  up(b->eval, heval.get(), sizeof(double) * o_ent);
  up(b->pval, hpval.get(), sizeof(double) * o_ent);
  up(b->ptr, hptr.get(), sizeof(int64_t) * o_ptr);
  b->upload_bytes = (int64_t)(sizeof(ProbDesc) * nprob + sizeof(BlockDesc) * nblk_total + sizeof(int32_t) * nprob +
                              sizeof(double) * o_dd + (3 * sizeof(int32_t) + 2 * sizeof(double)) * o_ent +
                              sizeof(int64_t) * o_ptr);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d64, 0, sizeof(double) * std::max<int64_t>(o64, 1), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d32, 0, sizeof(float) * std::max<int64_t>(o32, 1), st);
  // staging buffers are pageable: wait before they go out of scope
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    msdp_batch_destroy(b);
    return fail(ctx, MSDP_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(e));
  }
  int occ = std::max(msdp_ipm_occupancy(b->mixed ? 1 : 0), 1);
  b->grid = std::min(nprob, ctx->nsm * occ);
  *out = b;
  return MSDP_OK;
}

}  // extern "C"

namespace {

BatchDev make_dev(msdp_batch* b) {
  BatchDev B;
  std::memset(&B, 0, sizeof(B));
  B.nprob = b->nprob;
  B.prob = b->dprob; B.blk = b->dblk; B.order = b->dorder;
  B.dd = b->dd; B.d64 = b->d64; B.d32 = b->d32;
  B.e_row = b->erow; B.e_col = b->ecol; B.e_val = b->eval;
  B.p_con = b->pcon; B.p_val = b->pval; B.ptr = b->ptr;
  B.queue = b->queue;
  B.prm = b->prm;
  return B;
}

int launch(msdp_batch* b, int op, int max_iterations, double mu, int corrected) {
  msdp_context* ctx = b->ctx;
  b->prm.op = op;
  b->prm.max_iterations = max_iterations;
  b->prm.op_mu = mu;
  b->prm.op_corrected = corrected;
  BatchDev B = make_dev(b);
  CK(cudaMemsetAsync(b->queue, 0, sizeof(int32_t), ctx->stream));
  CK(msdp_ipm_launch(b->mixed ? 1 : 0, B, b->grid, ctx->stream));
  b->launches += 1;
  return MSDP_OK;
}

int sync(msdp_batch* b) {
  msdp_context* ctx = b->ctx;
  CK(cudaStreamSynchronize(ctx->stream));
  return MSDP_OK;
}

int gather(msdp_batch* b, std::vector<double>& sc) {
  msdp_context* ctx = b->ctx;
  BatchDev B = make_dev(b);
  CK(msdp_gather_launch(B, b->scal, ctx->stream));
  b->launches += 1;
  sc.resize((size_t)b->nprob * SC_COUNT);
  CK(cudaMemcpyAsync(sc.data(), b->scal, sizeof(double) * sc.size(), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return MSDP_OK;
}

void fill_stats(const double* sc, msdp_stats* s) {
  std::memset(s, 0, sizeof(*s));
  s->status = (int32_t)sc[SC_STATUS];
  s->iter = (int32_t)sc[SC_ITER];
  s->iter_fp32 = (int32_t)sc[SC_N32];
  s->iter_fp64 = (int32_t)sc[SC_N64];
  s->pobj = sc[SC_POBJ]; s->dobj = sc[SC_DOBJ];
  s->inf_pr = sc[SC_INFPR]; s->inf_du = sc[SC_INFDU]; s->gap = sc[SC_GAP];
  s->mu = sc[SC_MU]; s->sigma = sc[SC_SIGMA]; s->alpha = sc[SC_ALPHA]; s->beta = sc[SC_BETA];
  s->solve_ns = sc[SC_SOLVE_NS];
  s->n_newton = (int32_t)sc[SC_NNEWTON]; s->n_predictor = (int32_t)sc[SC_NPRED];
}

int copy_d2h(msdp_batch* b, void* dst, const void* src, size_t bytes) {
  msdp_context* ctx = b->ctx;
  if (!dst || !bytes) return MSDP_OK;
  CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return MSDP_OK;
}

int copy_h2d(msdp_batch* b, void* dst, const void* src, size_t bytes) {
  msdp_context* ctx = b->ctx;
  if (!src || !bytes) return MSDP_OK;
  CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return MSDP_OK;
}

bool bad_prob(msdp_batch* b, int32_t p) { return !b || p < 0 || p >= b->nprob; }

double* vec64(msdp_batch* b, int32_t p, int which_m) {
  const ProbDesc& d = b->hprob[p];
  return b->d64 + d.v64 + (int64_t)which_m * d.m;
}
double* svec64(msdp_batch* b, int32_t p, int which_s) {
  const ProbDesc& d = b->hprob[p];
  return b->d64 + d.v64 + (int64_t)V_MCOUNT * d.m + (int64_t)which_s * d.ns;
}
double* bmat64(msdp_batch* b, int32_t p, int i, int which) {
  const BlockDesc& bd = b->hblk[b->hprob[p].blk0 + i];
  return b->d64 + bd.m64 + (int64_t)which * bd.n * bd.n;
}

}  // namespace

extern "C" {

int msdp_batch_set_initial_point(msdp_batch* b, int32_t p, const double* const* X, const double* y,
                                 const double* x) {
  if (bad_prob(b, p)) return MSDP_ERR_INVALID_ARGUMENT;
  const ProbDesc& d = b->hprob[p];
  int rc;
  for (int i = 0; i < d.nblocks; ++i) {
    const int64_t n = b->hblk[d.blk0 + i].n;
    if (X && X[i] && (rc = copy_h2d(b, bmat64(b, p, i, M_X), X[i], sizeof(double) * n * n))) return rc;
  }
  if ((rc = copy_h2d(b, vec64(b, p, V_Y), y, sizeof(double) * d.m))) return rc;
  std::vector<double> ones(d.ns, 1.0);
  if ((rc = copy_h2d(b, svec64(b, p, S_X), x ? x : ones.data(), sizeof(double) * d.ns))) return rc;
  return MSDP_OK;
}

int msdp_batch_set_iterate(msdp_batch* b, int32_t p, const double* const* X, const double* const* S,
                           const double* y, const double* x, const double* z) {
  if (bad_prob(b, p)) return MSDP_ERR_INVALID_ARGUMENT;
  const ProbDesc& d = b->hprob[p];
  int rc;
  for (int i = 0; i < d.nblocks; ++i) {
    const int64_t n = b->hblk[d.blk0 + i].n;
    if (X && X[i] && (rc = copy_h2d(b, bmat64(b, p, i, M_X), X[i], sizeof(double) * n * n))) return rc;
    if (S && S[i] && (rc = copy_h2d(b, bmat64(b, p, i, M_S), S[i], sizeof(double) * n * n))) return rc;
  }
  if ((rc = copy_h2d(b, vec64(b, p, V_Y), y, sizeof(double) * d.m))) return rc;
  if ((rc = copy_h2d(b, svec64(b, p, S_X), x, sizeof(double) * d.ns))) return rc;
  if ((rc = copy_h2d(b, svec64(b, p, S_Z), z, sizeof(double) * d.ns))) return rc;
  return MSDP_OK;
}

int msdp_batch_initialize(msdp_batch* b) {
  if (!b) return MSDP_ERR_INVALID_ARGUMENT;
  int rc = launch(b, OP_INITIALIZE, 0, 0.0, 0);
  if (rc) return rc;
  if ((rc = sync(b))) return rc;
  std::vector<double> sc;
  if ((rc = gather(b, sc))) return rc;
  for (int p = 0; p < b->nprob; ++p)
    if ((int)sc[(size_t)p * SC_COUNT + SC_STATUS] == MSDP_STATUS_INITIAL_POINT_ERROR)
      return fail(b->ctx, MSDP_ERR_INITIAL_POINT,
                  "MadSDP: could not find a dual interior point `y = -rho 1` with rho <= max_shift; "
                  "use `InitialPoint` to give one.");
  return MSDP_OK;
}

int msdp_batch_launch_initialize(msdp_batch* b) {
  if (!b) return MSDP_ERR_INVALID_ARGUMENT;
  return launch(b, OP_INITIALIZE, 0, 0.0, 0);
}

int64_t msdp_batch_upload_bytes(const msdp_batch* b) { return b ? b->upload_bytes : 0; }

int msdp_batch_launch_solve(msdp_batch* b) {
  if (!b) return MSDP_ERR_INVALID_ARGUMENT;
  int rc = launch(b, OP_INITIALIZE, 0, 0.0, 0);
  return rc ? rc : launch(b, OP_ITERATE, 0, 0.0, 0);
}

int msdp_batch_iterate(msdp_batch* b, int32_t max_iterations) {
  if (!b) return MSDP_ERR_INVALID_ARGUMENT;
  return launch(b, OP_ITERATE, max_iterations, 0.0, 0);
}

int msdp_batch_solve(msdp_batch* b) {
  int rc = msdp_batch_initialize(b);
  if (rc) return rc;
  if ((rc = launch(b, OP_ITERATE, 0, 0.0, 0))) return rc;
  return sync(b);
}

int msdp_batch_synchronize(msdp_batch* b) {
  if (!b) return MSDP_ERR_INVALID_ARGUMENT;
  return sync(b);
}

int msdp_batch_get_stats(msdp_batch* b, int32_t p, msdp_stats* out) {
  if (bad_prob(b, p) || !out) return MSDP_ERR_INVALID_ARGUMENT;
  std::vector<double> sc(SC_COUNT);
  int rc = copy_d2h(b, sc.data(), b->d64 + b->hprob[p].v64 + (int64_t)V_MCOUNT * b->hprob[p].m +
                                      (int64_t)S_COUNT * b->hprob[p].ns,
                    sizeof(double) * SC_COUNT);
  if (rc) return rc;
  fill_stats(sc.data(), out);
  return MSDP_OK;
}

int msdp_batch_get_all_stats(msdp_batch* b, msdp_stats* out) {
  if (!b || !out) return MSDP_ERR_INVALID_ARGUMENT;
  std::vector<double> sc;
  int rc = gather(b, sc);
  if (rc) return rc;
  for (int p = 0; p < b->nprob; ++p) fill_stats(sc.data() + (size_t)p * SC_COUNT, out + p);
  return MSDP_OK;
}

namespace {
struct SolSeg {
  const double* src;
  int64_t dst, len;
};
// one block per segment: packed copy of the solution arrays
__global__ void k_gather_solutions(const SolSeg* __restrict__ seg, double* __restrict__ out) {
  const SolSeg s = seg[blockIdx.x];
  for (int64_t i = threadIdx.x; i < s.len; i += blockDim.x) out[s.dst + i] = s.src[i];
}

// Segments in problem order: X of every block (column-major n x n), y, x, z.
void solution_segments(msdp_batch* b, std::vector<SolSeg>* segs, int64_t* total) {
  int64_t off = 0;
  for (int p = 0; p < b->nprob; ++p) {
    const ProbDesc& d = b->hprob[p];
    for (int i = 0; i < d.nblocks; ++i) {
      const int64_t n = b->hblk[d.blk0 + i].n;
      segs->push_back({bmat64(b, p, i, M_X), off, n * n});
      off += n * n;
    }
    if (d.m) segs->push_back({vec64(b, p, V_Y), off, d.m});
    off += d.m;
    if (d.ns) {
      segs->push_back({svec64(b, p, S_X), off, d.ns});
      segs->push_back({svec64(b, p, S_Z), off + d.ns, d.ns});
    }
    off += 2 * (int64_t)d.ns;
  }
  *total = off;
}
}  // namespace

int64_t msdp_batch_solution_size(const msdp_batch* cb) {
  if (!cb) return 0;
  msdp_batch* b = const_cast<msdp_batch*>(cb);
  std::vector<SolSeg> segs;
  int64_t total = 0;
  solution_segments(b, &segs, &total);
  return total;
}

int msdp_batch_get_all_solutions(msdp_batch* b, double* out) {
  if (!b || !out) return MSDP_ERR_INVALID_ARGUMENT;
  msdp_context* ctx = b->ctx;
  if (!b->gsol) {
    std::vector<SolSeg> segs;
    int64_t total = 0;
    solution_segments(b, &segs, &total);
    CK(cudaMalloc((void**)&b->gsol, sizeof(double) * (size_t)std::max<int64_t>(total, 1)));
    CK(cudaMalloc(&b->gseg, sizeof(SolSeg) * std::max<size_t>(segs.size(), 1)));
    // on the batch's stream (the gather below reads the segments there);
    // the pageable source lives until the copy has completed
    CK(cudaMemcpyAsync(b->gseg, segs.data(), sizeof(SolSeg) * segs.size(), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    b->nseg = (int64_t)segs.size();
    b->sol_size = total;
    b->bytes += sizeof(double) * total + sizeof(SolSeg) * segs.size();
  }
  if (b->nseg) {
    k_gather_solutions<<<(unsigned)b->nseg, 128, 0, ctx->stream>>>((const SolSeg*)b->gseg, b->gsol);
    CK(cudaGetLastError());
    b->launches += 1;
  }
  CK(cudaMemcpyAsync(out, b->gsol, sizeof(double) * (size_t)b->sol_size, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return MSDP_OK;
}

int msdp_batch_get_solution(msdp_batch* b, int32_t p, double* const* X, double* y, double* x, double* z) {
  if (bad_prob(b, p)) return MSDP_ERR_INVALID_ARGUMENT;
  const ProbDesc& d = b->hprob[p];
  int rc;
  for (int i = 0; i < d.nblocks; ++i) {
    const int64_t n = b->hblk[d.blk0 + i].n;
    if (X && X[i] && (rc = copy_d2h(b, X[i], bmat64(b, p, i, M_X), sizeof(double) * n * n))) return rc;
  }
  if ((rc = copy_d2h(b, y, vec64(b, p, V_Y), sizeof(double) * d.m))) return rc;
  if ((rc = copy_d2h(b, x, svec64(b, p, S_X), sizeof(double) * d.ns))) return rc;
  if ((rc = copy_d2h(b, z, svec64(b, p, S_Z), sizeof(double) * d.ns))) return rc;
  return MSDP_OK;
}

int msdp_batch_get_trajectory(msdp_batch* b, int32_t p, msdp_iter_record* out, int32_t capacity,
                              int32_t* count) {
  if (bad_prob(b, p) || !count) return MSDP_ERR_INVALID_ARGUMENT;
  msdp_stats st;
  std::vector<double> sc(SC_COUNT);
  const ProbDesc& d = b->hprob[p];
  int rc = copy_d2h(b, sc.data(), b->d64 + d.v64 + (int64_t)V_MCOUNT * d.m + (int64_t)S_COUNT * d.ns,
                    sizeof(double) * SC_COUNT);
  if (rc) return rc;
  (void)st;
  const int n = std::min((int)sc[SC_NTRAJ], capacity);
  *count = (int)sc[SC_NTRAJ];
  if (out && n > 0) return copy_d2h(b, out, b->d64 + d.traj, sizeof(double) * TRAJ_FIELDS * n);
  return MSDP_OK;
}

int msdp_batch_update_residuals(msdp_batch* b) {
  if (!b) return MSDP_ERR_INVALID_ARGUMENT;
  int rc = launch(b, OP_UPDATE_RESIDUALS, 0, 0.0, 0);
  return rc ? rc : sync(b);
}

int msdp_batch_prepare(msdp_batch* b, int32_t* ok) {
  if (!b) return MSDP_ERR_INVALID_ARGUMENT;
  int rc = launch(b, OP_PREPARE, 0, 0.0, 0);
  if (rc || (rc = sync(b))) return rc;
  if (ok) {
    std::vector<double> sc;
    if ((rc = gather(b, sc))) return rc;
    for (int p = 0; p < b->nprob; ++p) ok[p] = sc[(size_t)p * SC_COUNT + SC_OK] != 0.0;
  }
  return MSDP_OK;
}

int msdp_batch_solve_directions(msdp_batch* b, double mu, int32_t corrected) {
  if (!b) return MSDP_ERR_INVALID_ARGUMENT;
  int rc = launch(b, OP_SOLVE_DIRECTIONS, 0, mu, corrected);
  return rc ? rc : sync(b);
}

int msdp_batch_correction(msdp_batch* b) {
  if (!b) return MSDP_ERR_INVALID_ARGUMENT;
  int rc = launch(b, OP_CORRECTION, 0, 0.0, 0);
  return rc ? rc : sync(b);
}

int msdp_batch_get_directions(msdp_batch* b, int32_t p, double* const* delX, double* const* delS, double* dely,
                              double* delx, double* delz) {
  if (bad_prob(b, p)) return MSDP_ERR_INVALID_ARGUMENT;
  const ProbDesc& d = b->hprob[p];
  int rc;
  for (int i = 0; i < d.nblocks; ++i) {
    const int64_t n = b->hblk[d.blk0 + i].n;
    if (delX && delX[i] && (rc = copy_d2h(b, delX[i], bmat64(b, p, i, M_DX), sizeof(double) * n * n))) return rc;
    if (delS && delS[i] && (rc = copy_d2h(b, delS[i], bmat64(b, p, i, M_DS), sizeof(double) * n * n))) return rc;
  }
  if ((rc = copy_d2h(b, dely, vec64(b, p, V_DELY), sizeof(double) * d.m))) return rc;
  if ((rc = copy_d2h(b, delx, svec64(b, p, S_DELX), sizeof(double) * d.ns))) return rc;
  if ((rc = copy_d2h(b, delz, svec64(b, p, S_DELZ), sizeof(double) * d.ns))) return rc;
  return MSDP_OK;
}

int msdp_batch_get_residuals(msdp_batch* b, int32_t p, double* Rp, double* const* Rd, double* Rd_lin) {
  if (bad_prob(b, p)) return MSDP_ERR_INVALID_ARGUMENT;
  const ProbDesc& d = b->hprob[p];
  int rc;
  for (int i = 0; i < d.nblocks; ++i) {
    const int64_t n = b->hblk[d.blk0 + i].n;
    if (Rd && Rd[i] && (rc = copy_d2h(b, Rd[i], bmat64(b, p, i, M_RD), sizeof(double) * n * n))) return rc;
  }
  if ((rc = copy_d2h(b, Rp, vec64(b, p, V_RP), sizeof(double) * d.m))) return rc;
  if ((rc = copy_d2h(b, Rd_lin, svec64(b, p, S_RDLIN), sizeof(double) * d.ns))) return rc;
  return MSDP_OK;
}

static const char* kProfileNames[] = {
    "cycles_cholesky", "cycles_triangular_inverse", "cycles_jacobi", "cycles_nt_products", "cycles_schur_assembly",
    "cycles_schur_factor", "cycles_rhs", "cycles_schur_solve", "cycles_directions", "cycles_step_length",
    "cycles_lanczos", "cycles_correction", "cycles_take_step", "cycles_termination", "cycles_iteration",
    "jacobi_sweeps", "jacobi_calls", "lanczos_steps", "lanczos_calls", "schur_factorizations"};

static std::string g_profile_names[2 * SC_PROFILE_N];

const char* msdp_profile_field_name(int32_t i) {
  if (i < 0 || i >= 2 * SC_PROFILE_N) return nullptr;
  if (g_profile_names[i].empty())
    g_profile_names[i] = std::string(i < SC_PROFILE_N ? "fp32." : "fp64.") + kProfileNames[i % SC_PROFILE_N];
  return g_profile_names[i].c_str();
}

int msdp_batch_get_profile(msdp_batch* b, int32_t p, double* out, int32_t capacity) {
  if (bad_prob(b, p) || !out) return MSDP_ERR_INVALID_ARGUMENT;
  const int n = std::min<int>(capacity, 2 * SC_PROFILE_N);
  const ProbDesc& d = b->hprob[p];
  std::vector<double> sc(SC_COUNT);
  int rc = copy_d2h(b, sc.data(), b->d64 + d.v64 + (int64_t)V_MCOUNT * d.m + (int64_t)S_COUNT * d.ns,
                    sizeof(double) * SC_COUNT);
  if (rc) return rc;
  for (int k = 0; k < n; ++k)
    out[k] = sc[SC_T_CHOL + (k % SC_PROFILE_N) + (k < SC_PROFILE_N ? 0 : SC_PROFILE_F64)];
  return n;
}

int msdp_batch_get_block_matrix(msdp_batch* b, int32_t p, int32_t block, int32_t which, double* out) {
  if (bad_prob(b, p) || !out) return MSDP_ERR_INVALID_ARGUMENT;
  const ProbDesc& d = b->hprob[p];
  if (block < 0 || block >= d.nblocks) return MSDP_ERR_INVALID_ARGUMENT;
  const BlockDesc& bd = b->hblk[d.blk0 + block];
  const int64_t nn = (int64_t)bd.n * bd.n;
  const double* src = nullptr;
  switch (which) {
    case MSDP_MAT_W: src = b->d64 + bd.w64 + (int64_t)W_W * nn; break;
    case MSDP_MAT_CORR: src = b->d64 + bd.w64 + (int64_t)W_CORR * nn; break;
    case MSDP_MAT_SI: src = b->d64 + bd.w64 + (int64_t)W_SI * nn; break;
    case MSDP_MAT_S: src = bmat64(b, p, block, M_S); break;
    case MSDP_MAT_X: src = bmat64(b, p, block, M_X); break;
    default: return MSDP_ERR_INVALID_ARGUMENT;
  }
  return copy_d2h(b, out, src, sizeof(double) * nn);
}

}  // extern "C"
