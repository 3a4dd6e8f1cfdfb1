// Continuous-batching solve server: requests of different sizes are
// admitted into one device arena as memory frees up, and every active
// request advances by a few interior-point iterations per persistent
// launch (a "wave").  Requests that arrive while others are on the GPU join
// at the next wave, so their work overlaps on the device; finished requests
// leave the arena and their memory is reused.  No device memory is
// allocated after msdp_server_create.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/madsdp_gpu.h"
#include "launch.h"
#include "freelist.h"
#include "stage.h"

struct msdp_context;  // defined in capi.cu; a server runs on its own streams

namespace {

constexpr int kMaxBlocks = 16;
inline int64_t a256(int64_t b) { return (b + 255) & ~int64_t(255); }
double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// One request staged on the host: the bytes to upload and the descriptors
// with offsets relative to the start of its arena region.
struct Staged {
  ProbDesc pd;
  BlockDesc bd[kMaxBlocks];
  int nblocks = 0;
  std::vector<unsigned char> image;  // main region bytes [0, upload_bytes)
  int64_t upload_bytes = 0;
  int64_t total_bytes = 0;           // main region bytes
  int64_t nnz = 0;                   // entries (one index range in the five entry arrays)
  std::vector<int32_t> erow, ecol, pcon;
  std::vector<double> eval, pval;
  std::vector<int> sides;
  int m = 0, ns = 0;
  // region-relative byte offsets of the typed sections
  int64_t o_dd = 0, o_ptr = 0, o_d64 = 0, o_d32 = 0;
};

// Layout and host image of one problem (same device format as
// msdp_batch_create: sorted coordinate lists, position lists, Hankel flag,
// data norms).
int stage_request(const msdp_problem_desc& d, const Params& prm, bool mixed, Staged& st) {
  if (d.nblocks < 0 || d.m < 0 || d.ns < 0 || (d.nblocks == 0 && d.ns == 0)) return MSDP_ERR_INVALID_ARGUMENT;
  if (d.nblocks > kMaxBlocks) return MSDP_ERR_TOO_LARGE;
  const int nb = d.nblocks;
  const int64_t m = d.m, ns = d.ns;
  st.nblocks = nb; st.m = d.m; st.ns = d.ns;
  st.sides.assign(d.sides, d.sides + nb);
  int64_t nnz_total = 0;
  for (int i = 0; i < nb; ++i) {
    if (d.sides[i] <= 0 || d.A_nnz[i] < 0) return MSDP_ERR_INVALID_ARGUMENT;
    nnz_total += d.A_nnz[i];
  }
  // element offsets inside the typed sections
  ProbDesc& pd = st.pd;
  std::memset(&pd, 0, sizeof(pd));
  std::memset(st.bd, 0, sizeof(st.bd));
  int64_t dd = 0, d64 = 0, d32 = 0, ent = 0, ptr = 0;
  pd.nblocks = nb; pd.m = d.m; pd.ns = d.ns; pd.blk0 = 0;
  pd.bdat = dd; dd += m + ns + m * ns + 3;
  pd.v64 = d64; d64 += (int64_t)V_MCOUNT * m + (int64_t)S_COUNT * ns + SC_COUNT;
  pd.H64 = d64; d64 += m * m;
  if (mixed) { pd.Hf = d32; d32 += m * m; pd.Lf = d32; d32 += m * m; } else { pd.Hf = -1; pd.Lf = -1; }
  pd.ntraj = 0;
  pd.traj = d64;
  int64_t K = ns;
  for (int i = 0; i < nb; ++i) K += (int64_t)d.sides[i] * (d.sides[i] + 1) / 2;
  pd.K = (int32_t)K;
  if (prm.schur == MSDP_QR_SCHUR) { pd.qr = d64; d64 += K * m + 2 * m + 2 * K; } else pd.qr = -1;
  if (prm.schur == MSDP_MADNLP_SCHUR) { pd.piv = d64; d64 += m; } else pd.piv = -1;
  for (int i = 0; i < nb; ++i) {
    const int64_t n = d.sides[i];
    BlockDesc& bd = st.bd[i];
    bd.n = (int32_t)n; bd.nnz = d.A_nnz[i];
    bd.cdat = dd; dd += n * n;
    bd.m64 = d64; d64 += (int64_t)M_COUNT * n * n + BS_COUNT;
    bd.w64 = d64; d64 += (int64_t)W_COUNT * n * n + (int64_t)WV_COUNT * (n + 1);
    if (mixed) { bd.w32 = d32; d32 += (int64_t)W_COUNT * n * n + (int64_t)WV_COUNT * (n + 1); } else bd.w32 = -1;
    bd.ent = ent; ent += bd.nnz;
    bd.conptr = ptr; ptr += m + 1;
    bd.posptr = ptr; ptr += n * n + 1;
  }
  // byte layout of the main region (the entries go to the entry pool)
  int64_t off = 0;
  st.o_dd = off; off = a256(off + 8 * dd);
  st.o_ptr = off; off = a256(off + 8 * ptr);
  st.upload_bytes = off;
  st.o_d64 = off; off = a256(off + 8 * d64);
  st.o_d32 = off; off = a256(off + 4 * d32);
  st.total_bytes = off;
  st.image.assign((size_t)st.upload_bytes, 0);
  st.nnz = nnz_total;
  st.erow.assign(nnz_total, 0); st.ecol.assign(nnz_total, 0); st.pcon.assign(nnz_total, 0);
  st.eval.assign(nnz_total, 0.0); st.pval.assign(nnz_total, 0.0);
  // the problem's data range is the whole dd section, its entries and
  // pointers the whole lists (stage.h)
  const StageBuffers sb{(double*)(st.image.data() + st.o_dd), dd, st.erow.data(), st.ecol.data(), st.eval.data(),
                        st.pcon.data(), st.pval.data(), (int64_t*)(st.image.data() + st.o_ptr)};
  std::vector<int64_t> idx, fill;
  if (!::stage_problem(d, pd, st.bd, dd, sb, idx, fill)) return MSDP_ERR_INVALID_ARGUMENT;
  return MSDP_OK;
}

// Shift a staged problem's element offsets to its main region at byte
// `base` and its entries to index `ent_base` of the entry pool.
void relocate(Staged& st, int64_t base, int64_t ent_base, int blk0) {
  ProbDesc& pd = st.pd;
  pd.blk0 = blk0;
  const int64_t dd = (base + st.o_dd) / 8, d64 = (base + st.o_d64) / 8, d32 = (base + st.o_d32) / 4;
  pd.bdat += dd; pd.v64 += d64; pd.H64 += d64; pd.traj += d64;
  if (pd.Hf >= 0) pd.Hf += d32;
  if (pd.Lf >= 0) pd.Lf += d32;
  if (pd.qr >= 0) pd.qr += d64;
  if (pd.piv >= 0) pd.piv += d64;
  for (int i = 0; i < st.nblocks; ++i) {
    BlockDesc& bd = st.bd[i];
    bd.cdat += dd; bd.m64 += d64; bd.w64 += d64;
    if (bd.w32 >= 0) bd.w32 += d32;
    bd.ent += ent_base;
    bd.conptr += (base + st.o_ptr) / 8;
    bd.posptr += (base + st.o_ptr) / 8;
  }
}

struct Request {
  int64_t id = 0;
  Staged st;
  double t_submit = 0, t_admit = 0, t_done = 0;
  int slot = -1;
  int64_t region = -1;
  int64_t entries = -1;
  int wave = -1;  // wave the request is running in, -1 when idle
  bool done = false;
  msdp_stats stats{};
  std::vector<std::vector<double>> X;
  std::vector<double> y, x, z;
};

}  // namespace

// One wave: a persistent launch over a set of requests on its own stream.
// Waves overlap on the device; a request belongs to at most one running
// wave, and the host only touches a wave's requests after its event.
constexpr int kWaves = 16;

struct Wave {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  int32_t *dorder = nullptr, *dinit = nullptr, *queue = nullptr, *pending = nullptr;
  double* scal = nullptr;   // device scalars of the wave's requests
  double* hscal = nullptr;  // pinned host copy
  // pinned staging of the wave's order and init lists and its pending
  // count (capacity, capacity, 1): host->device copies read their source
  // when the stream reaches them, and a wave is rewritten only once idle
  int32_t* hlist = nullptr;
  std::vector<int32_t> slots;
  bool busy = false;
};

struct msdp_server {
  msdp_context* ctx = nullptr;
  Params prm{};
  bool mixed = false;
  int capacity = 0;
  int sm_count = 0, occupancy = 1;
  unsigned char* arena = nullptr;
  int64_t arena_bytes = 0;
  std::map<int64_t, int64_t> free_blocks;  // main arena: offset -> size (bytes)
  // entry pool: five typed arrays addressed by one entry index
  int32_t *erow = nullptr, *ecol = nullptr, *pcon = nullptr;
  double *eval = nullptr, *pval = nullptr;
  int64_t entry_capacity = 0;
  std::map<int64_t, int64_t> free_entries;  // index -> count
  ProbDesc* dprob = nullptr;
  BlockDesc* dblk = nullptr;
  Wave waves[kWaves];
  std::vector<int> free_slots;
  std::deque<std::unique_ptr<Request>> pending;
  std::vector<Request*> active;              // by slot
  std::map<int64_t, std::unique_ptr<Request>> requests;
  int64_t next_id = 1;
  std::vector<int64_t> finished;             // harvested, not yet reported by msdp_server_finished
  int64_t launches = 0;
  int64_t completed = 0;
  std::string err;
};

namespace {

BatchDev server_dev(msdp_server* s, const Wave& w, const int32_t* order, int count) {
  BatchDev B;
  std::memset(&B, 0, sizeof(B));
  B.nprob = count;
  B.prob = s->dprob; B.blk = s->dblk; B.order = order;
  B.dd = (const double*)s->arena; B.d64 = (double*)s->arena; B.d32 = (float*)s->arena;
  B.e_row = s->erow; B.e_col = s->ecol; B.e_val = s->eval;
  B.p_con = s->pcon; B.p_val = s->pval; B.ptr = (const int64_t*)s->arena;
  B.queue = w.queue;
  B.prm = s->prm;
  return B;
}

void free_server(msdp_server* s) {
  for (auto& w : s->waves) {
    if (w.stream) cudaStreamSynchronize(w.stream);
    cudaFree(w.dorder); cudaFree(w.dinit); cudaFree(w.queue); cudaFree(w.pending); cudaFree(w.scal);
    if (w.hscal) cudaFreeHost(w.hscal);
    if (w.hlist) cudaFreeHost(w.hlist);
    if (w.done) cudaEventDestroy(w.done);
    if (w.stream) cudaStreamDestroy(w.stream);
  }
  cudaFree(s->arena); cudaFree(s->dprob); cudaFree(s->dblk);
  cudaFree(s->erow); cudaFree(s->ecol); cudaFree(s->pcon); cudaFree(s->eval); cudaFree(s->pval);
}

// Results of a finished wave: requests that terminated are copied to the
// host and leave the arena; the others become idle for the next wave.
cudaError_t harvest_wave(msdp_server* s, Wave& w, int* done_now) {
  cudaError_t e = cudaSuccess;
  std::vector<Request*> fin;
  for (size_t q = 0; q < w.slots.size(); ++q) {
    const double* v = w.hscal + q * SC_COUNT;
    Request* r = s->active[w.slots[q]];
    r->wave = -1;
    const int status = (int)v[SC_STATUS];
    if (status == MSDP_REGULAR) continue;
    msdp_stats& o = r->stats;
    std::memset(&o, 0, sizeof(o));
    o.status = status == MSDP_STATUS_INITIAL_POINT_ERROR ? MSDP_ERROR_IN_STEP_COMPUTATION : status;
    o.iter = (int32_t)v[SC_ITER]; o.iter_fp32 = (int32_t)v[SC_N32]; o.iter_fp64 = (int32_t)v[SC_N64];
    o.pobj = v[SC_POBJ]; o.dobj = v[SC_DOBJ]; o.inf_pr = v[SC_INFPR]; o.inf_du = v[SC_INFDU]; o.gap = v[SC_GAP];
    o.mu = v[SC_MU]; o.sigma = v[SC_SIGMA]; o.alpha = v[SC_ALPHA]; o.beta = v[SC_BETA]; o.solve_ns = v[SC_SOLVE_NS];
    const Staged& stg = r->st;
    const int64_t m = stg.m, ns = stg.ns;
    r->y.resize(m); r->x.resize(ns); r->z.resize(ns);
    const double* v64 = (const double*)s->arena + stg.pd.v64;
    if (e == cudaSuccess && m)
      e = cudaMemcpyAsync(r->y.data(), v64 + (int64_t)V_Y * m, 8 * m, cudaMemcpyDeviceToHost, w.stream);
    const double* sv = v64 + (int64_t)V_MCOUNT * m;
    if (e == cudaSuccess && ns)
      e = cudaMemcpyAsync(r->x.data(), sv + (int64_t)S_X * ns, 8 * ns, cudaMemcpyDeviceToHost, w.stream);
    if (e == cudaSuccess && ns)
      e = cudaMemcpyAsync(r->z.data(), sv + (int64_t)S_Z * ns, 8 * ns, cudaMemcpyDeviceToHost, w.stream);
    r->X.resize(stg.nblocks);
    for (int i = 0; i < stg.nblocks; ++i) {
      const int64_t n = stg.bd[i].n;
      r->X[i].resize(n * n);
      const double* Xd = (const double*)s->arena + stg.bd[i].m64 + (int64_t)M_X * n * n;
      if (e == cudaSuccess) e = cudaMemcpyAsync(r->X[i].data(), Xd, 8 * n * n, cudaMemcpyDeviceToHost, w.stream);
    }
    fin.push_back(r);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(w.stream);
  const double t = now_s();
  for (Request* r : fin) {
    r->t_done = t;
    r->done = true;
    list_free(s->free_blocks, r->region, r->st.total_bytes);
    list_free(s->free_entries, r->entries, r->st.nnz);
    s->active[r->slot] = nullptr;
    s->free_slots.push_back(r->slot);
    s->finished.push_back(r->id);
    ++s->completed;
    ++*done_now;
  }
  w.slots.clear();
  w.busy = false;
  return e;
}

int count_active(const msdp_server* s) {
  int a = 0;
  for (auto* r : s->active) a += (r != nullptr);
  return a;
}

// Harvest finished waves, admit pending requests, and start one wave over
// every idle request (on a free wave stream).  Returns without waiting.
int step_async(msdp_server* s, int32_t iterations, double budget_s, int* done_now) {
  cudaError_t e = cudaSuccess;
  for (auto& w : s->waves) {
    if (!w.busy) continue;
    const cudaError_t q = cudaEventQuery(w.done);
    if (q == cudaErrorNotReady) continue;
    if (q != cudaSuccess) { s->err = cudaGetErrorString(q); return MSDP_ERR_CUDA; }
    e = harvest_wave(s, w, done_now);
    if (e != cudaSuccess) { s->err = cudaGetErrorString(e); return MSDP_ERR_CUDA; }
  }
  int wi = -1;
  for (int k = 0; k < kWaves; ++k)
    if (!s->waves[k].busy) { wi = k; break; }
  if (wi < 0) return MSDP_OK;  // every wave stream is busy
  Wave& w = s->waves[wi];
  cudaStream_t st = w.stream;
  // ---- admission: arrival order, every pending request whose region fits
  std::vector<int32_t> fresh;
  for (auto it = s->pending.begin(); it != s->pending.end();) {
    if (s->free_slots.empty()) break;
    Request* r = it->get();
    const int64_t off = list_alloc(s->free_blocks, r->st.total_bytes);
    if (off < 0) { ++it; continue; }
    const int64_t ent = list_alloc(s->free_entries, r->st.nnz);
    if (ent < 0) { list_free(s->free_blocks, off, r->st.total_bytes); ++it; continue; }
    const int slot = s->free_slots.back();
    s->free_slots.pop_back();
    r->slot = slot;
    r->region = off;
    r->entries = ent;
    r->t_admit = now_s();
    relocate(r->st, off, ent, slot * kMaxBlocks);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s->arena + off, r->st.image.data(), (size_t)r->st.upload_bytes, cudaMemcpyHostToDevice, st);
    const size_t nz = (size_t)r->st.nnz;
    if (e == cudaSuccess && nz) e = cudaMemcpyAsync(s->erow + ent, r->st.erow.data(), 4 * nz, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nz) e = cudaMemcpyAsync(s->ecol + ent, r->st.ecol.data(), 4 * nz, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nz) e = cudaMemcpyAsync(s->pcon + ent, r->st.pcon.data(), 4 * nz, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nz) e = cudaMemcpyAsync(s->eval + ent, r->st.eval.data(), 8 * nz, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nz) e = cudaMemcpyAsync(s->pval + ent, r->st.pval.data(), 8 * nz, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemsetAsync(s->arena + off + r->st.upload_bytes, 0, (size_t)(r->st.total_bytes - r->st.upload_bytes), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->dprob + slot, &r->st.pd, sizeof(ProbDesc), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && r->st.nblocks)
      e = cudaMemcpyAsync(s->dblk + (int64_t)slot * kMaxBlocks, r->st.bd, sizeof(BlockDesc) * r->st.nblocks,
                          cudaMemcpyHostToDevice, st);
    fresh.push_back(slot);
    s->active[slot] = r;
    s->requests[r->id] = std::move(*it);
    it = s->pending.erase(it);
  }
  if (e != cudaSuccess) { s->err = cudaGetErrorString(e); return MSDP_ERR_CUDA; }
  // ---- the wave: every idle request (fresh ones initialized first)
  std::vector<int32_t> act;
  for (int k = 0; k < s->capacity; ++k)
    if (s->active[k] && s->active[k]->wave < 0) act.push_back(k);
  if (act.empty()) return MSDP_OK;
  const int mk = s->mixed ? 1 : 0;
  int32_t* horder = w.hlist;
  int32_t* hinit = w.hlist + s->capacity;
  int32_t* hpend = w.hlist + 2 * s->capacity;
  std::copy(act.begin(), act.end(), horder);
  std::copy(fresh.begin(), fresh.end(), hinit);
  if (!fresh.empty()) {
    e = cudaMemcpyAsync(w.dinit, hinit, sizeof(int32_t) * fresh.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(w.queue, 0, sizeof(int32_t), st);
    BatchDev B = server_dev(s, w, w.dinit, (int)fresh.size());
    B.prm.op = OP_INITIALIZE;
    const int grid = std::min((int)fresh.size(), std::max(1, s->sm_count * s->occupancy));
    if (e == cudaSuccess) e = msdp_ipm_launch(mk, B, grid, st);
    s->launches += 1;
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(w.dorder, horder, sizeof(int32_t) * act.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.queue, 0, sizeof(int32_t), st);
  BatchDev B = server_dev(s, w, w.dorder, (int)act.size());
  B.prm.op = OP_ITERATE;
  B.prm.max_iterations = iterations;
  B.prm.wave_ns = budget_s * 1e9;
  if (budget_s > 0.0) {
    *hpend = (int32_t)act.size();
    if (e == cudaSuccess) e = cudaMemcpyAsync(w.pending, hpend, sizeof(int32_t), cudaMemcpyHostToDevice, st);
    B.wave_pending = w.pending;
  }
  const int grid = std::min((int)act.size(), std::max(1, s->sm_count * s->occupancy));
  if (e == cudaSuccess) e = msdp_ipm_launch(mk, B, grid, st);
  s->launches += 1;
  BatchDev G = server_dev(s, w, w.dorder, (int)act.size());
  if (e == cudaSuccess) e = msdp_gather_launch_idx(G, w.dorder, (int)act.size(), w.scal, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(w.hscal, w.scal, sizeof(double) * SC_COUNT * act.size(), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaEventRecord(w.done, st);
  if (e != cudaSuccess) { s->err = cudaGetErrorString(e); return MSDP_ERR_CUDA; }
  for (int32_t k : act) s->active[k]->wave = wi;
  w.slots = act;
  w.busy = true;
  return MSDP_OK;
}

}  // namespace

extern "C" {

int msdp_server_create(msdp_context* ctx, const msdp_components* comp, const msdp_options* opt,
                       int64_t memory_budget_bytes, int32_t max_slots, msdp_server** out) {
  if (!ctx || !out || memory_budget_bytes <= 0 || max_slots <= 0) return MSDP_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  msdp_components c;
  msdp_options o;
  if (comp) c = *comp; else msdp_default_components(&c);
  if (opt) o = *opt; else msdp_default_options(&o);
  if (c.precision != MSDP_FP64 && c.precision != MSDP_MIXED) return MSDP_ERR_UNSUPPORTED;
  if (c.algorithm == MSDP_DUAL_CENTERING || (c.schur == MSDP_QR_SCHUR && c.precision != MSDP_FP64) ||
      (c.schur == MSDP_QR_SCHUR && c.direction != MSDP_NT) || !(c.shrink > 0.0 && c.shrink < 1.0) ||
      !(c.boundary > 0.0 && c.boundary <= 1.0) || !(c.tau > 0.0) || o.max_iter < 0 ||
      (c.initial_point == MSDP_INITIAL_POINT) || (c.initial_point == MSDP_DUAL_SHIFT && !(c.initial_shift > 0.0)))
    return MSDP_ERR_INVALID_ARGUMENT;
  auto s = std::make_unique<msdp_server>();
  s->ctx = ctx;
  s->mixed = (c.precision == MSDP_MIXED);
  s->capacity = max_slots;
  Params& prm = s->prm;
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
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, dev);
  s->occupancy = std::max(1, msdp_ipm_occupancy(s->mixed ? 1 : 0));
  // three quarters of the budget for the main arena, one quarter for the
  // constraint entries (28 bytes per entry over the five arrays)
  s->arena_bytes = a256(memory_budget_bytes / 4 * 3);
  s->entry_capacity = std::max<int64_t>(1, (memory_budget_bytes / 4) / 28);
  cudaError_t e = cudaMalloc((void**)&s->arena, (size_t)s->arena_bytes);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->erow, sizeof(int32_t) * s->entry_capacity);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->ecol, sizeof(int32_t) * s->entry_capacity);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->pcon, sizeof(int32_t) * s->entry_capacity);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->eval, sizeof(double) * s->entry_capacity);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->pval, sizeof(double) * s->entry_capacity);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->dprob, sizeof(ProbDesc) * max_slots);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->dblk, sizeof(BlockDesc) * max_slots * kMaxBlocks);
  for (auto& w : s->waves) {
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc((void**)&w.dorder, sizeof(int32_t) * max_slots);
    if (e == cudaSuccess) e = cudaMalloc((void**)&w.dinit, sizeof(int32_t) * max_slots);
    if (e == cudaSuccess) e = cudaMalloc((void**)&w.queue, sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc((void**)&w.pending, sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc((void**)&w.scal, sizeof(double) * SC_COUNT * max_slots);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&w.hscal, sizeof(double) * SC_COUNT * max_slots);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&w.hlist, sizeof(int32_t) * (2 * (size_t)max_slots + 1));
  }
  // every request descriptor starts empty (on a server stream: the legacy
  // default stream is not ordered with the non-blocking wave streams)
  if (e == cudaSuccess) e = cudaMemsetAsync(s->dprob, 0, sizeof(ProbDesc) * max_slots, s->waves[0].stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->waves[0].stream);
  if (e != cudaSuccess) {
    msdp_server* raw = s.release();
    free_server(raw);
    delete raw;
    return e == cudaErrorMemoryAllocation ? MSDP_ERR_OUT_OF_MEMORY : MSDP_ERR_CUDA;
  }
  s->free_blocks[0] = s->arena_bytes;
  s->free_entries[0] = s->entry_capacity;
  s->active.assign(max_slots, nullptr);
  for (int k = max_slots - 1; k >= 0; --k) s->free_slots.push_back(k);
  *out = s.release();
  return MSDP_OK;
}

int msdp_server_destroy(msdp_server* s) {
  if (!s) return MSDP_OK;
  // the server's own streams are synchronized; the context's stream is not
  // touched, so a server may outlive its context
  free_server(s);
  delete s;
  return MSDP_OK;
}

int msdp_server_submit(msdp_server* s, const msdp_problem_desc* prob, int64_t* request_id) {
  if (!s || !prob || !request_id) return MSDP_ERR_INVALID_ARGUMENT;
  auto r = std::make_unique<Request>();
  const int rc = stage_request(*prob, s->prm, s->mixed, r->st);
  if (rc) return rc;
  if (r->st.total_bytes > s->arena_bytes || r->st.nnz > s->entry_capacity) return MSDP_ERR_TOO_LARGE;
  r->id = s->next_id++;
  r->t_submit = now_s();
  *request_id = r->id;
  s->pending.push_back(std::move(r));
  return MSDP_OK;
}

int msdp_server_step_budget(msdp_server* s, int32_t iterations, double budget_s, int32_t* n_active,
                            int32_t* n_completed) {
  if (!s || iterations <= 0 || !(budget_s >= 0.0)) return MSDP_ERR_INVALID_ARGUMENT;
  int done_now = 0;
  const int rc = step_async(s, iterations, budget_s, &done_now);
  if (rc) return rc;
  if (n_active) *n_active = count_active(s);
  if (n_completed) *n_completed = done_now;
  return MSDP_OK;
}

int msdp_server_step(msdp_server* s, int32_t iterations, int32_t* n_active, int32_t* n_completed) {
  if (!s || iterations <= 0) return MSDP_ERR_INVALID_ARGUMENT;
  int done_now = 0;
  // finish every running wave first, so that the wave below covers every
  // active request, then wait for it
  for (auto& w : s->waves) {
    if (!w.busy) continue;
    cudaError_t e = cudaEventSynchronize(w.done);
    if (e == cudaSuccess) e = harvest_wave(s, w, &done_now);
    if (e != cudaSuccess) { s->err = cudaGetErrorString(e); return MSDP_ERR_CUDA; }
  }
  int rc = step_async(s, iterations, 0.0, &done_now);
  if (rc) return rc;
  for (auto& w : s->waves) {
    if (!w.busy) continue;
    cudaError_t e = cudaEventSynchronize(w.done);
    if (e == cudaSuccess) e = harvest_wave(s, w, &done_now);
    if (e != cudaSuccess) { s->err = cudaGetErrorString(e); return MSDP_ERR_CUDA; }
  }
  if (n_active) *n_active = count_active(s);
  if (n_completed) *n_completed = done_now;
  return MSDP_OK;
}

int msdp_server_counts(const msdp_server* s, int32_t* pending, int32_t* active, int64_t* completed) {
  if (!s) return MSDP_ERR_INVALID_ARGUMENT;
  if (pending) *pending = (int32_t)s->pending.size();
  if (active) *active = count_active(s);
  if (completed) *completed = s->completed;
  return MSDP_OK;
}

int msdp_server_result(msdp_server* s, int64_t id, msdp_stats* stats, double* const* X, double* y, double* x,
                       double* z, double* latency_s) {
  if (!s) return MSDP_ERR_INVALID_ARGUMENT;
  auto it = s->requests.find(id);
  if (it == s->requests.end()) {
    for (const auto& r : s->pending)
      if (r->id == id) return 1;  // not admitted yet
    return MSDP_ERR_INVALID_ARGUMENT;
  }
  Request* r = it->second.get();
  if (!r->done) return 1;  // not finished yet
  if (stats) *stats = r->stats;
  for (int i = 0; X && i < r->st.nblocks; ++i)
    if (X[i]) std::memcpy(X[i], r->X[i].data(), 8 * r->X[i].size());
  if (y) std::memcpy(y, r->y.data(), 8 * r->y.size());
  if (x) std::memcpy(x, r->x.data(), 8 * r->x.size());
  if (z) std::memcpy(z, r->z.data(), 8 * r->z.size());
  if (latency_s) *latency_s = r->t_done - r->t_submit;
  s->requests.erase(it);
  return MSDP_OK;
}

int msdp_server_finished(msdp_server* s, int64_t* ids, int32_t capacity, int32_t* count) {
  if (!s || !count || capacity < 0 || (capacity > 0 && !ids)) return MSDP_ERR_INVALID_ARGUMENT;
  const int32_t k = (int32_t)std::min<size_t>((size_t)capacity, s->finished.size());
  for (int32_t i = 0; i < k; ++i) ids[i] = s->finished[i];
  s->finished.erase(s->finished.begin(), s->finished.begin() + k);
  *count = k;
  return MSDP_OK;
}

int64_t msdp_server_launch_count(const msdp_server* s) { return s ? s->launches : 0; }

}  // extern "C"
