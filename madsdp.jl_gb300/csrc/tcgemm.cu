// Split-precision products on the tcgen05 tensor cores; see tcgemm.h.
#include "tcgemm.h"

#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <mutex>

#include "../../include/madsdp_gpu.h"

namespace tcg {
namespace {

constexpr int BM = 128, BK = 32;             // tile rows, K per stage (64 B of bf16)
constexpr int TILE = BM * BK * 2;            // bytes of one 128 x 32 bf16 slice tile of A
constexpr int kThreads = 128;
constexpr unsigned long long kWaitNs = 2000000000ull;  // bound of every wait (2 s)

// Slice pairs (t, u) with t + u <= NS - 1 in order of t + u; pairs of order
// s accumulate in group min(s, NG - 1).
template <int NS, int NG>
struct Pairs {
  static constexpr int N = NS * (NS + 1) / 2;
  int t[N], u[N], g[N], first[N];
  constexpr Pairs() : t(), u(), g(), first() {
    int p = 0;
    int seen[NG] = {};
    for (int s = 0; s < NS; ++s)
      for (int a = 0; a <= s; ++a) {
        t[p] = a;
        u[p] = s - a;
        g[p] = s < NG ? s : NG - 1;
        first[p] = seen[g[p]] ? 0 : 1;
        seen[g[p]] = 1;
        ++p;
      }
  }
};

struct Args {
  int64_t M, N, rpad_a, rpad_b, ldc, ldfix;
  int32_t tiles_m, tiles_n, lower, kblocks, chunk_kb, direct, U, alpha_exp, alpha_neg;
  const int32_t* exa;
  const int32_t* exb;
  double* C;
  unsigned long long* fix;
  int* err;
};

// ---------------------------------------------------------------- PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long gtime() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait on a phase parity: false when the deadline passed first.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned long long deadline) {
  for (uint32_t it = 0;; ++it) {
    if (mbar_try(bar, parity)) return true;
    if ((it & 255u) == 255u && gtime() > deadline) return false;
  }
}
__device__ __forceinline__ void tma_load_2d(const CUtensorMap* map, uint32_t dst, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"((unsigned long long)map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// K-major operand tile of 64 or 128 rows x 64 bytes with the 64-byte swizzle:
// 8-row groups 512 bytes apart, descriptor version 1, layout SWIZZLE_64B.
__device__ __forceinline__ unsigned long long smem_desc(uint32_t saddr) {
  unsigned long long d = (unsigned long long)((saddr & 0x3FFFFu) >> 4);
  d |= 1ull << 16;                 // leading byte offset (unused for swizzled K-major)
  d |= (unsigned long long)(512 >> 4) << 32;
  d |= 1ull << 46;
  d |= 4ull << 61;
  return d;
}
// kind::f16 instruction descriptor: FP32 accumulator, bf16 A and B, both
// K-major, N = BN, M = BM.
template <int BN>
constexpr uint32_t idesc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

template <int BN>
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, unsigned long long adesc, unsigned long long bdesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc<BN>()), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
        "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
        "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// v * 2^E for a fixed-point integer v, rounded once (int64 -> double).
__device__ __forceinline__ double fix_to_double(long long v, int E) {
  if (v == 0) return 0.0;
  const double d = __ll2double_rn(v);
  const long long b = __double_as_longlong(d);
  const int ex = (int)((b >> 52) & 0x7FF) + E;
  if (ex > 0 && ex < 2047) return __longlong_as_double(b + ((long long)E << 52));
  return scalbn(d, E);
}

// ---------------------------------------------------------------- the product
template <int NS, int NG, int BN, int NST>
__global__ void __launch_bounds__(kThreads, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap ma, const __grid_constant__ CUtensorMap mb, const Args a) {
  constexpr Pairs<NS, NG> P{};
  constexpr int TILE_B = BN * BK * 2;
  constexpr int STAGE = NS * (TILE + TILE_B);
  constexpr uint32_t TCOLS = NG * BN <= 128 ? 128u : (NG * BN <= 256 ? 256u : 512u);
  static_assert(NG * BN <= 512, "tensor memory holds 512 columns");

  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t sb = (raw + 1023u) & ~1023u;       // 1 KiB aligned stage buffers
  unsigned char* gb = smem_raw + (sb - raw);
  const uint32_t bar0 = sb + NST * STAGE;           // full[NST], empty[NST], done
  uint32_t* tslot = (uint32_t*)(gb + NST * STAGE + 8 * (2 * NST + 1));
  volatile int* abort_flag = (volatile int*)(tslot + 1);
  auto full = [&](int s) { return bar0 + 8u * s; };
  auto empty = [&](int s) { return bar0 + 8u * (NST + s); };
  const uint32_t done = bar0 + 8u * (2 * NST);
  auto tileA = [&](int s, int t) { return sb + (uint32_t)(s * STAGE + t * TILE); };
  auto tileB = [&](int s, int u) { return sb + (uint32_t)(s * STAGE + NS * TILE + u * TILE_B); };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tm = (int)(blockIdx.x / a.tiles_n), tn = (int)(blockIdx.x % a.tiles_n);
  // lower triangle only: tiles entirely above the diagonal have nothing to do
  if (a.lower && (int64_t)tn * BN > (int64_t)tm * BM + BM - 1) return;
  const int kb0 = blockIdx.y * a.chunk_kb;
  const int nkb = min(a.chunk_kb, a.kblocks - kb0);

  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(full(s), 1);
      mbar_init(empty(s), 1);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;
  const unsigned long long deadline = gtime() + kWaitNs;

  if (warp == 0 && lane == 0) {
    // TMA producer: every slice of A and B for one 32-wide K block per stage
    int issued = 0;
    for (int i = 0; i < nkb; ++i) {
      const int s = i % NST;
      if (i >= NST && !mbar_wait(empty(s), ((i / NST) & 1) ^ 1, deadline)) {
        *abort_flag = 1;
        atomicExch(a.err, 1);
        break;
      }
      if (*abort_flag) break;
      mbar_expect_tx(full(s), STAGE);
      const int x = (kb0 + i) * BK;
#pragma unroll
      for (int t = 0; t < NS; ++t) tma_load_2d(&ma, tileA(s, t), x, (int)(t * a.rpad_a + (int64_t)tm * BM), full(s));
#pragma unroll
      for (int u = 0; u < NS; ++u) tma_load_2d(&mb, tileB(s, u), x, (int)(u * a.rpad_b + (int64_t)tn * BN), full(s));
      issued = i + 1;
    }
    if (*abort_flag) {
      // let the copies already issued land before the block exits
      const unsigned long long d2 = gtime() + kWaitNs / 4;
      for (int i = max(0, issued - NST); i < issued; ++i) mbar_wait(full(i % NST), (i / NST) & 1, d2);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: all slice pairs of the stage into their group accumulators
    bool ok = true;
    for (int i = 0; i < nkb; ++i) {
      const int s = i % NST;
      if (!mbar_wait(full(s), (i / NST) & 1, deadline) || *abort_flag) {
        *abort_flag = 1;
        atomicExch(a.err, 2);
        ok = false;
        break;
      }
      tc_fence_after();
#pragma unroll
      for (int p = 0; p < Pairs<NS, NG>::N; ++p) {
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk) {
          const unsigned long long ad = smem_desc(tileA(s, P.t[p]) + kk * 32);
          const unsigned long long bd = smem_desc(tileB(s, P.u[p]) + kk * 32);
          mma_bf16<BN>(tbase + (uint32_t)(P.g[p] * BN), ad, bd, (i > 0 || !P.first[p] || kk > 0) ? 1u : 0u);
        }
      }
      mma_commit(empty(s));
    }
    if (ok) mma_commit(done);
  }
  __syncwarp();

  // epilogue: thread = one row of the tile (tensor-memory lane)
  const bool ok = mbar_wait(done, 0, deadline) && !*abort_flag;
  if (!ok && threadIdx.x == 0) atomicExch(a.err, 3);
  __syncwarp();
  tc_fence_after();
  if (ok) {
    const int64_t row = (int64_t)tm * BM + warp * 32 + lane;
    const bool row_ok = row < a.M;
    const int ea = row_ok ? a.exa[row] : 0;
    const float scaleU = __int_as_float((127 + a.U) << 23);
    const uint32_t tw = tbase + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
    for (int cc = 0; cc < BN / 32; ++cc) {
      long long acc[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) acc[j] = 0;
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        uint32_t v[32];
        tmem_ld32(tw + (uint32_t)(g * BN + cc * 32), v);
#pragma unroll
        for (int j = 0; j < 32; ++j) acc[j] += __float2ll_rn(__uint_as_float(v[j]) * scaleU);
      }
      if (row_ok) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int64_t col = (int64_t)tn * BN + cc * 32 + j;
          if (col >= a.N || (a.lower && row < col)) continue;
          if (a.direct) {
            double d = fix_to_double(acc[j], ea + a.exb[col] - a.U - 14 + a.alpha_exp);
            d = a.alpha_neg ? -d : d;
            double* o = a.C + row + col * a.ldc;
            *o = a.direct == 2 ? *o + d : d;
          } else {
            atomicAdd(a.fix + row + col * a.ldfix, (unsigned long long)acc[j]);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 2) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(TCOLS) : "memory");
  }
}

// C = alpha * fix * 2^(ea + eb - U - 14) + beta * C
__global__ void k_finish(int64_t M, int64_t N, const long long* __restrict__ fix, int64_t ldfix,
                         const int32_t* __restrict__ exa, const int32_t* __restrict__ exb, int U, double alpha,
                         double beta, double* C, int64_t ldc, int lower) {
  const int64_t total = M * N;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx / M, r = idx - c * M;
    if (lower && r < c) continue;
    const double v = alpha * fix_to_double(fix[r + c * ldfix], exa[r] + exb[c] - U - 14);
    double* o = C + r + c * ldc;
    *o = beta == 0.0 ? v : v + beta * *o;
  }
}

// ---------------------------------------------------------------- slicing
__device__ __forceinline__ double src_load(const Source& s, int64_t R, int64_t k) {
  const uint32_t j = (uint32_t)R / (uint32_t)s.nr;
  const int64_t i = R - (int64_t)j * s.nr;
  if (s.kmap) {
    const int2 ab = s.kmap[k];
    const double v = s.p[(int64_t)j * s.bs + ab.x * s.rs + ab.y * s.ks];
    return ab.x == ab.y ? v : v * 1.4142135623730951;
  }
  return s.p[(int64_t)j * s.bs + i * s.rs + k * s.ks];
}
// Row exponents, one warp per row (rows read along k).
__global__ void k_rowexp_warp(Source s, int64_t Rpad, int32_t* __restrict__ ex) {
  const int64_t R = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (R >= Rpad) return;
  int m = 0;
  if (R < s.rows)
    for (int64_t k = lane; k < s.K; k += 32) m = max(m, exp_field(src_load(s, R, k)));
#pragma unroll
  for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) ex[R] = row_exp(m);
}
// Row exponents, one thread per row (rows contiguous in memory).
__global__ void k_rowexp_thread(Source s, int64_t Rpad, int32_t* __restrict__ ex) {
  const int64_t R = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (R >= Rpad) return;
  int m = 0;
  if (R < s.rows)
    for (int64_t k = 0; k < s.K; ++k) m = max(m, exp_field(src_load(s, R, k)));
  ex[R] = row_exp(m);
}

// 32 x 32 tiles: read (through shared memory when rows are the contiguous
// direction), cut into NS slices, write K-major bf16 (zeros in the padding).
template <int NS>
__global__ void __launch_bounds__(256) k_slice(Source s, int64_t Rpad, int64_t Kpad, const int32_t* __restrict__ ex,
                                              __nv_bfloat16* __restrict__ out) {
  __shared__ double tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.x * 32, k0 = (int64_t)blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const bool along_k = s.kmap != nullptr || s.ks == 1 || s.rs != 1;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int rr = along_k ? ty + 8 * i : tx, kk = along_k ? tx : ty + 8 * i;
    const int64_t R = r0 + rr, k = k0 + kk;
    tile[rr][kk] = (R < s.rows && k < s.K) ? src_load(s, R, k) : 0.0;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int rr = ty + 8 * i;
    const int64_t R = r0 + rr, k = k0 + tx;
    write_slices<NS>(tile[rr][tx], R < s.rows ? ex[R] : 0, out + R * Kpad + k, Rpad * Kpad);
  }
}

int64_t rup(int64_t x, int64_t a) { return (std::max<int64_t>(x, 1) + a - 1) / a * a; }

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  });
  return fn;
}

template <int NS, int BN, int NST>
constexpr int smem_bytes() {
  return NST * NS * (TILE + BN * BK * 2) + 1024 + 8 * (2 * NST + 1) + 16;
}

template <int NS, int NG, int BN, int NST>
cudaError_t launch(const Sliced& A, const Sliced& B, const Args& a, int64_t ntiles, int nchunks, cudaStream_t st) {
  constexpr int smem = smem_bytes<NS, BN, NST>();
  static_assert(smem <= 232448, "shared memory per block");
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(k_tc_gemm<NS, NG, BN, NST>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  });
  if (attr != cudaSuccess) return attr;
  const CUtensorMap& mb = BN == 64 ? B.map64 : B.map;
  k_tc_gemm<NS, NG, BN, NST><<<dim3((unsigned)ntiles, (unsigned)nchunks), kThreads, smem, st>>>(A.map, mb, a);
  return cudaGetLastError();
}

}  // namespace

int slices_of(Mode m) { return m == kMixed ? 3 : 7; }

int64_t sliced_bytes(int64_t rows, int64_t K, int ns) {
  const int64_t Rpad = rup(rows, BM), Kpad = rup(K, BK);
  return rup(ns * Rpad * Kpad * 2, 256) + rup(Rpad * 4, 256);
}

cudaError_t sliced_init(Sliced* s, void* mem, int64_t rows, int64_t K, int ns, cudaStream_t st, bool zero) {
  s->rows = rows;
  s->K = K;
  s->ns = ns;
  s->Rpad = rup(rows, BM);
  s->Kpad = rup(K, BK);
  s->s = (__nv_bfloat16*)mem;
  s->ex = (int32_t*)((char*)mem + rup(ns * s->Rpad * s->Kpad * 2, 256));
  if (zero) {
    const cudaError_t e = cudaMemsetAsync(mem, 0, (size_t)sliced_bytes(rows, K, ns), st);
    if (e != cudaSuccess) return e;
  }
  auto enc = encode_fn();
  if (!enc) return cudaErrorNotSupported;
  const cuuint64_t dims[2] = {(cuuint64_t)s->Kpad, (cuuint64_t)(ns * s->Rpad)};
  const cuuint64_t strides[1] = {(cuuint64_t)(s->Kpad * 2)};
  const cuuint32_t box[2] = {BK, BM}, box64[2] = {BK, 64};
  const cuuint32_t es[2] = {1, 1};
  if (ns * s->Rpad >= (int64_t)1 << 31) return cudaErrorInvalidValue;
  CUresult r = enc(&s->map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, s->s, dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r == CUDA_SUCCESS)
    r = enc(&s->map64, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, s->s, dims, strides, box64, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t slice(const Source& src, Sliced* d, cudaStream_t st) {
  if (src.rows != d->rows || src.K != d->K || src.nr <= 0) return cudaErrorInvalidValue;
  const bool along_k = src.kmap != nullptr || src.ks == 1 || src.rs != 1;
  if (along_k)
    k_rowexp_warp<<<(unsigned)((d->Rpad + 7) / 8), 256, 0, st>>>(src, d->Rpad, d->ex);
  else
    k_rowexp_thread<<<(unsigned)((d->Rpad + 255) / 256), 256, 0, st>>>(src, d->Rpad, d->ex);
  const dim3 grid((unsigned)(d->Rpad / 32), (unsigned)(d->Kpad / 32));
  switch (d->ns) {
    case 3: k_slice<3><<<grid, 256, 0, st>>>(src, d->Rpad, d->Kpad, d->ex, d->s); break;
    case 7: k_slice<7><<<grid, 256, 0, st>>>(src, d->Rpad, d->Kpad, d->ex, d->s); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

int64_t fix_bytes(int64_t M, int64_t N) { return std::max<int64_t>(M, 1) * std::max<int64_t>(N, 1) * 8; }

namespace {
// K per chunk: the order-0 group (1 pair) of the mixed mode is exact up to
// 1024; the order-3 group (4 pairs) of the FP64 mode up to 256.
int chunk_kb_of(Mode m) { return m == kMixed ? 32 : 8; }
int bn_of(Mode m) { return m == kMixed ? 128 : 64; }
// The epilogue writes C itself (1: C = v, 2: C += v) for one K chunk and
// alpha = +-2^p with beta 0 or 1; otherwise fixed-point sums and a finish pass.
int direct_mode(int nchunks, const Out& o, int* aexp) {
  int e = 0;
  const double f = std::frexp(std::fabs(o.alpha), &e);
  *aexp = e - 1;
  if (nchunks != 1 || f != 0.5) return 0;
  return o.beta == 0.0 ? 1 : (o.beta == 1.0 ? 2 : 0);
}
}  // namespace

bool needs_fix(const Sliced& A, const Sliced&, Mode mode, const Out& o) {
  const int ck = chunk_kb_of(mode);
  const int nchunks = (int)((A.Kpad / BK + ck - 1) / ck);
  int aexp;
  return direct_mode(nchunks, o, &aexp) == 0;
}

cudaError_t gemm(const Sliced& A, const Sliced& B, Mode mode, const Out& o, cudaStream_t st, int64_t* launches) {
  const int ns = slices_of(mode);
  if (A.ns != ns || B.ns != ns || A.Kpad != B.Kpad || A.K != B.K) return cudaErrorInvalidValue;
  if (o.lower && A.rows != B.rows) return cudaErrorInvalidValue;
  const int64_t M = A.rows, N = B.rows;
  if (M == 0 || N == 0) return cudaSuccess;
  Args a{};
  a.M = M;
  a.N = N;
  a.rpad_a = A.Rpad;
  a.rpad_b = B.Rpad;
  a.kblocks = (int)(A.Kpad / BK);
  a.chunk_kb = chunk_kb_of(mode);
  const int nchunks = (a.kblocks + a.chunk_kb - 1) / a.chunk_kb;
  if (nchunks > 65535) return cudaErrorInvalidValue;
  int aexp = 0;
  a.direct = direct_mode(nchunks, o, &aexp);
  a.alpha_exp = aexp;
  a.alpha_neg = o.alpha < 0 ? 1 : 0;
  if (!a.direct && !o.fix) return cudaErrorInvalidValue;
  int lg = 0;
  while (((int64_t)1 << lg) < std::max<int64_t>(A.K, 2)) ++lg;
  a.U = std::max(16, std::min(46, 47 - lg));
  a.exa = A.ex;
  a.exb = B.ex;
  a.C = o.C;
  a.ldc = o.ldc;
  a.fix = (unsigned long long*)o.fix;
  a.ldfix = o.ldfix;
  a.err = o.err;
  a.lower = o.lower ? 1 : 0;
  const int BN = bn_of(mode);
  const int64_t tm = (M + BM - 1) / BM, tn = (N + BN - 1) / BN;
  a.tiles_m = (int32_t)tm;
  a.tiles_n = (int32_t)tn;
  const int64_t ntiles = tm * tn;
  if (ntiles >= ((int64_t)1 << 31)) return cudaErrorInvalidValue;
  cudaError_t e = cudaSuccess;
  if (!a.direct) {
    e = cudaMemset2DAsync(o.fix, (size_t)(o.ldfix * 8), 0, (size_t)(M * 8), (size_t)N, st);
    if (e != cudaSuccess) return e;
  }
  // mixed: orders 0 | 1-2 (2 groups, 128-column tiles, 4 stages);
  // FP64: orders 0 | 1 | 2 | 3 | 4-6 (5 groups, 64-column tiles, 2 stages)
  e = mode == kMixed ? launch<3, 2, 128, 4>(A, B, a, ntiles, nchunks, st)
                     : launch<7, 5, 64, 2>(A, B, a, ntiles, nchunks, st);
  if (e != cudaSuccess) return e;
  if (launches) *launches += 1;
  if (!a.direct) {
    const int64_t total = M * N;
    const unsigned grid = (unsigned)std::min<int64_t>((total + 255) / 256, 152 * 32);
    k_finish<<<grid, 256, 0, st>>>(M, N, o.fix, o.ldfix, A.ex, B.ex, a.U, o.alpha, o.beta, o.C, o.ldc, a.lower);
    if (launches) *launches += 1;
    e = cudaGetLastError();
  }
  return e;
}

}  // namespace tcg

// ---------------------------------------------------------------- C ABI
// C = alpha op(A) op(B) + beta C on the tensor cores (include/madsdp_gpu.h).
extern "C" int msdp_tc_gemm(int32_t precision, int32_t transa, int32_t transb, int64_t M, int64_t N, int64_t K,
                            double alpha, const double* A, int64_t lda, const double* B, int64_t ldb, double beta,
                            double* C, int64_t ldc, int32_t lower, void* stream) {
  using namespace tcg;
  if (M < 0 || N < 0 || K < 0 || (M && !C) || ldc < std::max<int64_t>(M, 1)) return MSDP_ERR_INVALID_ARGUMENT;
  if (precision != MSDP_FP64 && precision != MSDP_MIXED) return MSDP_ERR_INVALID_ARGUMENT;
  if (lower && M != N) return MSDP_ERR_INVALID_ARGUMENT;
  if (M == 0 || N == 0) return MSDP_OK;
  if (K == 0 || (!A || !B)) return MSDP_ERR_INVALID_ARGUMENT;
  if (lda < (transa ? K : M) || ldb < (transb ? N : K)) return MSDP_ERR_INVALID_ARGUMENT;
  const Mode mode = precision == MSDP_MIXED ? kMixed : kFp64;
  const int ns = slices_of(mode);
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t ba = sliced_bytes(M, K, ns), bb = sliced_bytes(N, K, ns), bf = fix_bytes(M, N);
  char* mem = nullptr;
  if (cudaMalloc(&mem, (size_t)(ba + bb + bf + 256)) != cudaSuccess) return MSDP_ERR_OUT_OF_MEMORY;
  Sliced SA, SB;
  int* err = (int*)(mem + ba + bb + bf);
  int rc = MSDP_OK;
  cudaError_t e = sliced_init(&SA, mem, M, K, ns, st);
  if (e == cudaSuccess) e = sliced_init(&SB, mem + ba, N, K, ns, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), st);
  Source sa, sb;
  // A operand rows = rows of op(A): op(A)(r, k)
  sa.p = A; sa.rows = M; sa.K = K; sa.nr = M; sa.bs = 0;
  sa.rs = transa ? lda : 1; sa.ks = transa ? 1 : lda;
  // B operand rows = columns of op(B): op(B)(k, c)
  sb.p = B; sb.rows = N; sb.K = K; sb.nr = N; sb.bs = 0;
  sb.rs = transb ? 1 : ldb; sb.ks = transb ? ldb : 1;
  if (e == cudaSuccess) e = slice(sa, &SA, st);
  if (e == cudaSuccess) e = slice(sb, &SB, st);
  Out o;
  o.C = C; o.ldc = ldc; o.alpha = alpha; o.beta = beta; o.lower = lower != 0;
  o.fix = (long long*)(mem + ba + bb); o.ldfix = M; o.err = err;
  if (e == cudaSuccess) e = gemm(SA, SB, mode, o, st, nullptr);
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) rc = MSDP_ERR_CUDA;
  else if (herr) rc = MSDP_ERR_CUDA;
  cudaFree(mem);
  return rc;
}
