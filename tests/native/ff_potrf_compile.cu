// Compile-only check: the CTA Cholesky of la.cuh instantiated with the
// float-float type of ff.cuh (no launch; the test reads ptxas's report).
#include "../../madsdp.jl_gb300/csrc/ff.cuh"
#include "../../madsdp.jl_gb300/csrc/la.cuh"

template <> struct Num<ff> {
  static __device__ __forceinline__ ff eps() { return ff(1.2325951644078310e-32); }
  static __device__ __forceinline__ ff sqrt_(ff x) { return sqrt(x); }
  static __device__ __forceinline__ ff rsqrt_(ff x) { return ff(1.0f) / sqrt(x); }
  static __device__ __forceinline__ bool finite(ff x) { return isfinite(x.hi) && isfinite(x.lo); }
};

__global__ void ff_potrf_probe(ff* a, int n, int* ok) {
  __shared__ int flag;
  const bool r = cta_potrf<ff>(n, a, n, &flag);
  if (threadIdx.x == 0) *ok = r ? 1 : 0;
}
