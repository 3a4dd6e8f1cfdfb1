// The FP64 variant of the persistent IPM kernel.
#define MSDP_DEFINE_GATHER
#include "kernel.cuh"
#include "launch.h"


cudaError_t msdp_ipm_setup_0() {
  return cudaFuncSetAttribute(msdp_ipm_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, MSDP_SMEM_BYTES);
}
int msdp_ipm_occupancy_0() {
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, msdp_ipm_kernel<0>, NTHREADS, MSDP_SMEM_BYTES) != cudaSuccess) return 1;
  return occ;
}
cudaError_t msdp_ipm_launch_0(const BatchDev& B, int grid, cudaStream_t stream) {
  msdp_ipm_kernel<0><<<grid, NTHREADS, MSDP_SMEM_BYTES, stream>>>(B);
  return cudaGetLastError();
}

cudaError_t msdp_gather_launch(const BatchDev& B, double* out, cudaStream_t stream) {
  msdp_gather_scalars<<<B.nprob, 64, 0, stream>>>(B, out);
  return cudaGetLastError();
}

cudaError_t msdp_gather_launch_idx(const BatchDev& B, const int32_t* idx, int count, double* out, cudaStream_t stream) {
  if (count <= 0) return cudaSuccess;
  msdp_gather_scalars_idx<<<count, 64, 0, stream>>>(B, idx, out);
  return cudaGetLastError();
}
