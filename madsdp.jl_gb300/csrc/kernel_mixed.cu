// The mixed-precision variant of the persistent IPM kernel.
#include "kernel.cuh"
#include "launch.h"


cudaError_t msdp_ipm_setup_1() {
  return cudaFuncSetAttribute(msdp_ipm_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, MSDP_SMEM_BYTES);
}
int msdp_ipm_occupancy_1() {
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, msdp_ipm_kernel<1>, NTHREADS, MSDP_SMEM_BYTES) != cudaSuccess) return 1;
  return occ;
}
cudaError_t msdp_ipm_launch_1(const BatchDev& B, int grid, cudaStream_t stream) {
  msdp_ipm_kernel<1><<<grid, NTHREADS, MSDP_SMEM_BYTES, stream>>>(B);
  return cudaGetLastError();
}
