// Host launchers of the device kernels; each kernel variant lives in its
// own translation unit (kernel_fp64.cu, kernel_mixed.cu) so the library
// builds in parallel.
#pragma once
#include <cuda_runtime.h>
#include "layout.h"
#include "la.cuh"

#ifndef MSDP_SMEM_BYTES
#ifndef MSDP_SMEM_KB
#define MSDP_SMEM_KB 72
#endif
#define MSDP_SMEM_BYTES (MSDP_SMEM_KB * 1024)
#endif

// mixed = 0: FP64 kernel; mixed = 1: FP32 phase + FP64 phase kernel



cudaError_t msdp_gather_launch(const BatchDev& B, double* out, cudaStream_t stream);
cudaError_t msdp_gather_launch_idx(const BatchDev& B, const int32_t* idx, int count, double* out, cudaStream_t stream);

cudaError_t msdp_ipm_setup_0();
cudaError_t msdp_ipm_setup_1();
int msdp_ipm_occupancy_0();
int msdp_ipm_occupancy_1();
cudaError_t msdp_ipm_launch_0(const BatchDev& B, int grid, cudaStream_t stream);
cudaError_t msdp_ipm_launch_1(const BatchDev& B, int grid, cudaStream_t stream);

inline cudaError_t msdp_ipm_setup(int mixed) { return mixed ? msdp_ipm_setup_1() : msdp_ipm_setup_0(); }
inline int msdp_ipm_occupancy(int mixed) { return mixed ? msdp_ipm_occupancy_1() : msdp_ipm_occupancy_0(); }
inline cudaError_t msdp_ipm_launch(int mixed, const BatchDev& B, int grid, cudaStream_t stream) {
  return mixed ? msdp_ipm_launch_1(B, grid, stream) : msdp_ipm_launch_0(B, grid, stream);
}
