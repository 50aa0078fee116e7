// Launchers of the GB300 DMCBS kernels (implemented in dmc_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "dmc_device.cuh"

namespace dmc {

// Bytes of dynamic shared memory of the walker kernel for these sizes; fills
// the on-chip layout.  limit_bytes is the per-CTA budget.
int walker_smem_bytes(const DevParams& p, int limit_bytes, SmemLayout* L);

cudaError_t launch_walker(const DevParams& p, const KernelArgs& a, const SmemLayout& L, int grid, cudaStream_t st,
                          bool mixed = false);

cudaError_t launch_estimators(const double* est, int n, int nest, double* valblk, double* valblk2, double* wtblk,
                              cudaStream_t st);

cudaError_t launch_branch(const DevStack& in, const DevStack& out, int n, int n3, int cap, double factor,
                          int* counts, int* offs, unsigned long long* irn1, unsigned long long* wtisto,
                          cudaStream_t st);

// FMA throughput of the FP64 (kind 0) or FP32 (kind 1) pipe, TFLOP/s
cudaError_t probe_fma_peak(int kind, int nsm, double* tflops);

}  // namespace dmc
