// The walker kernel instances for systems whose union region (orbital
// matrices U and D, orbital powers, the second inverse buffer and the pair
// vectors) does not fit one CTA's shared memory: that region lives in the
// CTA's slice of an L2-resident global scratch buffer (BIG = true), the pair
// matrix, positions and accumulators stay on chip.  Every idmc, both
// precisions, 256 threads; a translation unit of its own so that the
// on-chip instances keep their code and the units compile in parallel.
#include <cuda_runtime.h>

#include "dmc_attr.h"
#include "dmc_kernels.h"
#include "dmc_walker_kernel.cuh"

namespace dmc {

int walker_big_static_smem_bytes()
{
    cudaFuncAttributes a[4]{};
    if (cudaFuncGetAttributes(&a[0], walker_kernel<double, kThreads, false, true>) != cudaSuccess) return -1;
    if (cudaFuncGetAttributes(&a[1], walker_kernel<df, kThreads, false, true>) != cudaSuccess) return -1;
    if (cudaFuncGetAttributes(&a[2], walker_kernel<double, kThreads, true, true>) != cudaSuccess) return -1;
    if (cudaFuncGetAttributes(&a[3], walker_kernel<df, kThreads, true, true>) != cudaSuccess) return -1;
    size_t m = 0;
    for (const auto& x : a) m = x.sharedSizeBytes > m ? x.sharedSizeBytes : m;
    return (int)m;
}

// per-device record: kind 0 the carveout, 1..4 the dynamic shared-memory
// opt-in of <double / df> x <GF false / true>
static AttrCache g_attr_big;

template <class R, bool GF>
static int set_smem_attr_big(int v)
{
    return (int)cudaFuncSetAttribute(walker_kernel<R, kThreads, GF, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     v);
}

cudaError_t walker_big_attrs(int smem)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    int rc = g_attr_big.ensure(dev, 0, 1, [](int) {
        const int c = (int)cudaSharedmemCarveoutMaxShared;
        cudaError_t r = cudaFuncSetAttribute(walker_kernel<double, kThreads, false, true>,
                                             cudaFuncAttributePreferredSharedMemoryCarveout, c);
        if (r == cudaSuccess)
            r = cudaFuncSetAttribute(walker_kernel<df, kThreads, false, true>,
                                     cudaFuncAttributePreferredSharedMemoryCarveout, c);
        if (r == cudaSuccess)
            r = cudaFuncSetAttribute(walker_kernel<double, kThreads, true, true>,
                                     cudaFuncAttributePreferredSharedMemoryCarveout, c);
        if (r == cudaSuccess)
            r = cudaFuncSetAttribute(walker_kernel<df, kThreads, true, true>,
                                     cudaFuncAttributePreferredSharedMemoryCarveout, c);
        return (int)r;
    });
    if (!rc) rc = g_attr_big.ensure(dev, 1, smem, set_smem_attr_big<double, false>);
    if (!rc) rc = g_attr_big.ensure(dev, 2, smem, set_smem_attr_big<df, false>);
    if (!rc) rc = g_attr_big.ensure(dev, 3, smem, set_smem_attr_big<double, true>);
    if (!rc) rc = g_attr_big.ensure(dev, 4, smem, set_smem_attr_big<df, true>);
    return (cudaError_t)rc;
}

cudaError_t launch_walker_big(const DevParams& p, const KernelArgs& a, const SmemLayout& L, int grid, cudaStream_t st,
                              bool mixed, bool gf)
{
    const size_t smem = (size_t)L.total * 8;
    const cudaError_t e = walker_big_attrs((int)smem);
    if (e != cudaSuccess) return e;
    if (!a.gscratch) return cudaErrorInvalidValue;   // the union region needs the scratch slices
    if (gf) {
        if (mixed)
            walker_kernel<df, kThreads, true, true><<<grid, kThreads, smem, st>>>(p, a, L);
        else
            walker_kernel<double, kThreads, true, true><<<grid, kThreads, smem, st>>>(p, a, L);
    } else {
        if (mixed)
            walker_kernel<df, kThreads, false, true><<<grid, kThreads, smem, st>>>(p, a, L);
        else
            walker_kernel<double, kThreads, false, true><<<grid, kThreads, smem, st>>>(p, a, L);
    }
    return cudaGetLastError();
}

}   // namespace dmc
