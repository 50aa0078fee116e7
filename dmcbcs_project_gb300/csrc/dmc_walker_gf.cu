// The walker kernel instances for idmc = 10 (step.f90:231-279: direct
// sampling of the Green's function with importance sampling, two
// wavefunction evaluations per move), in a translation unit of their own:
// the other idmc values keep kernels without the second evaluation, and the
// two units compile in parallel.
#include <cuda_runtime.h>

#include "dmc_attr.h"
#include "dmc_kernels.h"
#include "dmc_walker_kernel.cuh"

namespace dmc {

int walker_gf_static_smem_bytes()
{
    cudaFuncAttributes a[3]{};
    if (cudaFuncGetAttributes(&a[0], walker_kernel<double, kThreads, true>) != cudaSuccess) return -1;
    if (cudaFuncGetAttributes(&a[1], walker_kernel<df, kThreads, true>) != cudaSuccess) return -1;
    if (cudaFuncGetAttributes(&a[2], walker_kernel<df, 2 * kThreads, true>) != cudaSuccess) return -1;
    size_t m = 0;
    for (const auto& x : a) m = x.sharedSizeBytes > m ? x.sharedSizeBytes : m;
    return (int)m;
}

// attribute kinds of the per-device record: the carveout, then the dynamic
// shared-memory opt-in of walker_kernel<double 256 / df 256 / df 512, GF>
static AttrCache g_attr_gf;

template <class R, int NT>
static int set_smem_attr_gf(int v)
{
    return (int)cudaFuncSetAttribute(walker_kernel<R, NT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
}

cudaError_t walker_gf_attrs(int smem, int nt, bool both, bool mixed)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    int rc = g_attr_gf.ensure(dev, 0, 1, [](int) {
        const int c = (int)cudaSharedmemCarveoutMaxShared;
        cudaError_t r =
            cudaFuncSetAttribute(walker_kernel<df, kThreads, true>, cudaFuncAttributePreferredSharedMemoryCarveout, c);
        if (r == cudaSuccess)
            r = cudaFuncSetAttribute(walker_kernel<double, kThreads, true>,
                                     cudaFuncAttributePreferredSharedMemoryCarveout, c);
        if (r == cudaSuccess)
            r = cudaFuncSetAttribute(walker_kernel<df, 2 * kThreads, true>,
                                     cudaFuncAttributePreferredSharedMemoryCarveout, c);
        return (int)r;
    });
    if (rc) return (cudaError_t)rc;
    const bool wide = nt != kThreads;
    if (both || mixed) {
        rc = g_attr_gf.ensure(dev, wide ? 3 : 2, smem,
                              wide ? set_smem_attr_gf<df, 2 * kThreads> : set_smem_attr_gf<df, kThreads>);
        if (rc) return (cudaError_t)rc;
    }
    if (both || !mixed) {
        rc = g_attr_gf.ensure(dev, 1, smem, set_smem_attr_gf<double, kThreads>);
        if (rc) return (cudaError_t)rc;
    }
    return cudaSuccess;
}

cudaError_t launch_walker_gf(const DevParams& p, const KernelArgs& a, const SmemLayout& L, int grid, cudaStream_t st,
                             bool mixed)
{
    const size_t smem = (size_t)L.total * 8;
    const cudaError_t e = walker_gf_attrs((int)smem, L.nt, false, mixed);
    if (e != cudaSuccess) return e;
    if (!mixed)
        walker_kernel<double, kThreads, true><<<grid, kThreads, smem, st>>>(p, a, L);
    else if (L.nt == 2 * kThreads)
        walker_kernel<df, 2 * kThreads, true><<<grid, 2 * kThreads, smem, st>>>(p, a, L);
    else
        walker_kernel<df, kThreads, true><<<grid, kThreads, smem, st>>>(p, a, L);
    return cudaGetLastError();
}

}   // namespace dmc
