// Branching without device allocation: dmc_branch_noalloc keeps its scratch
// (copy counts, prefix offsets, the walkers' random states after ran1) in a
// fixed file-scope device array instead of buffers obtained from cudaMalloc.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/dmcbcs_gpu.h"
#include "dmc_device.cuh"
#include "dmc_kernels.h"

namespace {

constexpr int kMax = DMC_NOALLOC_MAX_WALKERS;
// layout of the scratch, in bytes (each part 256-byte aligned)
constexpr size_t kCountsOff = 0;
constexpr size_t kOffsOff = kCountsOff + ((sizeof(int) * kMax + 255) / 256) * 256;
constexpr size_t kIrnOff = kOffsOff + ((sizeof(int) * (kMax + 1) + 255) / 256) * 256;
constexpr size_t kHistOff = kIrnOff + ((sizeof(unsigned long long) * kMax + 255) / 256) * 256;
constexpr size_t kBytes = kHistOff + ((sizeof(unsigned long long) * DMC_WTISTO + 255) / 256) * 256;

// The scratch itself.  Host code must not pass this name to a kernel: on the
// host it only stands for the symbol, so its device address is looked up
// with cudaGetSymbolAddress once per device.
static __device__ __align__(256) unsigned char g_branch_scratch[kBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_addr[kMaxDevices] = {};

// device address of the scratch on the current device (looked up once)
cudaError_t scratch_address(unsigned char** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_branch_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

dmc::DevStack view(const dmc_dev_stack& s)
{
    dmc::DevStack d;
    d.x = s.x; d.dpsi = s.dpsi; d.dpsig = s.dpsig; d.psil = s.psil; d.psigl = s.psigl; d.d2psi = s.d2psi;
    d.d2psig = s.d2psig; d.v = s.v; d.vext = s.vext; d.weight = s.weight; d.psil0 = s.psil0; d.psigl0 = s.psigl0;
    d.wt0 = s.wt0; d.is = s.is; d.irn = reinterpret_cast<unsigned long long*>(s.irn);
    return d;
}

}  // namespace

extern "C" int dmc_branch_noalloc(int n, int npart, int cap, double factor, const dmc_dev_stack* in,
                                  const dmc_dev_stack* out, uint64_t* wtisto, int* nout, void* stream)
{
    if (!in || !out || !nout || n < 0 || cap < 0 || npart < 1 || npart > DMC_MAX_PART) return DMC_ERR_INVALID;
    if (n > kMax || cap > kMax) return DMC_ERR_NOALLOC_LIMIT;
    *nout = 0;
    if (n == 0) return DMC_OK;
    unsigned char* base = nullptr;
    if (scratch_address(&base) != cudaSuccess) return DMC_ERR_CUDA;
    int* counts = reinterpret_cast<int*>(base + kCountsOff);
    int* offs = reinterpret_cast<int*>(base + kOffsOff);
    unsigned long long* irn1 = reinterpret_cast<unsigned long long*>(base + kIrnOff);
    unsigned long long* hist =
        wtisto ? reinterpret_cast<unsigned long long*>(wtisto) : reinterpret_cast<unsigned long long*>(base + kHistOff);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dmc::launch_branch(view(*in), view(*out), n, 3 * npart, cap, factor, counts, offs, irn1, hist, st) !=
        cudaSuccess)
        return DMC_ERR_CUDA;
    int total = 0;
    if (cudaMemcpyAsync(&total, offs + n, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return DMC_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return DMC_ERR_CUDA;
    if (total > cap) {
        *nout = cap;
        return DMC_ERR_OVERFLOW;
    }
    *nout = total;
    return DMC_OK;
}
