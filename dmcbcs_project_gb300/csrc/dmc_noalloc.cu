// Branching without device allocation: dmc_branch_noalloc keeps its scratch
// (copy counts, prefix offsets, the walkers' random states after ran1) in a
// fixed file-scope device array instead of buffers obtained from cudaMalloc.
#include <cuda_runtime.h>

#include <cstdint>
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

// byte ranges of the fields of a stack of `count` walkers
int ranges(const dmc_dev_stack& s, int count, int npart, uintptr_t (*r)[2])
{
    const size_t n3 = (size_t)count * 3 * npart * sizeof(double), n1 = (size_t)count * sizeof(double);
    const void* p[15] = {s.x, s.dpsi, s.dpsig, s.psil, s.psigl, s.d2psi, s.d2psig, s.v,
                         s.vext, s.weight, s.psil0, s.psigl0, s.wt0, s.is, s.irn};
    const size_t b[15] = {n3, n3, n3, n1, n1, n1, n1, n1, n1, n1, n1, n1, (size_t)count * sizeof(float),
                          (size_t)count * sizeof(int), (size_t)count * sizeof(uint64_t)};
    for (int k = 0; k < 15; ++k) {
        r[k][0] = reinterpret_cast<uintptr_t>(p[k]);
        r[k][1] = r[k][0] + b[k];
    }
    return 15;
}

// true when a field of the input stack (n walkers) overlaps a field of the
// output stack (cap walkers): the scatter would read walkers it overwrites
bool stacks_overlap(const dmc_dev_stack& in, int n, const dmc_dev_stack& out, int cap, int npart)
{
    uintptr_t a[15][2], b[15][2];
    ranges(in, n, npart, a);
    ranges(out, cap, npart, b);
    for (int i = 0; i < 15; ++i)
        for (int j = 0; j < 15; ++j)
            if (a[i][0] < b[j][1] && b[j][0] < a[i][1]) return true;
    return false;
}

}  // namespace

extern "C" int dmc_branch_noalloc(int n, int npart, int cap, double factor, const dmc_dev_stack* in,
                                  const dmc_dev_stack* out, uint64_t* wtisto, int* nout, void* stream)
{
    if (!in || !out || !nout || n < 0 || cap < 0 || npart < 1 || npart > DMC_MAX_PART) return DMC_ERR_INVALID;
    if (!(factor >= 0.0) || !(factor <= 1.0e6)) return DMC_ERR_INVALID;   // also rejects NaN
    if (n > kMax || cap > kMax) return DMC_ERR_NOALLOC_LIMIT;
    *nout = 0;
    if (n == 0) return DMC_OK;
    if (stacks_overlap(*in, n, *out, cap, npart)) return DMC_ERR_INVALID;
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
