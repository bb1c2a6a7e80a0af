// Newton error of a device-resident residual without any allocation.
//
// gbfv_newton_error_noalloc computes what gbfv_newton_error computes -- the
// maximum norm of the residual over the cells that are not constraint cells
// (NewtonMethod::preSolve_, newtonmethod.hh:572-598) -- for a
// residual that the caller already holds in device memory, and allocates
// nothing: no cudaMalloc, no cudaFree, no library routine that allocates.
// Its scratch is the fixed file-scope device array below.
//
//   pass 1 (kNewtonErrorPartials): one block per NOALLOC_CELLS_PER_BLOCK
//          cells writes its maximum (as the bit pattern of a non-negative
//          double; a non-finite value writes the all-ones pattern) to
//          partial[blockIdx.x];
//   pass 2 (kNewtonErrorCombine): one block folds the partials into
//          result, which is copied to the host.
//
// Every scratch word that a call reads is written earlier in the same call,
// so nothing in the scratch has to start at zero.  Two calls that overlap in
// time (on different streams or host threads) share the scratch and race.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/gbfv.h"
#include "gbfv_internal.cuh"

namespace gbfv {
void setLastError(const std::string& s);
}

namespace {

constexpr int NOALLOC_THREADS = 256;
constexpr int NOALLOC_CELLS_PER_BLOCK = NOALLOC_THREADS;
constexpr int NOALLOC_MAX_BLOCKS = GBFV_NOALLOC_MAX_CELLS / NOALLOC_CELLS_PER_BLOCK;
constexpr unsigned long long NONFINITE_BITS = ~0ull;  // above every finite or infinite double

struct NoAllocScratch {
    unsigned long long partial[NOALLOC_MAX_BLOCKS];
    unsigned long long result;
};
static_assert(GBFV_NOALLOC_MAX_CELLS % NOALLOC_CELLS_PER_BLOCK == 0, "whole blocks");

// 512 KiB + 8 B of device memory, part of the module image
static __device__ __align__(256) NoAllocScratch g_noallocScratch;

constexpr int MAX_DEVICES = 64;
NoAllocScratch* g_scratchOfDevice[MAX_DEVICES] = {};
std::mutex g_setupMutex;

__device__ __forceinline__ unsigned long long maxBits(unsigned long long a, unsigned long long b) { return a > b ? a : b; }

__device__ unsigned long long blockMaxBits(unsigned long long bits)
{
    __shared__ unsigned long long swarp[NOALLOC_THREADS / 32];
    for (int o = 16; o > 0; o >>= 1) bits = maxBits(bits, __shfl_down_sync(0xffffffffu, bits, o));
    if ((threadIdx.x & 31) == 0) swarp[threadIdx.x >> 5] = bits;
    __syncthreads();
    unsigned long long b = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < NOALLOC_THREADS / 32; ++w) b = maxBits(b, swarp[w]);
    return b;
}

// NewtonMethod::preSolve_'s error (newtonmethod.hh:572-607): per block the
// max |r| over the cells the caller does not skip, as a bit pattern
__global__ void __launch_bounds__(NOALLOC_THREADS) kNewtonErrorPartials(const double* __restrict__ r,
                                                                          const int32_t* __restrict__ skip, int n,
                                                                          int b, NoAllocScratch* scr)
{
    const int p = blockIdx.x * NOALLOC_CELLS_PER_BLOCK + threadIdx.x;
    unsigned long long bits = 0;
    if (p < n && (skip == nullptr || skip[p] == 0)) {
        double e = 0.0;
        bool bad = false;
        for (int k = 0; k < b; ++k) {
            const double v = r[(size_t)p * b + k];
            if (!isfinite(v)) bad = true;
            else e = fmax(e, fabs(v));
        }
        bits = bad ? NONFINITE_BITS : (unsigned long long)__double_as_longlong(e);
    }
    bits = blockMaxBits(bits);
    if (threadIdx.x == 0) scr->partial[blockIdx.x] = bits;
}

// the blocks' maxima combined into the error (newtonmethod.hh:572-607)
__global__ void __launch_bounds__(NOALLOC_THREADS) kNewtonErrorCombine(int nblocks, NoAllocScratch* scr)
{
    unsigned long long bits = 0;
    for (int i = threadIdx.x; i < nblocks; i += NOALLOC_THREADS) bits = maxBits(bits, scr->partial[i]);
    bits = blockMaxBits(bits);
    if (threadIdx.x == 0) scr->result = bits;
}

// Set-up, once per device, with that device current: the address of the
// scratch array on this device.  It is cached for the life of the process;
// a device reset after the first call would leave it stale (documented as
// unsupported in the header).
int scratchOfCurrentDevice(NoAllocScratch** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        gbfv::setLastError(std::string("gbfv_newton_error_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return GBFV_ERR_CUDA;
    }
    if (dev < 0 || dev >= MAX_DEVICES) {
        gbfv::setLastError("gbfv_newton_error_noalloc: device ordinal beyond 63");
        return GBFV_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(g_setupMutex);
    if (!g_scratchOfDevice[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess || p == nullptr) {
            gbfv::setLastError(std::string("gbfv_newton_error_noalloc: cudaGetSymbolAddress: ") +
                               cudaGetErrorString(e));
            return GBFV_ERR_CUDA;
        }
        g_scratchOfDevice[dev] = static_cast<NoAllocScratch*>(p);
    }
    *out = g_scratchOfDevice[dev];
    return GBFV_OK;
}

}  // namespace

extern "C" int gbfv_newton_error_noalloc(const double* residual, const int32_t* skip, int32_t num_cells,
                                         int32_t num_eq, void* stream, double* error)
{
    if (!residual || !error || num_cells < 0 || num_eq < 1 || num_eq > 8) {
        gbfv::setLastError("gbfv_newton_error_noalloc: null pointer, negative cell count or num_eq outside [1, 8]");
        return GBFV_ERR_ARG;
    }
    if (num_cells > GBFV_NOALLOC_MAX_CELLS) {
        gbfv::setLastError("gbfv_newton_error_noalloc: num_cells " + std::to_string(num_cells) +
                           " exceeds the scratch limit GBFV_NOALLOC_MAX_CELLS = " +
                           std::to_string(GBFV_NOALLOC_MAX_CELLS));
        return GBFV_ERR_ARG;
    }
    NoAllocScratch* scr = nullptr;
    int st = scratchOfCurrentDevice(&scr);
    if (st != GBFV_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nblocks = (num_cells + NOALLOC_CELLS_PER_BLOCK - 1) / NOALLOC_CELLS_PER_BLOCK;
    if (nblocks > 0) {
        kNewtonErrorPartials<<<nblocks, NOALLOC_THREADS, 0, s>>>(residual, skip, num_cells, num_eq, scr);
        gbfv::countLaunch();
    }
    kNewtonErrorCombine<<<1, NOALLOC_THREADS, 0, s>>>(nblocks, scr);
    gbfv::countLaunch();
    cudaError_t e = cudaGetLastError();
    unsigned long long bits = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bits, &scr->result, sizeof(bits), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        gbfv::setLastError(std::string("gbfv_newton_error_noalloc: ") + cudaGetErrorString(e));
        return GBFV_ERR_CUDA;
    }
    if (bits == NONFINITE_BITS) {
        *error = __builtin_nan("");
        return GBFV_ERR_NONFINITE;
    }
    double v;
    static_assert(sizeof(v) == sizeof(bits), "64-bit double");
    __builtin_memcpy(&v, &bits, sizeof(v));
    *error = v;
    return GBFV_OK;
}
