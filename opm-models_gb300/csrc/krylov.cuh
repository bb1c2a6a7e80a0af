// Device building blocks shared by the persistent solve kernels (ILU(0) and
// AMG preconditioned BiCGStab): bounded software grid barrier, block and
// grid reductions in a fixed order, small dense block inverse.
#pragma once

#include <cuda_runtime.h>

#include <cooperative_groups.h>

#include "../../include/gbfv.h"
#include "gbfv_internal.cuh"
#include "solver.cuh"

namespace gbfv {
namespace cg = cooperative_groups;

// every device-side wait gives up after 4e9 SM cycles (about two seconds)
// and reports GBFV_ERR_TIMEOUT instead of hanging
#define GB_TIMEOUT_CYCLES 4000000000LL

// loads of data written inside the kernel by other blocks go to L2 directly
// (ld.global.cg), so no block can hit a stale line in its own L1
__device__ __forceinline__ float ldcg(const float* p) { return __ldcg(p); }
__device__ __forceinline__ double ldcg(const double* p) { return __ldcg(p); }

__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// phase timer (only block 0 / thread 0 writes; no contention)
struct PhaseClock {
    unsigned long long* prof;
    unsigned long long t;
    bool on;
    __device__ PhaseClock(unsigned long long* p, int gt) : prof(p), t(0), on(p != nullptr && gt == 0)
    {
        if (on) t = gtimer();
    }
    __device__ __forceinline__ void tick(int k)
    {
        if (!on) return;
        const unsigned long long n = gtimer();
        prof[k] += n - t;
        t = n;
    }
};

// The set of blocks that cooperate on one system: the whole grid
// (cooperative launch, software barrier) or one thread-block cluster
// (hardware cluster barrier).
template <int MODE>
struct Team {
    int rank, nblk;
    __device__ Team()
    {
        if (MODE == SYNC_CLUSTER) {
            cg::cluster_group c = cg::this_cluster();
            rank = (int)c.block_rank();
            nblk = (int)c.num_blocks();
        }
        else {
            rank = blockIdx.x;
            nblk = gridDim.x;
        }
    }
};

// one arrival at the software grid barrier out of `expected`, bounded; false
// when this arrival or another one gave up (the abort word is then set)
__device__ __forceinline__ int gridArrive(const GridSync& g, unsigned expected)
{
    int ok = 1;
    volatile unsigned* vgen = g.gen;
    const unsigned my = *vgen;
    __threadfence();
    const unsigned arrived = atomicAdd(g.count, 1u);
    if (arrived == expected - 1) {
        atomicExch(g.count, 0u);
        __threadfence();
        atomicAdd(g.gen, 1u);
    }
    else {
        const long long t0 = clock64();
        while (*vgen == my) {
            if (*(volatile int*)g.abort) { ok = 0; break; }
            if (clock64() - t0 > GB_TIMEOUT_CYCLES) {
                atomicExch(g.abort, 1);
                ok = 0;
                break;
            }
            __nanosleep(64);
        }
    }
    __threadfence();
    return ok;
}

// Barrier over the whole cooperative grid.  A wait that gives up makes the
// blocks leave at different barriers; that is harmless when blocks share only
// global memory, but not inside a cluster whose blocks write into each
// other's shared memory (a block must not exit while a peer may still push
// into it).  So in a hybrid launch (g.perCluster > 0) each cluster arrives
// once, through its rank-0 block, and all blocks of the cluster take that
// block's decision: a cluster's blocks always leave together.
__device__ __forceinline__ bool gridBarrier(const GridSync& g)
{
    __shared__ int sOk;
    __syncthreads();
    if (gridDim.x == 1) return true;
    if (g.perCluster > 0) {
        cg::cluster_group cl = cg::this_cluster();
        if (threadIdx.x == 0) __threadfence();  // this block's writes are visible GPU-wide
        cl.sync();
        if (cl.block_rank() == 0 && threadIdx.x == 0) sOk = gridArrive(g, gridDim.x / cl.num_blocks());
        cl.sync();
        return *cl.map_shared_rank(&sOk, 0) != 0;
    }
    if (threadIdx.x == 0) sOk = gridArrive(g, gridDim.x);
    __syncthreads();
    return sOk != 0;
}

template <int MODE>
__device__ __forceinline__ bool teamSync(const GridSync& g)
{
    if (MODE == SYNC_CLUSTER) {
        cg::this_cluster().sync();
        return true;
    }
    return gridBarrier(g);
}

// block reduction of NV sums (or maxima) into partial[k*nblk + rank]
template <int NV, int MODE>
__device__ __forceinline__ void blockPartials(double (&v)[NV], const bool (&isMax)[NV], double* partial,
                                              const Team<MODE>& tm)
{
    __shared__ double sred[NV][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k)
        for (int o = 16; o > 0; o >>= 1) {
            const double t = __shfl_down_sync(0xffffffffu, v[k], o);
            v[k] = isMax[k] ? fmax(v[k], t) : v[k] + t;
        }
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) sred[k][w] = v[k];
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = lane < nw ? sred[k][lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) {
                const double u = __shfl_down_sync(0xffffffffu, t, o);
                t = isMax[k] ? fmax(t, u) : t + u;
            }
            if (lane == 0) __stcg(&partial[k * tm.nblk + tm.rank], t);
        }
    }
}

// after a team barrier: every block combines the partials in the same order
template <int NV, int MODE>
__device__ __forceinline__ void allCombine(const double* partial, const bool (&isMax)[NV], double (&out)[NV],
                                           const Team<MODE>& tm)
{
    __shared__ double sres[NV];
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = 0.0;
            for (int i = lane; i < tm.nblk; i += 32) {
                const double u = ldcg(&partial[k * tm.nblk + i]);
                t = isMax[k] ? fmax(t, u) : t + u;
            }
            for (int o = 16; o > 0; o >>= 1) {
                const double u = __shfl_xor_sync(0xffffffffu, t, o);
                t = isMax[k] ? fmax(t, u) : t + u;
            }
            if (lane == 0) sres[k] = t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = sres[k];
    __syncthreads();
}

// ----------------------------------------------------- block helpers -----
template <class T, int B>
__device__ __forceinline__ void ldBlock(const T* a, int slot, int ld, int row, T (&M)[B * B])
{
#pragma unroll
    for (int e = 0; e < B * B; ++e) M[e] = a[(slot * B * B + e) * ld + row];
}

template <class T, int B>
__device__ __forceinline__ bool invertBlock(const T (&A)[B * B], T (&R)[B * B])
{
    if (B == 2) {
        const T a = A[0], b = A[1], c = A[2], d = A[3];
        const T det = a * d - b * c;
        if (det == T(0) || !isfinite((double)det)) return false;
        const T id = T(1) / det;
        R[0] = d * id; R[1] = -b * id; R[2] = -c * id; R[3] = a * id;
        return true;
    }
    const T a00 = A[0], a01 = A[1], a02 = A[2];
    const T a10 = A[3], a11 = A[4], a12 = A[5];
    const T a20 = A[6], a21 = A[7], a22 = A[8];
    const T c00 = a11 * a22 - a12 * a21;
    const T c01 = a12 * a20 - a10 * a22;
    const T c02 = a10 * a21 - a11 * a20;
    const T det = a00 * c00 + a01 * c01 + a02 * c02;
    if (det == T(0) || !isfinite((double)det)) return false;
    const T id = T(1) / det;
    R[0] = c00 * id;
    R[1] = (a02 * a21 - a01 * a22) * id;
    R[2] = (a01 * a12 - a02 * a11) * id;
    R[3] = c01 * id;
    R[4] = (a00 * a22 - a02 * a20) * id;
    R[5] = (a02 * a10 - a00 * a12) * id;
    R[6] = c02 * id;
    R[7] = (a01 * a20 - a00 * a21) * id;
    R[8] = (a00 * a11 - a01 * a10) * id;
    return true;
}

}  // namespace gbfv
