// Arguments and launchers of the persistent BiCGStab / ILU(0) kernel and
// the FP64 helpers of the mixed-precision outer refinement.
#pragma once
#include <cuda_runtime.h>

#include "gbfv_internal.cuh"

namespace gbfv {

constexpr int SOLVER_THREADS = 256;   // blocks of the cooperative-grid variant
template <class T> constexpr int clusterThreads() { return sizeof(T) == 4 ? 512 : 256; }  // cluster variant
constexpr int MAX_PUSH_LEVELS = 2048;  // push sweeps keep the level pointers in shared memory
constexpr int PUSH_BUFFERS = 4;        // push sweeps: dependency buffers (levels in flight) per block
constexpr int PUSH_BARRIER_FLAG = 1 << 30;  // in levVals: a cluster barrier follows this level
// values per pushed dependency slot: a block of B values padded for one vector store
__host__ __device__ constexpr int padB(int B) { return B == 3 ? 4 : B; }
constexpr int SYNC_GRID = 0;     // whole grid, cooperative launch, software barrier
constexpr int SYNC_CLUSTER = 1;  // one thread-block cluster, hardware barrier
constexpr int SYNC_HYBRID = 2;   // launch mode: clusters over the whole GPU, cluster 0 sweeps, all share the rest
constexpr int HYBRID_CLUSTER = 16;  // cluster size of the hybrid launch
// or-ed into SYNC_HYBRID: blocks of SOLVER_THREADS threads (the FP32 solver
// otherwise runs clusterThreads<float>() per block); fewer threads make a
// level step cheaper where a level's share per block still fits
constexpr int SYNC_NARROW = 8;
// Spatial-tile sweeps (a flag or-ed into the cluster and hybrid modes): the
// rows of every level are dealt to the sweeping cluster's blocks by the
// spatial tile of their cell, so most dependencies stay inside a block.
constexpr int SYNC_TILES = 4;
constexpr int TILE_KEYS = 16;           // tiles the rows are ordered by (4 x 4)
constexpr int TILE_MAX_LEVELS = 1024;   // tile sweeps keep per-level data in shared memory
constexpr int TILE_HALO = 1 << 30;      // dependency code: a value pushed by another block (halo slot)
constexpr int TILE_MASK = (1 << 24) - 1;

// software grid barrier state (device memory, zero-initialised)
struct GridSync {
    unsigned* count;
    unsigned* gen;
    int* abort;
    int perCluster;     // hybrid launch: blocks per cluster; the cluster arrives once and
                        // its blocks share one decision (0: every block arrives)
};

// everything one solve needs; T is the Krylov/preconditioner precision
template <class T>
struct KArgs {
    int N, ldN, dim, nslot, numLev;
    const int* col;     // [s*ldN + p]
    const int* levPtr;  // [numLev+1]
    const T* A;         // [(s*b*b + e)*ldN + p]
    T* FL;              // lower factor blocks, slots [0, dim)
    T* FD;              // inverted pivots [e*ldN + p]
    const T* rhs;       // [p*b + e]
    T *x, *r, *p, *v, *y, *z;
    double* partial;    // [4*blocks]: two halves, alternately used
    GridSync gs;
    DevStatus* st;
    double redTol, absTol, maxRes;
    int maxIter;
    int factor;         // factorize before iterating
    unsigned long long* prof;  // optional per-phase nanoseconds (block 0, thread 0): factor,
                               // L sweep, U sweep, SpMV+dot, update+max, count of iterations
    int hybrid;         // hybrid launch: the sweeping cluster's blocks (0 = not hybrid)
    int grp;            // push sweeps: number of level-rotating thread groups
    int ownerMode;      // push sweeps: rows of a level dealt to blocks by warp round-robin (0) or contiguously (1)
    const int* pushL;   // push sweeps: consumer block/slot of each upper neighbour [q*ldN + p]
    const int* pushU;   // push sweeps: consumer block/slot of each lower neighbour [q*ldN + p]
    const int* levVals; // push sweeps: values block r receives at level l, [(r*numLev + l)*2 + fwd/bwd]
    int dsmem;          // cluster mode: every level fits one row per thread, so the
                        // previous level's results are exchanged in distributed shared memory
    int cluster;        // push sweeps: the cluster size the push tables were built for
    int tile;           // spatial-tile sweeps (instead of the push sweeps)
    const int4* tinfo;  // tile sweeps: [r*numLev + l] first row, rows, forward / backward halo slots
    const int* tdepF;   // tile sweeps: [q*ldN + p] row p's dependency q: -1 none, a position in the
    const int* tdepB;   //   block's previous level, or TILE_HALO | halo slot
    const int* tpushF;  // tile sweeps: [t*ldN + p] (consumer block << 24) | halo slot, or -1
    const int* tpushB;
    int thalo;          // tile sweeps: halo slots per block
    int twidth;         // tile sweeps: the most rows a block computes in one level
};

template <class T> int launchBicgstab(const KArgs<T>& a, int b, int mode, int nblocks, cudaStream_t s);
// dynamic shared memory of the tile sweeps, and the most a solve launch may use
template <class T> size_t tileSmemBytes(int b, int numLev, int haloSlots, int width, int dim);
template <class T> size_t solverSmemLimit(int b);

// One system of a batched mixed-precision refinement (FP64 true residual of
// the Newton system, FP32 inner solve)
struct SolveJob {
    int N, ld, nslot, b;
    long nval;              // nslot*b*b*ld matrix entries
    const int* col;
    const double* A64;      // FP64 Jacobian (block-ELL)
    float* A32;             // its FP32 copy
    const double* rhs;      // FP64 right-hand side (the Newton residual)
    double* xref;           // FP64 accumulated solution
    double* rref;           // FP64 true residual
    float* r32;             // its FP32 copy: right-hand side of the inner solve
    const float* dx32;      // inner solution added to xref
    DevStatus* st;
};
void launchBatchCast(const SolveJob* jobs, const int* active, int K, int gx, cudaStream_t s);
void launchBatchZeroX(const SolveJob* jobs, const int* active, int K, int gx, cudaStream_t s);
void launchBatchAccumulate(const SolveJob* jobs, const int* active, int K, int gx, cudaStream_t s);
void launchBatchResidual64(const SolveJob* jobs, const int* active, int K, int gx, int b, cudaStream_t s);
template <class T> int maxSolverBlocks(int b);
template <class T> int maxClusterBlocks(int b);
template <class T> int maxHybridBlocks(int b, bool narrow = false);
// batched solve: clusters of clusterSize blocks take systems args[order[q]],
// q = 0..*count-1 (device memory), from the queue counter (zero before the launch)
template <class T>
int launchBicgstabBatch(const KArgs<T>* args, const int* order, const int* count, int* queue, int b,
                        int clusterSize, int numClusters, int maxLev, cudaStream_t s);
template <class T> int maxActiveClusters(int b, int clusterSize);
void launchCastMatrix(const double* src, float* dst, long n, cudaStream_t s);
void launchWaitTimeoutProbe(DevStatus* st, cudaStream_t s);
void launchAccumulate(int n, double* x, const float* d, cudaStream_t s);
void launchResidual64(int N, int ld, int nslot, int b, const int* col, const double* A, const double* rhs,
                      const double* x, double* r, float* r32, DevStatus* st, cudaStream_t s);

// device-side decisions of a batched Newton round (batchround.cu)
void launchRoundBegin(RoundSys* ys, JobState* js, DevStatus* st, int K, cudaStream_t s);
void launchRoundAfterLin(RoundSys* ys, const JobState* js, DevStatus* st, int* act, KArgs<float>* ka32,
                         KArgs<double>* ka64, const SolveJob* sj, int* order, int* queue, const RoundParams& p, int K,
                         cudaStream_t s);
void launchRoundAfterRes0(RoundSys* ys, DevStatus* st, int* act, KArgs<float>* ka, const SolveJob* sj, int* order,
                          int* queue, const RoundParams& p, int K, cudaStream_t s);
void launchRoundAfterKrylov(RoundSys* ys, DevStatus* st, int* act, const RoundParams& p, int K, cudaStream_t s);
void launchRoundAfterRefine(RoundSys* ys, DevStatus* st, int* act, KArgs<float>* ka, const SolveJob* sj, int* order,
                            int* queue, const RoundParams& p, int K, int lastRefinement, cudaStream_t s);
void launchRoundBeforeCheck(RoundSys* ys, JobState* js, DevStatus* st, int K, cudaStream_t s);
void launchRoundAfterCheck(RoundSys* ys, JobState* js, DevStatus* st, int K, cudaStream_t s);
void launchRoundAfterUpdate(RoundSys* ys, const JobState* js, const RoundParams& p, int K, cudaStream_t s);
void launchRoundTimeLevel(const RoundSys* ys, const LinJob* jobs, int K, int gx, cudaStream_t s);

}  // namespace gbfv
