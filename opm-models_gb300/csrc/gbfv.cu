// Host side of libgbfv: the C ABI declared in include/gbfv.h.
//
// Set-up (gbfv_create) does once what the reference does once per grid in
// FvBaseLinearizer::createMatrix_ (fvbaselinearizer.hh:418-452) and
// ParallelBaseBackend::prepare (parallelbasebackend.hh:182-210): it builds
// the sparsity pattern, orders cells wavefront-major (see
// gbfv_internal.cuh), precomputes per-face geometry and transmissibility
// factors, boundary fluid states and the ILU(0) level sets, and uploads
// everything.  The Newton loop (gbfv_newton_apply) follows
// NewtonMethod::apply (newtonmethod.hh:228-438); each iteration reads back
// two scalars (Newton error, solver status).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/gbfv.h"
#include "gbfv_internal.cuh"
#include "amg.cuh"
#include "gilu.cuh"
#include "vcfv.cuh"
#include "solver.cuh"

namespace gbfv {
std::atomic<int64_t> g_launches{0};
thread_local int t_captureLaunches = -1;
}

using namespace gbfv;

namespace {

thread_local std::string t_lastError;

void setError(const std::string& s) { t_lastError = s; }

// NVTX range over a scope: one per Newton phase (linearize, Newton error,
// solve, update) and per time step, so an attached profiler shows the
// phases of NewtonMethod::apply (newtonmethod.hh:239-262 times the same ones);
// without a tool attached the calls return at once
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

#define CK(call)                                                                        \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            setError(std::string(#call) + ": " + cudaGetErrorString(e_));              \
            return e_ == cudaErrorMemoryAllocation ? GBFV_ERR_OOM : GBFV_ERR_CUDA;      \
        }                                                                               \
    } while (0)

// Device arrays are planes of ldN rows (the row count rounded up to 64),
// indexed with 32-bit ints in the kernels; the most planes one array holds
// is the block-ELL values / Jacobian's MAX_SLOTS x 3 x 3 = 63
static_assert(MAX_SLOTS * 3 * 3 < 64, "plane count of the largest device array");
static_assert(GBFV_MAX_CELLS % 64 == 0 && 64LL * GBFV_MAX_CELLS <= std::numeric_limits<int>::max(),
              "GBFV_MAX_CELLS keeps every device index within 32 bits");

template <class T>
int devAlloc(T** p, size_t n)
{
    *p = nullptr;
    if (n == 0) n = 1;
    CK(cudaMalloc((void**)p, n * sizeof(T)));
    return GBFV_OK;
}

template <class T>
int upload(T** p, const std::vector<T>& v)
{
    int st = devAlloc(p, v.size());
    if (st) return st;
    if (!v.empty()) CK(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return GBFV_OK;
}

double harmonicMean(double x, double y)
{
    if (x * y <= 0) return 0.0;
    return (2 * x * y) / (x + y);
}

// solver-side structure shared by the grid context and the stand-alone
// linear solver: ELL columns, level sets, factor and Krylov storage
struct SolverData {
    int N = 0, b = 0, dim = 0, nslot = 0, ldN = 0;
    std::vector<int> levPtr;  // host copy
    int* col = nullptr;
    int* levPtrD = nullptr;
    double* FL64 = nullptr;
    double* FD64 = nullptr;
    float* A32 = nullptr;
    float* FL32 = nullptr;
    float* FD32 = nullptr;
    double* v64[6] = {};  // x r p v y z
    float* v32[7] = {};   // rhs x r p v y z
    double* xref = nullptr;
    double* rref = nullptr;
    double* partial = nullptr;
    unsigned* bar = nullptr;  // count, gen, abort
    int nblocks64 = 1, nblocks32 = 1;
    // solver launch configuration per precision ([0] FP64, [1] FP32):
    // SYNC_CLUSTER with a cluster of nblk blocks, or SYNC_GRID (cooperative)
    int mode[2] = {SYNC_CLUSTER, SYNC_CLUSTER};
    int nblk[2] = {1, 1};
    int tuned[2] = {0, 0};
    int maxGrid[2] = {1, 1};
    int maxCluster[2] = {1, 1};
    int maxHybrid[2] = {0, 0};  // blocks of a hybrid launch (whole resident clusters of HYBRID_CLUSTER)
    int maxHybridNarrow = 0;    // the same for the FP32 hybrid launch with SOLVER_THREADS-thread blocks
    double tuneMs[2][16] = {};
    int adjacentLevels = 0;  // every dependency is exactly one level away
    std::vector<int> colHost;   // [s*ldN + p] host copy of the ELL columns
    int* pushL = nullptr;       // push targets for the current (C, G, NT)
    int* pushU = nullptr;
    int* levVals = nullptr;     // values each block receives per level and sweep
    int pushKey[4] = {0, 0, 0, 0};
    int ownerMode = 0;          // rows of a level to blocks: warp round-robin (0) / contiguous (1)
    // spatial-tile sweeps (see buildTileTables)
    std::vector<int> tileKey;   // [p] tile of row p out of TILE_KEYS (empty: no tiles)
    int4* tInfo = nullptr;      // [r*numLev + l]: first row, row count, forward / backward halo slots
    int* tDepF = nullptr;       // [q*ldN + p] dependency code of row p, forward sweep
    int* tDepB = nullptr;       // backward sweep
    int* tPushF = nullptr;      // [t*ldN + p] consumers of row p in other tiles, forward sweep
    int* tPushB = nullptr;
    int tHalo = 0;              // halo slots per block (the most any block receives in one sweep)
    int tWidth = 0;             // the most rows a block computes in one level
    int tileKeyC = 0;           // cluster size the tables were built for
    unsigned long long* prof = nullptr;  // per-phase timers of the solve kernel (GBFV_PROFILE=1)
    // AMG preconditioner (GBFV_LINSOLVER_AMG): the hierarchy, built at the
    // first AMG solve; natural row of every internal row
    AmgData* amg = nullptr;
    std::vector<int> natural;
    // block ILU(0) of a general pattern (vertex-centred grids), or of a
    // narrow structured system (giluRoute: every level at most 32 rows, see
    // createImpl), else NULL
    GiluData* gilu = nullptr;
    bool giluRoute = false;
    // wide structured system (giluWide): the general kernel's tagged sweeps
    // (no barrier per wavefront level) are a candidate of the autotuner for
    // the precisions in giluCand and serve the solves of those in giluUse
    // (bit 1 FP64, bit 2 the FP32 inner solve of the mixed form)
    bool giluWide = false;
    int giluCand = 0, giluUse = 0;
    // max-norm residual reduction the last solve reached: the FP64 true
    // residual for the mixed form, BiCGStab's residual for the plain one
    double lastReduction = 0.0, lastResidual = 0.0;
    // cumulative statistics of the persistent solve kernel
    cudaEvent_t evA = nullptr, evB = nullptr;
    double statMs = 0, statBytes = 0;
    int64_t statLaunches = 0, statIters = 0, statFactor = 0;
};

int allocSolver(SolverData& S, int maxBlocksOverride = 0)
{
    const size_t ld = S.ldN, bb = (size_t)S.b * S.b;
    int st;
    if ((st = devAlloc(&S.FL64, S.dim * bb * ld))) return st;
    if ((st = devAlloc(&S.FD64, bb * ld))) return st;
    if ((st = devAlloc(&S.A32, S.nslot * bb * ld))) return st;
    if ((st = devAlloc(&S.FL32, S.dim * bb * ld))) return st;
    if ((st = devAlloc(&S.FD32, bb * ld))) return st;
    // Krylov vectors padded by 16 values: the tile sweeps' bulk copies round a
    // run of rows up to a 16-byte boundary
    for (auto& p : S.v64)
        if ((st = devAlloc(&p, (size_t)S.N * S.b + 16))) return st;
    for (auto& p : S.v32)
        if ((st = devAlloc(&p, (size_t)S.N * S.b + 16))) return st;
    if ((st = devAlloc(&S.xref, (size_t)S.N * S.b))) return st;
    if ((st = devAlloc(&S.rref, (size_t)S.N * S.b))) return st;
    (void)maxBlocksOverride;
    S.maxGrid[0] = maxSolverBlocks<double>(S.b);
    S.maxGrid[1] = maxSolverBlocks<float>(S.b);
    S.maxCluster[0] = std::min(16, maxClusterBlocks<double>(S.b));
    S.maxCluster[1] = std::min(16, maxClusterBlocks<float>(S.b));
    // The hybrid launch (a cooperative grid of clusters) is left out under a
    // profiler that injects itself into the process (Nsight Compute sets
    // NV_COMPUTE_PROFILER_PERFWORKS_DIR and NV_NSIGHT_INJECTION_TRANSPORT_TYPE
    // in the profiled process; other tools CUDA_INJECTION64_PATH): a
    // kernel-replay capture of it ended in a device fault, while the same runs
    // without the profiler pass.  GBFV_NO_HYBRID leaves it out as well.
    bool profiled = false;
    for (const char* v : {"CUDA_INJECTION64_PATH", "NV_COMPUTE_PROFILER_PERFWORKS_DIR",
                          "NV_NSIGHT_INJECTION_TRANSPORT_TYPE"}) {
        const char* e = getenv(v);
        if (e && *e) profiled = true;
    }
    const bool hybridOk = !getenv("GBFV_NO_HYBRID") && !profiled;
    S.maxHybrid[0] = hybridOk && S.maxCluster[0] >= HYBRID_CLUSTER ? maxHybridBlocks<double>(S.b) : 0;
    S.maxHybrid[1] = hybridOk && S.maxCluster[1] >= HYBRID_CLUSTER ? maxHybridBlocks<float>(S.b) : 0;
    S.maxHybridNarrow = S.maxHybrid[1] > 0 ? maxHybridBlocks<float>(S.b, true) : 0;
    // default before tuning: one block for small systems, else a cluster of 8
    for (int k = 0; k < 2; ++k) {
        S.mode[k] = SYNC_CLUSTER;
        S.nblk[k] = S.N <= 12288 ? 1 : std::min(8, S.maxCluster[k]);
    }
    // forced configuration, e.g. GBFV_SOLVER=cluster:16 or grid:152
    if (const char* f = getenv("GBFV_SOLVER")) {
        int n = 0;
        // ":tiles" selects the spatial-tile sweeps, e.g. GBFV_SOLVER=cluster:16:tiles
        const int tf = strstr(f, "tiles") ? SYNC_TILES : 0;
        if (sscanf(f, "cluster:%d", &n) == 1 && n > 0)
            for (int k = 0; k < 2; ++k) {
                S.mode[k] = SYNC_CLUSTER | tf;
                S.nblk[k] = std::min(n, S.maxCluster[k]);
                S.tuned[k] = 1;
            }
        else if (strncmp(f, "hybrid", 6) == 0) {
            // "hybrid:256": FP32 blocks of SOLVER_THREADS threads
            const bool nw = strstr(f, ":256") != nullptr;
            for (int k = 0; k < 2; ++k) {
                const int mx = k == 1 && nw ? S.maxHybridNarrow : S.maxHybrid[k];
                if (mx > HYBRID_CLUSTER) {
                    S.mode[k] = SYNC_HYBRID | tf | (k == 1 && nw ? SYNC_NARROW : 0);
                    S.nblk[k] = mx;
                    S.tuned[k] = 1;
                }
            }
        }
        else if (sscanf(f, "grid:%d", &n) == 1 && n > 0)
            for (int k = 0; k < 2; ++k) { S.mode[k] = SYNC_GRID; S.nblk[k] = std::min(n, S.maxGrid[k]); S.tuned[k] = 1; }
    }
    const int nbMax = std::max(std::max(S.maxGrid[0], S.maxGrid[1]), 16);
    if ((st = devAlloc(&S.partial, 4 * (size_t)nbMax))) return st;
    if ((st = devAlloc(&S.bar, 4))) return st;
    CK(cudaMemset(S.bar, 0, 4 * sizeof(unsigned)));
    CK(cudaEventCreate(&S.evA));
    CK(cudaEventCreate(&S.evB));
    if (getenv("GBFV_PROFILE")) {
        CK(cudaMalloc((void**)&S.prof, 16 * sizeof(unsigned long long)));
        CK(cudaMemset(S.prof, 0, 16 * sizeof(unsigned long long)));
    }
    return GBFV_OK;
}

// algorithmic bytes of one persistent solve launch (see gbfv.h)
double solveBytes(const SolverData& S, int iters, int factor, int s)
{
    const double N = S.N, b = S.b, d = S.dim, Sl = S.nslot, bb = b * b;
    double B = 5.0 * N * b * s;  // rhs read, x r v p initialised
    if (factor) B += N * (Sl * bb + (d + 1) * bb) * s + 4.0 * N * d;
    B += (double)iters * (N * (2 * Sl * bb + 4 * d * bb + 2 * bb) * s + 4.0 * N * (2 * Sl + 4 * d) + 30.0 * N * b * s);
    return B;
}

// a batched or served system solves in the batch kernel: no general ILU(0)
void dropWideGilu(SolverData& S)
{
    if (!S.giluWide) return;
    giluDestroy(S.gilu);
    S.gilu = nullptr;
    S.giluWide = false;
    S.giluCand = S.giluUse = 0;
}

void freeSolver(SolverData& S)
{
    amgDestroy(S.amg);
    S.amg = nullptr;
    giluDestroy(S.gilu);
    S.gilu = nullptr;
    cudaFree(S.col);
    cudaFree(S.levPtrD);
    cudaFree(S.tInfo);
    cudaFree(S.tDepF);
    cudaFree(S.tDepB);
    cudaFree(S.tPushF);
    cudaFree(S.tPushB);
    cudaFree(S.FL64);
    cudaFree(S.FD64);
    cudaFree(S.A32);
    cudaFree(S.FL32);
    cudaFree(S.FD32);
    for (auto p : S.v64) cudaFree(p);
    for (auto p : S.v32) cudaFree(p);
    cudaFree(S.xref);
    cudaFree(S.rref);
    cudaFree(S.partial);
    cudaFree(S.bar);
    if (S.prof) cudaFree(S.prof);
    cudaFree(S.pushL);
    cudaFree(S.pushU);
    cudaFree(S.levVals);
    if (S.evA) cudaEventDestroy(S.evA);
    if (S.evB) cudaEventDestroy(S.evB);
}



}  // namespace

namespace gbfv {
// error message for gbfv_last_error from other translation units
void setLastError(const std::string& s) { setError(s); }
// problem.cu: consistency of a problem description (host only)
int checkProblem(const gbfv_problem* P, int maxMaterials, int maxTable);
}  // namespace gbfv

// ===================================================================== ctx
struct gbfv_ctx {
    int N = 0, b = 0, dim = 0, model = 0, ldN = 0;
    gbfv_params prm;
    cudaStream_t stream = nullptr;
    std::vector<int> perm, iperm;  // natural -> internal, internal -> natural
    DevMesh mesh{};
    DevPhysics hphys{};
    DevPhysics* dphys = nullptr;
    // device state
    double *x = nullptr, *xOld = nullptr, *storageOld = nullptr, *residual = nullptr, *jval = nullptr;
    int *meaning = nullptr, *meaningOld = nullptr, *wasSwitched = nullptr;
    IqBuffers iq{};
    std::string solveLog;  // GBFV_SOLVE_LOG at creation: per-solve JSON lines appended here
    // finite-difference linearizer (allocated on first use): deflected
    // states and their intensive quantities; the reference pressure
    FdIq fd{};
    double* fdX[6] = {};
    double* refP = nullptr;
    double* dx = nullptr;
    SolverData S;
    DevStatus* st = nullptr;
    DevStatus* hst = nullptr;  // pinned
    // owned device arrays of the mesh
    std::vector<void*> owned;
    // vertex-centred grid: element geometry, incidence and scratch (else NULL)
    VcfvDev* vcfv = nullptr;
    int numElements = 0;
    // natural BCRS view
    std::vector<int> bcrsRowPtr, bcrsCol, bcrsSlot, bcrsRow;
    double dt = 1.0;
    int newtonIter = 0;
    int numIterations = 0;
    double error = 0, lastError = 0;
    int haveDx = 0;
    cudaEvent_t ev[6];
    double phaseMs[4] = {0, 0, 0, 0};
    int lastIterations = 0, lastRefinements = 0;
    // snapshot
    double* xSave = nullptr;
    int* meaningSave = nullptr;
    int* switchedSave = nullptr;
    // linearization statistics
    cudaEvent_t evL0 = nullptr, evL1 = nullptr;
    int linPending = 0;
    double linMs = 0, linBytes = 0, linBytesPer = 0;
    int64_t linLaunches = 0;
};

struct gbfv_linsolver {
    int N = 0, b = 0;
    gbfv_params prm;
    cudaStream_t stream = nullptr;
    SolverData S;
    std::vector<int> perm, iperm;
    std::vector<int> rowPtr, colN;
    std::vector<int> entSlot, entRow;  // BCRS entry -> (slot, internal row)
    double* A64 = nullptr;
    double* A64host = nullptr;  // pinned staging
    double* rhs = nullptr;
    DevStatus* st = nullptr;
    DevStatus* hst = nullptr;
    double* stage = nullptr;    // pinned vector staging
};

namespace {

int syncStatus(cudaStream_t s, DevStatus* d, DevStatus* h)
{
    CK(cudaMemcpyAsync(h, d, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return GBFV_OK;
}

int resetStatus(cudaStream_t s, DevStatus* d)
{
    CK(cudaMemsetAsync(d, 0, sizeof(DevStatus), s));
    return GBFV_OK;
}

// levels and wavefront-major order from a lower-triangular dependency walk;
// inside a level, rows are ordered by key (when given), then naturally
void buildOrder(int N, const std::vector<std::vector<int>>& lower, std::vector<int>& perm,
                std::vector<int>& iperm, std::vector<int>& levPtr, const std::vector<int>* key = nullptr)
{
    std::vector<int> level(N, 0);
    int maxLev = 0;
    for (int i = 0; i < N; ++i) {
        int l = 0;
        for (int k : lower[i]) l = std::max(l, level[k] + 1);
        level[i] = l;
        maxLev = std::max(maxLev, l);
    }
    std::vector<int> cnt(maxLev + 2, 0);
    for (int i = 0; i < N; ++i) cnt[level[i] + 1]++;
    for (int l = 0; l <= maxLev; ++l) cnt[l + 1] += cnt[l];
    levPtr.assign(cnt.begin(), cnt.end());
    iperm.assign(N, 0);
    perm.assign(N, 0);
    std::vector<int> pos(cnt.begin(), cnt.end() - 1);
    if (key) {
        std::vector<int> idx(N);
        for (int i = 0; i < N; ++i) idx[i] = i;
        std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) {
            return level[x] != level[y] ? level[x] < level[y] : (*key)[x] < (*key)[y];
        });
        for (int p = 0; p < N; ++p) {
            iperm[p] = idx[p];
            perm[idx[p]] = p;
        }
        return;
    }
    for (int i = 0; i < N; ++i) {  // natural order inside a level
        const int p = pos[level[i]]++;
        iperm[p] = i;
        perm[i] = p;
    }
}

// Spatial tiles of the cluster sweeps: TILE_KEYS = 16 tiles, 4 x 4 over the
// two axes with the most cells, each cell's index along an axis counted from
// the lower boundary (natural order: the lower neighbour comes first).  For
// a cluster of C blocks (C dividing 16) block key / (16 / C) owns the cell,
// so rows ordered by key inside a level are contiguous per block.
std::vector<int> tileKeys(int N, int dim, int ndir, const std::vector<int>& nbrDir)
{
    std::vector<int> key(N, 0);
    if (dim < 2) return key;
    std::vector<int> idx((size_t)N * dim, 0);
    int ext[3] = {1, 1, 1};
    for (int I = 0; I < N; ++I)
        for (int a = 0; a < dim; ++a) {
            const int K = nbrDir[(size_t)I * ndir + 2 * a];
            idx[(size_t)I * dim + a] = K >= 0 ? idx[(size_t)K * dim + a] + 1 : 0;
            ext[a] = std::max(ext[a], idx[(size_t)I * dim + a] + 1);
        }
    int ax0 = 0, ax1 = 1;  // the two longest axes, ax0 >= ax1
    if (dim == 3) {
        int o[3] = {0, 1, 2};
        std::sort(o, o + 3, [&](int x, int y) { return ext[x] != ext[y] ? ext[x] > ext[y] : x < y; });
        ax0 = o[0];
        ax1 = o[1];
    }
    for (int I = 0; I < N; ++I) {
        const int t0 = (int)((long)idx[(size_t)I * dim + ax0] * 4 / ext[ax0]);
        const int t1 = (int)((long)idx[(size_t)I * dim + ax1] * 4 / ext[ax1]);
        key[I] = t0 * 4 + t1;
    }
    return key;
}

// Block and thread slot (within the level group) that own position t of a
// level of width W: warps dealt round-robin (mode 0) or contiguous shares
// rounded to whole warps (mode 1); the device side is SweepMap::pos.
inline void levelSlot(int t, int W, int C, int mode, int& owner, int& uu)
{
    if (mode == 0) {
        const int w = t >> 5;
        owner = w % C;
        uu = ((w / C) << 5) | (t & 31);
        return;
    }
    const int chunk = (((W + C - 1) / C) + 31) & ~31;
    owner = t / chunk;
    uu = t - owner * chunk;
}
// the most rows one block takes in a level of width W
inline int levelChunk(int W, int C, int mode)
{
    return mode == 0 ? 32 * ((W + 32 * C - 1) / (32 * C)) : (((W + C - 1) / C) + 31) & ~31;
}

// Which levels of a sweep need the cluster-wide level barrier.  A block
// pushes the results of level l into the consumer block's dependency buffer
// (l+1) mod PUSH_BUFFERS, which the consumer last read at level
// l+1-PUSH_BUFFERS; the push is safe once the consumer has finished that
// level.  Blocks finish their levels in order (a block-local barrier per
// level); a row starts after its block finished the previous level and after
// its dependencies were computed.  know[Y] = the latest level that block Y is
// known to have finished when a row starts, propagated along those two
// orderings and along the cluster barriers placed so far.  Where a push is
// not covered, a cluster barrier is placed after the previous level.
// barrierAfter[l] (level index, in the sweep's own order) is the result.
// The pattern: N rows in level order, levPtr, columns colHost[s*ld + p]
// (lower slots 0..dim-1, diagonal dim, upper dim+1..2dim, -1 for none);
// D dependency buffers per block.
void placeLevelBarriersCore(int N, int ld, int dim, const std::vector<int>& levPtr, const std::vector<int>& colHost,
                            int C, int mode, int D, const std::vector<int>& lev, bool forward,
                            std::vector<char>& barrierAfter)
{
    const int nl = (int)levPtr.size() - 1;
    barrierAfter.assign(nl, 0);
    auto owner = [&](int p) {
        int o, uu;
        const int l = lev[p];
        levelSlot(p - levPtr[l], levPtr[l + 1] - levPtr[l], C, mode, o, uu);
        return o;
    };
    std::vector<int> K((size_t)C * C, -1), Knew;   // K[X*C + Y]: known finished step of Y when X finished its last
    std::vector<int> know((size_t)N * C, -1);
    std::vector<int> acc(C);
    for (int step = 0; step < nl; ++step) {
        const int l = forward ? step : nl - 1 - step;
        auto attempt = [&]() -> bool {
            Knew = K;
            for (int X = 0; X < C; ++X) Knew[(size_t)X * C + X] = step;
            for (int p = levPtr[l]; p < levPtr[l + 1]; ++p) {
                const int X = owner(p);
                for (int Y = 0; Y < C; ++Y) acc[Y] = K[(size_t)X * C + Y];
                for (int q = 0; q < dim; ++q) {
                    const int sl = forward ? q : 2 * dim - q;   // dependencies of p in this sweep
                    const int j = colHost[(size_t)sl * ld + p];
                    if (j < 0) continue;
                    const int* kj = &know[(size_t)j * C];
                    for (int Y = 0; Y < C; ++Y) acc[Y] = std::max(acc[Y], kj[Y]);
                }
                for (int q = 0; q < dim; ++q) {
                    const int sl = forward ? dim + 1 + q : q;   // consumers of p
                    const int u = colHost[(size_t)sl * ld + p];
                    if (u >= 0 && acc[owner(u)] < step + 1 - D) return false;
                }
                std::copy(acc.begin(), acc.end(), &know[(size_t)p * C]);
                int* kx = &Knew[(size_t)X * C];
                for (int Y = 0; Y < C; ++Y) kx[Y] = std::max(kx[Y], acc[Y]);
                kx[X] = step;
            }
            return true;
        };
        if (!attempt()) {
            // a cluster barrier after the previous step: every block knows every
            // block finished it (then every push is covered, D >= 2)
            barrierAfter[forward ? l - 1 : l + 1] = 1;
            for (int& v : K) v = std::max(v, step - 1);
            attempt();
        }
        K.swap(Knew);
    }
}

void placeLevelBarriers(const SolverData& S, int C, int mode, const std::vector<int>& lev, bool forward,
                        std::vector<char>& barrierAfter)
{
    placeLevelBarriersCore(S.N, S.ldN, S.dim, S.levPtr, S.colHost, C, mode, PUSH_BUFFERS, lev, forward,
                           barrierAfter);
}

// Push targets of the cluster sweeps for cluster size C, G level groups and
// NT threads per block: for each row and each neighbour in the dependency
// direction, the consumer's block and the offset of its slot (see
// SweepMap in solver.cu).
int buildPushTargets(SolverData& S, int C, int G, int NT, int mode)
{
    if (S.pushKey[0] == C && S.pushKey[1] == G && S.pushKey[2] == NT && S.pushKey[3] == mode && S.pushL)
        return GBFV_OK;
    const int N = S.N, ld = S.ldN, dim = S.dim, B = S.b, NG = NT / G;
    const int PB = padB(B);  // values per dependency slot
    std::vector<int> lev(N);
    for (size_t l = 0; l + 1 < S.levPtr.size(); ++l)
        for (int p = S.levPtr[l]; p < S.levPtr[l + 1]; ++p) lev[p] = (int)l;
    auto target = [&](int j, int slot) {
        const int l = lev[j];
        int owner, uu;
        levelSlot(j - S.levPtr[l], S.levPtr[l + 1] - S.levPtr[l], C, mode, owner, uu);
        const int cslot = (l % G) * NG + uu;
        return (owner << 24) | ((cslot * 3 + slot) * PB);
    };
    const int nl = (int)S.levPtr.size() - 1;
    std::vector<int> hL((size_t)3 * ld, -1), hU((size_t)3 * ld, -1), hV((size_t)C * nl * 2, 0);
    auto ownerOf = [&](int p) {
        int o, uu;
        const int l = lev[p];
        levelSlot(p - S.levPtr[l], S.levPtr[l + 1] - S.levPtr[l], C, mode, o, uu);
        return o;
    };
    for (int p = 0; p < N; ++p) {
        const int owner = ownerOf(p);
        for (int q = 0; q < dim; ++q) {
            const int ju = S.colHost[(size_t)(dim + 1 + q) * ld + p];  // upper neighbour +q
            if (ju >= 0) {
                hL[(size_t)q * ld + p] = target(ju, dim - 1 - q);
                hV[((size_t)owner * nl + lev[p]) * 2 + 1] += PB;  // p receives ju in the backward sweep
            }
            const int jl = S.colHost[(size_t)q * ld + p];  // lower neighbour in slot q
            if (jl >= 0) {
                hU[(size_t)q * ld + p] = target(jl, q);
                hV[((size_t)owner * nl + lev[p]) * 2] += PB;  // p receives jl in the forward sweep
            }
        }
    }
    if (!getenv("GBFV_LEVEL_BARRIER")) {
        std::vector<char> barF, barB;
        placeLevelBarriers(S, C, mode, lev, true, barF);
        placeLevelBarriers(S, C, mode, lev, false, barB);
        for (int r = 0; r < C; ++r)
            for (int l = 0; l < nl; ++l) {
                if (barF[l]) hV[((size_t)r * nl + l) * 2] |= PUSH_BARRIER_FLAG;
                if (barB[l]) hV[((size_t)r * nl + l) * 2 + 1] |= PUSH_BARRIER_FLAG;
            }
    }
    else
        for (int& v : hV) v |= PUSH_BARRIER_FLAG;
    cudaFree(S.pushL);
    cudaFree(S.pushU);
    cudaFree(S.levVals);
    S.pushL = S.pushU = S.levVals = nullptr;
    int st;
    if ((st = upload(&S.pushL, hL)) || (st = upload(&S.pushU, hU)) || (st = upload(&S.levVals, hV))) return st;
    S.pushKey[0] = C;
    S.pushKey[1] = G;
    S.pushKey[2] = NT;
    S.pushKey[3] = mode;
    return GBFV_OK;
}

// Tables of the spatial-tile sweeps for a cluster of C blocks of NT threads.
// Block r owns the rows whose tile key / (TILE_KEYS / C) is r; inside a
// level they are contiguous (the order is by key), so block r computes rows
// first..first+count-1 of level l, one per thread (tileFits: at most NT).  A dependency on a row of
// the same block is read from the block's copy of the previous level (by
// its position there); one on another block's row arrives by a push into a
// halo slot, numbered per block and sweep, so no slot is written twice in a
// sweep and no flow control is needed.  Unsupported (no tiles, too many
// levels or halo slots): GBFV_ERR_UNSUPPORTED.
int buildTileTables(SolverData& S, int C)
{
    if (S.tileKeyC == C && S.tInfo) return GBFV_OK;
    const int N = S.N, ld = S.ldN, dim = S.dim, nl = (int)S.levPtr.size() - 1;
    if (S.tileKey.empty() || C < 2 || TILE_KEYS % C || !S.adjacentLevels || nl > TILE_MAX_LEVELS || dim > 3)
        return GBFV_ERR_UNSUPPORTED;
    const int per = TILE_KEYS / C;
    std::vector<int> lev(N), own(N), pos(N);
    for (int l = 0; l < nl; ++l)
        for (int p = S.levPtr[l]; p < S.levPtr[l + 1]; ++p) {
            lev[p] = l;
            own[p] = S.tileKey[p] / per;
        }
    std::vector<int4> info((size_t)C * nl, make_int4(0, 0, 0, 0));
    for (int l = 0; l < nl; ++l) {
        int prev = -1;
        for (int p = S.levPtr[l]; p < S.levPtr[l + 1]; ++p) {
            const int r = own[p];
            if (r < prev) return GBFV_ERR_UNSUPPORTED;  // not contiguous per block
            int4& f = info[(size_t)r * nl + l];
            if (r != prev) f.x = p;
            pos[p] = p - f.x;
            f.y++;
            prev = r;
        }
    }
    std::vector<int> depF((size_t)3 * ld, -1), depB((size_t)3 * ld, -1), pushF((size_t)3 * ld, -1),
        pushB((size_t)3 * ld, -1);
    std::vector<int> hF(C, 0), hB(C, 0);
    auto addPush = [&](std::vector<int>& push, int producer, int target) {
        for (int t = 0; t < 3; ++t)
            if (push[(size_t)t * ld + producer] < 0) {
                push[(size_t)t * ld + producer] = target;
                return true;
            }
        return false;
    };
    // forward sweep in level order, backward sweep in reverse level order, so
    // a block's halo slots are numbered in the order it uses them
    for (int p = 0; p < N; ++p) {
        const int r = own[p];
        for (int q = 0; q < dim; ++q) {
            const int j = S.colHost[(size_t)q * ld + p];  // lower neighbour in slot q
            if (j < 0) continue;
            if (own[j] == r) depF[(size_t)q * ld + p] = pos[j];
            else {
                const int h = hF[r]++;
                depF[(size_t)q * ld + p] = TILE_HALO | h;
                if (!addPush(pushF, j, (r << 24) | h)) return GBFV_ERR_UNSUPPORTED;
                info[(size_t)r * nl + lev[p]].z++;
            }
        }
    }
    for (int p = N - 1; p >= 0; --p) {
        const int r = own[p];
        for (int q = 0; q < dim; ++q) {
            const int j = S.colHost[(size_t)(2 * dim - q) * ld + p];  // upper neighbours, descending columns
            if (j < 0) continue;
            if (own[j] == r) depB[(size_t)q * ld + p] = pos[j];
            else {
                const int h = hB[r]++;
                depB[(size_t)q * ld + p] = TILE_HALO | h;
                if (!addPush(pushB, j, (r << 24) | h)) return GBFV_ERR_UNSUPPORTED;
                info[(size_t)r * nl + lev[p]].w++;
            }
        }
    }
    int halo = 1, wmax = 0;
    for (int r = 0; r < C; ++r) halo = std::max(halo, std::max(hF[r], hB[r]));
    for (const int4& f : info) wmax = std::max(wmax, f.y);
    if (halo > TILE_MASK) return GBFV_ERR_UNSUPPORTED;
    cudaFree(S.tInfo);
    cudaFree(S.tDepF);
    cudaFree(S.tDepB);
    cudaFree(S.tPushF);
    cudaFree(S.tPushB);
    S.tInfo = nullptr;
    S.tDepF = S.tDepB = S.tPushF = S.tPushB = nullptr;
    S.tileKeyC = 0;
    int st;
    if ((st = upload(&S.tInfo, info)) || (st = upload(&S.tDepF, depF)) || (st = upload(&S.tDepB, depB)) ||
        (st = upload(&S.tPushF, pushF)) || (st = upload(&S.tPushB, pushB)))
        return st;
    S.tHalo = halo;
    S.tWidth = wmax;
    S.tileKeyC = C;
    return GBFV_OK;
}

// the tile sweeps of precision T fit: one row per thread, shared memory
template <class T>
bool tileFits(const SolverData& S, int NT)
{
    const int nl = (int)S.levPtr.size() - 1;
    return S.tWidth <= NT && tileSmemBytes<T>(S.b, nl, S.tHalo, S.tWidth, S.dim) <= solverSmemLimit<T>(S.b);
}

// 1 if every lower dependency of a row sits exactly one level below it
int adjacentLevels(const std::vector<std::vector<int>>& lower, const std::vector<int>& perm,
                   const std::vector<int>& levPtr)
{
    const int N = (int)perm.size();
    std::vector<int> lev(N);
    for (size_t l = 0; l + 1 < levPtr.size(); ++l)
        for (int p = levPtr[l]; p < levPtr[l + 1]; ++p) lev[p] = (int)l;
    for (int i = 0; i < N; ++i)
        for (int k : lower[i])
            if (lev[perm[k]] != lev[perm[i]] - 1) return 0;
    return 1;
}

// kernel arguments of one solve of S in launch configuration (mode, nblocks)
template <class T>
int fillKArgs(SolverData& S, DevStatus* st, const T* A, T* FL, T* FD, const T* rhs, T* const* vec, int factor,
              double redTol, double absTol, double maxRes, int maxIter, int mode, int nblocks, KArgs<T>& a)
{
    const bool tiles = (mode & SYNC_TILES) != 0;
    const bool narrow = (mode & SYNC_NARROW) != 0;
    mode &= ~(SYNC_TILES | SYNC_NARROW);
    if (narrow && (mode != SYNC_HYBRID || tiles)) return GBFV_ERR_UNSUPPORTED;
    a.N = S.N;
    a.ldN = S.ldN;
    a.dim = S.dim;
    a.nslot = S.nslot;
    a.numLev = (int)S.levPtr.size() - 1;
    a.col = S.col;
    a.levPtr = S.levPtrD;
    a.A = A;
    a.FL = FL;
    a.FD = FD;
    a.rhs = rhs;
    a.x = vec[0];
    a.r = vec[1];
    a.p = vec[2];
    a.v = vec[3];
    a.y = vec[4];
    a.z = vec[5];
    a.partial = S.partial;
    a.gs.count = S.bar;
    a.gs.gen = S.bar + 1;
    a.gs.abort = (int*)(S.bar + 2);
    a.gs.perCluster = mode == SYNC_HYBRID ? HYBRID_CLUSTER : 0;
    a.st = st;
    a.redTol = redTol;
    a.absTol = absTol;
    a.maxRes = maxRes;
    a.maxIter = maxIter;
    a.factor = factor;
    a.prof = S.prof;
    {
        int omode = S.ownerMode;
        if (const char* e = getenv("GBFV_OWNER")) omode = strcmp(e, "contig") == 0 ? 1 : 0;
        a.ownerMode = omode;
        int maxChunk = 0;  // the most rows one block takes in a level
        // the cluster that sweeps: the whole launch, or the first cluster of a hybrid one
        const int C = mode == SYNC_HYBRID ? HYBRID_CLUSTER : nblocks;
        a.hybrid = mode == SYNC_HYBRID ? HYBRID_CLUSTER : 0;
        for (size_t l = 0; l + 1 < S.levPtr.size(); ++l)
            maxChunk = std::max(maxChunk, levelChunk(S.levPtr[l + 1] - S.levPtr[l], C, omode));
        // threads per block of the sweeping cluster
        const int NTC = narrow ? SOLVER_THREADS : clusterThreads<T>();
        a.tile = 0;
        a.tinfo = nullptr;
        a.tdepF = a.tdepB = a.tpushF = a.tpushB = nullptr;
        a.thalo = 0;
        a.twidth = 0;
        if (tiles) {
            if (mode != SYNC_CLUSTER && mode != SYNC_HYBRID) return GBFV_ERR_UNSUPPORTED;
            const int ts = buildTileTables(S, C);
            if (ts) return ts;
            if (!tileFits<T>(S, NTC)) return GBFV_ERR_UNSUPPORTED;
            a.tile = 1;
            a.dsmem = 0;
            a.grp = 1;
            a.pushL = a.pushU = a.levVals = nullptr;
            a.cluster = C;
            a.tinfo = S.tInfo;
            a.tdepF = S.tDepF;
            a.tdepB = S.tDepB;
            a.tpushF = S.tPushF;
            a.tpushB = S.tPushB;
            a.thalo = S.tHalo;
            a.twidth = S.tWidth;
            return GBFV_OK;
        }
        a.dsmem = ((mode == SYNC_CLUSTER || mode == SYNC_HYBRID) && S.adjacentLevels && maxChunk <= NTC &&
                   (int)S.levPtr.size() - 1 <= MAX_PUSH_LEVELS && !getenv("GBFV_NO_DSMEM")) ? 1 : 0;
        if (mode == SYNC_HYBRID && !a.dsmem) return GBFV_ERR_UNSUPPORTED;  // the hybrid sweeps need the push tables
        // two level groups where they fit (each group must cover a block's share
        // of the widest level): staging one level ahead hides the operand loads;
        // more groups were measured slower (hybrid solve of the 100x100x20
        // black-oil grid: 2 groups 135.4 ms, 4 groups 137.7 ms, 1 group 175.7 ms)
        a.grp = maxChunk <= NTC / 2 ? 2 : 1;
        if (const char* e = getenv("GBFV_GROUPS")) a.grp = std::max(1, std::min(a.grp, atoi(e)));
        a.pushL = a.pushU = a.levVals = nullptr;
        a.cluster = a.dsmem ? C : 0;
        if (a.dsmem) {
            const int ps = buildPushTargets(S, C, a.grp, NTC, omode);
            if (ps) return ps;
            a.pushL = S.pushL;
            a.pushU = S.pushU;
            a.levVals = S.levVals;
        }
    }
    return GBFV_OK;
}

// solver-precision iteration; returns status and fills iterations
template <class T>
int runKrylovCfg(SolverData& S, cudaStream_t stream, DevStatus* st, DevStatus* hst, const T* A, T* FL, T* FD,
                 const T* rhs, T* const* vec, int factor, double redTol, double absTol, double maxRes,
                 int maxIter, int mode, int nblocks, int& iters, float* msOut, bool stats)
{
    KArgs<T> a;
    int rs = fillKArgs<T>(S, st, A, FL, FD, rhs, vec, factor, redTol, absTol, maxRes, maxIter, mode, nblocks, a);
    if (rs) return rs;
    if ((rs = resetStatus(stream, st))) return rs;
    CK(cudaMemsetAsync(S.bar, 0, 4 * sizeof(unsigned), stream));
    cudaEventRecord(S.evA, stream);
    const int ls = launchBicgstab<T>(a, S.b, mode & ~SYNC_TILES, nblocks, stream);
    if (ls != GBFV_OK) {
        setError(std::string("cooperative launch failed: ") + cudaGetErrorString(cudaGetLastError()));
        return ls;
    }
    cudaEventRecord(S.evB, stream);
    if ((rs = syncStatus(stream, st, hst))) return rs;
    iters = hst->iterations;
    {
        float ms = 0;
        cudaEventElapsedTime(&ms, S.evA, S.evB);
        if (msOut) *msOut = ms;
        if (stats) {
            S.statMs += ms;
            S.statLaunches++;
            S.statIters += iters;
            S.statFactor += factor;
            S.statBytes += solveBytes(S, iters, factor, (int)sizeof(T));
        }
    }
    if (hst->code) return hst->code;
    return hst->converged ? GBFV_OK : GBFV_ERR_NOT_CONVERGED;
}

// Autotuner: time a factorization + 12 iterations of every candidate launch
// configuration on the system at hand and keep the fastest.
template <class T>
void tuneSolver(SolverData& S, cudaStream_t stream, DevStatus* st, DevStatus* hst, const T* A, T* FL, T* FD,
                const T* rhs, T* const* vec)
{
    const int k = sizeof(T) == 4 ? 1 : 0;
    if (S.tuned[k]) return;
    S.tuned[k] = 1;
    struct Cand { int mode, nb; };
    std::vector<Cand> cands;
    for (int c = 1; c <= S.maxCluster[k]; c *= 2) cands.push_back({SYNC_CLUSTER, c});
    int dev = 0, nsm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (S.N > 4 * 4096) {
        cands.push_back({SYNC_GRID, std::min(nsm, S.maxGrid[k])});
        cands.push_back({SYNC_GRID, std::min(2 * nsm, S.maxGrid[k])});
        if (S.maxHybrid[k] > HYBRID_CLUSTER) cands.push_back({SYNC_HYBRID, S.maxHybrid[k]});
        if (k == 1 && S.maxHybridNarrow > HYBRID_CLUSTER) cands.push_back({SYNC_HYBRID | SYNC_NARROW, S.maxHybridNarrow});
    }
    // The spatial-tile sweeps are not a candidate: on the black-oil workloads
    // they were slower than the push sweeps (a level's rows of one tile sit on
    // one SM), so they only run when asked for (GBFV_SOLVER=...:tiles,
    // gbfv_set_solver_config with GBFV_SOLVER_TILES).
    double best = 1e300;
    Cand pick = {S.mode[k], S.nblk[k]};
    int idx = 0;
    for (const Cand& c : cands) {
        int it = 0;
        float ms = 0;
        const int rs = runKrylovCfg<T>(S, stream, st, hst, A, FL, FD, rhs, vec, 1, 0.0, 0.0, 1e300, 12, c.mode,
                                       c.nb, it, &ms, false);
        if (rs != GBFV_OK && rs != GBFV_ERR_NOT_CONVERGED) {
            cudaGetLastError();
            continue;
        }
        if (idx < 16) S.tuneMs[k][idx++] = ms;
        if (ms < best) { best = ms; pick = c; }
    }
    S.mode[k] = pick.mode;
    S.nblk[k] = pick.nb;
    // the general kernel's tagged sweeps, timed the same way (last entry of
    // the timings); kept for this precision when they are the fastest
    const int bit = k ? 2 : 1;
    if (S.giluWide && (S.giluCand & bit)) {
        int it = 0;
        float ms = 0;
        const int rs = giluSolve<T>(S.gilu, A, rhs, vec[0], 1, 0.0, 0.0, 1e300, 12, stream, st, hst, it, &ms, nullptr);
        if (rs != GBFV_OK && rs != GBFV_ERR_NOT_CONVERGED) {
            cudaGetLastError();
            ms = 1e30f;
        }
        else if (idx < 16)
            S.tuneMs[k][idx++] = ms;
        if (ms < best) S.giluUse |= bit;
        else S.giluUse &= ~bit;
    }
}

template <class T>
int runGilu(SolverData& S, cudaStream_t stream, DevStatus* st, DevStatus* hst, const T* A, const T* rhs, T* x,
            int factor, double redTol, double absTol, double maxRes, int maxIter, int& iters);

template <class T>
int runKrylov(SolverData& S, cudaStream_t stream, DevStatus* st, DevStatus* hst, const T* A, T* FL, T* FD,
              const T* rhs, T* const* vec, int factor, double redTol, double absTol, double maxRes,
              int maxIter, int& iters)
{
    const int k = sizeof(T) == 4 ? 1 : 0;
    if (!S.tuned[k]) tuneSolver<T>(S, stream, st, hst, A, FL, FD, rhs, vec);
    if (S.giluWide && (S.giluUse & (k ? 2 : 1)))
        return runGilu<T>(S, stream, st, hst, A, rhs, vec[0], factor, redTol, absTol, maxRes, maxIter, iters);
    return runKrylovCfg<T>(S, stream, st, hst, A, FL, FD, rhs, vec, factor, redTol, absTol, maxRes, maxIter,
                           S.mode[k], S.nblk[k], iters, nullptr, true);
}

double absTolOf(const gbfv_params& p)
{
    return p.linear_abs_tolerance < 0 ? p.newton_tolerance / 100.0 : p.linear_abs_tolerance;
}

// the AMG hierarchy of S, built from the FP64 matrix A at its first AMG solve
int ensureAmg(SolverData& S, cudaStream_t stream, const double* A, const gbfv_params& prm)
{
    if (S.amg) return GBFV_OK;
    if ((int)S.natural.size() != S.N) {
        setError("AMG: the solver has no natural row order");
        return GBFV_ERR_UNSUPPORTED;
    }
    AmgSystem sys;
    sys.N = S.N;
    sys.b = S.b;
    sys.nslot = S.nslot;
    sys.ld = S.ldN;
    sys.colHost = S.colHost.data();
    sys.natural = S.natural.data();
    int st = GBFV_OK;
    S.amg = amgCreate(sys, A, prm.amg_coarsen_target, stream, &st);
    return S.amg ? GBFV_OK : (st ? st : GBFV_ERR_CUDA);
}

// BiCGStab + AMG V-cycle in precision T: statistics as the ILU(0) solves
template <class T>
int runAmg(SolverData& S, cudaStream_t stream, DevStatus* st, DevStatus* hst, const T* A, const T* rhs, T* x,
           double redTol, double absTol, double maxRes, int maxIter, int& iters)
{
    float ms = 0;
    double bytes = 0;
    const int rs = amgSolve<T>(S.amg, A, rhs, x, redTol, absTol, maxRes, maxIter, stream, st, hst, iters, &ms, &bytes);
    S.statMs += ms;
    S.statLaunches++;
    S.statIters += iters;
    S.statBytes += bytes;
    return rs;
}

// BiCGStab + general block ILU(0) in precision T: statistics as above
template <class T>
int runGilu(SolverData& S, cudaStream_t stream, DevStatus* st, DevStatus* hst, const T* A, const T* rhs, T* x,
            int factor, double redTol, double absTol, double maxRes, int maxIter, int& iters)
{
    float ms = 0;
    double bytes = 0;
    const int rs = giluSolve<T>(S.gilu, A, rhs, x, factor, redTol, absTol, maxRes, maxIter, stream, st, hst, iters,
                                &ms, &bytes);
    S.statMs += ms;
    S.statLaunches++;
    S.statIters += iters;
    S.statBytes += bytes;
    if (factor) S.statFactor++;
    return rs;
}

// FP64 BiCGStab + ILU0 or AMG (plain form): solves A x = rhs into S.v64[0]
int solvePlain(SolverData& S, cudaStream_t stream, DevStatus* st, DevStatus* hst, const double* A,
               const double* rhs, const gbfv_params& prm, int& iters)
{
    int rs;
    if (prm.linear_solver == GBFV_LINSOLVER_AMG) {
        if ((rs = ensureAmg(S, stream, A, prm))) return rs;
        rs = runAmg<double>(S, stream, st, hst, A, rhs, S.v64[0], prm.linear_tolerance, absTolOf(prm),
                            prm.linear_max_error, prm.linear_max_iterations, iters);
    }
    else if (S.gilu && !S.giluWide)
        rs = runGilu<double>(S, stream, st, hst, A, rhs, S.v64[0], 1, prm.linear_tolerance, absTolOf(prm),
                             prm.linear_max_error, prm.linear_max_iterations, iters);
    else
        rs = runKrylov<double>(S, stream, st, hst, A, S.FL64, S.FD64, rhs, S.v64, 1, prm.linear_tolerance,
                               absTolOf(prm), prm.linear_max_error, prm.linear_max_iterations, iters);
    S.lastReduction = hst->resid0 > 0 ? hst->resid / hst->resid0 : 0.0;
    S.lastResidual = hst->resid;
    return rs;
}

// FP32 BiCGStab + FP32 ILU0 under FP64 iterative refinement (mixed form):
// solution in S.xref (FP64)
int solveMixed(SolverData& S, cudaStream_t stream, DevStatus* st, DevStatus* hst, const double* A,
               const double* rhs, const gbfv_params& prm, int& iters, int& refinements)
{
    const long nval = (long)S.nslot * S.b * S.b * S.ldN;
    launchCastMatrix(A, S.A32, nval, stream);
    const int n = S.N * S.b;
    CK(cudaMemsetAsync(S.xref, 0, sizeof(double) * n, stream));
    // r = b - A*0 = b, its max-norm and FP32 copy
    int rs;
    if ((rs = resetStatus(stream, st))) return rs;
    launchResidual64(S.N, S.ldN, S.nslot, S.b, S.col, A, rhs, S.xref, S.rref, S.v32[0], st, stream);
    if ((rs = syncStatus(stream, st, hst))) return rs;
    const double eps = std::numeric_limits<double>::min() * 1e10;
    double resErr;
    {
        unsigned long long bits = hst->errorBits;
        std::memcpy(&resErr, &bits, sizeof(double));
    }
    resErr = std::max(resErr, eps);
    const double resErr0 = resErr;
    const double absTol = absTolOf(prm);
    auto converged = [&](double re) {
        return re / std::max(1e-20, resErr0) <= prm.linear_tolerance || re <= absTol;
    };
    iters = 0;
    refinements = 0;
    S.lastReduction = 1.0;
    S.lastResidual = resErr;
    if (converged(resErr)) return GBFV_OK;
    const bool amg = prm.linear_solver == GBFV_LINSOLVER_AMG;
    if (amg && (rs = ensureAmg(S, stream, A, prm))) return rs;
    for (int ref = 0; ref < std::max(1, prm.max_refinements); ++ref) {
        const double target = std::max(prm.linear_tolerance * resErr0, absTol);
        const double need = target / resErr;
        const double innerTol = std::min(0.5, std::max(0.5 * need, prm.inner_tolerance));
        int it = 0;
        float* vec[6] = {S.v32[1], S.v32[2], S.v32[3], S.v32[4], S.v32[5], S.v32[6]};
        const int ks = amg ? runAmg<float>(S, stream, st, hst, S.A32, S.v32[0], S.v32[1], innerTol, 0.0,
                                           prm.linear_max_error, prm.linear_max_iterations, it)
                       : S.gilu && !S.giluWide
                           ? runGilu<float>(S, stream, st, hst, S.A32, S.v32[0], S.v32[1], ref == 0, innerTol, 0.0,
                                                 prm.linear_max_error, prm.linear_max_iterations, it)
                           : runKrylov<float>(S, stream, st, hst, S.A32, S.FL32, S.FD32, S.v32[0], vec, ref == 0,
                                              innerTol, 0.0, prm.linear_max_error, prm.linear_max_iterations, it);
        iters += it;
        refinements++;
        if (ks != GBFV_OK && ks != GBFV_ERR_NOT_CONVERGED) return ks;
        launchAccumulate(n, S.xref, S.v32[1], stream);
        if ((rs = resetStatus(stream, st))) return rs;
        launchResidual64(S.N, S.ldN, S.nslot, S.b, S.col, A, rhs, S.xref, S.rref, S.v32[0], st, stream);
        if ((rs = syncStatus(stream, st, hst))) return rs;
        unsigned long long bits = hst->errorBits;
        std::memcpy(&resErr, &bits, sizeof(double));
        if (!std::isfinite(resErr)) return GBFV_ERR_NONFINITE;
        S.lastReduction = resErr / std::max(1e-20, resErr0);
        S.lastResidual = resErr;
        if (converged(resErr)) return GBFV_OK;
        if (resErr > prm.linear_max_error * resErr0) return GBFV_ERR_NOT_CONVERGED;
        if (ks == GBFV_ERR_NOT_CONVERGED && it >= prm.linear_max_iterations) return GBFV_ERR_NOT_CONVERGED;
    }
    return GBFV_ERR_NOT_CONVERGED;
}

}  // namespace

extern "C" {

void gbfv_default_params(gbfv_params* p)
{
    std::memset(p, 0, sizeof(*p));
    p->newton_tolerance = 1e-8;
    p->newton_max_iterations = 20;
    p->newton_target_iterations = 10;
    p->newton_max_error = 1e100;
    p->linear_tolerance = 1e-3;
    p->linear_abs_tolerance = -1.0;
    p->linear_max_iterations = 1000;
    p->linear_max_error = 1e7;
    p->precision = GBFV_PREC_FP64;
    p->inner_tolerance = 1e-3;
    p->max_refinements = 20;
    p->dp_max_rel = 0.3;
    p->ds_max = 0.2;
    p->pv_oscillation_threshold = 1e-5;
    p->pressure_min = -1e99;
    p->pressure_max = 1e99;
    p->max_water_saturation = 1.0;
    p->water_only_threshold = 1.0;
    p->min_time_step = 0.0;
    p->max_time_step = std::numeric_limits<double>::infinity();
    p->max_time_step_divisions = 10;
    p->local_linearizer = GBFV_LIN_AD;
    p->numeric_difference_method = 1;
    p->linear_solver = GBFV_LINSOLVER_ILU0;
    p->amg_coarsen_target = 5000;
    p->linearizer = GBFV_LINEARIZER_ELEMENT;
}

int64_t gbfv_kernel_launches(void) { return g_launches.load(); }
const char* gbfv_last_error(void) { return t_lastError.c_str(); }

// material laws, liquid properties and PVT tables of the problem
// (materialLawParams, the fluid system) in the device record
static int buildPhysics(const gbfv_problem* P, DevPhysics& ph)
{
    std::memset(&ph, 0, sizeof(ph));
    ph.numMaterials = P->num_materials;
    for (int m = 0; m < P->num_materials; ++m) {
        const double* mp = P->material_params + m * GBFV_MAT_STRIDE;
        const int law = (int)mp[0];
        TwoPhaseLaw& L = ph.law[m];
        std::memset(&L, 0, sizeof(L));
        if (law == GBFV_LAW_REG_VAN_GENUCHTEN || law == GBFV_LAW_REG_BROOKS_COREY) {
            L.law = law == GBFV_LAW_REG_VAN_GENUCHTEN ? 0 : 1;
            L.Swr = mp[1];
            L.Snr = mp[2];
            if (L.law == 0) { L.alpha = mp[3]; L.n = mp[4]; }
            else { L.pe = mp[3]; L.lambda = mp[4]; }
            finalizeLaw(L);
        }
        ph.coreyN[m] = law == GBFV_LAW_COREY3P ? mp[4] : 2.0;
    }
    ph.rho[0] = P->rho[0];
    ph.rho[1] = P->rho[1];
    ph.mu[0] = P->mu[0];
    ph.mu[1] = P->mu[1];
    if (P->pvt) {
        const gbfv_blackoil_pvt& t = *P->pvt;
        if (t.n_oil < 2 || t.n_oil > GBFV_MAX_TABLE || t.n_gas < 2 || t.n_gas > GBFV_MAX_TABLE) {
            setError("PVT table size outside [2, 32]");
            return GBFV_ERR_ARG;
        }
        BlackOilPvt& v = ph.pvt;
        v.rhoRefO = t.rho_ref_oil;
        v.rhoRefW = t.rho_ref_water;
        v.rhoRefG = t.rho_ref_gas;
        v.rsSat.n = v.pBubble.n = v.invBoSat.n = v.muoSat.n = t.n_oil;
        for (int i = 0; i < t.n_oil; ++i) {
            v.rsSat.x[i] = t.oil_p[i]; v.rsSat.y[i] = t.oil_rs[i];
            v.pBubble.x[i] = t.oil_rs[i]; v.pBubble.y[i] = t.oil_p[i];
            v.invBoSat.x[i] = t.oil_p[i]; v.invBoSat.y[i] = 1.0 / t.oil_bo[i];
            v.muoSat.x[i] = t.oil_p[i]; v.muoSat.y[i] = t.oil_mu[i];
        }
        v.oilComp = t.oil_compressibility;
        v.invBg.n = v.mug.n = t.n_gas;
        for (int i = 0; i < t.n_gas; ++i) {
            v.invBg.x[i] = t.gas_p[i]; v.invBg.y[i] = 1.0 / t.gas_bg[i];
            v.mug.x[i] = t.gas_p[i]; v.mug.y[i] = t.gas_mu[i];
        }
        v.pwRef = t.water_p_ref;
        v.bwRef = t.water_bw_ref;
        v.cw = t.water_compressibility;
        v.muw = t.water_mu;
    }
    return GBFV_OK;
}

// A context on a vertex-centred grid (VcfvDiscretization): the degrees of
// freedom are the vertices; the Jacobian has the 3 x 3 vertex neighbourhood
// in VCFV_SLOTS slots (ascending natural column, the diagonal in the middle)
// and is solved by the general block ILU(0) (or the AMG backend).  The
// per-vertex kernels (intensive quantities, Newton error and update,
// constraints, output fields) are the cell-centred ones.
static int createVcfvImpl(gbfv_ctx* C, const gbfv_problem* P)
{
    if (C->prm.linearizer != GBFV_LINEARIZER_ELEMENT) {
        setError("vertex-centred grids take the element linearizer");
        return GBFV_ERR_UNSUPPORTED;
    }
    if (P->model == GBFV_MODEL_BLACKOIL_3P && C->prm.local_linearizer != GBFV_LIN_AD) {
        setError("vertex-centred black-oil grids take the AD local linearizer");
        return GBFV_ERR_UNSUPPORTED;
    }
    VcfvSetup vs;
    if (const int st = vcfvSetup(P, vs)) return st;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        setError("no CUDA device");
        return GBFV_ERR_NO_DEVICE;
    }
    const int N = P->num_cells, b = P->model == GBFV_MODEL_BLACKOIL_3P ? 3 : 2, nslot = VCFV_SLOTS;
    C->N = N;
    C->model = P->model;
    C->b = b;
    C->dim = 2;
    const int ld = ((N + 63) / 64) * 64;
    C->ldN = ld;
    if ((int64_t)nslot * b * b * ld > std::numeric_limits<int>::max()) {
        setError("grid too large for the 9-slot Jacobian's 32-bit indexing");
        return GBFV_ERR_UNSUPPORTED;
    }
    // level-major order from the lower neighbours (natural index below)
    std::vector<std::vector<int>> lower(N);
    for (int i = 0; i < N; ++i)
        for (int sl = 0; sl < VCFV_DIAG; ++sl) {
            const int q = vs.nbr[(size_t)i * nslot + sl];
            if (q >= 0) lower[i].push_back(q);
        }
    std::vector<int> levPtr;
    buildOrder(N, lower, C->perm, C->iperm, levPtr);
    const std::vector<int>& perm = C->perm;
    const std::vector<int>& iperm = C->iperm;
    std::vector<int> hCol((size_t)nslot * ld, -1);
    for (int i = 0; i < N; ++i)
        for (int sl = 0; sl < nslot; ++sl) {
            const int q = vs.nbr[(size_t)i * nslot + sl];
            if (q >= 0) hCol[(size_t)sl * ld + perm[i]] = perm[q];
        }
    C->bcrsRowPtr.assign(N + 1, 0);
    for (int i = 0; i < N; ++i) {
        for (int sl = 0; sl < nslot; ++sl) {
            const int q = vs.nbr[(size_t)i * nslot + sl];
            if (q < 0) continue;
            C->bcrsCol.push_back(q);
            C->bcrsSlot.push_back(sl);
            C->bcrsRow.push_back(perm[i]);
        }
        C->bcrsRowPtr[i + 1] = (int)C->bcrsCol.size();
    }
    DevPhysics& ph = C->hphys;
    if (const int pst = buildPhysics(P, ph)) return pst;
    std::vector<double> hVol(ld, 1.0), hPor(ld, 0.0), hPerm((size_t)3 * ld, 0.0);
    std::vector<int> hMat(ld, 0), hCflag(ld, -1);
    for (int p = 0; p < N; ++p) {
        const int I = iperm[p];
        hVol[p] = vs.totalVolume[I];
        hPor[p] = P->porosity[I];
        for (int d = 0; d < 3; ++d) hPerm[(size_t)d * ld + p] = P->perm[3 * I + d];
        hMat[p] = P->material[I];
        hCflag[p] = P->constraint ? P->constraint[I] : -1;
    }
    // constraint vertices (the problem's constraints(), e.g. wells)
    std::vector<int> consCells, consOf;
    for (int p = 0; p < N; ++p)
        if (hCflag[p] >= 0) {
            consCells.push_back(p);
            consOf.push_back(hCflag[p]);
        }
    std::vector<double> consPv(P->constraint_pv, P->constraint_pv + 3 * (size_t)std::max(0, P->num_constraints));
    std::vector<int> consMeaning(P->constraint_meaning, P->constraint_meaning + std::max(0, P->num_constraints));
    CK(cudaStreamCreateWithFlags(&C->stream, cudaStreamNonBlocking));
    for (auto& e : C->ev) CK(cudaEventCreate(&e));
    DevMesh& m = C->mesh;
    std::memset(&m, 0, sizeof(m));
    m.N = N;
    m.ldN = ld;
    m.dim = 2;
    m.b = b;
    m.model = C->model;
    m.nslot = nslot;
    m.fluxModule = GBFV_FLUX_DARCY;
    int st;
    auto up = [&](auto** dst, const auto& vec) {
        int s2 = upload(dst, vec);
        if (!s2) C->owned.push_back((void*)*dst);
        return s2;
    };
    int *dMat, *dCflag, *dConsCells, *dConsOf, *dConsMeaning;
    double *dVol, *dPor, *dPerm, *dConsPv;
    if ((st = up(&dVol, hVol)) || (st = up(&dPor, hPor)) || (st = up(&dPerm, hPerm)) || (st = up(&dMat, hMat)) ||
        (st = up(&dCflag, hCflag)) || (st = up(&dConsCells, consCells)) || (st = up(&dConsOf, consOf)) ||
        (st = up(&dConsPv, consPv)) || (st = up(&dConsMeaning, consMeaning)))
        return st;
    m.volume = dVol;
    m.porosity = dPor;
    m.perm = dPerm;
    m.material = dMat;
    m.cflag = dCflag;
    m.consCells = dConsCells;
    m.consOf = dConsOf;
    m.consPv = dConsPv;
    m.consMeaning = dConsMeaning;
    m.numConsCells = (int)consCells.size();
    if ((st = devAlloc(&C->dphys, 1))) return st;
    CK(cudaMemcpy(C->dphys, &ph, sizeof(DevPhysics), cudaMemcpyHostToDevice));
    C->vcfv = vcfvUpload(P, vs, ph, perm, ld, &st);
    if (!C->vcfv) return st;
    C->numElements = P->num_elements;
    // state
    const size_t nb = (size_t)N * b;
    if ((st = devAlloc(&C->x, nb)) || (st = devAlloc(&C->xOld, nb)) || (st = devAlloc(&C->residual, nb)) ||
        (st = devAlloc(&C->dx, nb)) || (st = devAlloc(&C->storageOld, (size_t)b * ld)) ||
        (st = devAlloc(&C->meaning, (size_t)N)) || (st = devAlloc(&C->meaningOld, (size_t)N)) ||
        (st = devAlloc(&C->wasSwitched, (size_t)N)) || (st = devAlloc(&C->refP, 1)))
        return st;
    CK(cudaMemset(C->meaning, 0, sizeof(int) * N));
    CK(cudaMemset(C->meaningOld, 0, sizeof(int) * N));
    CK(cudaMemset(C->wasSwitched, 0, sizeof(int) * N));
    CK(cudaMemset(C->x, 0, sizeof(double) * nb));
    CK(cudaMemset(C->xOld, 0, sizeof(double) * nb));
    {
        const double one = 1.0;
        CK(cudaMemcpy(C->refP, &one, sizeof(double), cudaMemcpyHostToDevice));
    }
    if ((st = devAlloc(&C->iq.val, (size_t)iqValuePlanes(b) * ld)) ||
        (st = devAlloc(&C->iq.der, (size_t)iqDerivPlanes(b) * ld)) ||
        (st = devAlloc(&C->iq.sto, (size_t)iqStoragePlanes(b) * ld)))
        return st;
    if ((st = devAlloc(&C->jval, (size_t)nslot * b * b * ld))) return st;
    CK(cudaMemset(C->jval, 0, sizeof(double) * (size_t)nslot * b * b * ld));
    // solver: the general block ILU(0) (the AMG backend on the same layout)
    SolverData& S = C->S;
    S.N = N;
    S.b = b;
    S.dim = 2;
    S.nslot = nslot;
    S.ldN = ld;
    S.levPtr = levPtr;
    S.colHost = hCol;
    S.natural = iperm;
    if ((st = upload(&S.col, hCol)) || (st = upload(&S.levPtrD, levPtr))) return st;
    if ((st = allocSolver(S))) return st;
    S.gilu = giluCreate(N, b, nslot, ld, hCol, S.col, levPtr, &st);
    if (!S.gilu) return st;
    if ((st = devAlloc(&C->st, 1))) return st;
    CK(cudaMallocHost((void**)&C->hst, sizeof(DevStatus)));
    CK(cudaMemset(C->st, 0, sizeof(DevStatus)));
    if ((st = devAlloc(&C->xSave, nb)) || (st = devAlloc(&C->meaningSave, (size_t)N)) ||
        (st = devAlloc(&C->switchedSave, (size_t)N)))
        return st;
    CK(cudaEventCreate(&C->evL0));
    CK(cudaEventCreate(&C->evL1));
    {
        const double k1 = b * 8.0 + 8 + 4 + (iqValuePlanes(b) + iqDerivPlanes(b) + iqStoragePlanes(b)) * 8.0;
        C->linBytesPer = N * k1 + vcfvLinearizeBytes(C->vcfv);
    }
    return GBFV_OK;
}

static int createImpl(gbfv_ctx* C, const gbfv_problem* P)
{
    // counts, offsets, enums and tables first: everything below follows them
    if (const int chk = gbfv::checkProblem(P, MAX_MATERIALS, GBFV_MAX_TABLE)) return chk;
    if (P->num_elements > 0) return createVcfvImpl(C, P);
    const int N = P->num_cells;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        setError("no CUDA device");
        return GBFV_ERR_NO_DEVICE;
    }
    C->N = N;
    C->model = P->model;
    C->b = P->model == GBFV_MODEL_BLACKOIL_3P ? 3 : 2;
    const int b = C->b;
    // dimension from the face normals
    int dim = 2;
    for (int c = 0; c < P->num_conn && dim == 2; ++c)
        if (P->conn_normal[3 * c + 2] != 0.0) dim = 3;
    for (int f = 0; f < P->num_bfaces && dim == 2; ++f)
        if (P->bface_normal[3 * f + 2] != 0.0) dim = 3;
    if (P->model == GBFV_MODEL_BLACKOIL_3P) dim = 3;
    C->dim = dim;
    const int ndir = 2 * dim;
    // neighbour per (cell, direction); verify axis-aligned geometry
    std::vector<int> nbrDir((size_t)N * ndir, -1), connOf((size_t)N * ndir, -1);
    auto axisOf = [&](const double* n, int& axis, double& sgn) {
        int cnt = 0;
        for (int d = 0; d < 3; ++d)
            if (n[d] != 0.0) { axis = d; sgn = n[d]; ++cnt; }
        return cnt == 1 && (sgn == 1.0 || sgn == -1.0);
    };
    for (int I = 0; I < N; ++I) {
        for (int c = P->conn_ptr[I]; c < P->conn_ptr[I + 1]; ++c) {
            int axis = 0;
            double sgn = 0;
            if (!axisOf(&P->conn_normal[3 * c], axis, sgn) || axis >= dim) {
                setError("only axis-aligned (Cartesian) faces are supported");
                return GBFV_ERR_UNSUPPORTED;
            }
            const int J = P->conn_nbr[c];
            if (J < 0 || J >= N) return GBFV_ERR_ARG;
            for (int d = 0; d < 3; ++d) {
                if (d == axis) continue;
                if (P->center[3 * J + d] != P->center[3 * I + d] || P->conn_center[3 * c + d] != P->center[3 * I + d]) {
                    setError("face centres must share the off-axis coordinates of the cell centres");
                    return GBFV_ERR_UNSUPPORTED;
                }
            }
            const int dir = 2 * axis + (sgn > 0 ? 1 : 0);
            if (nbrDir[(size_t)I * ndir + dir] >= 0) {
                setError("two neighbours in one direction");
                return GBFV_ERR_UNSUPPORTED;
            }
            nbrDir[(size_t)I * ndir + dir] = J;
            connOf[(size_t)I * ndir + dir] = c;
        }
    }
    // symmetric pattern and natural column order matching the slot order
    for (int I = 0; I < N; ++I) {
        int prevLower = -1;
        for (int s = 0; s < dim; ++s) {  // slots -z..-x: dirs 2(dim-1-s)
            const int J = nbrDir[(size_t)I * ndir + 2 * (dim - 1 - s)];
            if (J < 0) continue;
            if (J >= I || J <= prevLower) {
                setError("cell numbering is not the structured natural order");
                return GBFV_ERR_UNSUPPORTED;
            }
            prevLower = J;
        }
        int prevUpper = I;
        for (int a = 0; a < dim; ++a) {
            const int J = nbrDir[(size_t)I * ndir + 2 * a + 1];
            if (J < 0) continue;
            if (J <= prevUpper) {
                setError("cell numbering is not the structured natural order");
                return GBFV_ERR_UNSUPPORTED;
            }
            prevUpper = J;
            if (nbrDir[(size_t)J * ndir + 2 * a] != I) {
                setError("asymmetric connectivity");
                return GBFV_ERR_UNSUPPORTED;
            }
        }
    }
    // ILU(0) update structure: lower entry k of row i may only update (i,i)
    for (int I = 0; I < N; ++I)
        for (int a = 0; a < dim; ++a) {
            const int K = nbrDir[(size_t)I * ndir + 2 * a];
            if (K < 0) continue;
            for (int a2 = 0; a2 < dim; ++a2) {
                const int Kup = nbrDir[(size_t)K * ndir + 2 * a2 + 1];
                if (Kup < 0 || Kup == I) continue;
                for (int d = 0; d < ndir; ++d)
                    if (nbrDir[(size_t)I * ndir + d] == Kup) {
                        setError("pattern has ILU(0) fill interactions beyond the diagonal");
                        return GBFV_ERR_UNSUPPORTED;
                    }
            }
        }
    // wavefront-major order
    std::vector<std::vector<int>> lower(N);
    for (int I = 0; I < N; ++I)
        for (int a = 0; a < dim; ++a) {
            const int K = nbrDir[(size_t)I * ndir + 2 * a];
            if (K >= 0) lower[I].push_back(K);
        }
    std::vector<int> levPtr;
    const std::vector<int> tkey = tileKeys(N, dim, ndir, nbrDir);
    buildOrder(N, lower, C->perm, C->iperm, levPtr, &tkey);
    const int ld = ((N + 63) / 64) * 64;
    C->ldN = ld;
    const auto& perm = C->perm;
    const auto& iperm = C->iperm;
    // per-direction geometry in internal order
    std::vector<int> hNbr((size_t)ndir * ld, -1);
    std::vector<double> hDTot((size_t)ndir * ld, 0), hGIn((size_t)ndir * ld, 0), hGEx((size_t)ndir * ld, 0),
        hKh((size_t)ndir * ld, 0), hArea((size_t)ndir * ld, 0);
    const double* g = P->gravity;
    for (int p = 0; p < N; ++p) {
        const int I = iperm[p];
        const double* xI = &P->center[3 * I];
        for (int dir = 0; dir < ndir; ++dir) {
            const int J = nbrDir[(size_t)I * ndir + dir];
            if (J < 0) continue;
            const int c = connOf[(size_t)I * ndir + dir];
            const int axis = dir / 2;
            const double* xJ = &P->center[3 * J];
            const double* xf = &P->conn_center[3 * c];
            const size_t o = (size_t)dir * ld + p;
            hNbr[o] = perm[J];
            hDTot[o] = xJ[axis] - xI[axis];
            double gIn = 0.0, gEx = 0.0;
            for (int d = 0; d < 3; ++d) gIn += g[d] * (xI[d] - xf[d]);
            for (int d = 0; d < 3; ++d) gEx += g[d] * (xJ[d] - xf[d]);
            hGIn[o] = gIn;
            hGEx[o] = gEx;
            hKh[o] = harmonicMean(P->perm[3 * I + axis], P->perm[3 * J + axis]);
            hArea[o] = P->conn_area[c];
        }
    }
    // transmissibility flux module (transfluxmodule.hh:201-480): face
    // transmissibilities, hydrostatic depth terms and upwind tie rules
    const int fluxModule = P->flux_module;
    if (fluxModule != GBFV_FLUX_DARCY && fluxModule != GBFV_FLUX_TRANS) return GBFV_ERR_ARG;
    if (fluxModule == GBFV_FLUX_TRANS && P->model != GBFV_MODEL_IMMISCIBLE_2P) {
        setError("the transmissibility flux module is supported for the immiscible model");
        return GBFV_ERR_UNSUPPORTED;
    }
    // TpfaLinearizer + BlackOilLocalResidualTPFA: black-oil, no constraint
    // cells, boundary faces no-flow or mass-rate; its neighbour records carry
    // the same face transmissibilities, depth terms and upwind ties
    const bool tpfa = C->prm.linearizer == GBFV_LINEARIZER_TPFA;
    if (tpfa) {
        if (P->model != GBFV_MODEL_BLACKOIL_3P) {
            setError("the TPFA linearizer is the black-oil model's (BlackOilLocalResidualTPFA)");
            return GBFV_ERR_UNSUPPORTED;
        }
        for (int i = 0; P->constraint && i < N; ++i)
            if (P->constraint[i] >= 0) {
                setError("the TPFA linearizer applies no constraints; cell " + std::to_string(i) + " has one");
                return GBFV_ERR_UNSUPPORTED;
            }
        for (int f = 0; f < P->num_bfaces; ++f)
            if (P->bface_type[f] != GBFV_BC_NOFLOW && P->bface_type[f] != GBFV_BC_MASSRATE) {
                setError("the TPFA linearizer takes no-flow and mass-rate boundary faces only");
                return GBFV_ERR_UNSUPPORTED;
            }
    }
    const bool needTrans = fluxModule == GBFV_FLUX_TRANS || tpfa;
    int dimWorld = 1;  // the highest coordinate axis the faces use, plus one
    for (int c = 0; c < P->num_conn; ++c)
        for (int d = 0; d < 3; ++d)
            if (P->conn_normal[3 * c + d] != 0.0) dimWorld = std::max(dimWorld, d + 1);
    auto axisOfNormal = [&](const double* n) {
        int idx = 0;
        double val = 0.0;
        for (int d = 0; d < dimWorld; ++d)
            if (std::abs(n[d]) > val) { val = std::abs(n[d]); idx = d; }
        return idx;
    };
    std::vector<double> hTrans, hDzg;
    std::vector<int> hTie;
    if (needTrans) {
        hTrans.assign((size_t)ndir * ld, 0.0);
        hDzg.assign((size_t)ndir * ld, 0.0);
        hTie.assign((size_t)ndir * ld, 1);
        const double gz = g[dimWorld - 1];
        for (int p = 0; p < N; ++p) {
            const int I = iperm[p];
            const double* xI = &P->center[3 * I];
            for (int dir = 0; dir < ndir; ++dir) {
                const int J = nbrDir[(size_t)I * ndir + dir];
                if (J < 0) continue;
                const int c = connOf[(size_t)I * ndir + dir];
                const double* xJ = &P->center[3 * J];
                const double* xf = &P->conn_center[3 * c];
                const double* n = &P->conn_normal[3 * c];
                double nd0 = 0, nd1 = 0, s0 = 0, s1 = 0;
                for (int d = 0; d < 3; ++d) {
                    const double d0 = xf[d] - xI[d], d1 = xf[d] - xJ[d];
                    nd0 += n[d] * d0;
                    nd1 += n[d] * d1;
                    s0 += d0 * d0;
                    s1 += d1 * d1;
                }
                nd0 = std::abs(nd0);
                nd1 = std::abs(nd1);
                const int idx = axisOfNormal(n);
                const double T0 = P->perm[3 * I + idx] * nd0 / s0;
                const double T1 = P->perm[3 * J + idx] * nd1 / s1;
                const size_t o = (size_t)dir * ld + p;
                hTrans[o] = T0 * T1 / (T0 + T1);
                const double distZ = xI[dimWorld - 1] - xJ[dimWorld - 1];
                hDzg[o] = distZ * gz;
                const double Vin = P->volume[I], Vex = P->volume[J];
                hTie[o] = Vin > Vex ? 1 : (Vin < Vex ? 0 : (I < J ? 1 : 0));
            }
        }
    }
    std::vector<double> hVol(ld, 1.0), hPor(ld, 0.0), hPerm((size_t)3 * ld, 0.0);
    std::vector<int> hMat(ld, 0), hCflag(ld, -1);
    for (int p = 0; p < N; ++p) {
        const int I = iperm[p];
        hVol[p] = P->volume[I];
        hPor[p] = P->porosity[I];
        for (int d = 0; d < 3; ++d) hPerm[(size_t)d * ld + p] = P->perm[3 * I + d];
        hMat[p] = P->material[I];
        if (hMat[p] < 0 || hMat[p] >= P->num_materials || P->num_materials > MAX_MATERIALS) {
            setError("material index out of range");
            return GBFV_ERR_ARG;
        }
        hCflag[p] = P->constraint ? P->constraint[I] : -1;
    }
    // physics parameters
    DevPhysics& ph = C->hphys;
    if (const int pst = buildPhysics(P, ph)) return pst;
    // boundary faces in internal order, free-flow states on the host
    std::vector<int> hBfPtr(N + 1, 0);
    std::vector<BFace> hBf;
    for (int p = 0; p < N; ++p) {
        const int I = iperm[p];
        hBfPtr[p] = (int)hBf.size();
        for (int f = P->bface_ptr[I]; f < P->bface_ptr[I + 1]; ++f) {
            const int type = P->bface_type ? P->bface_type[f] : GBFV_BC_NOFLOW;
            if (type == GBFV_BC_NOFLOW) continue;
            BFace bf;
            std::memset(&bf, 0, sizeof(bf));
            bf.p = p;
            bf.type = type;
            int axis = 0;
            double sgn = 0;
            if (!axisOf(&P->bface_normal[3 * f], axis, sgn)) return GBFV_ERR_UNSUPPORTED;
            bf.axis = axis;
            bf.nrm = sgn;
            const double* xI = &P->center[3 * I];
            const double* xf = &P->bface_center[3 * f];
            for (int d = 0; d < 3; ++d)
                if (d != axis && xf[d] != xI[d]) return GBFV_ERR_UNSUPPORTED;
            bf.tmpA = xf[axis] - xI[axis];
            bf.dInA = xI[axis] - xf[axis];
            double gtd = 0.0;
            for (int d = 0; d < 3; ++d) gtd += g[d] * (xI[d] - xf[d]);
            bf.gTimesDist = gtd;
            bf.area = P->bface_area[f];
            const double* val = &P->bface_value[4 * f];
            if (type == GBFV_BC_MASSRATE) {
                for (int e = 0; e < b; ++e) bf.rate[e] = val[e];
            }
            else if (type == GBFV_BC_FREEFLOW) {
                if (P->model != GBFV_MODEL_IMMISCIBLE_2P) return GBFV_ERR_UNSUPPORTED;
                const TwoPhaseLaw& L = ph.law[P->material[I]];
                const double pw = val[0], Swb = val[1];
                const double sumRes = L.Swr + L.Snr;
                const double SwE = (Swb - L.Swr) / (1.0 - sumRes);
                const double SnE = ((1 - Swb) - L.Snr) / (1.0 - sumRes);
                const double pcn = pcnw(L, SwE);
                bf.pb[0] = pw;
                bf.pb[1] = pw + pcn - 0.0;
                const double krb[2] = {krw(L, SwE), krn(L, 1.0 - SnE)};
                for (int a = 0; a < 2; ++a) {
                    bf.mobb[a] = krb[a] / P->mu[a];
                    bf.rhob[a] = P->rho[a];
                }
                if (fluxModule == GBFV_FLUX_TRANS) {
                    // transmissibilityBoundary_ (transfluxmodule.hh:457-480) takes the
                    // geometry of the cell's interior face with the boundary face's index
                    const int c = P->conn_ptr[I] + (f - P->bface_ptr[I]);
                    if (c >= P->conn_ptr[I + 1]) {
                        setError("transmissibility boundary face without an interior face of the same index");
                        return GBFV_ERR_UNSUPPORTED;
                    }
                    const double* n = &P->conn_normal[3 * c];
                    const double* xc = &P->conn_center[3 * c];
                    double nd = 0, s0 = 0;
                    for (int d = 0; d < 3; ++d) {
                        const double t = xc[d] - xI[d];
                        nd += n[d] * t;
                        s0 += t * t;
                    }
                    bf.transB = P->perm[3 * I + axisOfNormal(n)] * nd / s0;
                    bf.dzgB = (xI[dimWorld - 1] - xf[dimWorld - 1]) * g[dimWorld - 1];
                }
            }
            hBf.push_back(bf);
        }
    }
    hBfPtr[N] = (int)hBf.size();
    // constraints
    std::vector<int> consCells, consOf;
    for (int p = 0; p < N; ++p)
        if (hCflag[p] >= 0) {
            if (hCflag[p] >= P->num_constraints) return GBFV_ERR_ARG;
            consCells.push_back(p);
            consOf.push_back(hCflag[p]);
        }
    std::vector<double> consPv(P->constraint_pv, P->constraint_pv + 3 * (size_t)std::max(0, P->num_constraints));
    std::vector<int> consMeaning(P->constraint_meaning,
                                 P->constraint_meaning + std::max(0, P->num_constraints));
    // ELL columns of the Jacobian / solver matrix
    const int nslot = 2 * dim + 1;
    std::vector<int> hCol((size_t)nslot * ld, -1);
    int slotOfDir[6];
    for (int dir = 0; dir < 6; ++dir) {
        const int a = dir / 2;
        slotOfDir[dir] = (dir & 1) ? dim + 1 + a : dim - 1 - a;
    }
    for (int p = 0; p < N; ++p) {
        hCol[(size_t)dim * ld + p] = p;
        for (int dir = 0; dir < ndir; ++dir) {
            const int q = hNbr[(size_t)dir * ld + p];
            if (q >= 0) hCol[(size_t)slotOfDir[dir] * ld + p] = q;
        }
    }
    // natural BCRS view (columns ascending), entry -> (slot, internal row)
    C->bcrsRowPtr.assign(N + 1, 0);
    for (int I = 0; I < N; ++I) {
        std::vector<std::pair<int, int>> ent;  // (col, slot)
        ent.push_back({I, dim});
        for (int dir = 0; dir < ndir; ++dir) {
            const int J = nbrDir[(size_t)I * ndir + dir];
            if (J >= 0) ent.push_back({J, slotOfDir[dir]});
        }
        std::sort(ent.begin(), ent.end());
        for (auto& e : ent) {
            C->bcrsCol.push_back(e.first);
            C->bcrsSlot.push_back(e.second);
            C->bcrsRow.push_back(perm[I]);
        }
        C->bcrsRowPtr[I + 1] = (int)C->bcrsCol.size();
    }
    // ---------------------------------------------------------- upload
    CK(cudaStreamCreateWithFlags(&C->stream, cudaStreamNonBlocking));
    for (auto& e : C->ev) CK(cudaEventCreate(&e));
    DevMesh& m = C->mesh;
    m.N = N;
    m.ldN = ld;
    m.dim = dim;
    m.b = b;
    m.model = C->model;
    m.nslot = nslot;
    for (int d = 0; d < 6; ++d) m.slotOfDir[d] = slotOfDir[d];
    int st;
    auto up = [&](auto** dst, const auto& vec) {
        int s2 = upload(dst, vec);
        if (!s2) C->owned.push_back((void*)*dst);
        return s2;
    };
    int *dNbr, *dMat, *dCflag, *dBfPtr, *dConsCells, *dConsOf, *dConsMeaning;
    double *dDTot, *dGIn, *dGEx, *dKh, *dArea, *dVol, *dPor, *dPerm, *dConsPv;
    BFace* dBf;
    if ((st = up(&dNbr, hNbr)) || (st = up(&dDTot, hDTot)) || (st = up(&dGIn, hGIn)) || (st = up(&dGEx, hGEx)) ||
        (st = up(&dKh, hKh)) || (st = up(&dArea, hArea)) || (st = up(&dVol, hVol)) || (st = up(&dPor, hPor)) ||
        (st = up(&dPerm, hPerm)) || (st = up(&dMat, hMat)) || (st = up(&dCflag, hCflag)) ||
        (st = up(&dBfPtr, hBfPtr)) || (st = up(&dBf, hBf)) || (st = up(&dConsCells, consCells)) ||
        (st = up(&dConsOf, consOf)) || (st = up(&dConsPv, consPv)) || (st = up(&dConsMeaning, consMeaning)))
        return st;
    m.nbr = dNbr;
    m.dTot = dDTot;
    m.gIn = dGIn;
    m.gEx = dGEx;
    m.Kh = dKh;
    m.area = dArea;
    m.volume = dVol;
    m.porosity = dPor;
    m.perm = dPerm;
    m.material = dMat;
    m.cflag = dCflag;
    m.bfPtr = dBfPtr;
    m.bfaces = dBf;
    m.consCells = dConsCells;
    m.consOf = dConsOf;
    m.consPv = dConsPv;
    m.consMeaning = dConsMeaning;
    m.numConsCells = (int)consCells.size();
    m.inst = nullptr;
    m.fluxModule = fluxModule;
    m.tpfa = tpfa ? 1 : 0;
    m.trans = m.dzg = nullptr;
    m.tieUpI = nullptr;
    if (needTrans) {
        double *dTrans, *dDzg;
        int* dTie;
        if ((st = up(&dTrans, hTrans)) || (st = up(&dDzg, hDzg)) || (st = up(&dTie, hTie))) return st;
        m.trans = dTrans;
        m.dzg = dDzg;
        m.tieUpI = dTie;
    }
    if ((st = devAlloc(&C->dphys, 1))) return st;
    CK(cudaMemcpy(C->dphys, &ph, sizeof(DevPhysics), cudaMemcpyHostToDevice));
    // state
    const size_t nb = (size_t)N * b;
    if ((st = devAlloc(&C->x, nb)) || (st = devAlloc(&C->xOld, nb)) || (st = devAlloc(&C->residual, nb)) ||
        (st = devAlloc(&C->dx, nb)) || (st = devAlloc(&C->storageOld, (size_t)b * ld)) ||
        (st = devAlloc(&C->meaning, (size_t)N)) || (st = devAlloc(&C->meaningOld, (size_t)N)) ||
        (st = devAlloc(&C->wasSwitched, (size_t)N)))
        return st;
    CK(cudaMemset(C->meaning, 0, sizeof(int) * N));
    CK(cudaMemset(C->meaningOld, 0, sizeof(int) * N));
    if ((st = devAlloc(&C->refP, 1))) return st;
    {
        const double one = 1.0;
        CK(cudaMemcpy(C->refP, &one, sizeof(double), cudaMemcpyHostToDevice));
    }
    CK(cudaMemset(C->wasSwitched, 0, sizeof(int) * N));
    CK(cudaMemset(C->x, 0, sizeof(double) * nb));
    CK(cudaMemset(C->xOld, 0, sizeof(double) * nb));
    const int nv = iqValuePlanes(b);
    const int nd = iqDerivPlanes(b);
    const int ns = iqStoragePlanes(b);
    if ((st = devAlloc(&C->iq.val, (size_t)nv * ld)) || (st = devAlloc(&C->iq.der, (size_t)nd * ld)) ||
        (st = devAlloc(&C->iq.sto, (size_t)ns * ld)))
        return st;
    if ((st = devAlloc(&C->jval, (size_t)nslot * b * b * ld))) return st;
    CK(cudaMemset(C->jval, 0, sizeof(double) * (size_t)nslot * b * b * ld));
    // solver
    SolverData& S = C->S;
    S.N = N;
    S.b = b;
    S.dim = dim;
    S.nslot = nslot;
    S.ldN = ld;
    S.levPtr = levPtr;
    S.adjacentLevels = adjacentLevels(lower, C->perm, levPtr);
    S.colHost = hCol;
    S.natural = C->iperm;
    if (dim >= 2) {
        S.tileKey.resize(N);
        for (int p = 0; p < N; ++p) S.tileKey[p] = tkey[iperm[p]];
    }
    if ((st = upload(&S.col, hCol)) || (st = upload(&S.levPtrD, levPtr))) return st;
    if ((st = allocSolver(S))) return st;
    // Narrow systems (every wavefront level at most 32 rows, e.g. the 48 x 32
    // lens; two-phase systems) solve faster with the general kernel's
    // one-warp sweeps over shared memory than with the cluster sweeps: the
    // same ILU(0) (no fill interactions here, so the same factors), one
    // block.  A forced solver
    // configuration (GBFV_SOLVER, gbfv_set_solver_config) or GBFV_NARROW=0
    // keeps the structured solver.
    {
        int maxW = 0;
        for (size_t l = 0; l + 1 < levPtr.size(); ++l) maxW = std::max(maxW, levPtr[l + 1] - levPtr[l]);
        const char* nv = getenv("GBFV_NARROW");
        if (b == 2 && maxW <= 32 && N <= 16384 && !getenv("GBFV_SOLVER") && !(nv && atoi(nv) == 0)) {
            int gst = GBFV_OK;
            S.gilu = giluCreate(N, b, nslot, ld, hCol, S.col, levPtr, &gst);
            S.giluRoute = S.gilu != nullptr;
        }
    }
    // Wide systems (more rows than one block of the general kernel takes):
    // the general kernel's tagged sweeps publish every row's result with a
    // tag that its consumers wait for, instead of a barrier per wavefront
    // level, over every SM of the GPU -- measured 1.7x (FP32) and 1.5x
    // (FP64) faster than the best structured launch on the 1M-cell system,
    // slower on the 200k-cell one.  So they are one more candidate of the
    // autotuner, per precision.  GBFV_SOLVER=tagged takes them without
    // tuning; another GBFV_SOLVER, gbfv_set_solver_config of a precision or
    // GBFV_GILU_TAGGED=0 / GBFV_GILU_TAGGED64=0 leave them out.
    const char* forced = getenv("GBFV_SOLVER");
    const bool forceTagged = forced && strcmp(forced, "tagged") == 0;
    if (!S.gilu && N > 65536 && (!forced || forceTagged)) {
        int gst = GBFV_OK;
        S.gilu = giluCreate(N, b, nslot, ld, hCol, S.col, levPtr, &gst);
        S.giluCand = S.gilu ? (giluTagged(S.gilu, 0) ? 2 : 0) | (giluTagged(S.gilu, 1) ? 1 : 0) : 0;
        S.giluWide = S.giluCand != 0;
        if (!S.giluWide) {
            giluDestroy(S.gilu);
            S.gilu = nullptr;
        }
        else if (forceTagged) {  // GBFV_SOLVER=tagged: no autotuning
            S.giluUse = S.giluCand;
            S.tuned[0] = S.tuned[1] = 1;
        }
    }
    if ((st = devAlloc(&C->st, 1))) return st;
    CK(cudaMallocHost((void**)&C->hst, sizeof(DevStatus)));
    CK(cudaMemset(C->st, 0, sizeof(DevStatus)));
    if ((st = devAlloc(&C->xSave, nb)) || (st = devAlloc(&C->meaningSave, (size_t)N)) ||
        (st = devAlloc(&C->switchedSave, (size_t)N)))
        return st;
    CK(cudaEventCreate(&C->evL0));
    CK(cudaEventCreate(&C->evL1));
    // algorithmic bytes per cell of the IQ + assembly passes
    {
        const double s8 = 8.0;
        const double iqv = iqValuePlanes(b), iqd = iqDerivPlanes(b), iqs = iqStoragePlanes(b);
        const double k1 = b * s8 + 8 + 4 + (b == 3 ? 4 : 0) + (iqv + iqd + iqs) * s8;
        const double k2 = (iqv + iqd + iqs) * s8 + ndir * (4 + 5 * s8) + 8 + 4 + b * s8 + b * s8 +
                          nslot * b * b * s8;
        C->linBytesPer = N * (k1 + k2);
    }
    return GBFV_OK;
}

// the local linearizer settings are one of the supported ones
// the enum-valued parameters hold values of their enums
static bool paramsOk(const gbfv_params& p)
{
    if (p.precision != GBFV_PREC_FP64 && p.precision != GBFV_PREC_MIXED) {
        setError("precision is neither GBFV_PREC_FP64 nor GBFV_PREC_MIXED");
        return false;
    }
    if ((p.local_linearizer != GBFV_LIN_AD && p.local_linearizer != GBFV_LIN_FD) ||
        p.numeric_difference_method < -1 || p.numeric_difference_method > 1) {
        setError("unknown local linearizer or numeric difference method");
        return false;
    }
    if ((p.linear_solver != GBFV_LINSOLVER_ILU0 && p.linear_solver != GBFV_LINSOLVER_AMG) ||
        (p.linear_solver == GBFV_LINSOLVER_AMG && p.amg_coarsen_target < 1)) {
        setError("unknown linear solver, or an AMG coarsening target below 1");
        return false;
    }
    if (p.linearizer != GBFV_LINEARIZER_ELEMENT && p.linearizer != GBFV_LINEARIZER_TPFA) {
        setError("unknown linearizer");
        return false;
    }
    if (p.linearizer == GBFV_LINEARIZER_TPFA && p.local_linearizer != GBFV_LIN_AD) {
        setError("the TPFA linearizer differentiates automatically (local_linearizer GBFV_LIN_AD)");
        return false;
    }
    return true;
}

gbfv_ctx* gbfv_create(const gbfv_problem* prob, const gbfv_params* params, int* status)
{
    gbfv_ctx* C = new gbfv_ctx();
    if (params) C->prm = *params;
    else gbfv_default_params(&C->prm);
    if (!paramsOk(C->prm)) {
        if (status) *status = GBFV_ERR_ARG;
        delete C;
        return nullptr;
    }
    if (const char* lg = getenv("GBFV_SOLVE_LOG")) C->solveLog = lg;
    int st = GBFV_ERR_ARG;
    try {
        st = createImpl(C, prob);
    }
    catch (const std::bad_alloc&) {
        st = GBFV_ERR_OOM;
    }
    if (status) *status = st;
    if (st != GBFV_OK) {
        gbfv_destroy(C);
        return nullptr;
    }
    return C;
}

int gbfv_destroy(gbfv_ctx* C)
{
    if (!C) return GBFV_ERR_ARG;
    for (void* p : C->owned) cudaFree(p);
    cudaFree(C->dphys);
    cudaFree(C->x);
    cudaFree(C->xOld);
    cudaFree(C->residual);
    cudaFree(C->dx);
    cudaFree(C->storageOld);
    cudaFree(C->meaning);
    cudaFree(C->meaningOld);
    cudaFree(C->wasSwitched);
    cudaFree(C->iq.val);
    cudaFree(C->iq.der);
    cudaFree(C->iq.sto);
    for (int k = 0; k < 3; ++k)
        for (IqBuffers* q : {&C->fd.plus[k], &C->fd.minus[k]}) {
            cudaFree(q->val);
            cudaFree(q->der);
            cudaFree(q->sto);
        }
    for (double* p : C->fdX) cudaFree(p);
    cudaFree(C->refP);
    cudaFree(C->jval);
    freeSolver(C->S);
    vcfvDestroy(C->vcfv);
    cudaFree(C->st);
    cudaFree(C->xSave);
    cudaFree(C->meaningSave);
    cudaFree(C->switchedSave);
    if (C->evL0) cudaEventDestroy(C->evL0);
    if (C->evL1) cudaEventDestroy(C->evL1);
    if (C->hst) cudaFreeHost(C->hst);
    if (C->stream) {
        for (auto& e : C->ev) cudaEventDestroy(e);
        cudaStreamDestroy(C->stream);
    }
    delete C;
    return GBFV_OK;
}

int gbfv_set_params(gbfv_ctx* C, const gbfv_params* p)
{
    if (!C || !p || !paramsOk(*p)) return GBFV_ERR_ARG;
    if (p->linearizer != C->prm.linearizer) {
        setError("the linearizer is fixed when the context is created");
        return GBFV_ERR_UNSUPPORTED;
    }
    C->prm = *p;
    return GBFV_OK;
}

int gbfv_dims(const gbfv_ctx* C, int* n, int* b, int* nnz)
{
    if (!C) return GBFV_ERR_ARG;
    if (n) *n = C->N;
    if (b) *b = C->b;
    if (nnz) *nnz = (int)C->bcrsCol.size();
    return GBFV_OK;
}

int gbfv_set_solution(gbfv_ctx* C, const double* pv, const int32_t* meaning)
{
    if (!C || !pv) return GBFV_ERR_ARG;
    const int N = C->N, b = C->b;
    // black-oil: the gas meanings the model has (BlackOilPrimaryVariables::
    // GasMeaning without Disabled, blackoilprimaryvariables.hh:138-143)
    if (meaning && C->model == GBFV_MODEL_BLACKOIL_3P)
        for (int I = 0; I < N; ++I)
            if (meaning[I] != GBFV_GAS_SG && meaning[I] != GBFV_GAS_RS && meaning[I] != GBFV_GAS_RV) {
                setError("gas meaning of cell " + std::to_string(I) + " is not Sg, Rs or Rv");
                return GBFV_ERR_ARG;
            }
    std::vector<double> h((size_t)N * b);
    for (int I = 0; I < N; ++I)
        for (int e = 0; e < b; ++e) h[(size_t)C->perm[I] * b + e] = pv[(size_t)I * b + e];
    CK(cudaMemcpy(C->x, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(C->xOld, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice));
    std::vector<int> hm(N, 0);
    if (meaning)
        for (int I = 0; I < N; ++I) hm[C->perm[I]] = meaning[I];
    CK(cudaMemcpy(C->meaning, hm.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(C->meaningOld, hm.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    launchSetRefPressure(C->x, C->perm[0] * b, C->refP, C->stream);
    CK(cudaStreamSynchronize(C->stream));
    return GBFV_OK;
}

int gbfv_get_solution(gbfv_ctx* C, double* pv, int32_t* meaning)
{
    if (!C || !pv) return GBFV_ERR_ARG;
    const int N = C->N, b = C->b;
    std::vector<double> h((size_t)N * b);
    CK(cudaStreamSynchronize(C->stream));
    CK(cudaMemcpy(h.data(), C->x, sizeof(double) * h.size(), cudaMemcpyDeviceToHost));
    for (int I = 0; I < N; ++I)
        for (int e = 0; e < b; ++e) pv[(size_t)I * b + e] = h[(size_t)C->perm[I] * b + e];
    if (meaning) {
        std::vector<int> hm(N);
        CK(cudaMemcpy(hm.data(), C->meaning, sizeof(int) * N, cudaMemcpyDeviceToHost));
        for (int I = 0; I < N; ++I) meaning[I] = hm[C->perm[I]];
    }
    return GBFV_OK;
}

int gbfv_output_fields(gbfv_ctx* C, double* out)
{
    if (!C || !out) return GBFV_ERR_ARG;
    const int N = C->N;
    const size_t ld = C->ldN, n = (size_t)GBFV_OUTPUT_PLANES * ld;
    double* d = nullptr;
    int st;
    if ((st = devAlloc(&d, n))) return st;
    CK(cudaMemsetAsync(d, 0, sizeof(double) * n, C->stream));
    launchOutputFields(C->mesh, C->dphys, C->x, C->meaning, C->iq, d, C->stream);
    std::vector<double> h(n);
    const cudaError_t e = cudaMemcpyAsync(h.data(), d, sizeof(double) * n, cudaMemcpyDeviceToHost, C->stream);
    const cudaError_t e2 = cudaStreamSynchronize(C->stream);
    cudaFree(d);
    CK(e);
    CK(e2);
    for (int q = 0; q < GBFV_OUTPUT_PLANES; ++q)
        for (int I = 0; I < N; ++I) out[(size_t)q * N + I] = h[(size_t)q * ld + C->perm[I]];
    return GBFV_OK;
}

int gbfv_set_timestep(gbfv_ctx* C, double dt)
{
    if (!C || !(dt > 0)) return GBFV_ERR_ARG;
    C->dt = dt;
    return GBFV_OK;
}

int gbfv_set_newton_iteration(gbfv_ctx* C, int it)
{
    if (!C || it < 0) return GBFV_ERR_ARG;
    C->newtonIter = it;
    return GBFV_OK;
}

static void collectLinStats(gbfv_ctx* C)
{
    if (!C->linPending) return;
    float ms = 0;
    if (cudaEventElapsedTime(&ms, C->evL0, C->evL1) == cudaSuccess) {
        C->linMs += ms;
        C->linLaunches += 2;
        C->linBytes += C->linBytesPer;
    }
    C->linPending = 0;
}

// buffers of the finite-difference linearizer (once per context)
static int ensureFd(gbfv_ctx* C)
{
    if (C->fdX[0]) return GBFV_OK;
    const int b = C->b;
    const size_t ld = C->ldN, nv = iqValuePlanes(b), nd = iqDerivPlanes(b), ns = iqStoragePlanes(b);
    int st;
    for (int k = 0; k < b; ++k)
        for (IqBuffers* q : {&C->fd.plus[k], &C->fd.minus[k]})
            if ((st = devAlloc(&q->val, nv * ld)) || (st = devAlloc(&q->der, nd * ld)) ||
                (st = devAlloc(&q->sto, ns * ld)))
                return st;
    for (int k = 0; k < 2 * b; ++k)
        if ((st = devAlloc(&C->fdX[k], (size_t)C->N * b))) return st;
    return GBFV_OK;
}

static int linearizeImpl(gbfv_ctx* C)
{
    NvtxRange nr("gbfv linearize");
    collectLinStats(C);
    launchApplyConstraints(C->mesh, C->x, C->xOld, C->meaning, C->meaningOld, C->stream);
    if (C->prm.local_linearizer == GBFV_LIN_FD) {
        // FvBaseFdLocalLinearizer: the unperturbed intensive quantities, those
        // of the deflected states, then every element's columns
        int st = ensureFd(C);
        if (st) return st;
        const int method = C->prm.numeric_difference_method, b = C->b;
        cudaEventRecord(C->evL0, C->stream);
        launchIq(C->mesh, C->dphys, C->x, C->meaning, C->iq, C->stream);
        for (int pv = 0; pv < b; ++pv) {
            if (method >= 0) {
                launchFdDeflect(C->mesh, b, C->x, C->meaning, C->refP, pv, 1, C->fdX[pv], C->stream);
                launchIq(C->mesh, C->dphys, C->fdX[pv], C->meaning, C->fd.plus[pv], C->stream);
            }
            if (method <= 0) {
                launchFdDeflect(C->mesh, b, C->x, C->meaning, C->refP, pv, method == 0 ? 0 : -1, C->fdX[b + pv],
                                C->stream);
                launchIq(C->mesh, C->dphys, C->fdX[b + pv], C->meaning, C->fd.minus[pv], C->stream);
            }
        }
        if (C->vcfv)
            launchVcfvAssembleFd(C->vcfv, C->mesh, C->iq, C->fd, C->refP, method, C->storageOld, C->newtonIter == 0,
                                 C->dt, C->residual, C->jval, C->stream);
        else
            launchAssembleFd(C->mesh, C->dphys, C->iq, C->fd, C->meaning, C->refP, method, C->storageOld,
                             C->newtonIter == 0, C->dt, C->residual, C->jval, C->stream);
        cudaEventRecord(C->evL1, C->stream);
        C->linPending = 1;
        CK(cudaGetLastError());
        return GBFV_OK;
    }
    cudaEventRecord(C->evL0, C->stream);
    launchIq(C->mesh, C->dphys, C->x, C->meaning, C->iq, C->stream);
    if (C->vcfv)
        launchVcfvAssemble(C->vcfv, C->mesh, C->iq, C->storageOld, C->newtonIter == 0, C->dt, C->residual, C->jval,
                           C->stream);
    else
        launchAssemble(C->mesh, C->dphys, C->iq, C->storageOld, C->newtonIter == 0, C->dt, C->residual, C->jval,
                       C->stream);
    cudaEventRecord(C->evL1, C->stream);
    C->linPending = 1;
    CK(cudaGetLastError());
    return GBFV_OK;
}

int gbfv_linearize(gbfv_ctx* C)
{
    if (!C) return GBFV_ERR_ARG;
    int st = linearizeImpl(C);
    if (st) return st;
    CK(cudaStreamSynchronize(C->stream));
    return GBFV_OK;
}

int gbfv_get_residual(gbfv_ctx* C, double* r)
{
    if (!C || !r) return GBFV_ERR_ARG;
    const int N = C->N, b = C->b;
    std::vector<double> h((size_t)N * b);
    CK(cudaStreamSynchronize(C->stream));
    CK(cudaMemcpy(h.data(), C->residual, sizeof(double) * h.size(), cudaMemcpyDeviceToHost));
    for (int I = 0; I < N; ++I)
        for (int e = 0; e < b; ++e) r[(size_t)I * b + e] = h[(size_t)C->perm[I] * b + e];
    return GBFV_OK;
}

int gbfv_get_jacobian(gbfv_ctx* C, int32_t* rowPtr, int32_t* colIdx, double* blocks)
{
    if (!C) return GBFV_ERR_ARG;
    const int b = C->b, bb = b * b, ld = C->ldN;
    const size_t nval = (size_t)C->mesh.nslot * bb * ld;
    std::vector<double> h(nval);
    CK(cudaStreamSynchronize(C->stream));
    CK(cudaMemcpy(h.data(), C->jval, sizeof(double) * nval, cudaMemcpyDeviceToHost));
    if (rowPtr) std::copy(C->bcrsRowPtr.begin(), C->bcrsRowPtr.end(), rowPtr);
    if (colIdx) std::copy(C->bcrsCol.begin(), C->bcrsCol.end(), colIdx);
    if (blocks)
        for (size_t k = 0; k < C->bcrsCol.size(); ++k)
            for (int e = 0; e < bb; ++e)
                blocks[k * bb + e] = h[((size_t)C->bcrsSlot[k] * bb + e) * ld + C->bcrsRow[k]];
    return GBFV_OK;
}

static int newtonErrorImpl(gbfv_ctx* C, double* err)
{
    int st;
    if ((st = resetStatus(C->stream, C->st))) return st;
    launchNewtonError(C->mesh, C->residual, C->st, C->stream);
    if ((st = syncStatus(C->stream, C->st, C->hst))) return st;
    unsigned long long bits = C->hst->errorBits;
    std::memcpy(err, &bits, sizeof(double));
    if (C->hst->nonfinite) {
        *err = std::numeric_limits<double>::quiet_NaN();
        return GBFV_ERR_NONFINITE;
    }
    return GBFV_OK;
}

int gbfv_newton_error(gbfv_ctx* C, double* err)
{
    if (!C || !err) return GBFV_ERR_ARG;
    return newtonErrorImpl(C, err);
}

static int solveImpl(gbfv_ctx* C, int* iterations)
{
    NvtxRange nr("gbfv solve");
    const double ms0 = C->S.statMs, bytes0 = C->S.statBytes;
    int it = 0, ref = 0, st;
    if (C->prm.precision == GBFV_PREC_MIXED) {
        st = solveMixed(C->S, C->stream, C->st, C->hst, C->jval, C->residual, C->prm, it, ref);
        if (st == GBFV_OK || st == GBFV_ERR_NOT_CONVERGED)
            CK(cudaMemcpyAsync(C->dx, C->S.xref, sizeof(double) * C->N * C->b, cudaMemcpyDeviceToDevice,
                               C->stream));
    }
    else {
        st = solvePlain(C->S, C->stream, C->st, C->hst, C->jval, C->residual, C->prm, it);
        if (st == GBFV_OK || st == GBFV_ERR_NOT_CONVERGED)
            CK(cudaMemcpyAsync(C->dx, C->S.v64[0], sizeof(double) * C->N * C->b, cudaMemcpyDeviceToDevice,
                               C->stream));
    }
    C->lastIterations = it;
    C->lastRefinements = ref;
    if (iterations) *iterations = it;
    C->haveDx = 1;
    if (!C->solveLog.empty()) {
        // one JSON line per solve (GBFV_SOLVE_LOG): iterations, refinements,
        // the max-norm residual reduction reached and the residual (the FP64
        // true residual for the mixed form), device time and algorithmic
        // bytes of the solver launches
        const double ms = C->S.statMs - ms0, bytes = C->S.statBytes - bytes0;
        if (FILE* f = fopen(C->solveLog.c_str(), "a")) {
            fprintf(f,
                    "{\"cells\": %d, \"newton_iteration\": %d, \"precision\": \"%s\", \"status\": %d, "
                    "\"iterations\": %d, \"refinements\": %d, \"residual_reduction\": %.6g, \"residual\": %.6g, "
                    "\"solve_ms\": %.6g, \"bytes\": %.6g, \"achieved_gbs\": %.6g}\n",
                    C->N, C->newtonIter, C->prm.precision == GBFV_PREC_MIXED ? "mixed" : "fp64", st, it, ref,
                    C->S.lastReduction, C->S.lastResidual, ms, bytes, ms > 0 ? bytes / (ms * 1e6) : 0.0);
            fclose(f);
        }
    }
    return st;
}

int gbfv_solve(gbfv_ctx* C, double* dx, int* iterations)
{
    if (!C) return GBFV_ERR_ARG;
    const int st = solveImpl(C, iterations);
    if (dx) {
        const int N = C->N, b = C->b;
        std::vector<double> h((size_t)N * b);
        CK(cudaStreamSynchronize(C->stream));
        CK(cudaMemcpy(h.data(), C->dx, sizeof(double) * h.size(), cudaMemcpyDeviceToHost));
        for (int I = 0; I < N; ++I)
            for (int e = 0; e < b; ++e) dx[(size_t)I * b + e] = h[(size_t)C->perm[I] * b + e];
    }
    return st;
}

static int updateImpl(gbfv_ctx* C, int* switched)
{
    NvtxRange nr("gbfv update");
    int st;
    if ((st = resetStatus(C->stream, C->st))) return st;
    launchCheckUpdate(C->N * C->b, C->dx, C->st, C->stream);
    UpdateParams up;
    up.dsMax = C->prm.ds_max;
    up.dpMaxRel = C->prm.dp_max_rel;
    up.oscThreshold = C->prm.pv_oscillation_threshold;
    up.pMin = C->prm.pressure_min;
    up.pMax = C->prm.pressure_max;
    up.swMax = C->prm.max_water_saturation;
    up.waterOnly = C->prm.water_only_threshold;
    if ((st = syncStatus(C->stream, C->st, C->hst))) return st;
    if (C->hst->nonfinite) {
        setError("Non-finite update!");
        return GBFV_ERR_NONFINITE;
    }
    launchNewtonUpdate(C->mesh, C->dphys, C->dx, C->x, C->meaning, C->wasSwitched, up, C->st, C->stream);
    if (switched) {
        if ((st = syncStatus(C->stream, C->st, C->hst))) return st;
        *switched = C->hst->switched;
    }
    CK(cudaGetLastError());
    return GBFV_OK;
}

int gbfv_newton_update(gbfv_ctx* C, int* switched)
{
    if (!C || !C->haveDx) return GBFV_ERR_ARG;
    int st = updateImpl(C, switched);
    if (st) return st;
    CK(cudaStreamSynchronize(C->stream));
    return GBFV_OK;
}

void* gbfv_stream(gbfv_ctx* C) { return C ? (void*)C->stream : nullptr; }

}  // extern "C"

namespace gbfv {
void entitiesOf(const gbfv_ctx* C, int32_t& codim, int32_t& numElements)
{
    codim = C->vcfv ? C->dim : 0;
    numElements = C->vcfv ? C->numElements : 0;
}
}  // namespace gbfv

extern "C" {

int gbfv_save_state(gbfv_ctx* C)
{
    if (!C) return GBFV_ERR_ARG;
    CK(cudaMemcpyAsync(C->xSave, C->x, sizeof(double) * C->N * C->b, cudaMemcpyDeviceToDevice, C->stream));
    CK(cudaMemcpyAsync(C->meaningSave, C->meaning, sizeof(int) * C->N, cudaMemcpyDeviceToDevice, C->stream));
    CK(cudaMemcpyAsync(C->switchedSave, C->wasSwitched, sizeof(int) * C->N, cudaMemcpyDeviceToDevice, C->stream));
    CK(cudaStreamSynchronize(C->stream));
    return GBFV_OK;
}

int gbfv_restore_state(gbfv_ctx* C)
{
    if (!C) return GBFV_ERR_ARG;
    const size_t nb = sizeof(double) * C->N * C->b;
    CK(cudaMemcpyAsync(C->x, C->xSave, nb, cudaMemcpyDeviceToDevice, C->stream));
    CK(cudaMemcpyAsync(C->xOld, C->xSave, nb, cudaMemcpyDeviceToDevice, C->stream));
    CK(cudaMemcpyAsync(C->meaning, C->meaningSave, sizeof(int) * C->N, cudaMemcpyDeviceToDevice, C->stream));
    CK(cudaMemcpyAsync(C->meaningOld, C->meaningSave, sizeof(int) * C->N, cudaMemcpyDeviceToDevice, C->stream));
    CK(cudaMemcpyAsync(C->wasSwitched, C->switchedSave, sizeof(int) * C->N, cudaMemcpyDeviceToDevice, C->stream));
    return GBFV_OK;
}

int gbfv_get_kernel_stats(const gbfv_ctx* Cc, gbfv_kernel_stats* out)
{
    if (!Cc || !out) return GBFV_ERR_ARG;
    gbfv_ctx* C = const_cast<gbfv_ctx*>(Cc);
    cudaStreamSynchronize(C->stream);
    collectLinStats(C);
    out->solve_ms = C->S.statMs;
    out->solve_launches = C->S.statLaunches;
    out->solve_iterations = C->S.statIters;
    out->solve_factorizations = C->S.statFactor;
    out->solve_bytes = C->S.statBytes;
    out->linearize_ms = C->linMs;
    out->linearize_launches = C->linLaunches;
    out->linearize_bytes = C->linBytes;
    return GBFV_OK;
}

int gbfv_set_solver_config(gbfv_ctx* C, int precision, int mode, int blocks)
{
    const int base = mode & ~(SYNC_TILES | SYNC_NARROW);
    const int k = precision == GBFV_PREC_MIXED ? 1 : 0;
    if (!C || (base != SYNC_CLUSTER && base != SYNC_GRID && base != SYNC_HYBRID) || blocks < 1 ||
        (base == SYNC_GRID && mode != base) ||
        ((mode & SYNC_NARROW) && (base != SYNC_HYBRID || k != 1 || (mode & SYNC_TILES))))
        return GBFV_ERR_ARG;
    SolverData& S = C->S;
    if (S.gilu && !S.giluRoute && !S.giluWide) {
        setError("a vertex-centred context solves with the general block ILU(0) only");
        return GBFV_ERR_UNSUPPORTED;
    }
    const int maxH = (mode & SYNC_NARROW) ? S.maxHybridNarrow : S.maxHybrid[k];
    if (base == SYNC_CLUSTER && blocks > S.maxCluster[k]) return GBFV_ERR_UNSUPPORTED;
    if (base == SYNC_HYBRID && (blocks > maxH || blocks % HYBRID_CLUSTER || blocks <= HYBRID_CLUSTER))
        return GBFV_ERR_UNSUPPORTED;
    if (base == SYNC_GRID && blocks > S.maxGrid[k]) return GBFV_ERR_UNSUPPORTED;
    if (mode & SYNC_TILES) {
        const int c = base == SYNC_HYBRID ? HYBRID_CLUSTER : blocks;
        if (buildTileTables(S, c) != GBFV_OK) return GBFV_ERR_UNSUPPORTED;
        const bool fits = k ? tileFits<float>(S, clusterThreads<float>()) : tileFits<double>(S, clusterThreads<double>());
        if (!fits) return GBFV_ERR_UNSUPPORTED;
    }
    S.mode[k] = mode;
    S.nblk[k] = blocks;
    S.tuned[k] = 1;
    if (S.giluWide) {  // this precision now solves with the structured kernel
        S.giluUse &= ~(k ? 2 : 1);
        S.giluCand &= ~(k ? 2 : 1);
    }
    if (S.giluRoute || (S.giluWide && !S.giluCand)) {  // a forced configuration of the structured solver
        giluDestroy(S.gilu);
        S.gilu = nullptr;
        S.giluRoute = S.giluWide = false;
    }
    return GBFV_OK;
}

int gbfv_solver_config(const gbfv_ctx* C, int precision, int* mode, int* blocks, double* tuneMs, int* nt)
{
    if (!C) return GBFV_ERR_ARG;
    const int k = precision == GBFV_PREC_MIXED ? 1 : 0;
    const SolverData& S = C->S;
    if (S.gilu && (!S.giluWide || (S.giluUse & (k ? 2 : 1)))) {
        // the general block ILU(0) kernel
        if (mode) *mode = GBFV_SOLVER_GILU | (giluTagged(S.gilu, !k) ? GBFV_SOLVER_TAGGED : 0);
        if (blocks) *blocks = giluBlocks(S.gilu);
        if (nt) *nt = 0;
        return GBFV_OK;
    }
    if (mode) *mode = C->S.mode[k];
    if (blocks) *blocks = C->S.nblk[k];
    int n = 0;
    for (int i = 0; i < 16; ++i)
        if (C->S.tuneMs[k][i] > 0) n = i + 1;
    if (tuneMs)
        for (int i = 0; i < n; ++i) tuneMs[i] = C->S.tuneMs[k][i];
    if (nt) *nt = n;
    return GBFV_OK;
}

int gbfv_solver_phase_ns(gbfv_ctx* C, unsigned long long* ns8)
{
    if (!C || !ns8) return GBFV_ERR_ARG;
    if (!C->S.prof) { std::memset(ns8, 0, 8 * sizeof(unsigned long long)); return GBFV_OK; }
    CK(cudaStreamSynchronize(C->stream));
    CK(cudaMemcpy(ns8, C->S.prof, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    CK(cudaMemset(C->S.prof, 0, 8 * sizeof(unsigned long long)));
    return GBFV_OK;
}

int gbfv_solver_level_cycles(gbfv_ctx* C, unsigned long long* c8)
{
    if (!C || !c8) return GBFV_ERR_ARG;
    if (!C->S.prof) { std::memset(c8, 0, 8 * sizeof(unsigned long long)); return GBFV_OK; }
    CK(cudaStreamSynchronize(C->stream));
    CK(cudaMemcpy(c8, C->S.prof + 8, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    CK(cudaMemset(C->S.prof + 8, 0, 8 * sizeof(unsigned long long)));
    return GBFV_OK;
}

int gbfv_reset_kernel_stats(gbfv_ctx* C)
{
    if (!C) return GBFV_ERR_ARG;
    cudaStreamSynchronize(C->stream);
    C->linPending = 0;
    C->linMs = C->linBytes = 0;
    C->linLaunches = 0;
    C->S.statMs = C->S.statBytes = 0;
    C->S.statLaunches = C->S.statIters = C->S.statFactor = 0;
    return GBFV_OK;
}

int gbfv_phase_times(const gbfv_ctx* C, double* ms4)
{
    if (!C || !ms4) return GBFV_ERR_ARG;
    for (int i = 0; i < 4; ++i) ms4[i] = C->phaseMs[i];
    return GBFV_OK;
}

int gbfv_newton_apply(gbfv_ctx* C, double dt, gbfv_newton_report* rep)
{
    if (!C || !(dt > 0)) return GBFV_ERR_ARG;
    NvtxRange nr("gbfv newton_apply");
    gbfv_newton_report r;
    std::memset(&r, 0, sizeof(r));
    C->dt = dt;
    C->numIterations = 0;
    C->error = 0;
    C->lastError = 0;
    // FvBaseDiscretization::update -> updateBegin (the reference pressure of
    // the finite-difference linearizer) before NewtonMethod::apply
    if (C->prm.local_linearizer == GBFV_LIN_FD) launchSetRefPressure(C->x, C->perm[0] * C->b, C->refP, C->stream);
    const gbfv_params& prm = C->prm;
    auto converged = [&]() { return C->error <= prm.newton_tolerance; };
    auto proceed = [&]() {
        if (C->numIterations < 1) return true;
        if (converged()) return false;
        if (C->numIterations >= prm.newton_max_iterations) return C->error * 4.0 < C->lastError;
        return true;
    };
    for (int i = 0; i < 4; ++i) C->phaseMs[i] = 0;
    int status = GBFV_OK;
    bool failed = false;
    while (proceed()) {
        C->lastError = C->error;
        C->newtonIter = C->numIterations;
        cudaEventRecord(C->ev[0], C->stream);
        if ((status = linearizeImpl(C))) { failed = true; break; }
        cudaEventRecord(C->ev[1], C->stream);
        r.linearizations++;
        C->lastError = C->error;
        double err = 0;
        status = newtonErrorImpl(C, &err);
        C->error = err;
        if (status) { failed = true; break; }
        if (C->error > prm.newton_max_error) { status = GBFV_ERR_NUMERICAL; failed = true; break; }
        float ms = 0;
        cudaEventElapsedTime(&ms, C->ev[0], C->ev[1]);
        C->phaseMs[0] += ms;
        if (!proceed()) { C->numIterations++; break; }
        cudaEventRecord(C->ev[2], C->stream);
        int it = 0;
        status = solveImpl(C, &it);
        cudaEventRecord(C->ev[3], C->stream);
        r.linear_iterations += it;
        r.refinements += C->lastRefinements;
        if (status) { failed = true; break; }
        status = updateImpl(C, nullptr);
        cudaEventRecord(C->ev[4], C->stream);
        if (status) { failed = true; break; }
        cudaEventSynchronize(C->ev[4]);
        cudaEventElapsedTime(&ms, C->ev[2], C->ev[3]);
        C->phaseMs[2] += ms;
        cudaEventElapsedTime(&ms, C->ev[3], C->ev[4]);
        C->phaseMs[3] += ms;
        C->numIterations++;
    }
    if (!failed && !converged()) {
        failed = true;
        status = GBFV_ERR_NOT_CONVERGED;
    }
    if (failed) {
        C->numIterations = prm.newton_target_iterations * 2;
        // FvBaseDiscretization::updateFailed: solution(0) = solution(1)
        cudaMemcpyAsync(C->x, C->xOld, sizeof(double) * C->N * C->b, cudaMemcpyDeviceToDevice, C->stream);
        cudaMemcpyAsync(C->meaning, C->meaningOld, sizeof(int) * C->N, cudaMemcpyDeviceToDevice, C->stream);
        cudaStreamSynchronize(C->stream);
    }
    else
        r.converged = 1;
    r.iterations = C->numIterations;
    r.status = failed ? status : GBFV_OK;
    r.error = C->error;
    if (rep) *rep = r;
    return failed ? status : GBFV_OK;
}

double gbfv_suggest_time_step(const gbfv_ctx* C, double oldDt, int n)
{
    const int target = C->prm.newton_target_iterations;
    if (n > target) {
        const double percent = double(n - target) / target;
        return std::max(C->prm.min_time_step, oldDt / (1.0 + percent));
    }
    const double percent = double(target - n) / target;
    return std::max(C->prm.min_time_step, oldDt * (1.0 + percent / 1.2));
}

int gbfv_time_integration(gbfv_ctx* C, int numSteps, double dt0, double endTime, int fixedDt, double* stepDt,
                          int32_t* stepNewton, int32_t* stepLinear, int32_t* totalLin)
{
    if (!C || numSteps < 0 || !(dt0 > 0)) return GBFV_ERR_ARG;
    double dt = dt0, t = 0.0;
    int lin = 0;
    for (int step = 0; step < numSteps; ++step) {
        if (t >= endTime) break;
        bool ok = false;
        gbfv_newton_report rep;
        int linIt = 0;
        const int maxFails = C->prm.max_time_step_divisions;
        for (int i = 0; i < maxFails; ++i) {
            const int st = gbfv_newton_apply(C, dt, &rep);
            linIt += rep.linear_iterations;
            lin += rep.linearizations;
            ok = st == GBFV_OK;
            if (ok) break;
            if (st == GBFV_ERR_CUDA || st == GBFV_ERR_TIMEOUT || st == GBFV_ERR_OOM) return st;
            double nextDt = dt / 2.0;
            if (dt < C->prm.min_time_step * (1 + 1e-9)) return GBFV_ERR_NOT_CONVERGED;
            if (nextDt < C->prm.min_time_step) nextDt = C->prm.min_time_step;
            dt = nextDt;
        }
        if (!ok) return GBFV_ERR_NOT_CONVERGED;
        if (stepDt) stepDt[step] = dt;
        if (stepNewton) stepNewton[step] = C->numIterations;
        if (stepLinear) stepLinear[step] = linIt;
        // advanceTimeLevel: solution(1) = solution(0)
        CK(cudaMemcpyAsync(C->xOld, C->x, sizeof(double) * C->N * C->b, cudaMemcpyDeviceToDevice, C->stream));
        CK(cudaMemcpyAsync(C->meaningOld, C->meaning, sizeof(int) * C->N, cudaMemcpyDeviceToDevice, C->stream));
        t += dt;
        if (fixedDt) {
            dt = dt0;
            continue;
        }
        const double maxTs = std::max(0.0, endTime - t);
        double dtNext = std::min(C->prm.max_time_step, gbfv_suggest_time_step(C, dt, C->numIterations));
        if (dtNext < maxTs && maxTs < dtNext * 2) dtNext = maxTs / 2 * 1.01;
        dt = std::min(maxTs, dtNext);
    }
    CK(cudaStreamSynchronize(C->stream));
    if (totalLin) *totalLin = lin;
    return GBFV_OK;
}

// ============================================================ linsolver
gbfv_linsolver* gbfv_linsolver_create(int n, int b, const int32_t* rowPtr, const int32_t* col,
                                      const gbfv_params* params, int* status)
{
    auto fail = [&](gbfv_linsolver* L, int st) -> gbfv_linsolver* {
        if (status) *status = st;
        if (L) gbfv_linsolver_destroy(L);
        return nullptr;
    };
    if (n <= 0 || (b != 2 && b != 3) || !rowPtr || !col || (params && !paramsOk(*params)))
        return fail(nullptr, GBFV_ERR_ARG);
    if (n > GBFV_MAX_CELLS) {
        setError("more block rows than GBFV_MAX_CELLS (32-bit device indexing)");
        return fail(nullptr, GBFV_ERR_UNSUPPORTED);
    }
    // row pointers and column indices first: everything below follows them
    if (rowPtr[0] != 0) {
        setError("row_ptr[0] must be 0");
        return fail(nullptr, GBFV_ERR_ARG);
    }
    for (int i = 0; i < n; ++i)
        if (rowPtr[i + 1] < rowPtr[i]) {
            setError("row_ptr decreases at row " + std::to_string(i));
            return fail(nullptr, GBFV_ERR_ARG);
        }
    for (int k = 0; k < rowPtr[n]; ++k)
        if (col[k] < 0 || col[k] >= n) {
            setError("column index out of range at entry " + std::to_string(k));
            return fail(nullptr, GBFV_ERR_ARG);
        }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(nullptr, GBFV_ERR_NO_DEVICE);
    gbfv_linsolver* L = new gbfv_linsolver();
    if (params) L->prm = *params;
    else gbfv_default_params(&L->prm);
    L->N = n;
    L->b = b;
    L->rowPtr.assign(rowPtr, rowPtr + n + 1);
    L->colN.assign(col, col + rowPtr[n]);
    // slots from the distinct column offsets (symmetric, at most 7)
    std::vector<int> offs;
    for (int i = 0; i < n; ++i)
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k) offs.push_back(col[k] - i);
    std::sort(offs.begin(), offs.end());
    offs.erase(std::unique(offs.begin(), offs.end()), offs.end());
    const int nslot = (int)offs.size();
    if (nslot > GILU_MAX_SLOTS || nslot % 2 == 0) {
        setError("pattern needs at most 27 symmetric offsets");
        return fail(L, GBFV_ERR_UNSUPPORTED);
    }
    // patterns beyond the 5/7-point stencil's (more offsets, or ILU(0) fill
    // interactions) go to the general block ILU(0)
    bool general = nslot > MAX_SLOTS;
    const int dim = general ? 1 : nslot / 2;
    for (int s = 0; s < nslot; ++s)
        if (offs[s] != -offs[nslot - 1 - s]) { setError("asymmetric pattern offsets"); return fail(L, GBFV_ERR_UNSUPPORTED); }
    auto slotOf = [&](int off) { return (int)(std::lower_bound(offs.begin(), offs.end(), off) - offs.begin()); };
    std::vector<std::vector<int>> lower(n);
    for (int i = 0; i < n; ++i) {
        bool diag = false;
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k) {
            if (col[k] < i) lower[i].push_back(col[k]);
            if (col[k] == i) diag = true;
            if (k > rowPtr[i] && col[k] <= col[k - 1]) { setError("columns must be sorted"); return fail(L, GBFV_ERR_ARG); }
        }
        if (!diag) { setError("diagonal entry missing"); return fail(L, GBFV_ERR_ARG); }
    }
    // ILU(0) update structure: does a lower entry update more than the diagonal?
    for (int i = 0; i < n && !general; ++i)
        for (int k : lower[i])
            for (int kk = rowPtr[k]; kk < rowPtr[k + 1]; ++kk) {
                const int j = col[kk];
                if (j <= k || j == i) continue;
                for (int q = rowPtr[i]; q < rowPtr[i + 1]; ++q)
                    if (col[q] == j) general = true;
            }
    std::vector<int> levPtr;
    buildOrder(n, lower, L->perm, L->iperm, levPtr);
    const int ld = ((n + 63) / 64) * 64;
    std::vector<int> hCol((size_t)nslot * ld, -1);
    L->entSlot.resize(L->colN.size());
    L->entRow.resize(L->colN.size());
    for (int i = 0; i < n; ++i)
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k) {
            const int s = slotOf(col[k] - i);
            hCol[(size_t)s * ld + L->perm[i]] = L->perm[col[k]];
            L->entSlot[k] = s;
            L->entRow[k] = L->perm[i];
        }
    // every (i,k) lower entry must have its mirror (k,i)
    for (int i = 0; i < n; ++i)
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k) {
            const int j = col[k];
            bool found = false;
            for (int q = rowPtr[j]; q < rowPtr[j + 1]; ++q) found |= col[q] == i;
            if (!found) { setError("structurally asymmetric matrix"); return fail(L, GBFV_ERR_UNSUPPORTED); }
        }
    SolverData& S = L->S;
    S.N = n;
    S.b = b;
    S.dim = dim;
    S.nslot = nslot;
    S.ldN = ld;
    S.levPtr = levPtr;
    S.adjacentLevels = adjacentLevels(lower, L->perm, levPtr);
    S.colHost = hCol;
    S.natural = L->iperm;
    int st;
    if ((st = upload(&S.col, hCol)) || (st = upload(&S.levPtrD, levPtr)) || (st = allocSolver(S)))
        return fail(L, st);
    if (general) {
        S.gilu = giluCreate(n, b, nslot, ld, hCol, S.col, levPtr, &st);
        if (!S.gilu) return fail(L, st);
    }
    const size_t nval = (size_t)nslot * b * b * ld;
    if ((st = devAlloc(&L->A64, nval)) || (st = devAlloc(&L->rhs, (size_t)n * b)) || (st = devAlloc(&L->st, 1)))
        return fail(L, st);
    if (cudaMallocHost((void**)&L->hst, sizeof(DevStatus)) != cudaSuccess ||
        cudaMallocHost((void**)&L->A64host, sizeof(double) * nval) != cudaSuccess ||
        cudaMallocHost((void**)&L->stage, sizeof(double) * (size_t)n * b) != cudaSuccess ||
        cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(L, GBFV_ERR_CUDA);
    std::memset(L->A64host, 0, sizeof(double) * nval);
    if (status) *status = GBFV_OK;
    return L;
}

int gbfv_linsolver_destroy(gbfv_linsolver* L)
{
    if (!L) return GBFV_ERR_ARG;
    freeSolver(L->S);
    cudaFree(L->A64);
    cudaFree(L->rhs);
    cudaFree(L->st);
    if (L->hst) cudaFreeHost(L->hst);
    if (L->A64host) cudaFreeHost(L->A64host);
    if (L->stage) cudaFreeHost(L->stage);
    if (L->stream) cudaStreamDestroy(L->stream);
    delete L;
    return GBFV_OK;
}

int gbfv_linsolver_set_matrix(gbfv_linsolver* L, const double* blocks)
{
    if (!L || !blocks) return GBFV_ERR_ARG;
    const int bb = L->b * L->b, ld = L->S.ldN;
    for (size_t k = 0; k < L->colN.size(); ++k)
        for (int e = 0; e < bb; ++e)
            L->A64host[((size_t)L->entSlot[k] * bb + e) * ld + L->entRow[k]] = blocks[k * bb + e];
    CK(cudaMemcpyAsync(L->A64, L->A64host, sizeof(double) * (size_t)L->S.nslot * bb * ld, cudaMemcpyHostToDevice,
                       L->stream));
    return GBFV_OK;
}

int gbfv_linsolver_solve(gbfv_linsolver* L, const double* rhs, double* x, int* iterations)
{
    if (!L || !rhs || !x) return GBFV_ERR_ARG;
    const int n = L->N, b = L->b;
    for (int i = 0; i < n; ++i)
        for (int e = 0; e < b; ++e) L->stage[(size_t)L->perm[i] * b + e] = rhs[(size_t)i * b + e];
    CK(cudaMemcpyAsync(L->rhs, L->stage, sizeof(double) * n * b, cudaMemcpyHostToDevice, L->stream));
    int it = 0, ref = 0, st;
    const double* out;
    if (L->prm.precision == GBFV_PREC_MIXED) {
        st = solveMixed(L->S, L->stream, L->st, L->hst, L->A64, L->rhs, L->prm, it, ref);
        out = L->S.xref;
    }
    else {
        st = solvePlain(L->S, L->stream, L->st, L->hst, L->A64, L->rhs, L->prm, it);
        out = L->S.v64[0];
    }
    if (iterations) *iterations = it;
    CK(cudaMemcpyAsync(L->stage, out, sizeof(double) * n * b, cudaMemcpyDeviceToHost, L->stream));
    CK(cudaStreamSynchronize(L->stream));
    for (int i = 0; i < n; ++i)
        for (int e = 0; e < b; ++e) x[(size_t)i * b + e] = L->stage[(size_t)L->perm[i] * b + e];
    return st;
}

// The AMG hierarchy of a context (0 levels before its first AMG solve)
int gbfv_amg_levels(gbfv_ctx* C, int32_t* sizes, int32_t* colors)
{
    if (!C || !sizes) return -GBFV_ERR_ARG;
    if (!C->S.amg) return 0;
    int sz[AMG_MAX_LEVELS], co[AMG_MAX_LEVELS];
    const int n = amgLevelSizes(C->S.amg, sz);
    amgLevelColors(C->S.amg, co);
    for (int l = 0; l < n; ++l) {
        sizes[l] = sz[l];
        if (colors) colors[l] = co[l];
    }
    return n;
}

// The AMG hierarchy of the linear solver (built from the matrix last set
// when there is none yet): rows and colours of every level
int gbfv_linsolver_amg_levels(gbfv_linsolver* L, int32_t* sizes, int32_t* colors)
{
    if (!L || !sizes) return -GBFV_ERR_ARG;
    int st = ensureAmg(L->S, L->stream, L->A64, L->prm);
    if (st) return -st;
    int sz[AMG_MAX_LEVELS], co[AMG_MAX_LEVELS];
    const int n = amgLevelSizes(L->S.amg, sz);
    amgLevelColors(L->S.amg, co);
    for (int l = 0; l < n; ++l) {
        sizes[l] = sz[l];
        if (colors) colors[l] = co[l];
    }
    return n;
}

// one FP64 V-cycle of the AMG preconditioner, v = M^-1 d (natural order)
int gbfv_linsolver_ilu0_apply(gbfv_linsolver* L, const double* d, double* v)
{
    if (!L || !d || !v) return GBFV_ERR_ARG;
    if (!L->S.gilu) {
        setError("the matrix's pattern uses the structured ILU(0) solver, which has no separate apply");
        return GBFV_ERR_UNSUPPORTED;
    }
    const int n = L->N, b = L->b;
    for (int i = 0; i < n; ++i)
        for (int e = 0; e < b; ++e) L->stage[(size_t)L->perm[i] * b + e] = d[(size_t)i * b + e];
    CK(cudaMemcpyAsync(L->rhs, L->stage, sizeof(double) * n * b, cudaMemcpyHostToDevice, L->stream));
    int st = giluApply64(L->S.gilu, L->A64, L->rhs, L->S.v64[0], L->stream, L->st, L->hst);
    if (st) return st;
    CK(cudaMemcpyAsync(L->stage, L->S.v64[0], sizeof(double) * n * b, cudaMemcpyDeviceToHost, L->stream));
    CK(cudaStreamSynchronize(L->stream));
    for (int i = 0; i < n; ++i)
        for (int e = 0; e < b; ++e) v[(size_t)i * b + e] = L->stage[(size_t)L->perm[i] * b + e];
    return GBFV_OK;
}

int gbfv_linsolver_amg_apply(gbfv_linsolver* L, const double* d, double* v)
{
    if (!L || !d || !v) return GBFV_ERR_ARG;
    int st = ensureAmg(L->S, L->stream, L->A64, L->prm);
    if (st) return st;
    const int n = L->N, b = L->b;
    for (int i = 0; i < n; ++i)
        for (int e = 0; e < b; ++e) L->stage[(size_t)L->perm[i] * b + e] = d[(size_t)i * b + e];
    CK(cudaMemcpyAsync(L->rhs, L->stage, sizeof(double) * n * b, cudaMemcpyHostToDevice, L->stream));
    st = amgApply64(L->S.amg, L->A64, L->rhs, L->S.v64[0], L->stream, L->st, L->hst);
    if (st) return st;
    CK(cudaMemcpyAsync(L->stage, L->S.v64[0], sizeof(double) * n * b, cudaMemcpyDeviceToHost, L->stream));
    CK(cudaStreamSynchronize(L->stream));
    for (int i = 0; i < n; ++i)
        for (int e = 0; e < b; ++e) v[(size_t)i * b + e] = L->stage[(size_t)L->perm[i] * b + e];
    return GBFV_OK;
}

}  // extern "C"

// ================================================================ batch
// Many independent systems (ensemble realizations, served requests) advanced
// together.  Each system keeps its own context (device state, storage cache,
// solver data); the batch runs rounds, and in each round every system that
// needs it goes through one step of its own Newton / time-step state machine
// -- the same decisions as gbfv_newton_apply and gbfv_time_integration -- with
// the device work of all systems issued as one batched launch per phase:
//   L  constraints + intensive quantities + assembly + Newton error
//   S  FP64 residual, FP32 factorization + BiCGStab (one persistent launch,
//      clusters take systems from a work queue), refinement
//   U  update guard, Newton update with chopping / switching
// Each phase is a captured CUDA graph, replayed every round; which systems
// take part is data (an active flag per system), so the graphs never change.
// Every system runs the same device code as alone, with the same solver
// launch configuration, so its result does not depend on the batch.
namespace {

enum SysPhase { PH_LIN = 0, PH_SOLVE = 1, PH_UPDATE = 2, PH_DONE = 3, PH_FAILED = 4, PH_IDLE = 5 };

struct SysState {
    int phase = PH_IDLE;
    int status = GBFV_OK;
    // time integration
    int numSteps = 0, step = 0, fixedDt = 0, fails = 0, linItStep = 0, linearizations = 0;
    double dt = 0, dt0 = 0, t = 0, endTime = 1e100;
    std::vector<double> stepDt;
    std::vector<int> stepNewton, stepLinear;
    // Newton
    int numIterations = 0;
    double error = 0, lastError = 0;
    // mixed-precision refinement of the current solve
    double resErr = 0, resErr0 = 0;
    int solveIters = 0, refs = 0, lastKs = GBFV_OK, lastIt = 0, solveDone = 0, solveStatus = GBFV_OK;
};

struct GraphSet {
    cudaGraphExec_t exec = nullptr;
    int kernels = 0;
};

}  // namespace

struct gbfv_batch {
    int K = 0, b = 0, model = 0, precision = GBFV_PREC_MIXED;
    int dynamic = 0;          // slots admitted and released while running (serving)
    int maxCells = 0;         // largest admissible system of a dynamic batch
    int64_t footprint = 0;    // estimated device bytes of the admitted systems
    gbfv_params prm;
    cudaStream_t stream = nullptr;
    std::vector<gbfv_ctx*> ctx;
    std::vector<SysState> sys;
    int cluster = 0, numClusters = 1, maxLev = 1, gxLin = 16, gxSol = 16;
    // device tables and their pinned host mirrors
    LinJob* dLin = nullptr;
    SolveJob* dSol = nullptr;
    JobState *dJs = nullptr, *hJs = nullptr;
    int *dAct = nullptr, *hAct = nullptr;          // systems taking part in a solve phase
    DevStatus *dSt = nullptr, *hSt = nullptr;
    KArgs<float> *dK32 = nullptr, *hK32 = nullptr;
    KArgs<double> *dK64 = nullptr, *hK64 = nullptr;
    int *dOrder = nullptr, *hOrder = nullptr;      // [K] order, then the count at [K]
    int* dQueue = nullptr;
    GraphSet gLin, gCheck, gUpd, gRes0, gKry, gRef;
    // the whole Newton round as one graph: every phase and the per-system
    // decisions between them on the device (batchround.cu)
    RoundSys *dRound = nullptr, *hRound = nullptr;
    GraphSet gRound;
    int roundRefinements = 1;            // refinement launches captured in the round graph
    std::vector<cudaEvent_t> roundEv;    // [0,1] linearization, [2+2r, 3+2r] Krylov launch r
    int deviceRound = 1;                 // 0: the host-driven round (phase graphs, host decisions)
    UpdateParams up{};
    cudaEvent_t evA = nullptr, evB = nullptr;
    // statistics
    int64_t rounds = 0, graphLaunches = 0, kernelLaunches = 0;
    double solveMs = 0, solveBytes = 0, linMs = 0;
    int64_t solveLaunches = 0;
};

namespace {

template <class T>
int pinnedAlloc(T** p, size_t n)
{
    *p = nullptr;
    CK(cudaMallocHost((void**)p, sizeof(T) * std::max<size_t>(n, 1)));
    std::memset(*p, 0, sizeof(T) * std::max<size_t>(n, 1));
    return GBFV_OK;
}

// capture the work that fn issues on the batch stream into an executable graph
template <class F>
int captureGraph(gbfv_batch* B, GraphSet& g, F&& fn)
{
    struct CountScope {
        CountScope() { t_captureLaunches = 0; }
        ~CountScope() { t_captureLaunches = -1; }
    } scope;
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
    const int st = fn();
    const cudaError_t e = cudaStreamEndCapture(B->stream, &graph);
    if (st != GBFV_OK) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    CK(e);
    const cudaError_t ei = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    CK(ei);
    g.kernels = t_captureLaunches;  // counted when the graph is replayed
    return GBFV_OK;
}

int replay(gbfv_batch* B, GraphSet& g, bool sync)
{
    CK(cudaGraphLaunch(g.exec, B->stream));
    g_launches += g.kernels;
    B->kernelLaunches += g.kernels;
    B->graphLaunches++;
    if (sync) CK(cudaStreamSynchronize(B->stream));
    return GBFV_OK;
}

double bitsToDouble(unsigned long long bits)
{
    double v;
    std::memcpy(&v, &bits, sizeof(v));
    return v;
}

RoundParams roundParams(const gbfv_batch* B)
{
    const gbfv_params& prm = B->prm;
    RoundParams p{};
    p.newtonTol = prm.newton_tolerance;
    p.newtonMaxError = prm.newton_max_error;
    p.linTol = prm.linear_tolerance;
    p.absTol = absTolOf(prm);
    p.innerTol = prm.inner_tolerance;
    p.linMaxError = prm.linear_max_error;
    p.newtonMaxIt = prm.newton_max_iterations;
    p.linMaxIt = prm.linear_max_iterations;
    p.mixed = B->precision == GBFV_PREC_MIXED ? 1 : 0;
    return p;
}

// One Newton round of every system as one graph (the decisions of
// batchRound, made on the device by batchround.cu): per-system state in,
// linearize + Newton error, decide; mixed: FP32 matrix and FP64 residual,
// decide; the Krylov launch and, mixed, up to max_refinements refinement
// launches, each followed by its decision (a launch with an empty queue
// returns at once); update guard, decide; Newton update, decide; time level;
// per-system state out.
int buildRoundGraph(gbfv_batch* B)
{
    const int K = B->K;
    cudaStream_t s = B->stream;
    if (B->gRound.exec) {
        cudaGraphExecDestroy(B->gRound.exec);
        B->gRound.exec = nullptr;
    }
    const RoundParams p = roundParams(B);
    const bool mixed = p.mixed != 0;
    B->roundRefinements = mixed ? std::max(1, B->prm.max_refinements) : 1;
    const int nev = 2 + 2 * B->roundRefinements;
    while ((int)B->roundEv.size() < nev) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        B->roundEv.push_back(e);
    }
    return captureGraph(B, B->gRound, [&]() -> int {
        CK(cudaMemcpyAsync(B->dRound, B->hRound, sizeof(RoundSys) * K, cudaMemcpyHostToDevice, s));
        if (mixed) CK(cudaMemcpyAsync(B->dK32, B->hK32, sizeof(KArgs<float>) * K, cudaMemcpyHostToDevice, s));
        else CK(cudaMemcpyAsync(B->dK64, B->hK64, sizeof(KArgs<double>) * K, cudaMemcpyHostToDevice, s));
        launchRoundBegin(B->dRound, B->dJs, B->dSt, K, s);
        CK(cudaEventRecordWithFlags(B->roundEv[0], s, cudaEventRecordExternal));
        launchBatchLinearize(B->dLin, B->dJs, K, B->gxLin, s);
        launchBatchNewtonError(B->dLin, B->dJs, K, B->gxLin, s);
        CK(cudaEventRecordWithFlags(B->roundEv[1], s, cudaEventRecordExternal));
        launchRoundAfterLin(B->dRound, B->dJs, B->dSt, B->dAct, B->dK32, B->dK64, B->dSol, B->dOrder, B->dQueue, p,
                            K, s);
        if (mixed) {
            launchBatchCast(B->dSol, B->dAct, K, B->gxSol, s);
            launchBatchZeroX(B->dSol, B->dAct, K, B->gxSol, s);
            launchBatchResidual64(B->dSol, B->dAct, K, B->gxSol, B->b, s);
            launchRoundAfterRes0(B->dRound, B->dSt, B->dAct, B->dK32, B->dSol, B->dOrder, B->dQueue, p, K, s);
        }
        for (int r = 0; r < B->roundRefinements; ++r) {
            CK(cudaEventRecordWithFlags(B->roundEv[2 + 2 * r], s, cudaEventRecordExternal));
            int ls;
            if (mixed)
                ls = launchBicgstabBatch<float>(B->dK32, B->dOrder, B->dOrder + K, B->dQueue, B->b, B->cluster,
                                                B->numClusters, B->maxLev, s);
            else
                ls = launchBicgstabBatch<double>(B->dK64, B->dOrder, B->dOrder + K, B->dQueue, B->b, B->cluster,
                                                 B->numClusters, B->maxLev, s);
            if (ls) return ls;
            CK(cudaEventRecordWithFlags(B->roundEv[3 + 2 * r], s, cudaEventRecordExternal));
            launchRoundAfterKrylov(B->dRound, B->dSt, B->dAct, p, K, s);
            if (mixed) {
                launchBatchAccumulate(B->dSol, B->dAct, K, B->gxSol, s);
                launchBatchResidual64(B->dSol, B->dAct, K, B->gxSol, B->b, s);
                launchRoundAfterRefine(B->dRound, B->dSt, B->dAct, B->dK32, B->dSol, B->dOrder, B->dQueue, p, K,
                                       r + 1 == B->roundRefinements, s);
            }
        }
        launchRoundBeforeCheck(B->dRound, B->dJs, B->dSt, K, s);
        launchBatchCheckUpdate(B->dLin, B->dJs, K, B->gxLin, s);
        launchRoundAfterCheck(B->dRound, B->dJs, B->dSt, K, s);
        launchBatchNewtonUpdate(B->dLin, B->dJs, K, B->gxLin, B->up, s);
        launchRoundAfterUpdate(B->dRound, B->dJs, p, K, s);
        launchRoundTimeLevel(B->dRound, B->dLin, K, B->gxLin, s);
        CK(cudaMemcpyAsync(B->hRound, B->dRound, sizeof(RoundSys) * K, cudaMemcpyDeviceToHost, s));
        return GBFV_OK;
    });
}

int buildBatchGraphs(gbfv_batch* B)
{
    const int K = B->K;
    for (GraphSet* g : {&B->gLin, &B->gCheck, &B->gUpd, &B->gRes0, &B->gKry, &B->gRef})
        if (g->exec) {
            cudaGraphExecDestroy(g->exec);
            g->exec = nullptr;
        }
    cudaStream_t s = B->stream;
    int st;
    // L: constraints, IQ, assembly, Newton error; statuses to the host
    st = captureGraph(B, B->gLin, [&]() -> int {
        CK(cudaMemcpyAsync(B->dJs, B->hJs, sizeof(JobState) * K, cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(B->dSt, 0, sizeof(DevStatus) * K, s));
        launchBatchLinearize(B->dLin, B->dJs, K, B->gxLin, s);
        launchBatchNewtonError(B->dLin, B->dJs, K, B->gxLin, s);
        CK(cudaMemcpyAsync(B->hSt, B->dSt, sizeof(DevStatus) * K, cudaMemcpyDeviceToHost, s));
        return GBFV_OK;
    });
    if (st) return st;
    // U1: update guard
    st = captureGraph(B, B->gCheck, [&]() -> int {
        CK(cudaMemcpyAsync(B->dJs, B->hJs, sizeof(JobState) * K, cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(B->dSt, 0, sizeof(DevStatus) * K, s));
        launchBatchCheckUpdate(B->dLin, B->dJs, K, B->gxLin, s);
        CK(cudaMemcpyAsync(B->hSt, B->dSt, sizeof(DevStatus) * K, cudaMemcpyDeviceToHost, s));
        return GBFV_OK;
    });
    if (st) return st;
    // U2: Newton update
    st = captureGraph(B, B->gUpd, [&]() -> int {
        CK(cudaMemcpyAsync(B->dJs, B->hJs, sizeof(JobState) * K, cudaMemcpyHostToDevice, s));
        launchBatchNewtonUpdate(B->dLin, B->dJs, K, B->gxLin, B->up, s);
        return GBFV_OK;
    });
    if (st) return st;
    if (B->precision == GBFV_PREC_MIXED) {
        // S0: FP32 matrix, x = 0, FP64 residual of the Newton system
        st = captureGraph(B, B->gRes0, [&]() -> int {
            CK(cudaMemcpyAsync(B->dAct, B->hAct, sizeof(int) * K, cudaMemcpyHostToDevice, s));
            CK(cudaMemsetAsync(B->dSt, 0, sizeof(DevStatus) * K, s));
            launchBatchCast(B->dSol, B->dAct, K, B->gxSol, s);
            launchBatchZeroX(B->dSol, B->dAct, K, B->gxSol, s);
            launchBatchResidual64(B->dSol, B->dAct, K, B->gxSol, B->b, s);
            CK(cudaMemcpyAsync(B->hSt, B->dSt, sizeof(DevStatus) * K, cudaMemcpyDeviceToHost, s));
            return GBFV_OK;
        });
        if (st) return st;
        // S2: accumulate the inner solution, FP64 residual again
        st = captureGraph(B, B->gRef, [&]() -> int {
            CK(cudaMemcpyAsync(B->dAct, B->hAct, sizeof(int) * K, cudaMemcpyHostToDevice, s));
            CK(cudaMemsetAsync(B->dSt, 0, sizeof(DevStatus) * K, s));
            launchBatchAccumulate(B->dSol, B->dAct, K, B->gxSol, s);
            launchBatchResidual64(B->dSol, B->dAct, K, B->gxSol, B->b, s);
            CK(cudaMemcpyAsync(B->hSt, B->dSt, sizeof(DevStatus) * K, cudaMemcpyDeviceToHost, s));
            return GBFV_OK;
        });
        if (st) return st;
    }
    // S1: the persistent batched solve
    st = captureGraph(B, B->gKry, [&]() -> int {
        CK(cudaMemcpyAsync(B->dOrder, B->hOrder, sizeof(int) * (K + 1), cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(B->dQueue, 0, sizeof(int), s));
        CK(cudaMemsetAsync(B->dSt, 0, sizeof(DevStatus) * K, s));
        int ls;
        if (B->precision == GBFV_PREC_MIXED) {
            CK(cudaMemcpyAsync(B->dK32, B->hK32, sizeof(KArgs<float>) * K, cudaMemcpyHostToDevice, s));
            ls = launchBicgstabBatch<float>(B->dK32, B->dOrder, B->dOrder + K, B->dQueue, B->b, B->cluster,
                                            B->numClusters, B->maxLev, s);
        }
        else {
            CK(cudaMemcpyAsync(B->dK64, B->hK64, sizeof(KArgs<double>) * K, cudaMemcpyHostToDevice, s));
            ls = launchBicgstabBatch<double>(B->dK64, B->dOrder, B->dOrder + K, B->dQueue, B->b, B->cluster,
                                             B->numClusters, B->maxLev, s);
        }
        if (ls) return ls;
        CK(cudaMemcpyAsync(B->hSt, B->dSt, sizeof(DevStatus) * K, cudaMemcpyDeviceToHost, s));
        return GBFV_OK;
    });
    if (st) return st;
    return buildRoundGraph(B);
}

// the fail path of gbfv_newton_apply followed by the dt-halving of
// gbfv_time_integration (fvbaseproblem.hh:523-542)
void batchFail(gbfv_batch* B, int i, int status, bool deviceCopies = true)
{
    SysState& y = B->sys[i];
    gbfv_ctx* C = B->ctx[i];
    if (deviceCopies) {  // (the device round's time-level kernel has done them)
        cudaMemcpyAsync(C->x, C->xOld, sizeof(double) * C->N * C->b, cudaMemcpyDeviceToDevice, B->stream);
        cudaMemcpyAsync(C->meaning, C->meaningOld, sizeof(int) * C->N, cudaMemcpyDeviceToDevice, B->stream);
    }
    y.numIterations = B->prm.newton_target_iterations * 2;
    if (status == GBFV_ERR_CUDA || status == GBFV_ERR_TIMEOUT || status == GBFV_ERR_OOM) {
        y.phase = PH_FAILED;
        y.status = status;
        return;
    }
    y.fails++;
    const double nextDt0 = y.dt / 2.0;
    if (y.dt < B->prm.min_time_step * (1 + 1e-9) || y.fails >= B->prm.max_time_step_divisions) {
        y.phase = PH_FAILED;
        y.status = GBFV_ERR_NOT_CONVERGED;
        return;
    }
    y.dt = std::max(nextDt0, B->prm.min_time_step);
    y.numIterations = 0;
    y.error = y.lastError = 0;
    y.phase = PH_LIN;
}

// end of a converged Newton solve: advance the time level, next step size
void batchStepDone(gbfv_batch* B, int i, bool deviceCopies = true)
{
    SysState& y = B->sys[i];
    gbfv_ctx* C = B->ctx[i];
    y.stepDt.push_back(y.dt);
    y.stepNewton.push_back(y.numIterations);
    y.stepLinear.push_back(y.linItStep);
    if (deviceCopies) {
        cudaMemcpyAsync(C->xOld, C->x, sizeof(double) * C->N * C->b, cudaMemcpyDeviceToDevice, B->stream);
        cudaMemcpyAsync(C->meaningOld, C->meaning, sizeof(int) * C->N, cudaMemcpyDeviceToDevice, B->stream);
    }
    y.t += y.dt;
    y.step++;
    C->numIterations = y.numIterations;
    if (y.fixedDt) y.dt = y.dt0;
    else {
        const double maxTs = std::max(0.0, y.endTime - y.t);
        double dtNext = std::min(B->prm.max_time_step, gbfv_suggest_time_step(C, y.dt, y.numIterations));
        if (dtNext < maxTs && maxTs < dtNext * 2) dtNext = maxTs / 2 * 1.01;
        y.dt = std::min(maxTs, dtNext);
    }
    y.fails = 0;
    y.linItStep = 0;
    y.numIterations = 0;
    y.error = y.lastError = 0;
    y.phase = (y.step >= y.numSteps || y.t >= y.endTime) ? PH_DONE : PH_LIN;
}

bool batchProceed(const gbfv_batch* B, const SysState& y)
{
    if (y.numIterations < 1) return true;
    if (y.error <= B->prm.newton_tolerance) return false;
    if (y.numIterations >= B->prm.newton_max_iterations) return y.error * 4.0 < y.lastError;
    return true;
}

// the Newton loop has left the loop body: converged or not (newton_apply tail)
void batchNewtonEnd(gbfv_batch* B, int i)
{
    SysState& y = B->sys[i];
    if (y.error <= B->prm.newton_tolerance) batchStepDone(B, i);
    else batchFail(B, i, GBFV_ERR_NOT_CONVERGED);
}

// one solve phase for every system in PH_SOLVE; leaves them in PH_UPDATE or failed
int batchSolvePhase(gbfv_batch* B)
{
    const int K = B->K;
    std::vector<int> S;
    for (int i = 0; i < K; ++i)
        if (B->sys[i].phase == PH_SOLVE) S.push_back(i);
    if (S.empty()) return GBFV_OK;
    const gbfv_params& prm = B->prm;
    const double absTol = absTolOf(prm);
    const double eps = std::numeric_limits<double>::min() * 1e10;
    auto solveOrder = [&](const std::vector<int>& R) {
        std::vector<int> o(R);
        std::stable_sort(o.begin(), o.end(), [&](int a, int c) { return B->ctx[a]->N > B->ctx[c]->N; });
        for (size_t q = 0; q < o.size(); ++q) B->hOrder[q] = o[q];
        B->hOrder[K] = (int)o.size();
    };
    auto krylov = [&](const std::vector<int>& R, int ref) -> int {
        for (int i : R) {
            gbfv_ctx* C = B->ctx[i];
            SolverData& Sd = C->S;
            int rs;
            if (B->precision == GBFV_PREC_MIXED) {
                const SysState& y = B->sys[i];
                const double target = std::max(prm.linear_tolerance * y.resErr0, absTol);
                const double need = target / y.resErr;
                const double innerTol = std::min(0.5, std::max(0.5 * need, prm.inner_tolerance));
                float* vec[6] = {Sd.v32[1], Sd.v32[2], Sd.v32[3], Sd.v32[4], Sd.v32[5], Sd.v32[6]};
                rs = fillKArgs<float>(Sd, &B->dSt[i], Sd.A32, Sd.FL32, Sd.FD32, Sd.v32[0], vec, ref == 0, innerTol,
                                      0.0, prm.linear_max_error, prm.linear_max_iterations, SYNC_CLUSTER, B->cluster,
                                      B->hK32[i]);
            }
            else {
                rs = fillKArgs<double>(Sd, &B->dSt[i], C->jval, Sd.FL64, Sd.FD64, C->residual, Sd.v64, 1,
                                       prm.linear_tolerance, absTol, prm.linear_max_error, prm.linear_max_iterations,
                                       SYNC_CLUSTER, B->cluster, B->hK64[i]);
            }
            if (rs) return rs;
        }
        solveOrder(R);
        cudaEventRecord(B->evA, B->stream);
        int rs = replay(B, B->gKry, false);
        if (rs) return rs;
        cudaEventRecord(B->evB, B->stream);
        CK(cudaStreamSynchronize(B->stream));
        float ms = 0;
        cudaEventElapsedTime(&ms, B->evA, B->evB);
        B->solveMs += ms;
        B->solveLaunches++;
        for (int i : R) {
            const DevStatus& h = B->hSt[i];
            B->solveBytes += solveBytes(B->ctx[i]->S, h.iterations, B->precision == GBFV_PREC_MIXED ? ref == 0 : 1,
                                        B->precision == GBFV_PREC_MIXED ? 4 : 8);
        }
        return GBFV_OK;
    };
    if (B->precision != GBFV_PREC_MIXED) {
        int rs = krylov(S, 0);
        if (rs) return rs;
        for (int i : S) {
            const DevStatus& h = B->hSt[i];
            SysState& y = B->sys[i];
            y.linItStep += h.iterations;
            const int ks = h.code ? h.code : (h.converged ? GBFV_OK : GBFV_ERR_NOT_CONVERGED);
            if (ks != GBFV_OK) batchFail(B, i, ks);
            else y.phase = PH_UPDATE;
        }
        return GBFV_OK;
    }
    // mixed: r = b - A*0, then refinement rounds (solveMixed)
    for (int i = 0; i < K; ++i) B->hAct[i] = 0;
    for (int i : S) B->hAct[i] = 1;
    int rs = replay(B, B->gRes0, true);
    if (rs) return rs;
    std::vector<int> R;
    for (int i : S) {
        SysState& y = B->sys[i];
        y.resErr = std::max(bitsToDouble(B->hSt[i].errorBits), eps);
        y.resErr0 = y.resErr;
        y.solveIters = 0;
        y.refs = 0;
        if (y.resErr / std::max(1e-20, y.resErr0) <= prm.linear_tolerance || y.resErr <= absTol) y.phase = PH_UPDATE;
        else R.push_back(i);
    }
    for (int ref = 0; ref < std::max(1, prm.max_refinements) && !R.empty(); ++ref) {
        if ((rs = krylov(R, ref))) return rs;
        std::vector<int> R2;
        for (int i : R) {
            const DevStatus& h = B->hSt[i];
            SysState& y = B->sys[i];
            y.lastIt = h.iterations;
            y.solveIters += h.iterations;
            y.linItStep += h.iterations;
            y.refs++;
            y.lastKs = h.code ? h.code : (h.converged ? GBFV_OK : GBFV_ERR_NOT_CONVERGED);
            if (y.lastKs != GBFV_OK && y.lastKs != GBFV_ERR_NOT_CONVERGED) batchFail(B, i, y.lastKs);
            else R2.push_back(i);
        }
        R.swap(R2);
        if (R.empty()) break;
        for (int i = 0; i < K; ++i) B->hAct[i] = 0;
        for (int i : R) B->hAct[i] = 1;
        if ((rs = replay(B, B->gRef, true))) return rs;
        std::vector<int> R3;
        for (int i : R) {
            SysState& y = B->sys[i];
            y.resErr = bitsToDouble(B->hSt[i].errorBits);
            if (!std::isfinite(y.resErr)) batchFail(B, i, GBFV_ERR_NONFINITE);
            else if (y.resErr / std::max(1e-20, y.resErr0) <= prm.linear_tolerance || y.resErr <= absTol)
                y.phase = PH_UPDATE;
            else if (y.resErr > prm.linear_max_error * y.resErr0) batchFail(B, i, GBFV_ERR_NOT_CONVERGED);
            else if (y.lastKs == GBFV_ERR_NOT_CONVERGED && y.lastIt >= prm.linear_max_iterations)
                batchFail(B, i, GBFV_ERR_NOT_CONVERGED);
            else R3.push_back(i);
        }
        R.swap(R3);
    }
    for (int i : R) batchFail(B, i, GBFV_ERR_NOT_CONVERGED);
    return GBFV_OK;
}

// one round: L for systems in PH_LIN, S, U; returns a CUDA-level status
int batchRound(gbfv_batch* B)
{
    const int K = B->K;
    const gbfv_params& prm = B->prm;
    bool any = false;
    for (int i = 0; i < K; ++i) {
        SysState& y = B->sys[i];
        B->hJs[i].active = y.phase == PH_LIN;
        if (y.phase == PH_LIN) {
            any = true;
            B->hJs[i].dt = y.dt;
            B->hJs[i].iter0 = y.numIterations == 0;
            y.lastError = y.error;
        }
    }
    if (!any) return GBFV_OK;
    B->rounds++;
    cudaEventRecord(B->evA, B->stream);
    int rs = replay(B, B->gLin, false);
    if (rs) return rs;
    cudaEventRecord(B->evB, B->stream);
    CK(cudaStreamSynchronize(B->stream));
    {
        float ms = 0;
        cudaEventElapsedTime(&ms, B->evA, B->evB);
        B->linMs += ms;
    }
    for (int i = 0; i < K; ++i) {
        if (!B->hJs[i].active) continue;
        SysState& y = B->sys[i];
        y.linearizations++;
        const DevStatus& h = B->hSt[i];
        y.error = bitsToDouble(h.errorBits);
        if (h.nonfinite) batchFail(B, i, GBFV_ERR_NONFINITE);
        else if (y.error > prm.newton_max_error) batchFail(B, i, GBFV_ERR_NUMERICAL);
        else if (!batchProceed(B, y)) {
            y.numIterations++;
            batchNewtonEnd(B, i);
        }
        else y.phase = PH_SOLVE;
    }
    if ((rs = batchSolvePhase(B))) return rs;
    bool anyU = false;
    for (int i = 0; i < K; ++i) {
        B->hJs[i].active = B->sys[i].phase == PH_UPDATE;
        anyU |= B->hJs[i].active != 0;
    }
    if (!anyU) return GBFV_OK;
    if ((rs = replay(B, B->gCheck, true))) return rs;
    for (int i = 0; i < K; ++i) {
        if (!B->hJs[i].active) continue;
        if (B->hSt[i].nonfinite) {
            B->hJs[i].active = 0;
            batchFail(B, i, GBFV_ERR_NONFINITE);
        }
    }
    // synchronised: the graph reads the pinned per-system state, which the
    // next round rewrites
    if ((rs = replay(B, B->gUpd, true))) return rs;
    for (int i = 0; i < K; ++i)
        if (B->hJs[i].active) {
            SysState& y = B->sys[i];
            y.numIterations++;
            // the loop condition of gbfv_newton_apply, checked before the next linearization
            if (batchProceed(B, y)) y.phase = PH_LIN;
            else batchNewtonEnd(B, i);
        }
    return GBFV_OK;
}

// one round as one graph launch (buildRoundGraph): the host sets which
// systems start a Newton iteration, replays the graph, and does the
// time-step bookkeeping of the systems whose Newton loop ended
int batchRoundDevice(gbfv_batch* B)
{
    const int K = B->K;
    const gbfv_params& prm = B->prm;
    const bool mixed = B->precision == GBFV_PREC_MIXED;
    bool any = false;
    for (int i = 0; i < K; ++i) {
        SysState& y = B->sys[i];
        RoundSys& r = B->hRound[i];
        std::memset(&r, 0, sizeof(r));
        r.phase = y.phase == PH_LIN ? RS_LIN : RS_IDLE;
        r.dt = y.dt;
        r.numIterations = y.numIterations;
        r.error = y.error;
        r.lastError = y.lastError;
        r.linItStep = y.linItStep;
        r.linearizations = y.linearizations;
        if (y.phase != PH_LIN) continue;
        any = true;
        // the solve's launch arguments; the round's decisions set each
        // launch's reduction target and factorization flag on the device
        gbfv_ctx* C = B->ctx[i];
        SolverData& Sd = C->S;
        int rs;
        if (mixed) {
            float* vec[6] = {Sd.v32[1], Sd.v32[2], Sd.v32[3], Sd.v32[4], Sd.v32[5], Sd.v32[6]};
            rs = fillKArgs<float>(Sd, &B->dSt[i], Sd.A32, Sd.FL32, Sd.FD32, Sd.v32[0], vec, 1, prm.inner_tolerance, 0.0,
                                  prm.linear_max_error, prm.linear_max_iterations, SYNC_CLUSTER, B->cluster,
                                  B->hK32[i]);
        }
        else
            rs = fillKArgs<double>(Sd, &B->dSt[i], C->jval, Sd.FL64, Sd.FD64, C->residual, Sd.v64, 1,
                                   prm.linear_tolerance, absTolOf(prm), prm.linear_max_error,
                                   prm.linear_max_iterations, SYNC_CLUSTER, B->cluster, B->hK64[i]);
        if (rs) return rs;
    }
    if (!any) return GBFV_OK;
    B->rounds++;
    int rs = replay(B, B->gRound, true);
    if (rs) return rs;
    {
        float ms = 0;
        cudaEventElapsedTime(&ms, B->roundEv[0], B->roundEv[1]);
        B->linMs += ms;
        int launches = 0;
        for (int i = 0; i < K; ++i) launches = std::max(launches, B->hRound[i].kryLaunches);
        for (int r = 0; r < launches; ++r) {
            cudaEventElapsedTime(&ms, B->roundEv[2 + 2 * r], B->roundEv[3 + 2 * r]);
            B->solveMs += ms;
        }
        B->solveLaunches += launches;
        const int sz = mixed ? 4 : 8;
        for (int i = 0; i < K; ++i) {
            const RoundSys& r = B->hRound[i];
            if (!r.kryLaunches) continue;
            const SolverData& Sd = B->ctx[i]->S;
            const double b0 = solveBytes(Sd, 0, 0, sz);
            B->solveBytes += r.kryLaunches * b0 + r.kryFactors * (solveBytes(Sd, 0, 1, sz) - b0) +
                             (double)r.kryIters * (solveBytes(Sd, 1, 0, sz) - b0);
        }
    }
    for (int i = 0; i < K; ++i) {
        SysState& y = B->sys[i];
        const RoundSys& r = B->hRound[i];
        if (y.phase != PH_LIN) continue;
        y.numIterations = r.numIterations;
        y.error = r.error;
        y.lastError = r.lastError;
        y.linItStep = r.linItStep;
        y.linearizations = r.linearizations;
        if (r.phase == RS_LIN) continue;
        if (r.phase == RS_END_OK) batchStepDone(B, i, false);
        else if (r.phase == RS_FAIL) batchFail(B, i, r.status, false);
        else {
            setError("batched round ended with a system in phase " + std::to_string(r.phase));
            return GBFV_ERR_CUDA;
        }
    }
    return GBFV_OK;
}

void freeBatch(gbfv_batch* B)
{
    if (!B) return;
    for (GraphSet* g : {&B->gLin, &B->gCheck, &B->gUpd, &B->gRes0, &B->gKry, &B->gRef, &B->gRound})
        if (g->exec) cudaGraphExecDestroy(g->exec);
    for (cudaEvent_t e : B->roundEv) cudaEventDestroy(e);
    cudaFree(B->dRound);
    cudaFreeHost(B->hRound);
    cudaFree(B->dLin);
    cudaFree(B->dSol);
    cudaFree(B->dJs);
    cudaFree(B->dAct);
    cudaFree(B->dSt);
    cudaFree(B->dK32);
    cudaFree(B->dK64);
    cudaFree(B->dOrder);
    cudaFree(B->dQueue);
    cudaFreeHost(B->hJs);
    cudaFreeHost(B->hAct);
    cudaFreeHost(B->hSt);
    cudaFreeHost(B->hK32);
    cudaFreeHost(B->hK64);
    cudaFreeHost(B->hOrder);
    if (B->evA) cudaEventDestroy(B->evA);
    if (B->evB) cudaEventDestroy(B->evB);
    if (B->stream) cudaStreamDestroy(B->stream);
    for (gbfv_ctx* C : B->ctx)
        if (C) gbfv_destroy(C);
    delete B;
}

// the batched kernels' view of system i
void fillJobs(gbfv_batch* B, int i, LinJob& j, SolveJob& s)
{
    gbfv_ctx* C = B->ctx[i];
    std::memset(&j, 0, sizeof(j));
    std::memset(&s, 0, sizeof(s));
    j.m = C->mesh;
    j.phys = C->dphys;
    j.x = C->x;
    j.xOld = C->xOld;
    j.meaning = C->meaning;
    j.meaningOld = C->meaningOld;
    j.iq = C->iq;
    j.storageOld = C->storageOld;
    j.residual = C->residual;
    j.jval = C->jval;
    j.dx = B->precision == GBFV_PREC_MIXED ? C->S.xref : C->S.v64[0];
    j.wasSwitched = C->wasSwitched;
    j.st = &B->dSt[i];
    SolverData& S = C->S;
    s.N = S.N;
    s.ld = S.ldN;
    s.nslot = S.nslot;
    s.b = S.b;
    s.nval = (long)S.nslot * S.b * S.b * S.ldN;
    s.col = S.col;
    s.A64 = C->jval;
    s.A32 = S.A32;
    s.rhs = C->residual;
    s.xref = S.xref;
    s.rref = S.rref;
    s.r32 = S.v32[0];
    s.dx32 = S.v32[1];
    s.st = &B->dSt[i];
}

int setupBatch(gbfv_batch* B, int cluster)
{
    const int K = B->K;
    int st;
    CK(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&B->evA));
    CK(cudaEventCreate(&B->evB));
    if ((st = devAlloc(&B->dLin, K)) || (st = devAlloc(&B->dSol, K)) || (st = devAlloc(&B->dJs, K)) ||
        (st = devAlloc(&B->dAct, K)) || (st = devAlloc(&B->dSt, K)) || (st = devAlloc(&B->dK32, K)) ||
        (st = devAlloc(&B->dK64, K)) || (st = devAlloc(&B->dOrder, K + 1)) || (st = devAlloc(&B->dQueue, 1)))
        return st;
    if ((st = pinnedAlloc(&B->hJs, K)) || (st = pinnedAlloc(&B->hAct, K)) || (st = pinnedAlloc(&B->hSt, K)) ||
        (st = pinnedAlloc(&B->hK32, K)) || (st = pinnedAlloc(&B->hK64, K)) || (st = pinnedAlloc(&B->hOrder, K + 1)))
        return st;
    if ((st = devAlloc(&B->dRound, K)) || (st = pinnedAlloc(&B->hRound, K))) return st;
    if (const char* e = getenv("GBFV_BATCH_HOST_ROUND")) B->deviceRound = atoi(e) ? 0 : 1;
    std::vector<LinJob> lj(K);
    std::vector<SolveJob> sj(K);
    int maxN = 1, maxLev = 1, maxC = 16;
    for (int i = 0; i < K; ++i) {
        gbfv_ctx* C = B->ctx[i];
        if (!C) continue;
        fillJobs(B, i, lj[i], sj[i]);
        maxN = std::max(maxN, C->N);
        maxLev = std::max(maxLev, (int)C->S.levPtr.size() - 1);
        maxC = std::min(maxC, C->S.maxCluster[B->precision == GBFV_PREC_MIXED ? 1 : 0]);
    }
    if (B->dynamic) {
        // slots are filled later: size the launches for any admissible system
        maxN = std::max(maxN, B->maxCells);
        maxLev = MAX_PUSH_LEVELS;
        maxC = std::min(maxC, B->precision == GBFV_PREC_MIXED ? maxClusterBlocks<float>(B->b)
                                                              : maxClusterBlocks<double>(B->b));
    }
    B->maxLev = std::min(maxLev, MAX_PUSH_LEVELS);
    B->cluster = cluster > 0 ? std::min(cluster, maxC) : std::min(8, maxC);
    B->numClusters = B->precision == GBFV_PREC_MIXED ? maxActiveClusters<float>(B->b, B->cluster)
                                                     : maxActiveClusters<double>(B->b, B->cluster);
    if (B->numClusters < 1) B->numClusters = 1;
    B->numClusters = std::min(B->numClusters, K);
    B->gxLin = std::max(1, std::min((maxN + 127) / 128, std::max(16, (152 * 16 + K - 1) / K)));
    B->gxSol = std::max(1, std::min((maxN + 255) / 256, std::max(16, (152 * 8 + K - 1) / K)));
    CK(cudaMemcpy(B->dLin, lj.data(), sizeof(LinJob) * K, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B->dSol, sj.data(), sizeof(SolveJob) * K, cudaMemcpyHostToDevice));
    UpdateParams& up = B->up;
    up.dsMax = B->prm.ds_max;
    up.dpMaxRel = B->prm.dp_max_rel;
    up.oscThreshold = B->prm.pv_oscillation_threshold;
    up.pMin = B->prm.pressure_min;
    up.pMax = B->prm.pressure_max;
    up.swMax = B->prm.max_water_saturation;
    up.waterOnly = B->prm.water_only_threshold;
    CK(cudaDeviceSynchronize());
    return buildBatchGraphs(B);
}

}  // namespace

extern "C" {

gbfv_batch* gbfv_batch_create(const gbfv_problem* probs, int num_systems, const gbfv_params* params,
                              int cluster_size, int* status)
{
    auto fail = [&](gbfv_batch* B, int st) -> gbfv_batch* {
        if (status) *status = st;
        freeBatch(B);
        return nullptr;
    };
    if (!probs || num_systems <= 0 || (params && !paramsOk(*params))) return fail(nullptr, GBFV_ERR_ARG);
    if (params && params->local_linearizer != GBFV_LIN_AD) {
        setError("batched systems are linearized by automatic differentiation only");
        return fail(nullptr, GBFV_ERR_UNSUPPORTED);
    }
    if (params && params->linear_solver != GBFV_LINSOLVER_ILU0) {
        setError("batched systems are solved with the ILU(0) backend only");
        return fail(nullptr, GBFV_ERR_UNSUPPORTED);
    }
    if (params && params->linearizer != GBFV_LINEARIZER_ELEMENT) {
        setError("batched systems are linearized element by element only");
        return fail(nullptr, GBFV_ERR_UNSUPPORTED);
    }
    for (int i = 0; i < num_systems; ++i)
        if (probs[i].num_elements > 0) {
            setError("batched systems are cell-centred grids only");
            return fail(nullptr, GBFV_ERR_UNSUPPORTED);
        }
    gbfv_batch* B = new gbfv_batch();
    if (params) B->prm = *params;
    else gbfv_default_params(&B->prm);
    B->precision = B->prm.precision;
    B->K = num_systems;
    for (int i = 0; i < num_systems; ++i) {
        int st = GBFV_OK;
        gbfv_ctx* C = gbfv_create(&probs[i], &B->prm, &st);
        if (!C) return fail(B, st ? st : GBFV_ERR_ARG);
        dropWideGilu(C->S);
        B->ctx.push_back(C);
        if (i == 0) {
            B->b = C->b;
            B->model = C->model;
        }
        else if (C->b != B->b || C->model != B->model) {
            setError("all systems of a batch must use the same model");
            return fail(B, GBFV_ERR_ARG);
        }
    }
    B->sys.resize(num_systems);
    const int st = setupBatch(B, cluster_size);
    if (st) return fail(B, st);
    if (status) *status = GBFV_OK;
    return B;
}

int gbfv_batch_destroy(gbfv_batch* B)
{
    freeBatch(B);
    return GBFV_OK;
}

gbfv_ctx* gbfv_batch_system(gbfv_batch* B, int i)
{
    if (!B || i < 0 || i >= B->K) return nullptr;
    return B->ctx[i];
}

int gbfv_batch_time_integration(gbfv_batch* B, int num_steps, double dt0, double end_time, int fixed_dt)
{
    if (!B || num_steps < 0 || !(dt0 > 0)) return GBFV_ERR_ARG;
    for (int i = 0; i < B->K; ++i) {
        gbfv_ctx* C = B->ctx[i];
        CK(cudaStreamSynchronize(C->stream));  // set_solution etc. ran on the context's stream
        SysState& y = B->sys[i];
        y = SysState();
        y.numSteps = num_steps;
        y.dt = y.dt0 = dt0;
        y.endTime = end_time;
        y.fixedDt = fixed_dt;
        y.phase = num_steps > 0 ? PH_LIN : PH_DONE;
    }
    for (;;) {
        bool pending = false;
        for (const SysState& y : B->sys) pending |= y.phase == PH_LIN;
        if (!pending) break;
        const int rs = B->deviceRound ? batchRoundDevice(B) : batchRound(B);
        if (rs) return rs;
    }
    CK(cudaStreamSynchronize(B->stream));
    int worst = GBFV_OK;
    for (const SysState& y : B->sys)
        if (y.phase == PH_FAILED && worst == GBFV_OK) worst = y.status;
    return worst;
}

int gbfv_batch_autotune(gbfv_batch* B, double dt, int* cluster_out, double* ms_out, int* num_out)
{
    if (!B || !(dt > 0)) return GBFV_ERR_ARG;
    for (int i = 0; i < B->K; ++i) CK(cudaStreamSynchronize(B->ctx[i]->stream));
    int maxC = 16;
    for (gbfv_ctx* C : B->ctx) maxC = std::min(maxC, C->S.maxCluster[B->precision == GBFV_PREC_MIXED ? 1 : 0]);
    // linearize every system at its current state (Newton iteration 0)
    for (int i = 0; i < B->K; ++i) {
        B->hJs[i].active = 1;
        B->hJs[i].dt = dt;
        B->hJs[i].iter0 = 1;
    }
    int rs = replay(B, B->gLin, true);
    if (rs) return rs;
    const double ms0 = B->solveMs;
    double best = 1e300;
    int pick = B->cluster, n = 0;
    for (int c = 2; c <= maxC; c *= 2) {
        B->cluster = c;
        B->numClusters = std::max(1, std::min(B->K, B->precision == GBFV_PREC_MIXED ? maxActiveClusters<float>(B->b, c)
                                                                                  : maxActiveClusters<double>(B->b, c)));
        if (B->gKry.exec) cudaGraphExecDestroy(B->gKry.exec);
        B->gKry.exec = nullptr;
        if ((rs = buildBatchGraphs(B))) return rs;
        for (SysState& y : B->sys) {
            y = SysState();
            y.phase = PH_SOLVE;
        }
        const double before = B->solveMs;
        if ((rs = batchSolvePhase(B))) return rs;
        const double ms = B->solveMs - before;
        if (ms_out && n < 8) ms_out[n] = ms;
        n++;
        if (ms < best) { best = ms; pick = c; }
    }
    B->solveMs = ms0;
    B->solveBytes = 0;
    B->solveLaunches = 0;
    B->cluster = pick;
    B->numClusters = std::max(1, std::min(B->K, B->precision == GBFV_PREC_MIXED ? maxActiveClusters<float>(B->b, pick)
                                                                             : maxActiveClusters<double>(B->b, pick)));
    if ((rs = buildBatchGraphs(B))) return rs;
    for (SysState& y : B->sys) y = SysState();
    CK(cudaStreamSynchronize(B->stream));
    if (cluster_out) *cluster_out = pick;
    if (num_out) *num_out = n;
    return GBFV_OK;
}

int gbfv_batch_system_report(const gbfv_batch* B, int i, int* status, int* steps_done, double* step_dt,
                             int32_t* step_newton, int32_t* step_linear, int* linearizations)
{
    if (!B || i < 0 || i >= B->K) return GBFV_ERR_ARG;
    const SysState& y = B->sys[i];
    if (status) *status = y.phase == PH_FAILED ? y.status : GBFV_OK;
    if (steps_done) *steps_done = (int)y.stepDt.size();
    for (size_t k = 0; k < y.stepDt.size(); ++k) {
        if (step_dt) step_dt[k] = y.stepDt[k];
        if (step_newton) step_newton[k] = y.stepNewton[k];
        if (step_linear) step_linear[k] = y.stepLinear[k];
    }
    if (linearizations) *linearizations = y.linearizations;
    return GBFV_OK;
}

int gbfv_batch_get_stats(const gbfv_batch* B, gbfv_batch_stats* out)
{
    if (!B || !out) return GBFV_ERR_ARG;
    out->num_systems = B->K;
    out->cluster_size = B->cluster;
    out->num_clusters = B->numClusters;
    out->rounds = B->rounds;
    out->graph_launches = B->graphLaunches;
    out->kernel_launches = B->kernelLaunches;
    out->solve_ms = B->solveMs;
    out->solve_bytes = B->solveBytes;
    out->solve_launches = B->solveLaunches;
    out->linearize_ms = B->linMs;
    return GBFV_OK;
}

void* gbfv_batch_stream(gbfv_batch* B) { return B ? (void*)B->stream : nullptr; }

// ---------------------------------------------------------------- serving
int64_t gbfv_footprint_bytes(int num_cells, int block_size, int dim)
{
    if (num_cells <= 0 || num_cells > GBFV_MAX_CELLS || (block_size != 2 && block_size != 3) || (dim != 2 && dim != 3))
        return -1;
    const int64_t b = block_size, bb = b * b, ns = 2 * dim + 1, nd = 2 * dim;
    const int64_t iq = iqValuePlanes((int)b) + iqDerivPlanes((int)b) + iqStoragePlanes((int)b);
    // solver: FP64 + FP32 factors, FP32 matrix, Krylov vectors, columns, push tables
    const int64_t solver = dim * bb * 12 + bb * 12 + ns * bb * 4 + 6 * b * 8 + 7 * b * 4 + 2 * b * 8 + ns * 4 + 6 * 4;
    // context: state vectors, Jacobian, IQ buffers, mesh (faces, cells), snapshot
    const int64_t ctx = 5 * b * 8 + ns * bb * 8 + 3 * 4 + iq * 8 + nd * (4 + 5 * 8) + 64 + b * 8 + 8 + 64;
    return (int64_t)num_cells * (solver + ctx) + (4 << 20);
}

gbfv_batch* gbfv_serve_create(int capacity, int model, const gbfv_params* params, int cluster_size, int max_cells,
                              int* status)
{
    auto fail = [&](gbfv_batch* B, int st) -> gbfv_batch* {
        if (status) *status = st;
        freeBatch(B);
        return nullptr;
    };
    if (capacity <= 0 || max_cells <= 0 || (model != GBFV_MODEL_IMMISCIBLE_2P && model != GBFV_MODEL_BLACKOIL_3P) ||
        (params && !paramsOk(*params)))
        return fail(nullptr, GBFV_ERR_ARG);
    if (params && params->local_linearizer != GBFV_LIN_AD) {
        setError("served systems are linearized by automatic differentiation only");
        return fail(nullptr, GBFV_ERR_UNSUPPORTED);
    }
    if (max_cells > GBFV_MAX_CELLS) {
        setError("max_cells above GBFV_MAX_CELLS (32-bit device indexing)");
        return fail(nullptr, GBFV_ERR_UNSUPPORTED);
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(nullptr, GBFV_ERR_NO_DEVICE);
    gbfv_batch* B = new gbfv_batch();
    if (params) B->prm = *params;
    else gbfv_default_params(&B->prm);
    B->precision = B->prm.precision;
    B->K = capacity;
    B->dynamic = 1;
    B->maxCells = max_cells;
    B->model = model;
    B->b = model == GBFV_MODEL_IMMISCIBLE_2P ? 2 : 3;
    B->ctx.assign(capacity, nullptr);
    B->sys.resize(capacity);
    const int st = setupBatch(B, cluster_size);
    if (st) return fail(B, st);
    if (status) *status = GBFV_OK;
    return B;
}

int gbfv_serve_admit(gbfv_batch* B, const gbfv_problem* prob, const double* pv, const int32_t* meaning,
                     int num_steps, double dt0, int fixed_dt, int* slot)
{
    if (!B || !B->dynamic || !prob || !pv || num_steps <= 0 || !(dt0 > 0) || !slot) return GBFV_ERR_ARG;
    if (prob->num_cells > B->maxCells) {
        setError("system larger than the server's max_cells");
        return GBFV_ERR_ARG;
    }
    if (prob->num_elements > 0) {
        setError("served systems are cell-centred grids only");
        return GBFV_ERR_UNSUPPORTED;
    }
    int i = -1;
    for (int k = 0; k < B->K; ++k)
        if (!B->ctx[k]) { i = k; break; }
    if (i < 0) {
        setError("no free slot");
        return GBFV_ERR_UNSUPPORTED;
    }
    int st = GBFV_OK;
    gbfv_ctx* C = gbfv_create(prob, &B->prm, &st);
    if (!C) return st ? st : GBFV_ERR_ARG;
    if (C->b != B->b || C->model != B->model) {
        gbfv_destroy(C);
        setError("the system's model differs from the server's");
        return GBFV_ERR_ARG;
    }
    if ((st = gbfv_set_solution(C, pv, meaning))) {
        gbfv_destroy(C);
        return st;
    }
    // the same solver launch configuration as the rest of the batch
    const int k = B->precision == GBFV_PREC_MIXED ? 1 : 0;
    C->S.mode[k] = SYNC_CLUSTER;
    C->S.nblk[k] = B->cluster;
    C->S.tuned[k] = 1;
    dropWideGilu(C->S);
    B->ctx[i] = C;
    LinJob lj;
    SolveJob sj;
    fillJobs(B, i, lj, sj);
    CK(cudaMemcpy(&B->dLin[i], &lj, sizeof(LinJob), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(&B->dSol[i], &sj, sizeof(SolveJob), cudaMemcpyHostToDevice));
    SysState& y = B->sys[i];
    y = SysState();
    y.numSteps = num_steps;
    y.dt = y.dt0 = dt0;
    y.fixedDt = fixed_dt;
    y.phase = PH_LIN;
    B->footprint += gbfv_footprint_bytes(C->N, C->b, C->dim);
    *slot = i;
    return GBFV_OK;
}

int gbfv_serve_step(gbfv_batch* B, int* running)
{
    if (!B) return GBFV_ERR_ARG;
    const int rs = B->deviceRound ? batchRoundDevice(B) : batchRound(B);
    int n = 0;
    for (const SysState& y : B->sys) n += y.phase == PH_LIN;
    if (running) *running = n;
    return rs;
}

int gbfv_serve_slot(const gbfv_batch* B, int slot, int* state, int* status)
{
    if (!B || slot < 0 || slot >= B->K) return GBFV_ERR_ARG;
    const SysState& y = B->sys[slot];
    if (state) *state = !B->ctx[slot] ? 0 : (y.phase == PH_DONE ? 2 : (y.phase == PH_FAILED ? 3 : 1));
    if (status) *status = y.phase == PH_FAILED ? y.status : GBFV_OK;
    return GBFV_OK;
}

int gbfv_serve_release(gbfv_batch* B, int slot)
{
    if (!B || !B->dynamic || slot < 0 || slot >= B->K || !B->ctx[slot]) return GBFV_ERR_ARG;
    CK(cudaStreamSynchronize(B->stream));
    gbfv_ctx* C = B->ctx[slot];
    B->footprint -= gbfv_footprint_bytes(C->N, C->b, C->dim);
    gbfv_destroy(C);
    B->ctx[slot] = nullptr;
    B->sys[slot] = SysState();
    return GBFV_OK;
}

int64_t gbfv_serve_footprint(const gbfv_batch* B) { return B ? B->footprint : -1; }

int gbfv_selftest_level_barriers(int32_t num_rows, int32_t dim, const int32_t* lev_ptr, int32_t num_levels,
                                 const int32_t* col, int32_t cluster, int32_t owner_mode, int32_t buffers,
                                 int32_t forward, int8_t* barrier_after)
{
    if (num_rows < 1 || dim < 1 || dim > 3 || num_levels < 1 || !lev_ptr || !col || cluster < 1 ||
        cluster > 16 || (owner_mode != 0 && owner_mode != 1) || buffers < 2 || !barrier_after)
        return GBFV_ERR_ARG;
    std::vector<int> levPtr(lev_ptr, lev_ptr + num_levels + 1);
    if (levPtr[0] != 0 || levPtr[num_levels] != num_rows) return GBFV_ERR_ARG;
    std::vector<int> colHost(col, col + (size_t)(2 * dim + 1) * num_rows), lev(num_rows);
    for (int l = 0; l < num_levels; ++l)
        for (int p = levPtr[l]; p < levPtr[l + 1]; ++p) lev[p] = l;
    std::vector<char> out;
    placeLevelBarriersCore(num_rows, num_rows, dim, levPtr, colHost, cluster, owner_mode, buffers, lev,
                           forward != 0, out);
    for (int l = 0; l < num_levels; ++l) barrier_after[l] = (int8_t)out[l];
    return GBFV_OK;
}

int gbfv_selftest_wait_timeout(double* ms)
{
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GBFV_ERR_NO_DEVICE;
    DevStatus* d = nullptr;
    DevStatus h;
    cudaEvent_t e0, e1;
    CK(cudaMalloc((void**)&d, sizeof(DevStatus)));
    CK(cudaMemset(d, 0, sizeof(DevStatus)));
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    cudaEventRecord(e0, 0);
    launchWaitTimeoutProbe(d, 0);
    cudaEventRecord(e1, 0);
    const cudaError_t e = cudaMemcpy(&h, d, sizeof(DevStatus), cudaMemcpyDeviceToHost);
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    if (ms) *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    CK(e);
    if (h.iterations != 1) return GBFV_ERR_CUDA;
    return h.code;
}

}  // extern "C"
