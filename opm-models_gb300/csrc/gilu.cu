// Block ILU(0) + BiCGStab for a general block-ELL pattern.
//
// The structured solver (solver.cu) relies on the 5/7-point pattern, whose
// ILU(0) only modifies the diagonal.  The vertex-centred Jacobian couples
// every vertex with its 3 x 3 neighbourhood: there a lower entry (i, k)
// also updates the row's other entries that row k's upper part shares, so
// this kernel runs the full natural-order block ILU(0) (dune-istl's
// blockILU0Decomposition as Dune::SeqILU<..., 0> calls it from
// istlpreconditionerwrappers.hh:151-190; not vendored, restated):
//     for each lower entry k of row i, ascending:
//         A_ik <- A_ik * inv(U_kk)
//         A_ij <- A_ij - A_ik * A_kj   for every j > k in both rows
//     U_ii <- inv(A_ii)
// Rows of one level (rows whose lower neighbours are all in earlier levels)
// are independent; levels are separated by barriers.  The triangular
// sweeps and BiCGStab (bicgstabsolver.hh:120-330, the structured solver's
// iteration and criterion) run in the same persistent launch: one block
// (block barriers) for systems whose levels fit a block, else a cooperative
// grid with the bounded software barrier -- or, for such wide systems,
// tagged sweeps with no barrier per level (see the tagged-sweep section).  Block operations follow the
// reference's order (FieldMatrix::rightmultiply, mmv, the cofactor
// inverse); the products are contracted to FMAs (on this GPU an FP64 warp
// instruction is the scarce resource: contraction measured 1.6x faster
// sweeps), so the FP64 preconditioner is the oracle's to rounding.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/gbfv.h"
#include "gbfv_internal.cuh"
#include "gilu.cuh"
#include "krylov.cuh"

namespace gbfv {

void setLastError(const std::string& s);

namespace {

constexpr int GILU_THREADS = 256;

template <class T>
struct GiluArgs {
    int N, ld, nslot, diag, numLev, factor;
    const int* col;      // [s*ld + p] internal column or -1
    const int* levPtr;   // [numLev + 1]
    const int* updPtr;   // [N + 1] factorization updates of row p
    const int* upd;      // (s | t << 8 | u << 16): A_pt -= A_ps * A_ku, k = col[s][p]
    const T* A;
    T* F;                // factors, A's layout; the diagonal slot holds inv(U_pp)
    const T* rhs;
    T *x, *r, *p, *v, *y, *z;
    double* partial;
    GridSync gs;
    DevStatus* st;
    double redTol, absTol, maxRes;
    int maxIter;
    int warpSweep;       // one block, every level at most 32 rows, at most 4 lower / upper slots:
                         // the narrow sweeps with the vectors in shared memory
    unsigned long long* prof;  // optional phase timers (GBFV_GILU_PROFILE), 16 words
    int localFactor;     // at most 9 slots and GILU_MAX_UPD updates per row: factorRowLocal
    // tagged sweeps (several blocks): row chunks of at most 32 rows inside
    // one level, and the tagged words of every row component (one for
    // FP32, two for FP64), zeroed before the launch
    int tagged, numChunks, pollNs;  // pollNs: back-off between polls after the second
    const int* chunkPtr;      // [numChunks + 1]
    unsigned long long* tw;   // [N * b * words]: tag << 32 | value bits
};

constexpr int WARP_SLOTS = 4;  // lower (and upper) slots the warp sweeps take

template <class T, int B>
__device__ __forceinline__ void ldBlk(const T* M, int s, int ld, int p, T (&o)[B * B])
{
#pragma unroll
    for (int e = 0; e < B * B; ++e) o[e] = ldcg(&M[((size_t)s * B * B + e) * ld + p]);
}
template <class T, int B>
__device__ __forceinline__ void stBlk(T* M, int s, int ld, int p, const T (&o)[B * B])
{
#pragma unroll
    for (int e = 0; e < B * B; ++e) M[((size_t)s * B * B + e) * ld + p] = o[e];
}

// row p of the factorization (its lower neighbours are final)
template <class T, int B>
__device__ bool factorRow(const GiluArgs<T>& a, int p)
{
    const int ld = a.ld;
    for (int s = 0; s < a.nslot; ++s) {
        T blk[B * B];
        ldBlk<T, B>(a.A, s, ld, p, blk);
        stBlk<T, B>(a.F, s, ld, p, blk);
    }
    int q = a.updPtr[p];
    const int q1 = a.updPtr[p + 1];
    for (int s = 0; s < a.diag; ++s) {
        const int k = a.col[(size_t)s * ld + p];
        if (k < 0) continue;
        // A_ps <- A_ps * inv(U_kk)
        T L[B * B], Dk[B * B], C[B * B];
        ldBlk<T, B>(a.F, s, ld, p, C);
        ldBlk<T, B>(a.F, a.diag, ld, k, Dk);
#pragma unroll
        for (int i = 0; i < B; ++i)
#pragma unroll
            for (int j = 0; j < B; ++j) {
                T t = T(0);
#pragma unroll
                for (int m = 0; m < B; ++m) t += C[i * B + m] * Dk[m * B + j];
                L[i * B + j] = t;
            }
        stBlk<T, B>(a.F, s, ld, p, L);
        // A_pt -= L * A_ku for the entries the two rows share
        for (; q < q1 && (a.upd[q] & 0xff) == s; ++q) {
            const int t = (a.upd[q] >> 8) & 0xff, u = (a.upd[q] >> 16) & 0xff;
            T U[B * B], Tt[B * B];
            ldBlk<T, B>(a.F, u, ld, k, U);
            ldBlk<T, B>(a.F, t, ld, p, Tt);
#pragma unroll
            for (int i = 0; i < B; ++i)
#pragma unroll
                for (int j = 0; j < B; ++j) {
                    T acc = T(0);
#pragma unroll
                    for (int m = 0; m < B; ++m) acc += L[i * B + m] * U[m * B + j];
                    Tt[i * B + j] -= acc;
                }
            stBlk<T, B>(a.F, t, ld, p, Tt);
        }
    }
    T D[B * B], R[B * B];
    ldBlk<T, B>(a.F, a.diag, ld, p, D);
    if (!invertBlock<T, B>(D, R)) return false;
    stBlk<T, B>(a.F, a.diag, ld, p, R);
    return true;
}

template <class T, int B>
__device__ void narrowSweeps(const GiluArgs<T>& a, const T* d, T* v, unsigned char* smem);

// row p of the factorization for patterns of at most 9 slots and 16
// updates per row: the row's blocks, its lower neighbours' inverted pivots
// and every upper block its updates read are loaded up front (one round of
// independent loads), the row is factored in local arrays and stored once
// -- the operations and their order are factorRow's
constexpr int GILU_MAX_UPD = 16;
template <class T, int B>
__device__ bool factorRowLocal(const GiluArgs<T>& a, int p)
{
    const int ld = a.ld, ns = a.nslot, diag = a.diag;
    const int q0 = a.updPtr[p], nu = a.updPtr[p + 1] - q0;
    int k[9], up[GILU_MAX_UPD];
#pragma unroll
    for (int s = 0; s < 9; ++s) k[s] = s < ns ? a.col[(size_t)s * ld + p] : -1;
#pragma unroll
    for (int q = 0; q < GILU_MAX_UPD; ++q) up[q] = q < nu ? a.upd[q0 + q] : -1;
    T Fr[9][B * B], Dk[WARP_SLOTS][B * B], U[GILU_MAX_UPD][B * B];
#pragma unroll
    for (int s = 0; s < 9; ++s)
        if (s < ns)
#pragma unroll
            for (int e = 0; e < B * B; ++e) Fr[s][e] = a.A[((size_t)s * B * B + e) * ld + p];
#pragma unroll
    for (int s = 0; s < WARP_SLOTS; ++s)
        if (s < diag && k[s] >= 0)
#pragma unroll
            for (int e = 0; e < B * B; ++e) Dk[s][e] = ldcg(&a.F[((size_t)diag * B * B + e) * ld + k[s]]);
#pragma unroll
    for (int q = 0; q < GILU_MAX_UPD; ++q)
        if (up[q] >= 0) {
            const int s = up[q] & 0xff, u = (up[q] >> 16) & 0xff;
            const int kk = a.col[(size_t)s * ld + p];
#pragma unroll
            for (int e = 0; e < B * B; ++e) U[q][e] = ldcg(&a.F[((size_t)u * B * B + e) * ld + kk]);
        }
    int q = 0;
#pragma unroll
    for (int s = 0; s < WARP_SLOTS; ++s) {
        if (s >= diag || k[s] < 0) continue;
        T L[B * B];
#pragma unroll
        for (int i = 0; i < B; ++i)
#pragma unroll
            for (int j = 0; j < B; ++j) {
                T t = T(0);
#pragma unroll
                for (int m = 0; m < B; ++m) t += Fr[s][i * B + m] * Dk[s][m * B + j];
                L[i * B + j] = t;
            }
#pragma unroll
        for (int e = 0; e < B * B; ++e) Fr[s][e] = L[e];
        for (; q < nu && (up[q] & 0xff) == s; ++q) {
            const int t = (up[q] >> 8) & 0xff;
#pragma unroll
            for (int i = 0; i < B; ++i)
#pragma unroll
                for (int j = 0; j < B; ++j) {
                    T acc = T(0);
#pragma unroll
                    for (int m = 0; m < B; ++m) acc += L[i * B + m] * U[q][m * B + j];
                    Fr[t][i * B + j] -= acc;
                }
        }
    }
    T R[B * B];
    if (!invertBlock<T, B>(Fr[diag], R)) return false;
#pragma unroll
    for (int e = 0; e < B * B; ++e) Fr[diag][e] = R[e];
#pragma unroll
    for (int s = 0; s < 9; ++s)
        if (s < ns)
#pragma unroll
            for (int e = 0; e < B * B; ++e) a.F[((size_t)s * B * B + e) * ld + p] = Fr[s][e];
    return true;
}

// v = (LU)^-1 d: the forward sweep over the levels, then the backward one
// (dune-istl's blockILUBacksolve)
// ------------------------------------------------------ tagged sweeps --
// The FP32 sweeps of a system too wide for one block, without a barrier per
// level: a row publishes each component of its result as one 64-bit word
// {tag, value bits} (single-copy atomic: the value arrives with its tag),
// and a row reads the words of the rows it depends on until they carry the
// current sweep's tag.  The tags of one launch are 1, 2, 3, ... (forward
// and backward sweep of every application); the words are zeroed before
// the launch.  Rows are dealt to warps in chunks of at most 32 rows of one
// level, chunk c to warp c mod W, the forward sweep in ascending and the
// backward sweep in descending chunk order.  Every dependency lies in an
// earlier level (later, backward), so the lowest unfinished chunk can
// always proceed: the cooperative launch keeps every warp resident, and no
// wait closes a cycle.  Every wait is bounded and gives up with the grid's
// abort word.  Same operations in the same order as iluApply: the same
// results to the bit.
constexpr int TAG_SLOTS = 4;  // lower (upper) slots a tagged row takes

// words per value: an FP32 value rides in one word, an FP64 value in two
// (low and high half, each with the tag)
template <class T>
__host__ __device__ constexpr int tagWords() { return sizeof(T) / 4; }

__device__ __forceinline__ void stWord(unsigned long long* p, unsigned tag, unsigned bits)
{
    const unsigned long long w = ((unsigned long long)tag << 32) | bits;
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;\n" ::"l"(p), "l"(w) : "memory");
}

__device__ __forceinline__ unsigned long long ldWord(const unsigned long long* p)
{
    unsigned long long w;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];\n" : "=l"(w) : "l"(p) : "memory");
    return w;
}

__device__ __forceinline__ void stTagged(unsigned long long* p, unsigned tag, float v) { stWord(p, tag, __float_as_uint(v)); }
__device__ __forceinline__ void stTagged(unsigned long long* p, unsigned tag, double v)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    stWord(p, tag, (unsigned)u);
    stWord(p + 1, tag, (unsigned)(u >> 32));
}

// the B components of the rows k[0..TAG_SLOTS) (k < 0: none) once every
// word carries `tag`; false when the wait gave up
template <class T, int B>
__device__ __forceinline__ bool waitTagged(const unsigned long long* tw, const int (&k)[TAG_SLOTS], unsigned tag,
                                           T (&x)[TAG_SLOTS][B], int* abort, int pollNs)
{
    constexpr int NW = tagWords<T>(), RW = B * NW;  // words per component, per row
    static_assert(TAG_SLOTS * RW <= 32, "pending mask");
    unsigned pending = 0;
#pragma unroll
    for (int s = 0; s < TAG_SLOTS; ++s)
        if (k[s] >= 0) pending |= ((1u << RW) - 1u) << (s * RW);
    unsigned lo[TAG_SLOTS][RW];
    long long t0 = 0;
    for (int round = 0; pending; ++round) {
        unsigned long long w[TAG_SLOTS][RW];
#pragma unroll
        for (int s = 0; s < TAG_SLOTS; ++s)
#pragma unroll
            for (int q = 0; q < RW; ++q)
                if (pending & (1u << (s * RW + q))) w[s][q] = ldWord(&tw[(size_t)k[s] * RW + q]);
#pragma unroll
        for (int s = 0; s < TAG_SLOTS; ++s)
#pragma unroll
            for (int q = 0; q < RW; ++q)
                if ((pending & (1u << (s * RW + q))) && (unsigned)(w[s][q] >> 32) == tag) {
                    lo[s][q] = (unsigned)w[s][q];
                    pending &= ~(1u << (s * RW + q));
                }
        if (!pending) break;
        if (round == 0) t0 = clock64();
        else if ((round & 15) == 0) {
            if (*(volatile int*)abort) return false;
            if (clock64() - t0 > GB_TIMEOUT_CYCLES) {
                atomicExch(abort, 1);
                return false;
            }
        }
        if (round >= 2 && pollNs > 0) __nanosleep(pollNs);
    }
#pragma unroll
    for (int s = 0; s < TAG_SLOTS; ++s)
#pragma unroll
        for (int e = 0; e < B; ++e) {
            if constexpr (NW == 1)
                x[s][e] = __uint_as_float(lo[s][e]);
            else
                x[s][e] = __longlong_as_double(
                    (long long)(((unsigned long long)lo[s][2 * e + 1] << 32) | lo[s][2 * e]));
        }
    return true;
}

template <class T, int B>
__device__ __noinline__ bool taggedApply(const GiluArgs<T>& a, const T* d, T* v, unsigned& tag)
{
    constexpr int RW = B * tagWords<T>();
    const unsigned tf = ++tag, tb = ++tag;
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, W = (gridDim.x * blockDim.x) >> 5;
    const int ld = a.ld;
    unsigned long long* tw = a.tw;
    bool ok = true;
    for (int c = gw; c < a.numChunks; c += W) {
        const int p = a.chunkPtr[c] + lane;
        if (ok && p < a.chunkPtr[c + 1]) {
            T rhs[B];
#pragma unroll
            for (int e = 0; e < B; ++e) rhs[e] = ldcg(&d[p * B + e]);
            int k[TAG_SLOTS];
            T L[TAG_SLOTS][B * B];
#pragma unroll
            for (int s = 0; s < TAG_SLOTS; ++s) {
                k[s] = s < a.diag ? a.col[(size_t)s * ld + p] : -1;
                if (k[s] >= 0) ldBlk<T, B>(a.F, s, ld, p, L[s]);
            }
            T x[TAG_SLOTS][B];
            if (!waitTagged<T, B>(tw, k, tf, x, a.gs.abort, a.pollNs)) ok = false;
#pragma unroll
            for (int s = 0; s < TAG_SLOTS; ++s)
                if (k[s] >= 0)
#pragma unroll
                    for (int i = 0; i < B; ++i)
#pragma unroll
                        for (int j = 0; j < B; ++j) rhs[i] -= L[s][i * B + j] * x[s][j];
#pragma unroll
            for (int e = 0; e < B; ++e) {
                v[p * B + e] = rhs[e];
                stTagged(&tw[(size_t)p * RW + e * tagWords<T>()], tf, rhs[e]);
            }
        }
        __syncwarp();  // the warp's lanes move to the next chunk together
    }
    if (gw < a.numChunks) {
        for (int c = gw + ((a.numChunks - 1 - gw) / W) * W; c >= 0; c -= W) {
            const int p = a.chunkPtr[c] + lane;
            if (ok && p < a.chunkPtr[c + 1]) {
                T rhs[B];
#pragma unroll
                for (int e = 0; e < B; ++e) rhs[e] = v[p * B + e];
                // upper slots in descending order, as iluApply takes them
                int k[TAG_SLOTS];
                T U[TAG_SLOTS][B * B];
#pragma unroll
                for (int q = 0; q < TAG_SLOTS; ++q) {
                    const int s = a.nslot - 1 - q;
                    k[q] = s > a.diag ? a.col[(size_t)s * ld + p] : -1;
                    if (k[q] >= 0) ldBlk<T, B>(a.F, s, ld, p, U[q]);
                }
                T Di[B * B];
                ldBlk<T, B>(a.F, a.diag, ld, p, Di);
                T x[TAG_SLOTS][B];
                if (!waitTagged<T, B>(tw, k, tb, x, a.gs.abort, a.pollNs)) ok = false;
#pragma unroll
                for (int q = 0; q < TAG_SLOTS; ++q)
                    if (k[q] >= 0)
#pragma unroll
                        for (int i = 0; i < B; ++i)
#pragma unroll
                            for (int j = 0; j < B; ++j) rhs[i] -= U[q][i * B + j] * x[q][j];
#pragma unroll
                for (int i = 0; i < B; ++i) {
                    T t = T(0);
#pragma unroll
                    for (int j = 0; j < B; ++j) t += Di[i * B + j] * rhs[j];
                    v[p * B + i] = t;
                    stTagged(&tw[(size_t)p * RW + i * tagWords<T>()], tb, t);
                }
            }
            __syncwarp();
        }
    }
    // the grid barrier after the sweeps makes v visible to every block
    return gridBarrier(a.gs) && ok;
}

template <class T, int B, bool TG, class Bar>
__device__ bool iluApply(const GiluArgs<T>& a, const T* d, T* v, int gt, int gs, const Bar& bar, unsigned& tag)
{
    if constexpr (TG) return taggedApply<T, B>(a, d, v, tag);
    if (a.warpSweep) {
        extern __shared__ __align__(16) unsigned char gsmem[];
        narrowSweeps<T, B>(a, d, v, gsmem);
        return bar();
    }
    const int ld = a.ld;
    for (int l = 0; l < a.numLev; ++l) {
        for (int p = a.levPtr[l] + gt; p < a.levPtr[l + 1]; p += gs) {
            T rhs[B];
#pragma unroll
            for (int e = 0; e < B; ++e) rhs[e] = ldcg(&d[p * B + e]);
            for (int s = 0; s < a.diag; ++s) {
                const int k = a.col[(size_t)s * ld + p];
                if (k < 0) continue;
                T L[B * B];
                ldBlk<T, B>(a.F, s, ld, p, L);
#pragma unroll
                for (int i = 0; i < B; ++i)
#pragma unroll
                    for (int j = 0; j < B; ++j) rhs[i] -= L[i * B + j] * ldcg(&v[k * B + j]);
            }
#pragma unroll
            for (int e = 0; e < B; ++e) v[p * B + e] = rhs[e];
        }
        if (!bar()) return false;
    }
    for (int l = a.numLev - 1; l >= 0; --l) {
        for (int p = a.levPtr[l] + gt; p < a.levPtr[l + 1]; p += gs) {
            T rhs[B];
#pragma unroll
            for (int e = 0; e < B; ++e) rhs[e] = ldcg(&v[p * B + e]);
            for (int s = a.nslot - 1; s > a.diag; --s) {
                const int k = a.col[(size_t)s * ld + p];
                if (k < 0) continue;
                T U[B * B];
                ldBlk<T, B>(a.F, s, ld, p, U);
#pragma unroll
                for (int i = 0; i < B; ++i)
#pragma unroll
                    for (int j = 0; j < B; ++j) rhs[i] -= U[i * B + j] * ldcg(&v[k * B + j]);
            }
            T Di[B * B];
            ldBlk<T, B>(a.F, a.diag, ld, p, Di);
#pragma unroll
            for (int i = 0; i < B; ++i) {
                T t = T(0);
#pragma unroll
                for (int j = 0; j < B; ++j) t += Di[i * B + j] * rhs[j];
                v[p * B + i] = t;
            }
        }
        if (!bar()) return false;
    }
    return true;
}

// ------------------------------------------------ narrow-system sweeps --
// A system whose levels all have at most 32 rows sweeps with one warp: lane
// r takes row r of every level (an FP64 warp instruction costs the same
// with 5 active lanes as with 17, so spreading a level's rows over more
// warps measured slower).  The sweep's input and output vectors live in
// shared memory, and the block's other warps stream each level's column
// indices and factor blocks into a shared-memory ring with cp.async,
// GILU_AHEAD levels ahead of the sweep, so a level costs its FP64 work, a
// few shared-memory round trips and one block barrier instead of a chain of
// L2 loads (the sweeping warp staging its own copies measured slower).
// Same operations in the same order as iluApply.
constexpr int GILU_RING = 8;                // ring slots (levels in flight + 2)
constexpr int GILU_AHEAD = GILU_RING - 2;   // a slot is refilled two levels after its use

__device__ __forceinline__ void cpAsync(void* dst, const void* src, int bytes)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if (bytes == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cpCommit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cpWaitAhead() { asm volatile("cp.async.wait_group %0;\n" ::"n"(GILU_AHEAD) : "memory"); }
__device__ __forceinline__ void cpWaitAll() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// planes of one ring slot: WARP_SLOTS blocks (and, backward, the inverted
// pivot) of T per row, WARP_SLOTS column indices per row, 32 rows each
template <class T, int B>
struct Ring {
    static constexpr int TP = (WARP_SLOTS + 1) * B * B;  // T planes
    static constexpr int IP = WARP_SLOTS;                // int planes
    static constexpr size_t bytes = (size_t)GILU_RING * 32 * (TP * sizeof(T) + IP * sizeof(int));
    T* t;    // [slot][TP][32]
    int* c;  // [slot][IP][32]
};

// shared-memory bytes of the narrow path: the ring, two vectors, the level pointers
template <class T, int B>
size_t narrowBytes(int N, int numLev)
{
    return Ring<T, B>::bytes + 2 * sizeof(T) * (size_t)N * B + sizeof(int) * (size_t)(numLev + 1);
}

// the staging warps: level l's data into ring slot l % GILU_RING (forward:
// the lower slots in ascending order; backward: the upper slots in
// descending order and the inverted pivot); one commit group per call,
// empty past the ends
template <class T, int B>
__device__ __forceinline__ void stageLevel(const GiluArgs<T>& a, const Ring<T, B>& R, const int* lp, int l,
                                           bool forward, int pt, int ps)
{
    if (l >= 0 && l < a.numLev) {
        const int p0 = lp[l], rows = lp[l + 1] - p0, ld = a.ld, sl = l % GILU_RING;
        T* rt = R.t + (size_t)sl * Ring<T, B>::TP * 32;
        int* rc = R.c + (size_t)sl * Ring<T, B>::IP * 32;
        const int nT = (forward ? WARP_SLOTS : WARP_SLOTS + 1) * B * B;
        for (int q = pt; q < (nT + WARP_SLOTS) * rows; q += ps) {
            const int plane = q / rows, r = q - plane * rows;
            if (plane < nT) {
                const int u = plane / (B * B), e = plane - u * B * B;
                int slot;
                if (forward) slot = u < a.diag ? u : -1;
                else slot = u < WARP_SLOTS ? (a.nslot - 1 - u > a.diag ? a.nslot - 1 - u : -1) : a.diag;
                if (slot >= 0) cpAsync(&rt[plane * 32 + r], &a.F[((size_t)slot * B * B + e) * ld + p0 + r], sizeof(T));
            }
            else {
                const int u = plane - nT;
                const int slot = forward ? u : a.nslot - 1 - u;
                const bool ok = forward ? slot < a.diag : slot > a.diag;
                if (ok) cpAsync(&rc[u * 32 + r], &a.col[(size_t)slot * ld + p0 + r], 4);
                else rc[u * 32 + r] = -1;
            }
        }
    }
    cpCommit();
}

template <class T, int B>
__device__ void narrowSweeps(const GiluArgs<T>& a, const T* d, T* v, unsigned char* smem)
{
    Ring<T, B> R;
    R.t = reinterpret_cast<T*>(smem);
    R.c = reinterpret_cast<int*>(smem + (size_t)GILU_RING * 32 * Ring<T, B>::TP * sizeof(T));
    T* sd = reinterpret_cast<T*>(smem + Ring<T, B>::bytes);
    T* sv = sd + (size_t)a.N * B;
    int* lp = reinterpret_cast<int*>(sv + (size_t)a.N * B);  // the level pointers
    const int lane = threadIdx.x & 31, nL = a.numLev;
    const bool sweeper = threadIdx.x < 32;
    const int pt = threadIdx.x - 32, ps = blockDim.x - 32;  // staging rank / count
    for (int i = threadIdx.x; i < a.N * B; i += blockDim.x) sd[i] = ldcg(&d[i]);
    for (int i = threadIdx.x; i <= nL; i += blockDim.x) lp[i] = a.levPtr[i];
    __syncthreads();
    for (int dir = 0; dir < 2; ++dir) {
        const bool fw = dir == 0;
        auto lev = [&](int step) { return fw ? step : nL - 1 - step; };
        if (!sweeper)
            for (int k = 0; k < GILU_AHEAD; ++k) stageLevel<T, B>(a, R, lp, lev(k), fw, pt, ps);
        for (int step = 0; step < nL; ++step) {
            if (!sweeper) {
                stageLevel<T, B>(a, R, lp, lev(step + GILU_AHEAD), fw, pt, ps);
                cpWaitAhead();  // the group of level `step` has landed
            }
            __syncthreads();
            if (sweeper) {
                const int l = lev(step), p0 = lp[l], rows = lp[l + 1] - p0, sl = l % GILU_RING;
                if (lane < rows) {
                    const int p = p0 + lane;
                    const T* rt = R.t + (size_t)sl * Ring<T, B>::TP * 32;
                    const int* rc = R.c + (size_t)sl * Ring<T, B>::IP * 32;
                    T x[B];
#pragma unroll
                    for (int e = 0; e < B; ++e) x[e] = fw ? sd[p * B + e] : sv[p * B + e];
#pragma unroll
                    for (int u = 0; u < WARP_SLOTS; ++u) {
                        const int k = rc[u * 32 + lane];
                        if (k < 0) continue;
#pragma unroll
                        for (int i = 0; i < B; ++i)
#pragma unroll
                            for (int j = 0; j < B; ++j) x[i] -= rt[(u * B * B + i * B + j) * 32 + lane] * sv[k * B + j];
                    }
                    if (fw) {
#pragma unroll
                        for (int e = 0; e < B; ++e) sv[p * B + e] = x[e];
                    }
                    else {
#pragma unroll
                        for (int i = 0; i < B; ++i) {
                            T t = T(0);
#pragma unroll
                            for (int j = 0; j < B; ++j) t += rt[(WARP_SLOTS * B * B + i * B + j) * 32 + lane] * x[j];
                            sv[p * B + i] = t;
                        }
                    }
                }
            }
        }
        if (!sweeper) cpWaitAll();
        __syncthreads();
    }
    for (int i = threadIdx.x; i < a.N * B; i += blockDim.x) v[i] = sv[i];
}

template <class T, int B, class Bar>
__device__ bool factorAll(const GiluArgs<T>& a, int gt, int gs, const Bar& bar)
{
    // one block: a level's rows round-robin over the warps, so its FP64 work
    // spreads over the SM's sub-partitions
    if (gridDim.x == 1) gt = (threadIdx.x & 31) * (blockDim.x >> 5) + (threadIdx.x >> 5);
    for (int l = 0; l < a.numLev; ++l) {
        for (int p = a.levPtr[l] + gt; p < a.levPtr[l + 1]; p += gs)
            if (!(a.localFactor ? factorRowLocal<T, B>(a, p) : factorRow<T, B>(a, p))) {
                atomicCAS(&a.st->code, 0, (int)GBFV_ERR_SINGULAR);
                a.st->where = p;
            }
        if (!bar()) return false;
    }
    return true;
}

// y = A x, row p, slots in ascending column order (BCRSMatrix::mv)
template <class T, int B>
__device__ __forceinline__ void spmvRow(const GiluArgs<T>& a, const T* xin, int p, T (&acc)[B])
{
#pragma unroll
    for (int e = 0; e < B; ++e) acc[e] = T(0);
    if (a.nslot <= 9) {
        // up to nine slots: every column index, then every block and
        // gathered value, issued before the first product
        int k[9];
#pragma unroll
        for (int s = 0; s < 9; ++s) k[s] = s < a.nslot ? a.col[(size_t)s * a.ld + p] : -1;
        T M[9][B * B], X[9][B];
#pragma unroll
        for (int s = 0; s < 9; ++s)
            if (k[s] >= 0) {
#pragma unroll
                for (int e = 0; e < B * B; ++e) M[s][e] = a.A[((size_t)s * B * B + e) * a.ld + p];
#pragma unroll
                for (int j = 0; j < B; ++j) X[s][j] = ldcg(&xin[k[s] * B + j]);
            }
#pragma unroll
        for (int s = 0; s < 9; ++s)
            if (k[s] >= 0)
#pragma unroll
                for (int i = 0; i < B; ++i)
#pragma unroll
                    for (int j = 0; j < B; ++j) acc[i] += M[s][i * B + j] * X[s][j];
        return;
    }
    for (int s = 0; s < a.nslot; ++s) {
        const int k = a.col[(size_t)s * a.ld + p];
        if (k < 0) continue;
        T M[B * B];
#pragma unroll
        for (int e = 0; e < B * B; ++e) M[e] = a.A[((size_t)s * B * B + e) * a.ld + p];
#pragma unroll
        for (int i = 0; i < B; ++i)
#pragma unroll
            for (int j = 0; j < B; ++j) acc[i] += M[i * B + j] * ldcg(&xin[k * B + j]);
    }
}

struct GBar {
    const GridSync* g;
    __device__ bool operator()() const { return gridBarrier(*g); }
};

// BiCGStabSolver::apply (bicgstabsolver.hh:120-330) with the block ILU(0)
// preconditioner, factorization included, in one cooperative launch
template <class T, int B, bool TG>
__global__ void __launch_bounds__(GILU_THREADS) kGiluBicgstab(const GiluArgs<T> a)
{
    const Team<SYNC_GRID> tm;
    const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
    const int N = a.N;
    const GBar bar{&a.gs};
    const double eps = 2.2250738585072014e-308 * 1e10;  // numeric_limits<double>::min()*1e10
    // optional timers: [0] factorization, [1] set-up, [2] p, [3] first
    // preconditioner, [4] SpMV + dot, [5] x / r update, [6] second
    // preconditioner, [7] SpMV + dots, [8] last update
    PhaseClock clk(a.prof, gt);
    unsigned tag = 0;  // tagged sweeps: the last tag used
    if (a.factor) {
        if (!factorAll<T, B>(a, gt, gs, bar)) goto timeout;
        if (*(volatile int*)&a.st->code != 0) return;
    }
    clk.tick(0);
    {
        double mx[1] = {0.0};
        const bool isMax1[1] = {true};
        for (int i = gt; i < N; i += gs)
#pragma unroll
            for (int e = 0; e < B; ++e) {
                const T bi = a.rhs[i * B + e];
                a.x[i * B + e] = T(0);
                a.r[i * B + e] = bi;
                a.v[i * B + e] = T(0);
                a.p[i * B + e] = T(0);
                mx[0] = fmax(mx[0], fabs((double)bi));
            }
        blockPartials<1, SYNC_GRID>(mx, isMax1, a.partial, tm);
        if (!gridBarrier(a.gs)) goto timeout;
    }
    {
        double tot[1];
        const bool isMax1[1] = {true};
        allCombine<1, SYNC_GRID>(a.partial, isMax1, tot, tm);
        double resErr = fmax(tot[0], eps);
        const double initErr = resErr;
        auto converged = [&](double re) { return re / fmax(1e-20, initErr) <= a.redTol || re <= a.absTol; };
        if (converged(resErr)) {
            if (gt == 0) {
                a.st->converged = 1;
                a.st->iterations = 0;
                a.st->resid = resErr;
                a.st->resid0 = initErr;
            }
            return;
        }
        double rho = 1.0, alpha = 1.0, omega = 1.0;
        {
            double dd[1] = {0.0};
            const bool isSum1[1] = {false};
            for (int i = gt; i < N; i += gs) {
                double t = 0.0;
#pragma unroll
                for (int e = 0; e < B; ++e) t += (double)(a.rhs[i * B + e] * a.rhs[i * B + e]);
                dd[0] += t;
            }
            blockPartials<1, SYNC_GRID>(dd, isSum1, a.partial + 2 * tm.nblk, tm);
            if (!gridBarrier(a.gs)) goto timeout;
        }
        int it = 0;
        int buf = 1;
        for (; it < a.maxIter; ++it) {
            double rho_i;
            {
                const bool isSum1[1] = {false};
                double tot1[1];
                allCombine<1, SYNC_GRID>(a.partial + 2 * tm.nblk * buf, isSum1, tot1, tm);
                rho_i = tot1[0];
            }
            if (fabs(rho) <= eps || fabs(omega) <= eps) {
                if (gt == 0) a.st->code = GBFV_ERR_BREAKDOWN;
                break;
            }
            clk.tick(1);
            const double beta = (rho_i / rho) * (alpha / omega);
            rho = rho_i;
            {
                // p = r - beta (p - omega v), in the reference's steps
                const T tb = (T)beta, to = (T)omega;
                for (int i = gt; i < N; i += gs)
#pragma unroll
                    for (int e = 0; e < B; ++e) {
                        T tmp = ldcg(&a.v[i * B + e]);
                        tmp *= to;
                        tmp -= ldcg(&a.p[i * B + e]);
                        tmp *= -tb;
                        a.p[i * B + e] = ldcg(&a.r[i * B + e]) + tmp;
                    }
                if (!gridBarrier(a.gs)) goto timeout;
            }
            clk.tick(2);
            if (!iluApply<T, B, TG>(a, a.p, a.y, gt, gs, bar, tag)) goto timeout;
            clk.tick(3);
            {
                double dd[1] = {0.0};
                const bool isSum1[1] = {false};
                for (int i = gt; i < N; i += gs) {
                    T acc[B];
                    spmvRow<T, B>(a, a.y, i, acc);
                    double t = 0.0;
#pragma unroll
                    for (int e = 0; e < B; ++e) {
                        a.v[i * B + e] = acc[e];
                        t += (double)(a.rhs[i * B + e] * acc[e]);
                    }
                    dd[0] += t;
                }
                buf ^= 1;
                blockPartials<1, SYNC_GRID>(dd, isSum1, a.partial + 2 * tm.nblk * buf, tm);
                if (!gridBarrier(a.gs)) goto timeout;
                double tot1[1];
                allCombine<1, SYNC_GRID>(a.partial + 2 * tm.nblk * buf, isSum1, tot1, tm);
                const double denom = tot1[0];
                if (fabs(denom) <= eps) {
                    if (gt == 0) a.st->code = GBFV_ERR_BREAKDOWN;
                    break;
                }
                alpha = rho_i / denom;
                clk.tick(4);
                if (fabs(alpha) <= eps) {
                    if (gt == 0) a.st->code = GBFV_ERR_BREAKDOWN;
                    break;
                }
            }
            {
                double red[2] = {0.0, 0.0};
                const bool kinds[2] = {true, true};
                const T ta = (T)alpha;
                for (int i = gt; i < N; i += gs)
#pragma unroll
                    for (int e = 0; e < B; ++e) {
                        T tmp = ldcg(&a.y[i * B + e]);
                        if (tmp != T(0)) red[1] = 1.0;
                        tmp *= ta;
                        tmp += ldcg(&a.x[i * B + e]);
                        a.x[i * B + e] = tmp;
                        tmp = ldcg(&a.v[i * B + e]);
                        tmp *= ta;
                        const T si = ldcg(&a.r[i * B + e]) - tmp;
                        a.r[i * B + e] = si;
                        red[0] = fmax(red[0], fabs((double)si));
                    }
                buf ^= 1;
                blockPartials<2, SYNC_GRID>(red, kinds, a.partial + 2 * tm.nblk * buf, tm);
                if (!gridBarrier(a.gs)) goto timeout;
                double tot2[2];
                allCombine<2, SYNC_GRID>(a.partial + 2 * tm.nblk * buf, kinds, tot2, tm);
                resErr = tot2[0];
                const bool stag = tot2[1] == 0.0;
                if (converged(resErr)) {
                    if (gt == 0) a.st->converged = 1;
                    break;
                }
                if (stag || resErr > a.maxRes) break;
            }
            clk.tick(5);
            if (!iluApply<T, B, TG>(a, a.r, a.z, gt, gs, bar, tag)) goto timeout;
            clk.tick(6);
            {
                double dd[2] = {0.0, 0.0};
                const bool isSum2[2] = {false, false};
                for (int i = gt; i < N; i += gs) {
                    T acc[B];
                    spmvRow<T, B>(a, a.z, i, acc);
                    double t0 = 0.0, t1 = 0.0;
#pragma unroll
                    for (int e = 0; e < B; ++e) {
                        a.y[i * B + e] = acc[e];
                        t0 += (double)(acc[e] * acc[e]);
                        t1 += (double)(acc[e] * ldcg(&a.r[i * B + e]));
                    }
                    dd[0] += t0;
                    dd[1] += t1;
                }
                buf ^= 1;
                blockPartials<2, SYNC_GRID>(dd, isSum2, a.partial + 2 * tm.nblk * buf, tm);
                if (!gridBarrier(a.gs)) goto timeout;
                double tot2[2];
                allCombine<2, SYNC_GRID>(a.partial + 2 * tm.nblk * buf, isSum2, tot2, tm);
                const double denom = tot2[0];
                if (fabs(denom) <= eps) {
                    if (gt == 0) a.st->code = GBFV_ERR_BREAKDOWN;
                    break;
                }
                omega = tot2[1] / denom;
                clk.tick(7);
                if (fabs(omega) <= eps) {
                    if (gt == 0) a.st->code = GBFV_ERR_BREAKDOWN;
                    break;
                }
            }
            {
                double red[2] = {0.0, 0.0};
                const bool kinds[2] = {false, true};
                const T to = (T)omega;
                for (int i = gt; i < N; i += gs) {
                    double t = 0.0;
#pragma unroll
                    for (int e = 0; e < B; ++e) {
                        const T zi = ldcg(&a.z[i * B + e]);
                        if (zi != T(0)) red[1] = 1.0;
                        a.x[i * B + e] = ldcg(&a.x[i * B + e]) + to * zi;
                        const T ri = ldcg(&a.r[i * B + e]) + (-to) * ldcg(&a.y[i * B + e]);
                        a.r[i * B + e] = ri;
                        t += (double)(a.rhs[i * B + e] * ri);
                    }
                    red[0] += t;
                }
                buf ^= 1;
                blockPartials<2, SYNC_GRID>(red, kinds, a.partial + 2 * tm.nblk * buf, tm);
                if (!gridBarrier(a.gs)) goto timeout;
                double tot2[2];
                allCombine<2, SYNC_GRID>(a.partial + 2 * tm.nblk * buf, kinds, tot2, tm);
                clk.tick(8);
                if (tot2[1] == 0.0) break;
            }
        }
        if (gt == 0) {
            a.st->iterations = it;
            a.st->resid = resErr;
            a.st->resid0 = initErr;
        }
    }
    return;
timeout:
    if (gt == 0) a.st->code = GBFV_ERR_TIMEOUT;
}

// factorization and one preconditioner application alone (tests)
template <class T, int B, bool TG>
__global__ void __launch_bounds__(GILU_THREADS) kGiluApply(const GiluArgs<T> a)
{
    const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
    const GBar bar{&a.gs};
    unsigned tag = 0;
    if (!factorAll<T, B>(a, gt, gs, bar)) {
        if (gt == 0) a.st->code = GBFV_ERR_TIMEOUT;
        return;
    }
    if (*(volatile int*)&a.st->code != 0) return;
    if (!iluApply<T, B, TG>(a, a.rhs, a.x, gt, gs, bar, tag) && gt == 0) a.st->code = GBFV_ERR_TIMEOUT;
}

}  // namespace

struct GiluData {
    int N = 0, b = 0, nslot = 0, ld = 0, numLev = 0, blocks = 1, maxWidth = 0;
    int warp = 0;  // narrow system: warp sweeps with the vector in shared memory
    int localFactor = 0;  // rows factored in local arrays (factorRowLocal)
    const int* col = nullptr;  // not owned
    int* levPtr = nullptr;
    int* updPtr = nullptr;
    int* upd = nullptr;
    double* F64 = nullptr;
    float* F32 = nullptr;
    double* vec64 = nullptr;  // x r p v y z
    float* vec32 = nullptr;
    double* partial = nullptr;
    unsigned* bar = nullptr;
    cudaEvent_t evA = nullptr, evB = nullptr;
    size_t nnz = 0;
    unsigned long long* prof = nullptr;  // GBFV_GILU_PROFILE phase timers
    int tagged = 0, tagged64 = 0;  // tagged sweeps of FP32 / FP64 solves (several blocks)
    // back-off of a waiting row between polls (GBFV_GILU_POLL_NS): none --
    // on the 1M-cell FP32 solve 0 / 16 / 32 / 100 / 250 ns measured 295 /
    // 304 / 309 / 310 / 310 ms, so the polls' L2 traffic does not slow the
    // producers and a sleep only adds latency
    int pollNs = 0;
    int numChunks = 0;
    int* chunkPtr = nullptr;
    unsigned long long* tw = nullptr;
};

GiluData* giluCreate(int N, int b, int nslot, int ld, const std::vector<int>& colHost, const int* colDev,
                     const std::vector<int>& levPtr, int* status)
{
    GiluData* d = new GiluData();
    auto fail = [&](int st, const std::string& msg) -> GiluData* {
        if (!msg.empty()) setLastError("ILU(0): " + msg);
        if (status) *status = st;
        giluDestroy(d);
        return nullptr;
    };
    if ((b != 2 && b != 3) || nslot < 1 || nslot > 255 || nslot % 2 == 0) return fail(GBFV_ERR_UNSUPPORTED, "layout");
    d->N = N;
    d->b = b;
    d->nslot = nslot;
    d->ld = ld;
    d->col = colDev;
    d->numLev = (int)levPtr.size() - 1;
    const int diag = nslot / 2;
    // layout checks, the level of every row, and the update lists
    std::vector<int> levOf(N, -1);
    for (int l = 0; l < d->numLev; ++l) {
        d->maxWidth = std::max(d->maxWidth, levPtr[l + 1] - levPtr[l]);
        for (int p = levPtr[l]; p < levPtr[l + 1]; ++p) levOf[p] = l;
    }
    auto C = [&](int s, int p) { return colHost[(size_t)s * ld + p]; };
    std::vector<int> updPtr(N + 1, 0), upd;
    for (int p = 0; p < N; ++p) {
        if (levOf[p] < 0 || C(diag, p) != p) return fail(GBFV_ERR_UNSUPPORTED, "diagonal or level missing");
        for (int s = 0; s < nslot; ++s) {
            const int k = C(s, p);
            if (k < 0 || s == diag) continue;
            if (k >= N || (s < diag) != (levOf[k] < levOf[p]) || levOf[k] == levOf[p])
                return fail(GBFV_ERR_UNSUPPORTED, "a lower entry outside the earlier levels");
        }
        for (int s = 0; s < diag; ++s) {
            const int k = C(s, p);
            if (k < 0) continue;
            for (int u = diag + 1; u < nslot; ++u) {
                const int j = C(u, k);
                if (j < 0) continue;
                for (int t = 0; t < nslot; ++t)
                    if (C(t, p) == j) {
                        upd.push_back(s | (t << 8) | (u << 16));
                        break;
                    }
            }
        }
        updPtr[p + 1] = (int)upd.size();
    }
    for (int s = 0; s < nslot; ++s)
        for (int p = 0; p < N; ++p) d->nnz += C(s, p) >= 0;
    {
        int maxUpd = 0;
        for (int p = 0; p < N; ++p) maxUpd = std::max(maxUpd, updPtr[p + 1] - updPtr[p]);
        d->localFactor = nslot <= 9 && diag <= WARP_SLOTS && maxUpd <= GILU_MAX_UPD;
    }
    auto up = [&](int** dst, const std::vector<int>& v) {
        if (cudaMalloc((void**)dst, sizeof(int) * std::max<size_t>(1, v.size())) != cudaSuccess) return false;
        return v.empty() || cudaMemcpy(*dst, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice) == cudaSuccess;
    };
    if (!up(&d->levPtr, levPtr) || !up(&d->updPtr, updPtr) || !up(&d->upd, upd)) return fail(GBFV_ERR_OOM, "");
    // one block when every level fits it (block barriers only), else a
    // cooperative grid (GBFV_GILU_BLOCKS overrides)
    int dev = 0, nsm = 1, occ = 1 << 20;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    for (const void* fn : {b == 2 ? (const void*)kGiluBicgstab<double, 2, false> : (const void*)kGiluBicgstab<double, 3, false>,
                           b == 2 ? (const void*)kGiluBicgstab<float, 2, false> : (const void*)kGiluBicgstab<float, 3, false>,
                           b == 2 ? (const void*)kGiluApply<double, 2, false> : (const void*)kGiluApply<double, 3, false>,
                           b == 2 ? (const void*)kGiluBicgstab<double, 2, true> : (const void*)kGiluBicgstab<double, 3, true>,
                           b == 2 ? (const void*)kGiluBicgstab<float, 2, true> : (const void*)kGiluBicgstab<float, 3, true>,
                           b == 2 ? (const void*)kGiluApply<double, 2, true> : (const void*)kGiluApply<double, 3, true>}) {
        int o = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, fn, GILU_THREADS, 0);
        occ = std::min(occ, o);
    }
    const int maxCoop = std::max(1, occ) * nsm;
    int blocks = N <= 65536 ? 1 : std::min(maxCoop, std::max(1, (N + 4095) / 4096));
    if (const char* e = getenv("GBFV_GILU_BLOCKS")) blocks = std::max(1, std::min(maxCoop, atoi(e)));
    d->blocks = blocks;
    // narrow systems: one block, every level within a warp, the ring and
    // both sweep vectors (FP64) within 200 KB of shared memory
    // (GBFV_GILU_WARP=0: off)
    const int diagSlot = nslot / 2;
    const size_t nb = b == 2 ? narrowBytes<double, 2>(N, d->numLev) : narrowBytes<double, 3>(N, d->numLev);
    d->warp = blocks == 1 && d->maxWidth <= 32 && diagSlot <= WARP_SLOTS && nslot - 1 - diagSlot <= WARP_SLOTS &&
              nb <= 200 * 1024;
    if (const char* e = getenv("GBFV_GILU_WARP")) d->warp = d->warp && atoi(e) != 0;
    if (d->warp) {
        const int bytes = (int)nb;
        for (const void* fn : {b == 2 ? (const void*)kGiluBicgstab<double, 2, false> : (const void*)kGiluBicgstab<double, 3, false>,
                               b == 2 ? (const void*)kGiluBicgstab<float, 2, false> : (const void*)kGiluBicgstab<float, 3, false>,
                               b == 2 ? (const void*)kGiluApply<double, 2, false> : (const void*)kGiluApply<double, 3, false>})
            if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess)
                d->warp = 0;
    }
    // tagged sweeps for systems on several blocks whose rows have at most
    // TAG_SLOTS lower and upper entries: FP32 (GBFV_GILU_TAGGED=0: off) and
    // FP64 (GBFV_GILU_TAGGED64=0: off); chunks of at most 32 rows inside
    // one level
    d->tagged = d->tagged64 = blocks > 1 && diagSlot <= TAG_SLOTS && nslot - 1 - diagSlot <= TAG_SLOTS;
    if (const char* e = getenv("GBFV_GILU_TAGGED64")) d->tagged64 = d->tagged64 && atoi(e) != 0;
    if (const char* e = getenv("GBFV_GILU_TAGGED")) d->tagged = d->tagged && atoi(e) != 0;
    if (const char* e = getenv("GBFV_GILU_POLL_NS")) d->pollNs = std::max(0, std::min(1000, atoi(e)));
    // the tagged sweeps take every SM (more warps in flight per level: 139
    // against 158 ms for a 200k-cell FP32 solve on 152 against 49 blocks)
    if ((d->tagged || d->tagged64) && !getenv("GBFV_GILU_BLOCKS")) d->blocks = blocks = maxCoop;
    if (d->tagged || d->tagged64) {
        std::vector<int> chunks;
        for (int l = 0; l < d->numLev; ++l)
            for (int p = levPtr[l]; p < levPtr[l + 1]; p += 32) chunks.push_back(p);
        chunks.push_back(N);
        d->numChunks = (int)chunks.size() - 1;
        if (!up(&d->chunkPtr, chunks)) return fail(GBFV_ERR_OOM, "");
    }
    // the factors and vectors of a precision are allocated at its first solve
    if (cudaMalloc((void**)&d->partial, sizeof(double) * 4 * (size_t)std::max(blocks, 16)) != cudaSuccess ||
        cudaMalloc((void**)&d->bar, 4 * sizeof(unsigned)) != cudaSuccess)
        return fail(GBFV_ERR_OOM, "");
    cudaMemset(d->bar, 0, 4 * sizeof(unsigned));
    cudaEventCreate(&d->evA);
    cudaEventCreate(&d->evB);
    if (status) *status = GBFV_OK;
    return d;
}

int giluTagged(const GiluData* d, int fp64) { return d ? (fp64 ? d->tagged64 : d->tagged) : 0; }
int giluBlocks(const GiluData* d) { return d ? d->blocks : 0; }

void giluDestroy(GiluData* d)
{
    if (!d) return;
    cudaFree(d->levPtr);
    cudaFree(d->updPtr);
    cudaFree(d->upd);
    cudaFree(d->F64);
    cudaFree(d->F32);
    cudaFree(d->vec64);
    cudaFree(d->vec32);
    cudaFree(d->partial);
    cudaFree(d->bar);
    cudaFree(d->prof);
    cudaFree(d->chunkPtr);
    cudaFree(d->tw);
    if (d->evA) cudaEventDestroy(d->evA);
    if (d->evB) cudaEventDestroy(d->evB);
    delete d;
}

namespace {

template <class T>
int args(GiluData& d, GiluArgs<T>& a, const T* A, const T* rhs, DevStatus* st)
{
    const size_t nv = (size_t)d.N * d.b + 16;
    T* vec;
    T* F;
    if (sizeof(T) == 8) {
        if (!d.vec64 && (cudaMalloc((void**)&d.vec64, sizeof(double) * 6 * nv) != cudaSuccess ||
                         cudaMalloc((void**)&d.F64, sizeof(double) * (size_t)d.nslot * d.b * d.b * d.ld) != cudaSuccess))
            return GBFV_ERR_OOM;
        vec = (T*)d.vec64;
        F = (T*)d.F64;
    }
    else {
        if (!d.vec32 && (cudaMalloc((void**)&d.vec32, sizeof(float) * 6 * nv) != cudaSuccess ||
                         cudaMalloc((void**)&d.F32, sizeof(float) * (size_t)d.nslot * d.b * d.b * d.ld) != cudaSuccess))
            return GBFV_ERR_OOM;
        vec = (T*)d.vec32;
        F = (T*)d.F32;
    }
    const bool tagged = sizeof(T) == 4 ? d.tagged : d.tagged64;
    // tagged words: two per component (enough for FP64)
    if (tagged && !d.tw && cudaMalloc((void**)&d.tw, sizeof(unsigned long long) * 2 * (size_t)d.N * d.b) != cudaSuccess)
        return GBFV_ERR_OOM;
    a.N = d.N;
    a.ld = d.ld;
    a.nslot = d.nslot;
    a.diag = d.nslot / 2;
    a.numLev = d.numLev;
    a.col = d.col;
    a.levPtr = d.levPtr;
    a.updPtr = d.updPtr;
    a.upd = d.upd;
    a.A = A;
    a.F = F;
    a.rhs = rhs;
    a.x = vec;
    a.r = vec + nv;
    a.p = vec + 2 * nv;
    a.v = vec + 3 * nv;
    a.y = vec + 4 * nv;
    a.z = vec + 5 * nv;
    a.partial = d.partial;
    a.gs.count = d.bar;
    a.gs.gen = d.bar + 1;
    a.gs.abort = (int*)(d.bar + 2);
    a.gs.perCluster = 0;
    a.st = st;
    a.warpSweep = d.warp;
    a.prof = d.prof;
    a.localFactor = d.localFactor;
    a.tagged = tagged;
    a.pollNs = d.pollNs;
    a.numChunks = d.numChunks;
    a.chunkPtr = d.chunkPtr;
    a.tw = d.tw;
    return GBFV_OK;
}

// the sweep vector of the warp sweeps in shared memory: N * b values of T
template <class T>
int launch(const void* fn, GiluArgs<T>& a, int blocks, int b, cudaStream_t s)
{
    void* argv[] = {(void*)&a};
    const size_t smem = !a.warpSweep ? 0 : b == 2 ? narrowBytes<T, 2>(a.N, a.numLev) : narrowBytes<T, 3>(a.N, a.numLev);
    const cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(GILU_THREADS), argv, smem, s);
    countLaunch();
    if (e != cudaSuccess) {
        setLastError(std::string("ILU(0) cooperative launch failed: ") + cudaGetErrorString(e));
        return GBFV_ERR_CUDA;
    }
    return GBFV_OK;
}

}  // namespace

template <class T>
int giluSolve(GiluData* d, const T* A, const T* rhs, T* x, int factor, double redTol, double absTol, double maxRes,
              int maxIter, cudaStream_t s, DevStatus* st, DevStatus* hst, int& iters, float* ms, double* bytes)
{
    GiluArgs<T> a;
    int rs;
    if ((rs = args<T>(*d, a, A, rhs, st))) return rs;
    a.factor = factor;
    a.redTol = redTol;
    a.absTol = absTol;
    a.maxRes = maxRes;
    a.maxIter = maxIter;
    const char* profFile = getenv("GBFV_GILU_PROFILE");
    if (profFile && !d->prof) {
        if (cudaMalloc((void**)&d->prof, 16 * sizeof(unsigned long long)) != cudaSuccess) return GBFV_ERR_OOM;
        a.prof = d->prof;
    }
    if (d->prof && cudaMemsetAsync(d->prof, 0, 16 * sizeof(unsigned long long), s) != cudaSuccess)
        return GBFV_ERR_CUDA;
    if (cudaMemsetAsync(st, 0, sizeof(DevStatus), s) != cudaSuccess ||
        cudaMemsetAsync(d->bar, 0, 4 * sizeof(unsigned), s) != cudaSuccess)
        return GBFV_ERR_CUDA;
    if (a.tagged && cudaMemsetAsync(d->tw, 0, sizeof(T) * 2 * (size_t)d->N * d->b, s) != cudaSuccess)
        return GBFV_ERR_CUDA;
    cudaEventRecord(d->evA, s);
    const void* fn = a.tagged ? (d->b == 2 ? (const void*)kGiluBicgstab<T, 2, true> : (const void*)kGiluBicgstab<T, 3, true>)
                              : (d->b == 2 ? (const void*)kGiluBicgstab<T, 2, false> : (const void*)kGiluBicgstab<T, 3, false>);
    if ((rs = launch<T>(fn, a, d->blocks, d->b, s))) return rs;
    if (cudaMemcpyAsync(x, a.x, sizeof(T) * (size_t)d->N * d->b, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return GBFV_ERR_CUDA;
    cudaEventRecord(d->evB, s);
    if (cudaMemcpyAsync(hst, st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        setLastError(std::string("ILU(0) solve: ") + cudaGetErrorString(cudaGetLastError()));
        return GBFV_ERR_CUDA;
    }
    iters = hst->iterations;
    if (ms) cudaEventElapsedTime(ms, d->evA, d->evB);
    if (profFile && d->prof) {
        // one JSON line per solve: nanoseconds per phase
        unsigned long long h[16];
        if (cudaMemcpy(h, d->prof, sizeof(h), cudaMemcpyDeviceToHost) == cudaSuccess)
            if (FILE* f = std::fopen(profFile, "a")) {
                std::fprintf(f, "{\"rows\": %d, \"levels\": %d, \"narrow\": %d, \"iterations\": %d, \"ns\": [", d->N,
                             d->numLev, d->warp, iters);
                for (int k = 0; k < 9; ++k) std::fprintf(f, "%s%llu", k ? ", " : "", h[k]);
                std::fprintf(f, "]}\n");
                std::fclose(f);
            }
    }
    if (bytes) {
        // per iteration: 2 sweeps over the factors (every stored block once
        // per application) and 2 SpMVs over A, plus the vector updates
        const double sz = sizeof(T), bb = (double)d->b * d->b, nb = (double)d->N * d->b;
        const double mat = (double)d->nnz * (bb * sz + 4);
        *bytes = iters * (4.0 * mat + 30.0 * nb * sz) + (factor ? 3.0 * mat : 0.0);
    }
    if (hst->code) return hst->code;
    return hst->converged ? GBFV_OK : GBFV_ERR_NOT_CONVERGED;
}

int giluApply64(GiluData* d, const double* A, const double* dv, double* v, cudaStream_t s, DevStatus* st,
                DevStatus* hst)
{
    GiluArgs<double> a;
    int rs;
    if ((rs = args<double>(*d, a, A, dv, st))) return rs;
    a.factor = 1;
    if (cudaMemsetAsync(st, 0, sizeof(DevStatus), s) != cudaSuccess ||
        cudaMemsetAsync(d->bar, 0, 4 * sizeof(unsigned), s) != cudaSuccess ||
        (a.tagged && cudaMemsetAsync(d->tw, 0, sizeof(double) * 2 * (size_t)d->N * d->b, s) != cudaSuccess))
        return GBFV_ERR_CUDA;
    const void* fn = a.tagged ? (d->b == 2 ? (const void*)kGiluApply<double, 2, true> : (const void*)kGiluApply<double, 3, true>)
                              : (d->b == 2 ? (const void*)kGiluApply<double, 2, false> : (const void*)kGiluApply<double, 3, false>);
    if ((rs = launch<double>(fn, a, d->blocks, d->b, s))) return rs;
    if (cudaMemcpyAsync(v, a.x, sizeof(double) * (size_t)d->N * d->b, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(hst, st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GBFV_ERR_CUDA;
    return hst->code;
}

template int giluSolve<double>(GiluData*, const double*, const double*, double*, int, double, double, double, int,
                               cudaStream_t, DevStatus*, DevStatus*, int&, float*, double*);
template int giluSolve<float>(GiluData*, const float*, const float*, float*, int, double, double, double, int,
                              cudaStream_t, DevStatus*, DevStatus*, int&, float*, double*);

}  // namespace gbfv
