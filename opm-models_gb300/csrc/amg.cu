// Algebraic multigrid preconditioner for BiCGStab: the reference's
// ParallelAmgBackend (parallelamgbackend.hh:85-330), which hands the system
// to dune-istl's Dune::Amg::AMG with these settings (:262-305):
// coarsening to AmgCoarsenTarget rows (5000) over at most 15 levels with a
// minimum coarsen rate of 1.05, symmetric strength criterion on the blocks'
// Frobenius norms, SOR smoothing (one step of relaxation 1.0 per smoothing
// step), dune's defaults of 2 pre- and 2 post-smoothing steps, V-cycle,
// Galerkin coarse matrices over aggregates, prolongation damped by 1.6.
//
// GB300 form.  The setup that decides structure runs on the host once per
// solver (first matrix): strength of connection, greedy aggregation
// (Vanek-Mandel-Brezina: a root with its strong neighbours, left-over rows
// join their strongest aggregated neighbour, the rest root aggregates of
// their own), the Galerkin patterns with, for every coarse block, the list of
// fine blocks it sums, and a greedy colouring of every level (row order on
// the finest, smallest-last order on the coarse ones).  Each level is
// then renumbered colour by colour, so one colour of an SOR sweep is one
// contiguous, coalesced range of rows: a dependent chain of rows (dune's
// natural-order sweep) becomes a handful of parallel passes.  Every solve
// recomputes the values on the device (gather of the fine matrix into the
// colour order, Galerkin sums in a fixed order, inverted diagonals) and runs
// BiCGStab with the V-cycle inside one persistent cooperative launch, grid
// barriers between dependent passes.
//
// Deviations from dune-istl, the same in the oracle (oracle/amg.hh): the
// aggregation scheme; the colour-ordered sweeps; the coarsest level smoothed
// by 2 forward + backward sweep pairs instead of a direct solve; structure
// kept from the first matrix while the reference rebuilds it every solve.
// The operation orders are the oracle's, and this file is compiled without
// FMA contraction, so one FP64 V-cycle equals the oracle's bit for bit.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <set>
#include <string>
#include <vector>

#include "../../include/gbfv.h"
#include "amg.cuh"
#include "gbfv_internal.cuh"
#include "krylov.cuh"
#include "solver.cuh"

namespace gbfv {

void setLastError(const std::string& s);  // gbfv.cu: the message gbfv_last_error returns

namespace {

constexpr double AMG_ALPHA = 1.0 / 3.0;
constexpr double AMG_MIN_COARSEN_RATE = 1.05;
constexpr double AMG_PROLONG_DAMP = 1.6;
constexpr int AMG_PRE = 2, AMG_POST = 2, AMG_COARSEST_PAIRS = 2;
constexpr int AMG_THREADS = 256;
constexpr int AMG_TAIL_ROWS = 0;  // levels this small run in one block (0: none)

// ------------------------------------------------------------ host setup --
// one level's matrix in natural order (the level's own numbering)
struct Csr {
    int n = 0;
    std::vector<int> ptr, col;
    std::vector<double> val;  // nnz * bb
    int find(int r, int c) const
    {
        const auto b = col.begin() + ptr[r], e = col.begin() + ptr[r + 1];
        const auto it = std::lower_bound(b, e, c);
        return (it != e && *it == c) ? (int)(it - col.begin()) : -1;
    }
};

// strong neighbours (ascending) by the symmetric Frobenius-norm criterion
void strongGraph(const Csr& A, int bb, std::vector<double>& nrm, std::vector<int>& sPtr, std::vector<int>& sCol)
{
    const int n = A.n;
    nrm.assign(A.col.size(), 0.0);
    std::vector<double> mx(n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            double s = 0;
            for (int e = 0; e < bb; ++e) s += A.val[(size_t)k * bb + e] * A.val[(size_t)k * bb + e];
            nrm[k] = std::sqrt(s);
            if (A.col[k] != i) mx[i] = std::max(mx[i], nrm[k]);
        }
    sPtr.assign(n + 1, 0);
    sCol.clear();
    for (int i = 0; i < n; ++i) {
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            const int j = A.col[k];
            if (j == i) continue;
            const int kt = A.find(j, i);
            const bool si = mx[i] > 0 && nrm[k] >= AMG_ALPHA * mx[i];
            const bool sj = kt >= 0 && mx[j] > 0 && nrm[kt] >= AMG_ALPHA * mx[j];
            if (si || sj) sCol.push_back(j);
        }
        sPtr[i + 1] = (int)sCol.size();
    }
}

// greedy aggregation; aggregates numbered in creation order
int aggregate(const Csr& A, int bb, std::vector<int>& agg)
{
    const int n = A.n;
    std::vector<double> nrm;
    std::vector<int> sPtr, sCol;
    strongGraph(A, bb, nrm, sPtr, sCol);
    agg.assign(n, -1);
    int na = 0;
    for (int i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        bool free = true;
        for (int q = sPtr[i]; q < sPtr[i + 1] && free; ++q) free = agg[sCol[q]] < 0;
        if (!free) continue;
        agg[i] = na;
        for (int q = sPtr[i]; q < sPtr[i + 1]; ++q) agg[sCol[q]] = na;
        ++na;
    }
    const std::vector<int> first = agg;
    for (int i = 0; i < n; ++i) {
        if (first[i] >= 0) continue;
        double best = -1;
        int pick = -1;
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            const int j = A.col[k];
            if (j == i || first[j] < 0) continue;
            if (!std::binary_search(sCol.begin() + sPtr[i], sCol.begin() + sPtr[i + 1], j)) continue;
            const int kt = A.find(j, i);
            const double s = std::max(nrm[k], kt >= 0 ? nrm[kt] : 0.0);
            if (s > best) {
                best = s;
                pick = first[j];
            }
        }
        if (pick >= 0) agg[i] = pick;
    }
    for (int i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        agg[i] = na;
        for (int q = sPtr[i]; q < sPtr[i + 1]; ++q)
            if (agg[sCol[q]] < 0) agg[sCol[q]] = na;
        ++na;
    }
    return na;
}

// Galerkin pattern of the coarse level, its FP64 values (needed to
// aggregate the next level) and, for every coarse entry, the fine entries it
// sums: members ascending, each member's entries ascending
void galerkin(const Csr& A, int bb, const std::vector<int>& agg, int nc, Csr& Ac, std::vector<int>& lPtr,
              std::vector<int>& lIdx)
{
    std::vector<int> mPtr(nc + 1, 0), mIdx(A.n);
    for (int i = 0; i < A.n; ++i) mPtr[agg[i] + 1]++;
    for (int I = 0; I < nc; ++I) mPtr[I + 1] += mPtr[I];
    {
        std::vector<int> pos(mPtr.begin(), mPtr.end() - 1);
        for (int i = 0; i < A.n; ++i) mIdx[pos[agg[i]]++] = i;
    }
    Ac.n = nc;
    Ac.ptr.assign(nc + 1, 0);
    Ac.col.clear();
    std::vector<int> cols;
    for (int I = 0; I < nc; ++I) {
        cols.clear();
        for (int m = mPtr[I]; m < mPtr[I + 1]; ++m) {
            const int i = mIdx[m];
            for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) cols.push_back(agg[A.col[k]]);
        }
        std::sort(cols.begin(), cols.end());
        cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
        Ac.col.insert(Ac.col.end(), cols.begin(), cols.end());
        Ac.ptr[I + 1] = (int)Ac.col.size();
    }
    const int nnzc = Ac.ptr[nc];
    std::vector<int> cnt(nnzc + 1, 0);
    std::vector<int> target(A.col.size());
    for (int I = 0; I < nc; ++I)
        for (int m = mPtr[I]; m < mPtr[I + 1]; ++m) {
            const int i = mIdx[m];
            for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
                target[k] = Ac.find(I, agg[A.col[k]]);
                cnt[target[k] + 1]++;
            }
        }
    lPtr.assign(nnzc + 1, 0);
    for (int k = 0; k < nnzc; ++k) lPtr[k + 1] = lPtr[k] + cnt[k + 1];
    lIdx.assign(A.col.size(), 0);
    std::vector<int> pos(lPtr.begin(), lPtr.end() - 1);
    for (int I = 0; I < nc; ++I)
        for (int m = mPtr[I]; m < mPtr[I + 1]; ++m) {
            const int i = mIdx[m];
            for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) lIdx[pos[target[k]]++] = k;
        }
    Ac.val.assign((size_t)nnzc * bb, 0.0);
    for (int k = 0; k < nnzc; ++k)
        for (int e = 0; e < bb; ++e) {
            double s = 0.0;
            for (int q = lPtr[k]; q < lPtr[k + 1]; ++q) s += A.val[(size_t)lIdx[q] * bb + e];
            Ac.val[(size_t)k * bb + e] = s;
        }
}

// the rows by smallest-last order (Matula, Beck): the row of least degree
// among those left is removed next (ties: lowest row), and the rows are
// coloured in the reverse order of removal
std::vector<int> smallestLast(const Csr& A)
{
    const int n = A.n;
    std::vector<int> deg(n, 0);
    for (int i = 0; i < n; ++i)
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) deg[i] += A.col[k] != i;
    std::set<std::pair<int, int>> left;
    for (int i = 0; i < n; ++i) left.emplace(deg[i], i);
    std::vector<char> gone(n, 0);
    std::vector<int> order(n);
    for (int t = n - 1; t >= 0; --t) {
        const int v = left.begin()->second;
        left.erase(left.begin());
        gone[v] = 1;
        order[t] = v;
        for (int k = A.ptr[v]; k < A.ptr[v + 1]; ++k) {
            const int j = A.col[k];
            if (j == v || gone[j]) continue;
            left.erase({deg[j], j});
            left.emplace(--deg[j], j);
        }
    }
    return order;
}

// greedy colouring (the smallest colour no coloured neighbour has) in row
// order on the finest level, in smallest-last order on the coarse ones;
// returns the colour count
int colourRows(const Csr& A, bool finest, std::vector<int>& color)
{
    color.assign(A.n, -1);
    int nc = 0;
    std::vector<char> seen;
    std::vector<int> order;
    if (!finest) order = smallestLast(A);
    for (int t = 0; t < A.n; ++t) {
        const int i = finest ? t : order[t];
        seen.assign(nc + 1, 0);
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            const int j = A.col[k];
            if (j != i && color[j] >= 0) seen[color[j]] = 1;
        }
        int c = 0;
        while (seen[c]) ++c;
        color[i] = c;
        nc = std::max(nc, c + 1);
    }
    return nc;
}

// -------------------------------------------------------- device layout --
template <class T>
struct AmgLevelDev {
    int n, ld, W, nColors;
    const int* col;     // [k*ld + q] device column of entry k of row q (ascending natural column), or -1
    const T* val;       // [(k*B*B + e)*ld + q]
    const T* dinv;      // [e*ld + q] inverted diagonal block
    T* x;               // [q*B + e] (levels > 0)
    T* rhs;             // [q*B + e] (levels > 0)
    const int* agg;     // [q] coarse device row (levels but the coarsest)
    const int* mPtr;    // members of next-level row Q: mIdx[mPtr[Q] .. mPtr[Q+1]), ascending natural row
    const int* mIdx;
    T* def;             // [q*B + e] the defects rhs - A x before restriction (levels but the coarsest)
    int tpr;            // lanes that share one row of this level (1: a thread per row)
    int colorPtr[AMG_MAX_COLORS + 1];
};

template <class T>
struct AmgKArgs {
    int L, N;
    const AmgLevelDev<T>* lv;  // [L], device memory
    const T* rhs;              // level-0 right-hand side
    T *x, *r, *p, *v, *y, *z;  // Krylov vectors (level-0 order)
    double* partial;           // [4*blocks]
    GridSync gs;
    DevStatus* st;
    double redTol, absTol, maxRes;
    int maxIter;
    T damp;
    int tail;  // levels [tail, L) run in block 0 alone (tail >= L: none)
    unsigned long long* prof;  // optional V-cycle timers (GBFV_AMG_PROFILE), 32 words
};

}  // namespace

// per level: structure (both precisions) and values (per precision)
struct AmgLevelHost {
    int n = 0, ld = 0, W = 0, nColors = 0;
    std::vector<int> colorPtr;
    int* col = nullptr;
    int* agg = nullptr;
    int* mPtr = nullptr;
    int* mIdx = nullptr;
    int* diagSlot = nullptr;  // [q] entry index of the diagonal
    int* gPtr = nullptr;      // Galerkin lists of this level's entries (levels > 0): [k*ld + q] ...
    int* gIdx = nullptr;      // ... fine entries k_f*ld_f + q_f of the level above
    double *valD = nullptr, *dinvD = nullptr, *xD = nullptr, *rhsD = nullptr, *defD = nullptr;
    float *valF = nullptr, *dinvF = nullptr, *xF = nullptr, *rhsF = nullptr, *defF = nullptr;
    int tpr = 1;              // lanes per row of the last precision set up
    size_t nnzDev = 0;        // stored entries (W * n, including padding)
    size_t galerkinTerms = 0;
};

struct AmgData {
    int N = 0, b = 0, nslot = 0, ldSys = 0;
    std::vector<AmgLevelHost> lv;
    int* map0 = nullptr;      // [q] internal row of level-0 device row q
    int* gather0 = nullptr;   // unused (level 0 keeps the system's slots)
    void* lvDev[2] = {nullptr, nullptr};  // AmgLevelDev<double> / <float> arrays
    double* vecD = nullptr;   // 7 level-0 vectors: rhs x r p v y z
    float* vecF = nullptr;
    double* partial = nullptr;
    unsigned* bar = nullptr;
    int blocks[2] = {0, 0};
    cudaEvent_t evA = nullptr, evB = nullptr;
    unsigned long long* prof = nullptr;  // V-cycle timers when GBFV_AMG_PROFILE names a file
};

namespace {

template <class T>
int dalloc(T** p, size_t n)
{
    if (n == 0) n = 1;
    if (cudaMalloc((void**)p, sizeof(T) * n) != cudaSuccess) return GBFV_ERR_OOM;
    return GBFV_OK;
}

template <class T>
int upload(T** p, const std::vector<T>& h)
{
    int st = dalloc(p, h.size());
    if (st) return st;
    if (!h.empty() && cudaMemcpy(*p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return GBFV_ERR_CUDA;
    return GBFV_OK;
}

// ------------------------------------------------------ device kernels --
template <class T>
__global__ void kAmgGather0(int n, int ld0, int ldS, int nslot, int bb, const int* __restrict__ map0,
                            const T* __restrict__ A, T* __restrict__ val0)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int p = map0[q];
    for (int k = 0; k < nslot * bb; ++k) val0[(size_t)k * ld0 + q] = A[(size_t)k * ldS + p];
}

// coarse entry (k, Q) = sum of its fine entries, in list order, from 0
template <class T>
__global__ void kAmgGalerkin(int nc, int ldc, int Wc, int ldf, int bb, const int* __restrict__ gPtr,
                             const int* __restrict__ gIdx, const T* __restrict__ valF, T* __restrict__ valC)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= Wc * ldc) return;
    const int k = t / ldc, Q = t - k * ldc;
    if (Q >= nc) return;
    const int g0 = gPtr[t], g1 = gPtr[t + 1];
    for (int e = 0; e < bb; ++e) {
        T s = T(0);
        for (int g = g0; g < g1; ++g) {
            const int f = gIdx[g];
            const int kf = f / ldf, qf = f - kf * ldf;
            s += valF[((size_t)kf * bb + e) * ldf + qf];
        }
        valC[((size_t)k * bb + e) * ldc + Q] = s;
    }
}

template <class T, int B>
__global__ void kAmgInvert(int n, int ld, const int* __restrict__ diagSlot, const T* __restrict__ val,
                           T* __restrict__ dinv, DevStatus* st)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int k = diagSlot[q];
    T D[B * B], R[B * B];
#pragma unroll
    for (int e = 0; e < B * B; ++e) D[e] = val[((size_t)k * B * B + e) * ld + q];
    if (!invertBlock<T, B>(D, R)) {
        atomicExch(&st->code, GBFV_ERR_SINGULAR);
#pragma unroll
        for (int e = 0; e < B * B; ++e) R[e] = T(0);
    }
#pragma unroll
    for (int e = 0; e < B * B; ++e) dinv[(size_t)e * ld + q] = R[e];
}

template <class T, int B>
__global__ void kAmgPermute(int n, const int* __restrict__ map0, const T* __restrict__ in, T* __restrict__ out,
                            int toLevel)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int p = map0[q];
#pragma unroll
    for (int e = 0; e < B; ++e) {
        if (toLevel) out[q * B + e] = in[p * B + e];
        else out[p * B + e] = in[q * B + e];
    }
}

// the new search direction, formed where a row first needs it (the first
// colour pass of the first smoothing sweep): p = r - beta (p - omega v)
template <class T>
struct FormP {
    T* p;
    const T *r, *v;
    T beta, omega;
};

// Row q's sum over its stored entries of A_qj x_j, in entry order, into
// acc (SUB: acc -= A_qj x_j, the SOR update, skipping the diagonal and, with
// fromZero, the columns >= c0 not visited yet; otherwise acc += A_qj x_j,
// every column).  Entries go in chunks of U: the chunk's column indices,
// then its matrix blocks and gathers, all issued before the first use, so a
// row costs a few memory latencies instead of two per entry.
template <class T, int B, bool SUB>
__device__ __forceinline__ void rowProduct(const int* __restrict__ col, const T* __restrict__ val, int W, int ld,
                                          int q, const T* x, int c0, bool fromZero, T (&acc)[B])
{
    constexpr int BB = B * B, U = sizeof(T) == 4 ? 8 : 4;
    for (int k0 = 0; k0 < W; k0 += U) {
        int j[U];
#pragma unroll
        for (int u = 0; u < U; ++u) j[u] = k0 + u < W ? __ldg(&col[(k0 + u) * ld + q]) : -1;
        bool use[U];
#pragma unroll
        for (int u = 0; u < U; ++u) use[u] = j[u] >= 0 && (!SUB || (j[u] != q && !(fromZero && j[u] >= c0)));
        T a[U][BB], xv[U][B];
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
            for (int e = 0; e < BB; ++e) a[u][e] = use[u] ? __ldg(&val[((size_t)(k0 + u) * BB + e) * ld + q]) : T(0);
#pragma unroll
            for (int c = 0; c < B; ++c) xv[u][c] = use[u] ? ldcg(&x[j[u] * B + c]) : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (!use[u]) continue;
#pragma unroll
            for (int r = 0; r < B; ++r)
#pragma unroll
                for (int c = 0; c < B; ++c) {
                    if (SUB) acc[r] -= a[u][r * B + c] * xv[u][c];
                    else acc[r] += a[u][r * B + c] * xv[u][c];
                }
        }
    }
}

// The same sum with the row shared by a group of TPR lanes (TPR > 1, for the
// small levels, where a thread per row leaves most of the GPU idle and a
// row's W entries are a long chain of dependent loads): lane g of the group
// loads entries k0 + u*TPR + g, and every lane of the group then applies all
// entries in entry order from the group's shuffled values -- the same
// operations in the same order as one thread, on every lane of the group.
template <class T, int B, bool SUB, int TPR>
__device__ __forceinline__ void rowProductGroup(const int* __restrict__ col, const T* __restrict__ val, int W, int ld,
                                               int q, bool valid, const T* x, int c0, bool fromZero, int g, int lane0,
                                               T (&acc)[B])
{
    constexpr int BB = B * B, U = 2;
    for (int k0 = 0; k0 < W; k0 += TPR * U) {
        bool use[U];
        T a[U][BB], xv[U][B];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int k = k0 + u * TPR + g;
            const int j = (valid && k < W) ? __ldg(&col[k * ld + q]) : -1;
            use[u] = j >= 0 && (!SUB || (j != q && !(fromZero && j >= c0)));
#pragma unroll
            for (int e = 0; e < BB; ++e) a[u][e] = use[u] ? __ldg(&val[((size_t)k * BB + e) * ld + q]) : T(0);
#pragma unroll
            for (int c = 0; c < B; ++c) xv[u][c] = use[u] ? ldcg(&x[j * B + c]) : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll 1
            for (int t = 0; t < TPR; ++t) {
                const int src = lane0 + t;
                const bool ut = __shfl_sync(0xffffffffu, use[u], src);
                T av[BB], xt[B];
#pragma unroll
                for (int e = 0; e < BB; ++e) av[e] = __shfl_sync(0xffffffffu, a[u][e], src);
#pragma unroll
                for (int c = 0; c < B; ++c) xt[c] = __shfl_sync(0xffffffffu, xv[u][c], src);
                if (!ut) continue;
#pragma unroll
                for (int r = 0; r < B; ++r)
#pragma unroll
                    for (int c = 0; c < B; ++c) {
                        if (SUB) acc[r] -= av[r * B + c] * xt[c];
                        else acc[r] += av[r * B + c] * xt[c];
                    }
            }
    }
}

// A pass over rows [r0, r1) of a level with TPR lanes per row: body(q, valid,
// g, lane0) once per row slot, on every lane (warp-uniform trip counts, so
// the group shuffles see every lane).
template <int TPR, class F>
__device__ __forceinline__ void forRows(int r0, int r1, int gt, int gs, F&& body)
{
    if (TPR == 1) {
        for (int q = r0 + gt; q < r1; q += gs) body(q, true, 0, 0);
        return;
    }
    const int lane = threadIdx.x & 31, g = lane % TPR, lane0 = lane - g;
    const int warp = gt >> 5, nWarps = gs >> 5;
    constexpr int GPW = 32 / TPR;  // row groups per warp
    for (int base = r0 + warp * GPW; base < r1; base += nWarps * GPW) {
        const int q = base + lane / TPR;
        body(q < r1 ? q : r0, q < r1, g, lane0);
    }
}

// One colour of an SOR sweep (relaxation 1) on rows [c0, c1) of a level:
// x_q = D_q^-1 (rhs_q - sum_{j != q} A_qj x_j).  With fromZero the rows not
// yet visited in this sweep (device index >= c0) count as zero.
template <class T, int B, int TPR>
__device__ __forceinline__ void sorColourT(const AmgLevelDev<T>& L, const T* rhs, T* x, int c0, int c1, bool fromZero,
                                           const FormP<T>* fp, int gt, int gs)
{
    const int W = L.W, ld = L.ld;
    const int* __restrict__ col = L.col;
    const T* __restrict__ val = L.val;
    const T* __restrict__ dinv = L.dinv;
    forRows<TPR>(c0, c1, gt, gs, [&](int q, bool valid, int g, int lane0) {
        T v[B];
        if (fp) {  // level 0 only, a thread per row
#pragma unroll
            for (int e = 0; e < B; ++e) {
                T tmp = ldcg(&fp->v[q * B + e]);
                tmp *= fp->omega;
                tmp -= ldcg(&fp->p[q * B + e]);
                tmp *= -fp->beta;
                T pe = ldcg(&fp->r[q * B + e]);
                pe += tmp;
                fp->p[q * B + e] = pe;
                v[e] = pe;
            }
        }
        else {
#pragma unroll
            for (int e = 0; e < B; ++e) v[e] = ldcg(&rhs[q * B + e]);
        }
        T d[B * B];
#pragma unroll
        for (int e = 0; e < B * B; ++e) d[e] = __ldg(&dinv[(size_t)e * ld + q]);
        if (TPR == 1) rowProduct<T, B, true>(col, val, W, ld, q, x, c0, fromZero, v);
        else rowProductGroup<T, B, true, TPR>(col, val, W, ld, q, valid, x, c0, fromZero, g, lane0, v);
        if (valid && g == 0) {
#pragma unroll
            for (int r = 0; r < B; ++r) {
                T s = T(0);
#pragma unroll
                for (int c = 0; c < B; ++c) s += d[r * B + c] * v[c];
                x[q * B + r] = s;
            }
        }
    });
}

template <class T, int B>
__device__ __noinline__ void sorColour(const AmgLevelDev<T>& L, const T* rhs, T* x, int c0, int c1, bool fromZero,
                                       const FormP<T>* fp, int gt, int gs)
{
    switch (fp ? 1 : L.tpr) {
    case 8: sorColourT<T, B, 8>(L, rhs, x, c0, c1, fromZero, nullptr, gt, gs); break;
    case 4: sorColourT<T, B, 4>(L, rhs, x, c0, c1, fromZero, nullptr, gt, gs); break;
    default: sorColourT<T, B, 1>(L, rhs, x, c0, c1, fromZero, fp, gt, gs); break;
    }
}

// the defects d_q = rhs_q - A_q x of every row of a level (spmv order), a
// coalesced pass over the level's rows
template <class T, int B, int TPR>
__device__ __forceinline__ void defectsT(const AmgLevelDev<T>& L, const T* rhs, const T* x, int gt, int gs)
{
    const int W = L.W, ld = L.ld;
    forRows<TPR>(0, L.n, gt, gs, [&](int q, bool valid, int g, int lane0) {
        T y[B];
#pragma unroll
        for (int e = 0; e < B; ++e) y[e] = T(0);
        if (TPR == 1) rowProduct<T, B, false>(L.col, L.val, W, ld, q, x, 0, false, y);
        else rowProductGroup<T, B, false, TPR>(L.col, L.val, W, ld, q, valid, x, 0, false, g, lane0, y);
        if (valid && g == 0)
#pragma unroll
            for (int e = 0; e < B; ++e) L.def[q * B + e] = ldcg(&rhs[q * B + e]) - y[e];
    });
}

template <class T, int B>
__device__ __noinline__ void defects(const AmgLevelDev<T>& L, const T* rhs, const T* x, int gt, int gs)
{
    switch (L.tpr) {
    case 8: defectsT<T, B, 8>(L, rhs, x, gt, gs); break;
    case 4: defectsT<T, B, 4>(L, rhs, x, gt, gs); break;
    default: defectsT<T, B, 1>(L, rhs, x, gt, gs); break;
    }
}

// coarse right-hand side: each coarse row's members' defects, in ascending
// member order from 0
template <class T, int B>
__device__ __forceinline__ void restrictDefects(const AmgLevelDev<T>& L, T* rc, int nc, int gt, int gs)
{
    const int* __restrict__ mPtr = L.mPtr;
    const int* __restrict__ mIdx = L.mIdx;
    for (int Q = gt; Q < nc; Q += gs) {
        const int m0 = __ldg(&mPtr[Q]), m1 = __ldg(&mPtr[Q + 1]);
        T s[B];
#pragma unroll
        for (int e = 0; e < B; ++e) s[e] = T(0);
        for (int m = m0; m < m1; ++m) {
            const int q = __ldg(&mIdx[m]);
#pragma unroll
            for (int e = 0; e < B; ++e) s[e] += ldcg(&L.def[q * B + e]);
        }
#pragma unroll
        for (int e = 0; e < B; ++e) rc[Q * B + e] = s[e];
    }
}

template <class T, int B>
__device__ __forceinline__ void prolongate(const AmgLevelDev<T>& L, T* x, const T* xc, T damp, int gt, int gs)
{
    for (int q = gt; q < L.n; q += gs) {
        const int Q = __ldg(&L.agg[q]);
#pragma unroll
        for (int e = 0; e < B; ++e) {
            const T t = damp * ldcg(&xc[Q * B + e]);
            x[q * B + e] = ldcg(&x[q * B + e]) + t;
        }
    }
}

// barrier between dependent passes: the whole grid, or (the tail levels
// that block 0 runs alone) the block
struct GridBar {
    const GridSync* g;
    __device__ bool operator()() const { return gridBarrier(*g); }
};
struct BlockBar {
    __device__ bool operator()() const
    {
        __syncthreads();
        return true;
    }
};

// one sweep of every colour, forward or backward, a barrier after each
template <class T, int B, class Bar>
__device__ __forceinline__ bool sweep(const AmgLevelDev<T>& L, const T* rhs, T* x, bool forward, bool fromZero,
                                      const FormP<T>* fp, int gt, int gs, const Bar& bar)
{
    const int nc = L.nColors;
    for (int s = 0; s < nc; ++s) {
        const int c = forward ? s : nc - 1 - s;
        sorColour<T, B>(L, rhs, x, L.colorPtr[c], L.colorPtr[c + 1], fromZero, fp, gt, gs);
        if (!bar()) return false;
    }
    return true;
}

// level l on the way down: pre-smoothing, then the restricted defect into l + 1
template <class T, int B, class Bar>
__device__ __forceinline__ bool downLevel(const AmgKArgs<T>& a, int l, const T* rhs0, T* x0, const FormP<T>* fp,
                                          int gt, int gs, const Bar& bar)
{
    const AmgLevelDev<T>& lv = a.lv[l];
    const T* rhs = l == 0 ? rhs0 : lv.rhs;
    T* x = l == 0 ? x0 : lv.x;
    for (int s = 0; s < AMG_PRE; ++s)
        if (!sweep<T, B>(lv, rhs, x, true, s == 0, (l == 0 && s == 0) ? fp : nullptr, gt, gs, bar)) return false;
    defects<T, B>(lv, rhs, x, gt, gs);
    if (!bar()) return false;
    const AmgLevelDev<T>& nx = a.lv[l + 1];
    restrictDefects<T, B>(lv, nx.rhs, nx.n, gt, gs);
    return bar();
}

// the coarsest level: forward + backward sweep pairs from a zero guess
template <class T, int B, class Bar>
__device__ __forceinline__ bool coarsest(const AmgKArgs<T>& a, const T* rhs0, T* x0, const FormP<T>* fp, int gt,
                                         int gs, const Bar& bar)
{
    const int L = a.L;
    const AmgLevelDev<T>& lv = a.lv[L - 1];
    const T* rhs = L == 1 ? rhs0 : lv.rhs;
    T* x = L == 1 ? x0 : lv.x;
    for (int s = 0; s < AMG_COARSEST_PAIRS; ++s) {
        if (!sweep<T, B>(lv, rhs, x, true, s == 0, (L == 1 && s == 0) ? fp : nullptr, gt, gs, bar)) return false;
        if (!sweep<T, B>(lv, rhs, x, false, false, nullptr, gt, gs, bar)) return false;
    }
    return true;
}

// level l on the way up: the prolongated correction, then post-smoothing
template <class T, int B, class Bar>
__device__ __forceinline__ bool upLevel(const AmgKArgs<T>& a, int l, const T* rhs0, T* x0, int gt, int gs,
                                        const Bar& bar)
{
    const AmgLevelDev<T>& lv = a.lv[l];
    const T* rhs = l == 0 ? rhs0 : lv.rhs;
    T* x = l == 0 ? x0 : lv.x;
    prolongate<T, B>(lv, x, a.lv[l + 1].x, a.damp, gt, gs);
    if (!bar()) return false;
    for (int s = 0; s < AMG_POST; ++s)
        if (!sweep<T, B>(lv, rhs, x, false, false, nullptr, gt, gs, bar)) return false;
    return true;
}

// AMG::mgc (gamma 1) on x0 = M^-1 rhs0, zero initial guess on every level.
// Levels [a.tail, L) -- the small coarse end of the hierarchy -- run in
// block 0 alone with block barriers (a pass over a few thousand rows costs
// less there than a grid barrier); the other blocks wait at the grid
// barrier that follows.  The passes and their order are the same either way.
template <class T, int B>
__device__ bool vcycle(const AmgKArgs<T>& a, const T* rhs0, T* x0, const FormP<T>* fp, int gt, int gs)
{
    const int L = a.L, split = a.tail < L - 1 ? a.tail : L - 1;
    const GridBar gbar{&a.gs};
    // optional timers (block 0, thread 0; every block passes the same
    // barriers): [l] down level l, [15] coarsest / tail, [16 + l] up level l
    unsigned long long* pr = (a.prof && gt == 0) ? a.prof : nullptr;
    unsigned long long t = pr ? gtimer() : 0;
    auto tick = [&](int k) {
        if (!pr) return;
        const unsigned long long n = gtimer();
        pr[k] += n - t;
        t = n;
    };
    for (int l = 0; l < split; ++l) {
        if (!downLevel<T, B>(a, l, rhs0, x0, fp, gt, gs, gbar)) return false;
        tick(l);
    }
    if (a.tail < L) {
        if (blockIdx.x == 0) {
            const BlockBar bbar;
            const int bt = threadIdx.x, bs = blockDim.x;
            for (int l = a.tail; l + 1 < L; ++l) downLevel<T, B>(a, l, rhs0, x0, fp, bt, bs, bbar);
            coarsest<T, B>(a, rhs0, x0, fp, bt, bs, bbar);
            for (int l = L - 2; l >= a.tail; --l) upLevel<T, B>(a, l, rhs0, x0, bt, bs, bbar);
        }
        if (!gbar()) return false;
    }
    else if (!coarsest<T, B>(a, rhs0, x0, fp, gt, gs, gbar))
        return false;
    tick(15);
    for (int l = split - 1; l >= 0; --l) {
        if (!upLevel<T, B>(a, l, rhs0, x0, gt, gs, gbar)) return false;
        tick(16 + l);
    }
    if (pr) pr[31] += 1;
    return true;
}

// y = A x on level 0 (spmv order), one row
template <class T, int B>
__device__ __forceinline__ void spmvRow0(const AmgLevelDev<T>& L, const T* in, int q, T (&acc)[B])
{
#pragma unroll
    for (int e = 0; e < B; ++e) acc[e] = T(0);
    rowProduct<T, B, false>(L.col, L.val, L.W, L.ld, q, in, 0, false, acc);
}

// BiCGStabSolver::apply (bicgstabsolver.hh:120-330) with the AMG V-cycle as
// the preconditioner: the ILU(0) solve kernel's iteration (same reductions,
// criterion and breakdown tests), every preconditioner application a
// V-cycle; the whole solve in one cooperative launch.
template <class T, int B>
__global__ void __launch_bounds__(AMG_THREADS) kAmgBicgstab(const AmgKArgs<T> a)
{
    const Team<SYNC_GRID> tm;
    const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
    const int N = a.N;
    const AmgLevelDev<T>& L0 = a.lv[0];
    const double eps = 2.2250738585072014e-308 * 1e10;  // numeric_limits<double>::min()*1e10
    if (*(volatile int*)&a.st->code != 0) return;        // a singular diagonal block
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
    {
        double tot[1];
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
            const double beta = (rho_i / rho) * (alpha / omega);
            rho = rho_i;
            {
                const FormP<T> fp = {a.p, a.r, a.v, (T)beta, (T)omega};
                if (!vcycle<T, B>(a, a.p, a.y, &fp, gt, gs)) goto timeout;
            }
            {
                double dd[1] = {0.0};
                const bool isSum1[1] = {false};
                for (int i = gt; i < N; i += gs) {
                    T acc[B];
                    spmvRow0<T, B>(L0, a.y, i, acc);
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
            if (!vcycle<T, B>(a, a.r, a.z, nullptr, gt, gs)) goto timeout;
            {
                double dd[2] = {0.0, 0.0};
                const bool isSum2[2] = {false, false};
                for (int i = gt; i < N; i += gs) {
                    T acc[B];
                    spmvRow0<T, B>(L0, a.z, i, acc);
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

// one V-cycle v = M^-1 d alone (unit tests: compared with the oracle's)
template <class T, int B>
__global__ void __launch_bounds__(AMG_THREADS) kAmgApply(const AmgKArgs<T> a)
{
    const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
    if (*(volatile int*)&a.st->code != 0) return;
    if (!vcycle<T, B>(a, a.rhs, a.x, nullptr, gt, gs) && gt == 0) a.st->code = GBFV_ERR_TIMEOUT;
}

template <class T>
T* lvVal(AmgLevelHost& h);
template <>
double* lvVal<double>(AmgLevelHost& h) { return h.valD; }
template <>
float* lvVal<float>(AmgLevelHost& h) { return h.valF; }

// per-precision device arrays (values, diagonals, vectors) on first use
template <class T>
int ensurePrecision(AmgData& d)
{
    const int k = sizeof(T) == 4 ? 1 : 0;
    if (d.lvDev[k]) return GBFV_OK;
    const int bb = d.b * d.b;
    int st;
    // blocks of the cooperative launch: as many as fit, at most 8 per SM
    // (GBFV_AMG_BLOCKS_PER_SM caps it lower)
    {
        int dev = 0, nsm = 1, occ = 0, occA = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (d.b == 2) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kAmgBicgstab<T, 2>, AMG_THREADS, 0);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occA, kAmgApply<T, 2>, AMG_THREADS, 0);
        }
        else {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kAmgBicgstab<T, 3>, AMG_THREADS, 0);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occA, kAmgApply<T, 3>, AMG_THREADS, 0);
        }
        occ = std::min(std::min(occ, occA), 8);
        if (const char* e = getenv("GBFV_AMG_BLOCKS_PER_SM")) occ = std::max(1, std::min(occ, atoi(e)));
        if (occ < 1) {
            setLastError("AMG solve kernel does not fit an SM");
            return GBFV_ERR_UNSUPPORTED;
        }
        d.blocks[k] = nsm * occ;
        // reduction partials: two halves of two values per block, for the
        // largest grid either precision launches
        if (!d.partial && ((st = dalloc(&d.partial, (size_t)4 * 8 * nsm)) || (st = dalloc(&d.bar, 4)))) return st;
    }
    const long threads = (long)d.blocks[k] * AMG_THREADS;
    std::vector<AmgLevelDev<T>> hl(d.lv.size());
    for (size_t l = 0; l < d.lv.size(); ++l) {
        AmgLevelHost& h = d.lv[l];
        T *val, *dinv, *x = nullptr, *rhs = nullptr, *def = nullptr;
        if ((st = dalloc(&val, (size_t)h.W * bb * h.ld)) || (st = dalloc(&dinv, (size_t)bb * h.ld))) return st;
        if (l > 0 && ((st = dalloc(&x, (size_t)h.ld * d.b)) || (st = dalloc(&rhs, (size_t)h.ld * d.b)))) return st;
        if (l + 1 < d.lv.size() && (st = dalloc(&def, (size_t)h.ld * d.b))) return st;
        if (cudaMemset(val, 0, sizeof(T) * (size_t)h.W * bb * h.ld) != cudaSuccess) return GBFV_ERR_CUDA;
        if (sizeof(T) == 8) {
            h.valD = (double*)val; h.dinvD = (double*)dinv; h.xD = (double*)x; h.rhsD = (double*)rhs;
            h.defD = (double*)def;
        }
        else {
            h.valF = (float*)val; h.dinvF = (float*)dinv; h.xF = (float*)x; h.rhsF = (float*)rhs;
            h.defF = (float*)def;
        }
        AmgLevelDev<T>& g = hl[l];
        g.n = h.n;
        g.ld = h.ld;
        g.W = h.W;
        g.nColors = h.nColors;
        g.col = h.col;
        g.val = val;
        g.dinv = dinv;
        g.x = x;
        g.rhs = rhs;
        g.def = def;
        g.agg = h.agg;
        g.mPtr = h.mPtr;
        g.mIdx = h.mIdx;
        for (int c = 0; c <= AMG_MAX_COLORS; ++c) g.colorPtr[c] = c <= h.nColors ? h.colorPtr[c] : h.n;
        // lanes per row: 8 where a colour has rows for at most one in eight
        // threads, else a thread per row (measured: 4 lanes slowed the
        // mid-size levels, 32 the small ones -- the in-order combine grows
        // with the group); the finest level always a thread per row
        const long perColour = std::max(1L, ((long)h.n + h.nColors - 1) / h.nColors);
        const int tpr = 8 * perColour <= threads ? 8 : 1;
        g.tpr = (l == 0 || getenv("GBFV_AMG_ROW_PER_THREAD")) ? 1 : tpr;
        h.tpr = g.tpr;
    }
    void* p = nullptr;
    if (cudaMalloc(&p, sizeof(AmgLevelDev<T>) * hl.size()) != cudaSuccess) return GBFV_ERR_OOM;
    if (cudaMemcpy(p, hl.data(), sizeof(AmgLevelDev<T>) * hl.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return GBFV_ERR_CUDA;
    d.lvDev[k] = p;
    T* vec;
    if ((st = dalloc(&vec, (size_t)7 * d.lv[0].ld * d.b))) return st;
    if (sizeof(T) == 8) d.vecD = (double*)vec;
    else d.vecF = (float*)vec;
    return GBFV_OK;
}

// coarse values and inverted diagonals of every level from A (solver layout)
template <class T, int B>
int amgValues(AmgData& d, const T* A, cudaStream_t s, DevStatus* st)
{
    const int bb = B * B;
    AmgLevelHost& h0 = d.lv[0];
    T* v0 = lvVal<T>(h0);
    kAmgGather0<T><<<(h0.n + 255) / 256, 256, 0, s>>>(h0.n, h0.ld, d.ldSys, d.nslot, bb, d.map0, A, v0);
    countLaunch();
    for (size_t l = 1; l < d.lv.size(); ++l) {
        AmgLevelHost& f = d.lv[l - 1];
        AmgLevelHost& c = d.lv[l];
        const long nt = (long)c.W * c.ld;
        kAmgGalerkin<T><<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(c.n, c.ld, c.W, f.ld, bb, c.gPtr, c.gIdx,
                                                                      lvVal<T>(f), lvVal<T>(c));
        countLaunch();
    }
    for (size_t l = 0; l < d.lv.size(); ++l) {
        AmgLevelHost& h = d.lv[l];
        T* dinv = sizeof(T) == 8 ? (T*)h.dinvD : (T*)h.dinvF;
        kAmgInvert<T, B><<<(h.n + 255) / 256, 256, 0, s>>>(h.n, h.ld, h.diagSlot, lvVal<T>(h), dinv, st);
        countLaunch();
    }
    return cudaGetLastError() == cudaSuccess ? GBFV_OK : GBFV_ERR_CUDA;
}

template <class T>
AmgKArgs<T> kargs(AmgData& d, DevStatus* st)
{
    const int k = sizeof(T) == 4 ? 1 : 0;
    AmgKArgs<T> a;
    a.L = (int)d.lv.size();
    a.N = d.N;
    a.lv = (const AmgLevelDev<T>*)d.lvDev[k];
    T* vec = sizeof(T) == 8 ? (T*)d.vecD : (T*)d.vecF;
    const size_t n = (size_t)d.lv[0].ld * d.b;
    a.rhs = vec;
    a.x = vec + n;
    a.r = vec + 2 * n;
    a.p = vec + 3 * n;
    a.v = vec + 4 * n;
    a.y = vec + 5 * n;
    a.z = vec + 6 * n;
    a.partial = d.partial;
    a.gs.count = d.bar;
    a.gs.gen = d.bar + 1;
    a.gs.abort = (int*)(d.bar + 2);
    a.gs.perCluster = 0;
    a.st = st;
    a.damp = (T)AMG_PROLONG_DAMP;
    a.prof = d.prof;
    // the coarse end of the hierarchy that block 0 runs alone: levels of at
    // most GBFV_AMG_TAIL rows (default AMG_TAIL_ROWS), never the finest
    a.tail = a.L;
    {
        int rows = AMG_TAIL_ROWS;
        if (const char* e = getenv("GBFV_AMG_TAIL")) rows = atoi(e);
        for (int l = 1; l < a.L; ++l)
            if (d.lv[l].n <= rows) {
                a.tail = l;
                break;
            }
    }
    return a;
}

template <class T>
int launchCoop(const void* fn, AmgKArgs<T>& a, int blocks, cudaStream_t s)
{
    void* args[] = {(void*)&a};
    const cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(AMG_THREADS), args, 0, s);
    countLaunch();
    if (e != cudaSuccess) {
        setLastError(std::string("AMG cooperative launch failed: ") + cudaGetErrorString(e));
        return GBFV_ERR_CUDA;
    }
    return GBFV_OK;
}

// bytes one BiCGStab iteration moves by the algorithm: 2 V-cycles (per level
// (pre + post + coarsest) sweeps read the level's matrix, diagonals and x;
// the restriction reads the matrix again), 2 level-0 SpMVs and the vector
// updates
double iterationBytes(const AmgData& d, int sz)
{
    const int b = d.b, bb = b * b;
    double v = 0;
    const int L = (int)d.lv.size();
    for (int l = 0; l < L; ++l) {
        const AmgLevelHost& h = d.lv[l];
        const double mat = (double)h.nnzDev * (bb * sz + 4) + (double)h.n * bb * sz;
        const double vec = (double)h.n * b * sz * 3;
        const int sweeps = l + 1 == L ? 2 * AMG_COARSEST_PAIRS : AMG_PRE + AMG_POST;
        v += sweeps * (mat + vec);
        if (l + 1 < L) v += mat + vec + (double)h.n * b * sz * 2;  // restriction, prolongation
    }
    const AmgLevelHost& h0 = d.lv[0];
    const double spmv = (double)h0.nnzDev * (bb * sz + 4) + (double)h0.n * b * sz * 2;
    return 2 * v + 2 * spmv + (double)h0.n * b * sz * 20;
}

}  // namespace

AmgData* amgCreate(const AmgSystem& sys, const double* A64, int coarsenTarget, cudaStream_t s, int* status)
{
    auto fail = [&](AmgData* d, int st, const std::string& msg) -> AmgData* {
        if (!msg.empty()) setLastError(msg);
        if (status) *status = st;
        amgDestroy(d);
        return nullptr;
    };
    const int N = sys.N, b = sys.b, bb = b * b, ld = sys.ld, ns = sys.nslot;
    AmgData* d = new AmgData();
    d->N = N;
    d->b = b;
    d->nslot = ns;
    d->ldSys = ld;
    // the FP64 matrix of this solve, in natural order
    std::vector<double> hA((size_t)ns * bb * ld);
    if (cudaMemcpyAsync(hA.data(), A64, sizeof(double) * hA.size(), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return fail(d, GBFV_ERR_CUDA, "AMG set-up: copy of the matrix failed");
    std::vector<int> perm(N);
    for (int p = 0; p < N; ++p) perm[sys.natural[p]] = p;
    std::vector<Csr> A(1);
    std::vector<std::vector<int>> slotOf(1);  // level 0: slot of each natural entry
    A[0].n = N;
    A[0].ptr.assign(N + 1, 0);
    for (int i = 0; i < N; ++i) {
        const int p = perm[i];
        for (int sl = 0; sl < ns; ++sl) {
            const int c = sys.colHost[(size_t)sl * ld + p];
            if (c < 0) continue;
            A[0].col.push_back(sys.natural[c]);
            slotOf[0].push_back(sl);
            for (int e = 0; e < bb; ++e) A[0].val.push_back(hA[((size_t)sl * bb + e) * ld + p]);
        }
        A[0].ptr[i + 1] = (int)A[0].col.size();
        for (int k = A[0].ptr[i] + 1; k < A[0].ptr[i + 1]; ++k)
            if (A[0].col[k] <= A[0].col[k - 1]) return fail(d, GBFV_ERR_UNSUPPORTED, "AMG: slots out of column order");
    }
    // coarsening
    std::vector<std::vector<int>> aggs, lPtrs, lIdxs;
    while ((int)A.size() < AMG_MAX_LEVELS && A.back().n > coarsenTarget) {
        std::vector<int> agg;
        const int nc = aggregate(A.back(), bb, agg);
        if ((double)A.back().n / nc < AMG_MIN_COARSEN_RATE) break;
        Csr Ac;
        std::vector<int> lPtr, lIdx;
        galerkin(A.back(), bb, agg, nc, Ac, lPtr, lIdx);
        aggs.push_back(std::move(agg));
        lPtrs.push_back(std::move(lPtr));
        lIdxs.push_back(std::move(lIdx));
        A.push_back(std::move(Ac));
    }
    const int L = (int)A.size();
    d->lv.resize(L);
    // colour order of every level: pos[l][natural] and row[l][device]
    std::vector<std::vector<int>> pos(L), rowOf(L);
    for (int l = 0; l < L; ++l) {
        std::vector<int> color;
        const int nc = colourRows(A[l], l == 0, color);
        if (nc > AMG_MAX_COLORS)
            return fail(d, GBFV_ERR_UNSUPPORTED, "AMG: a level needs more than " + std::to_string(AMG_MAX_COLORS) +
                                                     " colours");
        AmgLevelHost& h = d->lv[l];
        h.n = A[l].n;
        h.ld = ((h.n + 63) / 64) * 64;
        h.nColors = nc;
        h.colorPtr.assign(nc + 1, 0);
        for (int i = 0; i < h.n; ++i) h.colorPtr[color[i] + 1]++;
        for (int c = 0; c < nc; ++c) h.colorPtr[c + 1] += h.colorPtr[c];
        pos[l].assign(h.n, 0);
        rowOf[l].assign(h.n, 0);
        std::vector<int> next(h.colorPtr.begin(), h.colorPtr.end() - 1);
        for (int i = 0; i < h.n; ++i) {
            const int q = next[color[i]]++;
            pos[l][i] = q;
            rowOf[l][q] = i;
        }
    }
    int st;
    for (int l = 0; l < L; ++l) {
        AmgLevelHost& h = d->lv[l];
        const Csr& M = A[l];
        int W = 0;
        if (l == 0) W = ns;
        else
            for (int i = 0; i < M.n; ++i) W = std::max(W, M.ptr[i + 1] - M.ptr[i]);
        h.W = W;
        h.nnzDev = (size_t)W * h.n;
        std::vector<int> col((size_t)W * h.ld, -1), diag(h.ld, 0);
        // entry slot of natural entry k (level 0: the system's slot; coarse: its rank in the row)
        std::vector<int> slot(M.col.size());
        for (int i = 0; i < M.n; ++i) {
            const int q = pos[l][i];
            for (int k = M.ptr[i]; k < M.ptr[i + 1]; ++k) {
                const int sl = l == 0 ? slotOf[0][k] : k - M.ptr[i];
                slot[k] = sl;
                col[(size_t)sl * h.ld + q] = pos[l][M.col[k]];
                if (M.col[k] == i) diag[q] = sl;
            }
        }
        if ((st = upload(&h.col, col)) || (st = upload(&h.diagSlot, diag))) return fail(d, st, "");
        if (l == 0) {
            std::vector<int> map0(h.n);
            for (int q = 0; q < h.n; ++q) map0[q] = perm[rowOf[0][q]];
            if ((st = upload(&d->map0, map0))) return fail(d, st, "");
        }
        if (l + 1 < L) {
            const std::vector<int>& agg = aggs[l];
            const int nc = A[l + 1].n;
            std::vector<int> aggD(h.ld, 0), mPtr(nc + 1, 0), mIdx(h.n);
            for (int i = 0; i < h.n; ++i) {
                aggD[pos[l][i]] = pos[l + 1][agg[i]];
                mPtr[pos[l + 1][agg[i]] + 1]++;
            }
            for (int Q = 0; Q < nc; ++Q) mPtr[Q + 1] += mPtr[Q];
            std::vector<int> nx(mPtr.begin(), mPtr.end() - 1);
            for (int i = 0; i < h.n; ++i) mIdx[nx[pos[l + 1][agg[i]]]++] = pos[l][i];  // ascending natural i
            if ((st = upload(&h.agg, aggD)) || (st = upload(&h.mPtr, mPtr)) || (st = upload(&h.mIdx, mIdx)))
                return fail(d, st, "");
            // Galerkin lists of the next level, by its device entry (slot*ld_c + Q)
            const Csr& C = A[l + 1];
            AmgLevelHost& hc = d->lv[l + 1];
            int Wc = 0;
            for (int I = 0; I < C.n; ++I) Wc = std::max(Wc, C.ptr[I + 1] - C.ptr[I]);
            const int ldc = ((C.n + 63) / 64) * 64;
            std::vector<int> cnt((size_t)Wc * ldc + 1, 0);
            const std::vector<int>& lPtr = lPtrs[l];
            const std::vector<int>& lIdx = lIdxs[l];
            std::vector<int> dev(C.col.size());
            for (int I = 0; I < C.n; ++I)
                for (int k = C.ptr[I]; k < C.ptr[I + 1]; ++k) {
                    dev[k] = (k - C.ptr[I]) * ldc + pos[l + 1][I];
                    cnt[dev[k] + 1] = lPtr[k + 1] - lPtr[k];
                }
            std::vector<int> gPtr((size_t)Wc * ldc + 1, 0);
            for (size_t t = 0; t < (size_t)Wc * ldc; ++t) gPtr[t + 1] = gPtr[t] + cnt[t + 1];
            std::vector<int> gIdx(lIdx.size());
            for (size_t k = 0; k < C.col.size(); ++k) {
                int o = gPtr[dev[k]];
                for (int g = lPtr[k]; g < lPtr[k + 1]; ++g) {
                    const int kf = lIdx[g];
                    // the fine entry kf of natural row i_f: its device slot and row
                    int lo = 0, hi = M.n;  // row of kf by binary search on M.ptr
                    while (hi - lo > 1) {
                        const int mid = (lo + hi) / 2;
                        if (M.ptr[mid] <= kf) lo = mid;
                        else hi = mid;
                    }
                    gIdx[o++] = slot[kf] * h.ld + pos[l][lo];
                }
            }
            if ((st = upload(&hc.gPtr, gPtr)) || (st = upload(&hc.gIdx, gIdx))) return fail(d, st, "");
            hc.galerkinTerms = gIdx.size();
        }
    }
    cudaEventCreate(&d->evA);
    cudaEventCreate(&d->evB);
    if (status) *status = GBFV_OK;
    return d;
}

void amgDestroy(AmgData* d)
{
    if (!d) return;
    for (AmgLevelHost& h : d->lv) {
        for (int* p : {h.col, h.agg, h.mPtr, h.mIdx, h.diagSlot, h.gPtr, h.gIdx}) cudaFree(p);
        for (double* p : {h.valD, h.dinvD, h.xD, h.rhsD, h.defD}) cudaFree(p);
        for (float* p : {h.valF, h.dinvF, h.xF, h.rhsF, h.defF}) cudaFree(p);
    }
    cudaFree(d->map0);
    cudaFree(d->lvDev[0]);
    cudaFree(d->lvDev[1]);
    cudaFree(d->vecD);
    cudaFree(d->vecF);
    cudaFree(d->partial);
    cudaFree(d->bar);
    cudaFree(d->prof);
    if (d->evA) cudaEventDestroy(d->evA);
    if (d->evB) cudaEventDestroy(d->evB);
    delete d;
}

int amgLevelSizes(const AmgData* d, int* sizes)
{
    for (size_t l = 0; l < d->lv.size(); ++l) sizes[l] = d->lv[l].n;
    return (int)d->lv.size();
}

int amgLevelColors(const AmgData* d, int* colors)
{
    for (size_t l = 0; l < d->lv.size(); ++l) colors[l] = d->lv[l].nColors;
    return (int)d->lv.size();
}

template <class T>
int amgSolve(AmgData* d, const T* A, const T* rhs, T* x, double redTol, double absTol, double maxRes, int maxIter,
             cudaStream_t s, DevStatus* st, DevStatus* hst, int& iters, float* ms, double* bytes)
{
    int rs;
    if ((rs = ensurePrecision<T>(*d))) return rs;
    const int k = sizeof(T) == 4 ? 1 : 0;
    if (cudaMemsetAsync(st, 0, sizeof(DevStatus), s) != cudaSuccess) return GBFV_ERR_CUDA;
    if (cudaMemsetAsync(d->bar, 0, 4 * sizeof(unsigned), s) != cudaSuccess) return GBFV_ERR_CUDA;
    cudaEventRecord(d->evA, s);
    rs = d->b == 2 ? amgValues<T, 2>(*d, A, s, st) : amgValues<T, 3>(*d, A, s, st);
    if (rs) return rs;
    const char* profFile = getenv("GBFV_AMG_PROFILE");
    if (profFile && !d->prof && cudaMalloc((void**)&d->prof, 32 * sizeof(unsigned long long)) != cudaSuccess)
        return GBFV_ERR_OOM;
    if (d->prof && cudaMemsetAsync(d->prof, 0, 32 * sizeof(unsigned long long), s) != cudaSuccess)
        return GBFV_ERR_CUDA;
    AmgKArgs<T> a = kargs<T>(*d, st);
    a.redTol = redTol;
    a.absTol = absTol;
    a.maxRes = maxRes;
    a.maxIter = maxIter;
    const int n = d->N;
    if (d->b == 2) kAmgPermute<T, 2><<<(n + 255) / 256, 256, 0, s>>>(n, d->map0, rhs, (T*)a.rhs, 1);
    else kAmgPermute<T, 3><<<(n + 255) / 256, 256, 0, s>>>(n, d->map0, rhs, (T*)a.rhs, 1);
    countLaunch();
    const void* fn = d->b == 2 ? (const void*)kAmgBicgstab<T, 2> : (const void*)kAmgBicgstab<T, 3>;
    if ((rs = launchCoop<T>(fn, a, d->blocks[k], s))) return rs;
    if (d->b == 2) kAmgPermute<T, 2><<<(n + 255) / 256, 256, 0, s>>>(n, d->map0, a.x, x, 0);
    else kAmgPermute<T, 3><<<(n + 255) / 256, 256, 0, s>>>(n, d->map0, a.x, x, 0);
    countLaunch();
    cudaEventRecord(d->evB, s);
    if (cudaMemcpyAsync(hst, st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        setLastError(std::string("AMG solve: ") + cudaGetErrorString(cudaGetLastError()));
        return GBFV_ERR_CUDA;
    }
    iters = hst->iterations;
    if (ms) cudaEventElapsedTime(ms, d->evA, d->evB);
    if (profFile && d->prof) {
        // one JSON line per solve: V-cycles, nanoseconds per level down / up,
        // coarsest (or tail), and the whole solve
        unsigned long long h[32];
        float solveMs = 0;
        cudaEventElapsedTime(&solveMs, d->evA, d->evB);
        if (cudaMemcpy(h, d->prof, sizeof(h), cudaMemcpyDeviceToHost) == cudaSuccess)
            if (FILE* f = std::fopen(profFile, "a")) {
                const int L = (int)d->lv.size();
                std::fprintf(f, "{\"precision\": %d, \"iterations\": %d, \"solve_ms\": %.4f, \"vcycles\": %llu, \"rows\": [",
                             (int)sizeof(T) * 8, iters, solveMs, h[31]);
                for (int l = 0; l < L; ++l) std::fprintf(f, "%s%d", l ? ", " : "", d->lv[l].n);
                std::fprintf(f, "], \"colors\": [");
                for (int l = 0; l < L; ++l) std::fprintf(f, "%s%d", l ? ", " : "", d->lv[l].nColors);
                std::fprintf(f, "], \"width\": [");
                for (int l = 0; l < L; ++l) std::fprintf(f, "%s%d", l ? ", " : "", d->lv[l].W);
                std::fprintf(f, "], \"tpr\": [");
                for (int l = 0; l < L; ++l) std::fprintf(f, "%s%d", l ? ", " : "", d->lv[l].tpr);
                std::fprintf(f, "], \"down_ns\": [");
                for (int l = 0; l + 1 < L; ++l) std::fprintf(f, "%s%llu", l ? ", " : "", h[l]);
                std::fprintf(f, "], \"coarsest_ns\": %llu, \"up_ns\": [", h[15]);
                for (int l = 0; l + 1 < L; ++l) std::fprintf(f, "%s%llu", l ? ", " : "", h[16 + l]);
                std::fprintf(f, "], \"tail\": %d}\n", a.tail);
                std::fclose(f);
            }
    }
    if (bytes) *bytes = iterationBytes(*d, (int)sizeof(T)) * iters;
    if (hst->code) return hst->code;
    return hst->converged ? GBFV_OK : GBFV_ERR_NOT_CONVERGED;
}

// one V-cycle v = M^-1 d in FP64 (both vectors in internal order), for tests
int amgApply64(AmgData* d, const double* A, const double* dv, double* v, cudaStream_t s, DevStatus* st,
               DevStatus* hst)
{
    int rs;
    if ((rs = ensurePrecision<double>(*d))) return rs;
    if (cudaMemsetAsync(st, 0, sizeof(DevStatus), s) != cudaSuccess) return GBFV_ERR_CUDA;
    if (cudaMemsetAsync(d->bar, 0, 4 * sizeof(unsigned), s) != cudaSuccess) return GBFV_ERR_CUDA;
    rs = d->b == 2 ? amgValues<double, 2>(*d, A, s, st) : amgValues<double, 3>(*d, A, s, st);
    if (rs) return rs;
    AmgKArgs<double> a = kargs<double>(*d, st);
    const int n = d->N;
    if (d->b == 2) kAmgPermute<double, 2><<<(n + 255) / 256, 256, 0, s>>>(n, d->map0, dv, (double*)a.rhs, 1);
    else kAmgPermute<double, 3><<<(n + 255) / 256, 256, 0, s>>>(n, d->map0, dv, (double*)a.rhs, 1);
    countLaunch();
    const void* fn = d->b == 2 ? (const void*)kAmgApply<double, 2> : (const void*)kAmgApply<double, 3>;
    if ((rs = launchCoop<double>(fn, a, d->blocks[0], s))) return rs;
    if (d->b == 2) kAmgPermute<double, 2><<<(n + 255) / 256, 256, 0, s>>>(n, d->map0, a.x, v, 0);
    else kAmgPermute<double, 3><<<(n + 255) / 256, 256, 0, s>>>(n, d->map0, a.x, v, 0);
    countLaunch();
    if (cudaMemcpyAsync(hst, st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GBFV_ERR_CUDA;
    return hst->code;
}

template int amgSolve<double>(AmgData*, const double*, const double*, double*, double, double, double, int,
                              cudaStream_t, DevStatus*, DevStatus*, int&, float*, double*);
template int amgSolve<float>(AmgData*, const float*, const float*, float*, double, double, double, int, cudaStream_t,
                             DevStatus*, DevStatus*, int&, float*, double*);

}  // namespace gbfv
