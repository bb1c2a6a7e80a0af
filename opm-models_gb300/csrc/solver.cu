// Linear solver kernels: block ILU(0) factorization, level-scheduled
// triangular sweeps and BiCGStab, all inside one persistent cooperative
// kernel per solve; plus the FP64 kernels of the mixed-precision outer
// iterative refinement.
//
// The algorithm is the reference's (ParallelBiCGStabSolverBackend ->
// BiCGStabSolver with Dune::SeqILU<...,0> and CombinedCriterion;
// bicgstabsolver.hh:120-330, combinedcriterion.hh:116-209,
// istlpreconditionerwrappers.hh:151-190): zero initial guess, r0hat = b,
// right preconditioning, max-norm criterion on the recursively updated
// residual, breakdown threshold numeric_limits<double>::min()*1e10.
//
// ILU(0) of the 5/7-point TPFA pattern: every lower entry (i,k) only updates
// the diagonal of row i (row k's upper entries other than (k,i) are outside
// row i's pattern), so the factorization is
//     L_ik = A_ik * D_k^-1 ;  D_i = A_ii - sum_k L_ik A_ki  (k ascending)
// and the upper factor is A's own upper part.  Rows of one wavefront level
// are independent; levels are separated by grid barriers.  Every wait on a
// barrier is bounded: on timeout the kernel records GBFV_ERR_TIMEOUT and all
// blocks leave.
#include <cuda_runtime.h>

#include "../../include/gbfv.h"
#include "gbfv_internal.cuh"
#include "solver.cuh"
#include "krylov.cuh"

namespace gbfv {

// --------------------------------------------------------- phases ---------
template <class T, int B, int MODE>
__device__ bool phaseFactor(const KArgs<T>& a, const Team<MODE>& tm)
{
    const int gt = tm.rank * blockDim.x + threadIdx.x, gs = tm.nblk * blockDim.x;
    const int dim = a.dim, ld = a.ldN;
    for (int l = 0; l < a.numLev; ++l) {
        const int i0 = a.levPtr[l], i1 = a.levPtr[l + 1];
        for (int i = i0 + gt; i < i1; i += gs) {
            T D[B * B];
            ldBlock<T, B>(a.A, dim, ld, i, D);
            for (int s = 0; s < dim; ++s) {
                const int k = a.col[s * ld + i];
                if (k < 0) continue;
                T As[B * B], Dk[B * B], L[B * B], U[B * B];
                ldBlock<T, B>(a.A, s, ld, i, As);
#pragma unroll
                for (int e = 0; e < B * B; ++e) Dk[e] = ldcg(&a.FD[e * ld + k]);
#pragma unroll
                for (int r = 0; r < B; ++r)
#pragma unroll
                    for (int c = 0; c < B; ++c) {
                        T t = T(0);
#pragma unroll
                        for (int q = 0; q < B; ++q) t += As[r * B + q] * Dk[q * B + c];
                        L[r * B + c] = t;
                    }
#pragma unroll
                for (int e = 0; e < B * B; ++e) a.FL[(s * B * B + e) * ld + i] = L[e];
                ldBlock<T, B>(a.A, 2 * dim - s, ld, k, U);
#pragma unroll
                for (int r = 0; r < B; ++r)
#pragma unroll
                    for (int c = 0; c < B; ++c) {
                        T t = T(0);
#pragma unroll
                        for (int q = 0; q < B; ++q) t += L[r * B + q] * U[q * B + c];
                        D[r * B + c] -= t;
                    }
            }
            T R[B * B];
            if (!invertBlock<T, B>(D, R)) {
                atomicExch(&a.st->code, GBFV_ERR_SINGULAR);
#pragma unroll
                for (int e = 0; e < B * B; ++e) R[e] = T(0);
            }
#pragma unroll
            for (int e = 0; e < B * B; ++e) a.FD[e * ld + i] = R[e];
        }
        if (!teamSync<MODE>(a.gs)) return false;
    }
    return true;
}

// forward sweep: y = L^-1 d.  With fuseP the right-hand side is the BiCGStab
// direction p = r + (-beta)(omega v - p), formed and stored here.
template <class T, int B, int MODE>
__device__ bool sweepLower(const KArgs<T>& a, const T* d, T* y, bool fuseP, T beta, T omega,
                           const Team<MODE>& tm)
{
    const int gt = tm.rank * blockDim.x + threadIdx.x, gs = tm.nblk * blockDim.x;
    const int dim = a.dim, ld = a.ldN;
    for (int l = 0; l < a.numLev; ++l) {
        const int i0 = a.levPtr[l], i1 = a.levPtr[l + 1];
        for (int i = i0 + gt; i < i1; i += gs) {
            T acc[B];
            if (fuseP) {
#pragma unroll
                for (int e = 0; e < B; ++e) {
                    T tmp = ldcg(&a.v[i * B + e]);
                    tmp *= omega;
                    tmp -= ldcg(&a.p[i * B + e]);
                    tmp *= -beta;
                    T pe = ldcg(&a.r[i * B + e]);
                    pe += tmp;
                    a.p[i * B + e] = pe;
                    acc[e] = pe;
                }
            }
            else {
#pragma unroll
                for (int e = 0; e < B; ++e) acc[e] = ldcg(&d[i * B + e]);
            }
            for (int s = 0; s < dim; ++s) {
                const int k = a.col[s * ld + i];
                if (k < 0) continue;
                T yk[B];
#pragma unroll
                for (int e = 0; e < B; ++e) yk[e] = ldcg(&y[k * B + e]);
#pragma unroll
                for (int r = 0; r < B; ++r)
#pragma unroll
                    for (int c = 0; c < B; ++c) acc[r] -= ldcg(&a.FL[(s * B * B + r * B + c) * ld + i]) * yk[c];
            }
#pragma unroll
            for (int e = 0; e < B; ++e) y[i * B + e] = acc[e];
        }
        if (!teamSync<MODE>(a.gs)) return false;
    }
    return true;
}

// backward sweep in place: y = D^-1 (y - U y)
template <class T, int B, int MODE>
__device__ bool sweepUpper(const KArgs<T>& a, T* y, const Team<MODE>& tm)
{
    const int gt = tm.rank * blockDim.x + threadIdx.x, gs = tm.nblk * blockDim.x;
    const int dim = a.dim, ld = a.ldN;
    for (int l = a.numLev - 1; l >= 0; --l) {
        const int i0 = a.levPtr[l], i1 = a.levPtr[l + 1];
        for (int i = i0 + gt; i < i1; i += gs) {
            T acc[B];
#pragma unroll
            for (int e = 0; e < B; ++e) acc[e] = ldcg(&y[i * B + e]);
            for (int s = 2 * dim; s > dim; --s) {
                const int k = a.col[s * ld + i];
                if (k < 0) continue;
                T yk[B];
#pragma unroll
                for (int e = 0; e < B; ++e) yk[e] = ldcg(&y[k * B + e]);
#pragma unroll
                for (int r = 0; r < B; ++r)
#pragma unroll
                    for (int c = 0; c < B; ++c) acc[r] -= a.A[(s * B * B + r * B + c) * ld + i] * yk[c];
            }
            T out[B];
#pragma unroll
            for (int r = 0; r < B; ++r) {
                T t = T(0);
#pragma unroll
                for (int c = 0; c < B; ++c) t += ldcg(&a.FD[(r * B + c) * ld + i]) * acc[c];
                out[r] = t;
            }
#pragma unroll
            for (int e = 0; e < B; ++e) y[i * B + e] = out[e];
        }
        if (!teamSync<MODE>(a.gs)) return false;
    }
    return true;
}

// ---------------------------------------------- cluster / DSMEM sweeps ---
// One row per thread: row levPtr[l] + (rank*NT + tid).  Each block keeps the
// results of the level it just computed in shared memory; the next level reads
// its (structured-grid: all) dependencies from the previous level through
// distributed shared memory instead of L2.  The cluster barrier is split:
// after a level is stored the block arrives, loads the next level's matrix
// blocks and column indices (which do not depend on the sweep), then waits.
__device__ __forceinline__ void clusterArrive() { asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory"); }
__device__ __forceinline__ void clusterWait() { asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory"); }

// ----------------------------------------------- cluster push sweeps ----
// Rows of a level are dealt to the blocks of the cluster a warp at a time:
// position t belongs to block (t/32) % C, local slot ((t/32)/C)*32 + t%32,
// so each warp reads 32 consecutive rows.  A row's dependencies (its lower
// neighbours in the forward sweep, upper ones in the backward sweep) are all
// in the previous level.  Each producer pushes its result into the
// consumers' shared memory with st.async; the bytes are counted on the
// consumer block's mbarrier (expect_tx / complete_tx), which the consumer
// waits on -- a point-to-point handshake, no release barrier per level.  A
// relaxed cluster barrier per level only keeps the blocks within one level of
// each other, so two dependency buffers suffice.
__device__ __forceinline__ void clusterArriveRelaxed()
{
    asm volatile("barrier.cluster.arrive.relaxed.aligned;\n" ::: "memory");
}
__device__ __forceinline__ unsigned smemAddr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned mapaRank(unsigned a, int rank)
{
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ void mbarInit(unsigned a, int count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbarArriveTx(unsigned a, unsigned bytes)
{
    // relaxed: arming publishes nothing, so it must not wait for this thread's
    // loads in flight (a release arrive would)
    asm volatile("mbarrier.arrive.expect_tx.relaxed.cta.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
// bounded wait for the phase with the given parity, relaxed: orders nothing,
// so it does not wait for this thread's loads in flight; false on timeout
__device__ __forceinline__ bool mbarWaitRelaxed(unsigned a, unsigned parity)
{
    const long long t0 = clock64();
    for (;;) {
        unsigned done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.relaxed.cta.shared::cta.b64 p, [%1], %2; "
            "selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > GB_TIMEOUT_CYCLES) return false;
    }
}
// bounded wait (acquire) for the phase with the given parity; false on timeout
__device__ __forceinline__ bool mbarWait(unsigned a, unsigned parity)
{
    const long long t0 = clock64();
    for (;;) {
        unsigned done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; "
            "selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > GB_TIMEOUT_CYCLES) return false;
    }
}
// A pushed block of B values occupies a slot of padB(B) values (3 -> 4), so
// that one vector st.async carries it (16-byte aligned for float, two 16-byte
// stores for double).
// remote push of one slot: vector st.async, bytes counted on the consumer's mbarrier
template <class T, int B>
__device__ __forceinline__ void stAsyncSlot(unsigned dst, const T (&v)[B], unsigned mbar)
{
    if constexpr (sizeof(T) == 4 && B == 3) {
        asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(dst),
                     "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(0u),
                     "r"(mbar)
                     : "memory");
    }
    else if constexpr (sizeof(T) == 4 && B == 2) {
        asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.b32 [%0], {%1, %2}, [%3];" ::"r"(dst),
                     "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(mbar)
                     : "memory");
    }
    else {
#pragma unroll
        for (int e = 0; e < B; e += 2) {
            const double hi = (e + 1 < B) ? (double)v[e + 1] : 0.0;
            asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.b64 [%0], {%1, %2}, [%3];" ::"r"(
                             dst + e * 8u),
                         "l"(__double_as_longlong((double)v[e])), "l"(__double_as_longlong(hi)), "r"(mbar)
                         : "memory");
        }
    }
}

struct PushState {
    unsigned mb[PUSH_BUFFERS];   // shared addresses of the data mbarriers, one per dependency buffer
    unsigned ph[PUSH_BUFFERS];   // parity of the next phase to wait for
    unsigned dep;     // shared address of the dependency buffers [PUSH_BUFFERS][NT][3][padB(B)]
    unsigned lev;     // shared address of the level-done mbarrier (C arrivals)
    unsigned levPh;
    unsigned tph;     // tile sweeps: parity of the current sweep's phase of every level's halo mbarrier
    int sbuf;         // tile sweeps: the staging buffer of the next level
    int ok;
};

// All-to-all level barrier of the cluster without acquire at cluster scope:
// thread t < C of every block arrives (relaxed) on block t's level-done
// mbarrier, then every thread waits on its own.  Data ordering is not its job
// (the st.async transaction counts do that); it only keeps the blocks within
// one level of each other.
__device__ __forceinline__ void levelBarrier(PushState& ps, int C, int rank)
{
    __syncthreads();
    const int t = threadIdx.x;
    if (t < C) {
        if (t == rank)
            asm volatile("mbarrier.arrive.relaxed.cta.shared::cta.b64 _, [%0];" ::"r"(ps.lev) : "memory");
        else
            asm volatile("mbarrier.arrive.relaxed.cluster.shared::cluster.b64 _, [%0];" ::"r"(mapaRank(ps.lev, t))
                         : "memory");
    }
    if (ps.ok && !mbarWaitRelaxed(ps.lev, ps.levPh)) ps.ok = 0;
    ps.levPh ^= 1u;
}

__device__ __forceinline__ void levelSlot(int t, int C, int& owner, int& loc)
{
    const int w = t >> 5;
    owner = w % C;
    loc = ((w / C) << 5) | (t & 31);
}

// Level-rotating thread groups: the block's threads form G groups of NT/G;
// group (l mod G) computes level l.  Right after computing a level a group
// loads the matrix blocks and right-hand sides of its next level (l + G), so
// those loads have G-1 levels to complete before they are used.  Every
// thread takes part in each level's mbarrier phase (idle groups expect zero
// bytes) and in the relaxed cluster barrier.
template <class T, int B, int NT>
struct SweepMap {
    int C, G, NG, rank, tid, grp, u;
    __device__ SweepMap(const Team<SYNC_CLUSTER>& tm, int G_) : C(tm.nblk), G(G_), rank(tm.rank)
    {
        tid = threadIdx.x;
        NG = NT / G;
        grp = tid / NG;
        u = tid - grp * NG;
    }
    // this thread's position inside level l of width W, or -1: warps dealt
    // round-robin to the blocks (ownerMode 0), or each block a contiguous
    // share rounded to whole warps (ownerMode 1)
    __device__ __forceinline__ int pos(int W, int ownerMode) const
    {
        if (ownerMode == 0) return ((((u >> 5) * C) + rank) << 5) | (u & 31);
        const int chunk = (((W + C - 1) / C) + 31) & ~31;
        return u < chunk ? rank * chunk + u : -1;
    }
};

// A push target is the consumer block (bits 24..31) and the element offset
// of the consumer's slot inside one half of the dependency buffer
// (precomputed on the host for the launch configuration).
template <class T, int B>
__device__ __forceinline__ void pushValues(int target, int half, const T (&out)[B], const Team<SYNC_CLUSTER>& tm,
                                           const T* dep, PushState& ps, int mbIdx)
{
    // also a consumer in this block gets its values by st.async (to this block's
    // own shared memory): the transaction count orders them, no fence needed
    const int owner = target >> 24;
    if (owner >= tm.nblk) {  // a table for another cluster size: no push outside the cluster
        ps.ok = 0;
        return;
    }
    const int off = (target & 0xffffff) + half;
    const unsigned dst = mapaRank(ps.dep + (unsigned)(off * sizeof(T)), owner);
    const unsigned mb = mapaRank(ps.mb[mbIdx], owner);
    stAsyncSlot<T, B>(dst, out, mb);
}

// Asynchronous global -> shared copies (no registers held, not waited for by
// barriers or fences); each thread waits for its own with wait_all.
template <int S>
__device__ __forceinline__ void cpAsync(unsigned dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(dst), "l"(src), "n"(S) : "memory");
}
// 16-byte copy, both addresses 16-byte aligned, not cached in L1
__device__ __forceinline__ void cpAsync16(unsigned dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cpCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cpWaitAll() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Shared memory of the push sweeps beyond the dependency buffer: one staging
// slot per thread for the operands of the next level it computes (field f of
// thread t at [f*NT + t]), the level pointers and this block's expected bytes
// per level (forward and backward sweep).
template <class T, int B, int NT>
struct PushSmem {
    static constexpr int NDEP = PUSH_BUFFERS * NT * 3 * padB(B);  // dependency buffers
    // staged fields: forward sweep 3 factor blocks + 3 vectors, backward
    // sweep 3 matrix blocks + inverted pivot + 1 vector
    static constexpr int NF = 4 * B * B + B > 3 * B * B + 3 * B ? 4 * B * B + B : 3 * B * B + 3 * B;
    static constexpr int NI = 6;                   // 3 neighbour columns, 3 push targets
    T* dep;      // [PUSH_BUFFERS][NT][3][padB(B)]: values pushed by the producers of a level's rows
    T* st;
    int* sn;
    int* lev;    // [numLev + 1]
    int* nval;   // [2*l + 0/1]: values this block receives at level l (forward/backward), and
                 // PUSH_BARRIER_FLAG if a cluster barrier follows level l in that sweep
    __device__ PushSmem(unsigned char* base, int numLev)
    {
        dep = reinterpret_cast<T*>(base);
        st = dep + NDEP;
        sn = reinterpret_cast<int*>(st + NF * NT);
        lev = sn + NI * NT;
        nval = lev + numLev + 1;
    }
    static constexpr size_t bytes(int numLev)
    {
        return sizeof(T) * ((size_t)NDEP + (size_t)NF * NT) +
               sizeof(int) * ((size_t)NI * NT + 3 * (size_t)numLev + 1);
    }
};
constexpr int PUSH_COUNT_MASK = PUSH_BARRIER_FLAG - 1;

// Shared memory of the tile sweeps: per level this block's (first row, rows,
// forward / backward halo slots) and the mbarrier that counts the bytes
// pushed into it for that level; the halo slots; two copies of this block's
// results of a level (the current and the previous one); two staging
// buffers.  A level's operands of one block are contiguous runs (its rows
// are), staged in 16-byte chunks, the next level's while the current one is
// computed.  A run starts at the 16-byte boundary below its first row, so a
// few elements precede the first row's.
template <class T, int B, int NT>
struct TileSmem {
    static constexpr int E = 16 / sizeof(T);  // elements of T per 16 bytes
    int4* info;
    unsigned long long* mb;   // [nl] halo data of a level
    T* halo;                  // [slot][padB(B)]
    T* loc;                   // [2][NT][padB(B)]: results of levels of parity 0 and 1
    T* stT;                   // [2][regT]: matrix blocks and vectors of a level
    int* stI;                 // [2][regI]: dependency codes and push targets of a level
    int* bad;                 // block rank 0's copy: a wait of some block of the cluster gave up (sticky)
    int capS, capA, capI, regT, regI;
    __host__ __device__ static constexpr int rup(int x, int m) { return (x + m - 1) / m * m; }
    // capacities for levels of at most w rows: a field of one value per row
    // (T or int), a vector of B values per row; per buffer the larger of the
    // forward sweep's (dim*B*B fields, 3 vectors) and the backward sweep's
    // ((dim+1)*B*B fields, 1 vector), and 2*dim int fields
    __host__ __device__ static void caps(int w, int dim, int& cS, int& cA, int& cI, int& rT, int& rI)
    {
        cS = rup(w + E, E);
        cA = rup(w * B + E, E);
        cI = rup(w + 4, 4);
        const int f = dim * B * B * cS + 3 * cA, g = (dim + 1) * B * B * cS + cA;
        rT = f > g ? f : g;
        rI = 2 * dim * cI;
    }
    __host__ __device__ static size_t a16(size_t x) { return (x + 15) & ~(size_t)15; }
    struct Off {
        size_t mb, halo, loc, stT, stI, bad, end;
    };
    __host__ __device__ static Off offsets(int nl, int hs, int w, int dim)
    {
        int cS, cA, cI, rT, rI;
        caps(w, dim, cS, cA, cI, rT, rI);
        Off o;
        o.mb = a16(16 * (size_t)nl);
        o.halo = a16(o.mb + 8 * (size_t)nl);
        o.loc = a16(o.halo + sizeof(T) * (size_t)hs * padB(B));
        o.stT = a16(o.loc + sizeof(T) * 2 * (size_t)NT * padB(B));
        o.stI = a16(o.stT + sizeof(T) * 2 * (size_t)rT);
        o.bad = a16(o.stI + sizeof(int) * 2 * (size_t)rI);
        o.end = o.bad + 16;
        return o;
    }
    __host__ __device__ static size_t bytes(int nl, int hs, int w, int dim) { return offsets(nl, hs, w, dim).end; }
    __device__ TileSmem(unsigned char* base, int nl, int hs, int w, int dim)
    {
        const Off o = offsets(nl, hs, w, dim);
        caps(w, dim, capS, capA, capI, regT, regI);
        info = reinterpret_cast<int4*>(base);
        mb = reinterpret_cast<unsigned long long*>(base + o.mb);
        halo = reinterpret_cast<T*>(base + o.halo);
        loc = reinterpret_cast<T*>(base + o.loc);
        stT = reinterpret_cast<T*>(base + o.stT);
        stI = reinterpret_cast<int*>(base + o.stI);
        bad = reinterpret_cast<int*>(base + o.bad);
    }
};

// forward sweep y = L^-1 d (fuseP: d is the BiCGStab direction p, formed here).
// The group that computed the previous level stages the operands of its next
// level while the current group works, so those copies stay off the current
// level's critical path.
template <class T, int B, int NT>
__device__ __forceinline__ void sweepLowerPush(const KArgs<T>& a, const T* d, T* y, bool fuseP, T beta, T omega,
                                               const Team<SYNC_CLUSTER>& tm, const T* dep, PushState& ps,
                                               const PushSmem<T, B, NT>& sm)
{
    constexpr int BB = B * B, VB = 3 * BB, PB = padB(B);
    const SweepMap<T, B, NT> mp(tm, a.grp);
    const int dim = a.dim, ld = a.ldN, nl = a.numLev, G = mp.G, tid = mp.tid;
    const int half = NT * 3 * PB;
    const T* st = sm.st;
    const int* sn = sm.sn;
    const unsigned stA = smemAddr(sm.st) + tid * sizeof(T), snA = smemAddr(sm.sn) + tid * sizeof(int);
    int iCur = -1;
    auto load = [&](int l) {
        iCur = -1;
        if (l >= nl) return;
        const int t = mp.pos(sm.lev[l + 1] - sm.lev[l], a.ownerMode);
        const int i = sm.lev[l] + t;
        if (t < 0 || i >= sm.lev[l + 1]) return;
        iCur = i;
#pragma unroll
        for (int s = 0; s < 3; ++s) {
            if (s >= dim) break;
            cpAsync<4>(snA + (s * NT) * 4, &a.col[s * ld + i]);
            cpAsync<4>(snA + ((3 + s) * NT) * 4, &a.pushL[s * ld + i]);
#pragma unroll
            for (int e = 0; e < BB; ++e)
                cpAsync<sizeof(T)>(stA + ((s * BB + e) * NT) * sizeof(T), &a.FL[(s * BB + e) * ld + i]);
        }
        if (fuseP) {
#pragma unroll
            for (int e = 0; e < B; ++e) {
                cpAsync<sizeof(T)>(stA + ((VB + e) * NT) * sizeof(T), &a.v[i * B + e]);
                cpAsync<sizeof(T)>(stA + ((VB + B + e) * NT) * sizeof(T), &a.p[i * B + e]);
                cpAsync<sizeof(T)>(stA + ((VB + 2 * B + e) * NT) * sizeof(T), &a.r[i * B + e]);
            }
        }
        else {
#pragma unroll
            for (int e = 0; e < B; ++e) cpAsync<sizeof(T)>(stA + ((VB + e) * NT) * sizeof(T), &d[i * B + e]);
        }
        cpCommit();
    };
    load(mp.grp);
    if (tid == 0) mbarArriveTx(ps.mb[0], (unsigned)((sm.nval[0] & PUSH_COUNT_MASK) * sizeof(T)));
    // optional cycle counts of one working thread (GBFV_PROFILE): data wait,
    // compute, pushes + stores, level barrier
    const bool probe = a.prof != nullptr && tm.rank == 0 && tid == 0;
    unsigned long long cyc[4] = {0, 0, 0, 0}, t0 = 0, t1 = 0, t2 = 0, t3 = 0, nprobe = 0;
    for (int l = 0; l < nl; ++l) {
        const int k = l & (PUSH_BUFFERS - 1), kn = (l + 1) & (PUSH_BUFFERS - 1);
        const bool mine = mp.grp == l % G;
        if (mine) {
            const int i = iCur;
            // the row's staged operands go to registers before the data wait
            T out[B];
            bool has[3] = {false, false, false};
            int tg[3] = {-1, -1, -1};
            if (i >= 0) {
                cpWaitAll();
                if (fuseP) {
#pragma unroll
                    for (int e = 0; e < B; ++e) {
                        T tmp = st[(VB + e) * NT + tid];
                        tmp *= omega;
                        tmp -= st[(VB + B + e) * NT + tid];
                        tmp *= -beta;
                        T pe = st[(VB + 2 * B + e) * NT + tid];
                        pe += tmp;
                        a.p[i * B + e] = pe;  // the new direction p = r - beta (p - omega v)
                        out[e] = pe;
                    }
                }
                else {
#pragma unroll
                    for (int e = 0; e < B; ++e) out[e] = st[(VB + e) * NT + tid];
                }
#pragma unroll
                for (int s = 0; s < 3; ++s) {
                    if (s >= dim) break;
                    has[s] = sn[s * NT + tid] >= 0;
                    tg[s] = sn[(3 + s) * NT + tid];
                }
            }
            if (probe) t0 = clock64();
            // after a timeout: no more waits and no more pushes
            if (ps.ok && !mbarWait(ps.mb[k], ps.ph[k])) ps.ok = 0;
            if (probe) t1 = t2 = clock64();
            if (i >= 0) {
                const T* md = dep + (k * NT + tid) * 3 * PB;
#pragma unroll
                for (int s = 0; s < 3; ++s) {
                    if (s >= dim) break;
                    if (!has[s]) continue;
                    T m[B];
#pragma unroll
                    for (int c = 0; c < B; ++c) m[c] = md[s * PB + c];
#pragma unroll
                    for (int r = 0; r < B; ++r)
#pragma unroll
                        for (int c = 0; c < B; ++c) out[r] -= st[(s * BB + r * B + c) * NT + tid] * m[c];
                }
                if (probe) t2 = clock64();
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    if (q >= dim) break;
                    if (tg[q] >= 0 && ps.ok) pushValues<T, B>(tg[q], kn * half, out, tm, dep, ps, kn);
                }
#pragma unroll
                for (int e = 0; e < B; ++e) y[i * B + e] = out[e];
            }
            if (G == 1) load(l + 1);
        }
        else if (G > 1 && l >= 1 && mp.grp == (l - 1) % G) {
            load(l - 1 + G);
        }
        ps.ph[k] ^= 1u;
        if (probe && mine) t3 = clock64();
        if (tid == 0 && l + 1 < nl)
            mbarArriveTx(ps.mb[kn], (unsigned)((sm.nval[2 * (l + 1)] & PUSH_COUNT_MASK) * sizeof(T)));
        if (sm.nval[2 * l] & PUSH_BARRIER_FLAG) levelBarrier(ps, mp.C, mp.rank);
        else __syncthreads();
        if (probe && mine) {
            const unsigned long long t4 = clock64();
            cyc[0] += t1 - t0;
            cyc[1] += t2 - t1;
            cyc[2] += t3 - t2;
            cyc[3] += t4 - t3;
            nprobe++;
        }
    }
    if (probe) {
        for (int j = 0; j < 4; ++j) a.prof[8 + j] += cyc[j];
        a.prof[12] += nprobe;
    }
    cg::this_cluster().sync();  // publish the global stores to the next phase
}

// backward sweep in place: y = D^-1 (y - U y)
template <class T, int B, int NT>
__device__ __forceinline__ void sweepUpperPush(const KArgs<T>& a, T* y, const Team<SYNC_CLUSTER>& tm, const T* dep,
                                               PushState& ps, const PushSmem<T, B, NT>& sm)
{
    constexpr int BB = B * B, VB = 4 * BB, PB = padB(B);
    const SweepMap<T, B, NT> mp(tm, a.grp);
    const int dim = a.dim, ld = a.ldN, nl = a.numLev, G = mp.G, tid = mp.tid;
    const int half = NT * 3 * PB;
    const T* st = sm.st;
    const int* sn = sm.sn;
    const unsigned stA = smemAddr(sm.st) + tid * sizeof(T), snA = smemAddr(sm.sn) + tid * sizeof(int);
    int iCur = -1;
    auto load = [&](int l) {
        iCur = -1;
        if (l < 0) return;
        const int t = mp.pos(sm.lev[l + 1] - sm.lev[l], a.ownerMode);
        const int i = sm.lev[l] + t;
        if (t < 0 || i >= sm.lev[l + 1]) return;
        iCur = i;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            if (q >= dim) break;
            const int s = 2 * dim - q;  // descending column order
            cpAsync<4>(snA + (q * NT) * 4, &a.col[s * ld + i]);
            cpAsync<4>(snA + ((3 + q) * NT) * 4, &a.pushU[q * ld + i]);
#pragma unroll
            for (int e = 0; e < BB; ++e)
                cpAsync<sizeof(T)>(stA + ((q * BB + e) * NT) * sizeof(T), &a.A[(s * BB + e) * ld + i]);
        }
#pragma unroll
        for (int e = 0; e < BB; ++e) cpAsync<sizeof(T)>(stA + ((3 * BB + e) * NT) * sizeof(T), &a.FD[e * ld + i]);
#pragma unroll
        for (int e = 0; e < B; ++e) cpAsync<sizeof(T)>(stA + ((VB + e) * NT) * sizeof(T), &y[i * B + e]);
        cpCommit();
    };
    // group of level l is l % G, also for the descending sweep
    {
        int first = -1;
        for (int l = nl - 1; l >= 0 && l >= nl - G; --l)
            if (l % G == mp.grp) first = l;
        load(first);
        if (tid == 0)
            mbarArriveTx(ps.mb[(nl - 1) & (PUSH_BUFFERS - 1)],
                         (unsigned)((sm.nval[2 * (nl - 1) + 1] & PUSH_COUNT_MASK) * sizeof(T)));
    }
    for (int l = nl - 1; l >= 0; --l) {
        const int k = l & (PUSH_BUFFERS - 1), kn = (l + PUSH_BUFFERS - 1) & (PUSH_BUFFERS - 1);
        const bool mine = mp.grp == l % G;
        if (mine) {
            const int i = iCur;
            // the row's staged operands go to registers before the data wait
            T acc[B];
            bool has[3] = {false, false, false};
            int tg[3] = {-1, -1, -1};
            if (i >= 0) {
                cpWaitAll();
#pragma unroll
                for (int e = 0; e < B; ++e) acc[e] = st[(VB + e) * NT + tid];
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    if (q >= dim) break;
                    has[q] = sn[q * NT + tid] >= 0;
                    tg[q] = sn[(3 + q) * NT + tid];
                }
            }
            if (ps.ok && !mbarWait(ps.mb[k], ps.ph[k])) ps.ok = 0;
            if (i >= 0) {
                const T* md = dep + (k * NT + tid) * 3 * PB;
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    if (q >= dim) break;
                    if (!has[q]) continue;
                    T m[B];
#pragma unroll
                    for (int c = 0; c < B; ++c) m[c] = md[q * PB + c];
#pragma unroll
                    for (int r = 0; r < B; ++r)
#pragma unroll
                        for (int c = 0; c < B; ++c) acc[r] -= st[(q * BB + r * B + c) * NT + tid] * m[c];
                }
                T out[B];
#pragma unroll
                for (int r = 0; r < B; ++r) {
                    T t = T(0);
#pragma unroll
                    for (int c = 0; c < B; ++c) t += st[(3 * BB + r * B + c) * NT + tid] * acc[c];
                    out[r] = t;
                }
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    if (q >= dim) break;
                    if (tg[q] >= 0 && ps.ok) pushValues<T, B>(tg[q], kn * half, out, tm, dep, ps, kn);
                }
#pragma unroll
                for (int e = 0; e < B; ++e) y[i * B + e] = out[e];
            }
            if (G == 1) load(l - 1);
        }
        else if (G > 1 && l <= nl - 2 && mp.grp == (l + 1) % G) {
            load(l + 1 - G);
        }
        ps.ph[k] ^= 1u;
        if (tid == 0 && l > 0)
            mbarArriveTx(ps.mb[kn], (unsigned)((sm.nval[2 * (l - 1) + 1] & PUSH_COUNT_MASK) * sizeof(T)));
        if (sm.nval[2 * l + 1] & PUSH_BARRIER_FLAG) levelBarrier(ps, mp.C, mp.rank);
        else __syncthreads();
    }
    cg::this_cluster().sync();
}

// ------------------------------------------------ spatial-tile sweeps ----
// Block r of the cluster owns the rows of one spatial tile (all levels); at
// level l its thread u computes row first(l) + u.  Dependencies inside the
// tile come from the block's copy of the previous level (a __syncthreads
// apart); those across a tile boundary are pushed by the producing block
// with st.async into a halo slot of the consumer, counted on the consumer's
// mbarrier of that level.  Each halo slot is written once per sweep, so a
// block runs ahead of its downstream neighbours as far as its own
// dependencies allow: the sweep is a pipeline over the tiles, and the
// critical path crosses a block boundary only at tile edges.

// push of a row's result into a halo slot of another block of the cluster
template <class T, int B>
__device__ __forceinline__ void tilePush(int target, const T (&out)[B], unsigned mbLevel, unsigned halo0,
                                         const Team<SYNC_CLUSTER>& tm, int hcap, PushState& ps)
{
    const int owner = target >> 24, h = target & TILE_MASK;
    if (owner >= tm.nblk || h >= hcap) {  // tables for another cluster: push nothing
        ps.ok = 0;
        return;
    }
    const unsigned dst = mapaRank(halo0 + (unsigned)(h * padB(B) * sizeof(T)), owner);
    stAsyncSlot<T, B>(dst, out, mapaRank(mbLevel, owner));
}

// the dependency value of code c: this block's previous level or a halo slot
template <class T, int B>
__device__ __forceinline__ const T* tileDep(int c, const T* prev, const T* halo, int hcap, int NT, PushState& ps)
{
    if (c & TILE_HALO) {
        const int h = c & TILE_MASK;
        if (h < hcap) return halo + h * padB(B);
    }
    else if (c < NT)
        return prev + c * padB(B);
    ps.ok = 0;
    return nullptr;
}

// End of a tile sweep: the cluster barrier publishes the global stores and
// frees the halo slots for the next sweep.  A wait that gave up anywhere in
// the cluster is made known to every thread of it (block rank 0 keeps the
// flag); from then on no block arms, waits or pushes, so no mbarrier phase
// is armed twice, and the solve ends with GBFV_ERR_TIMEOUT.
template <class T, int B, int NT>
__device__ __forceinline__ void tileSweepEnd(const TileSmem<T, B, NT>& ts, PushState& ps)
{
    cg::cluster_group cl = cg::this_cluster();
    if (!ps.ok) *cl.map_shared_rank(ts.bad, 0) = 1;
    ps.tph ^= 1u;
    cl.sync();
    if (*cl.map_shared_rank(ts.bad, 0)) ps.ok = 0;
}

// The block stages level l's operands into buffer bf with 16-byte cp.async
// chunks spread over its threads (one commit group per level).  Forward
// sweep: the dim*B*B factor fields, nv vectors, dependency codes and push
// targets; backward sweep: the dim*B*B upper blocks, the B*B inverted pivot
// fields, the vector y, codes and targets.
template <class T, int B, int NT>
__device__ __forceinline__ void tileStage(const KArgs<T>& a, const TileSmem<T, B, NT>& ts, int l, int bf, bool fwd,
                                          const T* v0, const T* v1, const T* v2, int nv)
{
    constexpr int E = TileSmem<T, B, NT>::E, BB = B * B;
    const int dim = a.dim, ld = a.ldN;
    const int4 f = ts.info[l];
    const int first = f.x, cnt = f.y;
    const int a0S = first & ~(E - 1), a0A = (first * B) & ~(E - 1), a0I = first & ~3;
    // 16-byte chunks per field of each kind
    const int cS = TileSmem<T, B, NT>::rup((first - a0S + cnt) * (int)sizeof(T), 16) / 16;
    const int cA = TileSmem<T, B, NT>::rup((first * B - a0A + cnt * B) * (int)sizeof(T), 16) / 16;
    const int cI = TileSmem<T, B, NT>::rup((first - a0I + cnt) * 4, 16) / 16;
    const int nS = fwd ? dim * BB : (dim + 1) * BB;
    const int n1 = nS * cS, n2 = n1 + nv * cA, n3 = n2 + 2 * dim * cI;
    const unsigned sT = smemAddr(ts.stT + bf * ts.regT), sI = smemAddr(ts.stI + bf * ts.regI);
    for (int k = threadIdx.x; k < n3; k += NT) {
        if (k < n1) {
            const int j = k / cS, c = k - j * cS;
            const T* src;
            if (fwd)
                src = a.FL + (size_t)j * ld;  // field s*B*B + e of the lower factor
            else if (j < dim * BB) {
                const int q = j / BB, e = j - q * BB;
                src = a.A + (size_t)((2 * dim - q) * BB + e) * ld;  // descending column order
            }
            else
                src = a.FD + (size_t)(j - dim * BB) * ld;
            cpAsync16(sT + (unsigned)((j * ts.capS) * sizeof(T) + c * 16), src + a0S + c * E);
        }
        else if (k < n2) {
            const int v = (k - n1) / cA, c = k - n1 - v * cA;
            const T* src = v == 0 ? v0 : v == 1 ? v1 : v2;
            cpAsync16(sT + (unsigned)((nS * ts.capS + v * ts.capA) * sizeof(T) + c * 16), src + a0A + c * E);
        }
        else {
            const int m = (k - n2) / cI, c = k - n2 - m * cI;  // dependency codes, then push targets
            const int* src = m < dim ? (fwd ? a.tdepF : a.tdepB) + (size_t)m * ld
                                     : (fwd ? a.tpushF : a.tpushB) + (size_t)(m - dim) * ld;
            cpAsync16(sI + (unsigned)(m * ts.capI * 4 + c * 16), src + a0I + c * 4);
        }
    }
    cpCommit();
}

// Before level l is computed: stage it unless the previous level did, then
// the next level of this block into the other buffer (read two levels ago:
// every thread is past that level's barrier); wait for level l's copies and
// make them visible to the whole block.  Returns the buffer of level l.
template <class T, int B, int NT>
__device__ __forceinline__ int tileStageStep(const KArgs<T>& a, const TileSmem<T, B, NT>& ts, int l, int next,
                                             int& staged, bool fwd, const T* v0, const T* v1, const T* v2, int nv,
                                             PushState& ps)
{
    const int bf = ps.sbuf;
    if (staged != l) tileStage<T, B, NT>(a, ts, l, bf, fwd, v0, v1, v2, nv);
    if (next >= 0) {
        tileStage<T, B, NT>(a, ts, next, bf ^ 1, fwd, v0, v1, v2, nv);
        asm volatile("cp.async.wait_group 1;" ::: "memory");
    }
    else
        cpWaitAll();
    staged = next;
    ps.sbuf = bf ^ 1;
    __syncthreads();
    return bf;
}

// forward sweep y = L^-1 d (fuseP: d is the BiCGStab direction p, formed here)
template <class T, int B, int NT>
__device__ __forceinline__ void sweepLowerTile(const KArgs<T>& a, const T* d, T* y, bool fuseP, T beta, T omega,
                                               const Team<SYNC_CLUSTER>& tm, const TileSmem<T, B, NT>& ts,
                                               PushState& ps)
{
    constexpr int BB = B * B, PB = padB(B), E = TileSmem<T, B, NT>::E;
    const int dim = a.dim, nl = a.numLev, u = threadIdx.x, hcap = a.thalo;
    const int capS = ts.capS, capA = ts.capA, capI = ts.capI, nS = dim * BB;
    const unsigned mb0 = smemAddr(ts.mb), halo0 = smemAddr(ts.halo);
    const unsigned par = ps.tph;
    // this sweep's phase of every level's mbarrier: one arrival carrying the
    // bytes the other blocks push into this one at that level
    if (ps.ok)
        for (int l = u; l < nl; l += NT) mbarArriveTx(mb0 + 8u * l, (unsigned)(ts.info[l].z * PB * sizeof(T)));
    const T* v0 = fuseP ? a.v : d;
    const int nv = fuseP ? 3 : 1;
    // optional cycle counts of thread 0 of block 5 (GBFV_PROFILE): staging,
    // halo wait, compute + pushes + stores, level barrier
    const bool probe = a.prof != nullptr && tm.rank == 5 % tm.nblk && u == 0;
    unsigned long long cyc[4] = {0, 0, 0, 0}, nprobe = 0, t0 = 0, t1 = 0, t2 = 0, t3 = 0;
    int staged = -1;
    for (int l = 0; l < nl; ++l) {
        const int4 f = ts.info[l];
        if (f.y == 0) continue;  // no rows of this tile at this level (the same for the whole block)
        const int next = l + 1 < nl && ts.info[l + 1].y > 0 ? l + 1 : -1;
        if (probe) t0 = clock64();
        const int bf = tileStageStep<T, B, NT>(a, ts, l, next, staged, true, v0, a.p, a.r, nv, ps);
        if (probe) t1 = clock64();
        const T* sT = ts.stT + bf * ts.regT;
        const int* sI = ts.stI + bf * ts.regI;
        const int shS = f.x & (E - 1), shA = (f.x * B) & (E - 1), shI = f.x & 3;
        const bool act = u < f.y;
        const int i = f.x + u;
        T out[B];
        int code[3] = {-1, -1, -1}, tg[3] = {-1, -1, -1};
        if (act) {
            const T* vs = sT + nS * capS + shA + u * B;
            if (fuseP) {
#pragma unroll
                for (int e = 0; e < B; ++e) {
                    T tmp = vs[e];
                    tmp *= omega;
                    tmp -= vs[capA + e];
                    tmp *= -beta;
                    T pe = vs[2 * capA + e];
                    pe += tmp;
                    a.p[i * B + e] = pe;  // the new direction p = r - beta (p - omega v)
                    out[e] = pe;
                }
            }
            else {
#pragma unroll
                for (int e = 0; e < B; ++e) out[e] = vs[e];
            }
#pragma unroll
            for (int s = 0; s < 3; ++s) {
                if (s >= dim) break;
                code[s] = sI[s * capI + shI + u];
                tg[s] = sI[(dim + s) * capI + shI + u];
            }
        }
        // after a timeout: no more waits and no more pushes
        if (f.z > 0 && ps.ok && !mbarWait(mb0 + 8u * l, par)) ps.ok = 0;
        if (probe) t2 = clock64();
        if (act) {
            const T* prev = ts.loc + ((l + 1) & 1) * NT * PB;  // level l - 1
            const T* fl = sT + shS + u;
#pragma unroll
            for (int s = 0; s < 3; ++s) {
                if (s >= dim) break;
                if (code[s] < 0) continue;
                const T* md = tileDep<T, B>(code[s], prev, ts.halo, hcap, NT, ps);
                if (!md) continue;
                T m[B];
#pragma unroll
                for (int c = 0; c < B; ++c) m[c] = md[c];
#pragma unroll
                for (int r = 0; r < B; ++r)
#pragma unroll
                    for (int c = 0; c < B; ++c) out[r] -= fl[(s * BB + r * B + c) * capS] * m[c];
            }
            T* mine = ts.loc + (l & 1) * NT * PB + u * PB;
#pragma unroll
            for (int e = 0; e < B; ++e) mine[e] = out[e];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                if (q >= dim) break;
                if (tg[q] >= 0 && ps.ok && l + 1 < nl)
                    tilePush<T, B>(tg[q], out, mb0 + 8u * (l + 1), halo0, tm, hcap, ps);
            }
#pragma unroll
            for (int e = 0; e < B; ++e) y[i * B + e] = out[e];
        }
        if (probe) t3 = clock64();
        __syncthreads();
        if (probe) {
            const unsigned long long t4 = clock64();
            cyc[0] += t1 - t0;
            cyc[1] += t2 - t1;
            cyc[2] += t3 - t2;
            cyc[3] += t4 - t3;
            nprobe++;
        }
    }
    if (probe) {
        for (int j = 0; j < 4; ++j) a.prof[8 + j] += cyc[j];
        a.prof[12] += nprobe;
    }
    tileSweepEnd<T, B, NT>(ts, ps);
}

// backward sweep in place: y = D^-1 (y - U y)
template <class T, int B, int NT>
__device__ __forceinline__ void sweepUpperTile(const KArgs<T>& a, T* y, const Team<SYNC_CLUSTER>& tm,
                                               const TileSmem<T, B, NT>& ts, PushState& ps)
{
    constexpr int BB = B * B, PB = padB(B), E = TileSmem<T, B, NT>::E;
    const int dim = a.dim, nl = a.numLev, u = threadIdx.x, hcap = a.thalo;
    const int capS = ts.capS, capI = ts.capI, nS = (dim + 1) * BB;
    const unsigned mb0 = smemAddr(ts.mb), halo0 = smemAddr(ts.halo);
    const unsigned par = ps.tph;
    if (ps.ok)
        for (int l = u; l < nl; l += NT) mbarArriveTx(mb0 + 8u * l, (unsigned)(ts.info[l].w * PB * sizeof(T)));
    int staged = -1;
    for (int l = nl - 1; l >= 0; --l) {
        const int4 f = ts.info[l];
        if (f.y == 0) continue;
        const int next = l > 0 && ts.info[l - 1].y > 0 ? l - 1 : -1;
        const int bf = tileStageStep<T, B, NT>(a, ts, l, next, staged, false, y, nullptr, nullptr, 1, ps);
        const T* sT = ts.stT + bf * ts.regT;
        const int* sI = ts.stI + bf * ts.regI;
        const int shS = f.x & (E - 1), shA = (f.x * B) & (E - 1), shI = f.x & 3;
        const bool act = u < f.y;
        const int i = f.x + u;
        T acc[B];
        int code[3] = {-1, -1, -1}, tg[3] = {-1, -1, -1};
        if (act) {
#pragma unroll
            for (int e = 0; e < B; ++e) acc[e] = sT[nS * capS + shA + u * B + e];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                if (q >= dim) break;
                code[q] = sI[q * capI + shI + u];
                tg[q] = sI[(dim + q) * capI + shI + u];
            }
        }
        if (f.w > 0 && ps.ok && !mbarWait(mb0 + 8u * l, par)) ps.ok = 0;
        if (act) {
            const T* prev = ts.loc + ((l + 1) & 1) * NT * PB;  // level l + 1
            const T* au = sT + shS + u;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                if (q >= dim) break;
                if (code[q] < 0) continue;
                const T* md = tileDep<T, B>(code[q], prev, ts.halo, hcap, NT, ps);
                if (!md) continue;
                T m[B];
#pragma unroll
                for (int c = 0; c < B; ++c) m[c] = md[c];
#pragma unroll
                for (int r = 0; r < B; ++r)
#pragma unroll
                    for (int c = 0; c < B; ++c) acc[r] -= au[(q * BB + r * B + c) * capS] * m[c];
            }
            const T* fd = au + dim * BB * capS;
            T out[B];
#pragma unroll
            for (int r = 0; r < B; ++r) {
                T t = T(0);
#pragma unroll
                for (int c = 0; c < B; ++c) t += fd[(r * B + c) * capS] * acc[c];
                out[r] = t;
            }
            T* mine = ts.loc + (l & 1) * NT * PB + u * PB;
#pragma unroll
            for (int e = 0; e < B; ++e) mine[e] = out[e];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                if (q >= dim) break;
                if (tg[q] >= 0 && ps.ok && l > 0)
                    tilePush<T, B>(tg[q], out, mb0 + 8u * (l - 1), halo0, tm, hcap, ps);
            }
#pragma unroll
            for (int e = 0; e < B; ++e) y[i * B + e] = out[e];
        }
        __syncthreads();
    }
    tileSweepEnd<T, B, NT>(ts, ps);
}

template <class T, int B>
__device__ __forceinline__ void spmvRow(const KArgs<T>& a, const T* in, int i, T (&acc)[B])
{
    // all column indices first, then every gather and matrix load without a
    // branch in between (more loads in flight); a missing neighbour (column
    // -1) contributes zero through the selects, its block is never trusted
    const int ld = a.ldN, ns = a.nslot;
    int k[MAX_SLOTS];
#pragma unroll
    for (int s = 0; s < MAX_SLOTS; ++s) k[s] = s < ns ? __ldg(&a.col[s * ld + i]) : -1;
#pragma unroll
    for (int e = 0; e < B; ++e) acc[e] = T(0);
#pragma unroll
    for (int s = 0; s < MAX_SLOTS; ++s) {
        if (s >= ns) break;
        const bool has = k[s] >= 0;
        const int kk = has ? k[s] : 0;
        T xk[B];
#pragma unroll
        for (int e = 0; e < B; ++e) xk[e] = has ? ldcg(&in[kk * B + e]) : T(0);
#pragma unroll
        for (int r = 0; r < B; ++r)
#pragma unroll
            for (int c = 0; c < B; ++c) {
                const T av = a.A[(s * B * B + r * B + c) * ld + i];
                acc[r] += (has ? av : T(0)) * xk[c];
            }
    }
}

// The whole solve of one system by one team (a cluster, or the cooperative
// grid): optional ILU(0) factorization, then BiCGStab to the tolerance.
template <class T, int B, int MODE, int NT>
__device__ __forceinline__ void bicgstabBody(const KArgs<T>& a, const Team<MODE>& tm, unsigned long long* mbar,
                                             unsigned char* dynSmem)
{
    const int gt = tm.rank * blockDim.x + threadIdx.x, gs = tm.nblk * blockDim.x;
    const int N = a.N;
    PushState ps;
    ps.ok = 1;
    const PushSmem<T, B, NT> psm(dynSmem, a.numLev);
    const TileSmem<T, B, NT> tsm(dynSmem, a.numLev, a.thalo, a.twidth, a.dim);  // the same memory, tile layout
    T* const dep = psm.dep;
    ps.tph = 0;
    ps.sbuf = 0;
    // hybrid launch (grid of clusters): cluster 0 factorizes and sweeps, every
    // block of the grid shares SpMV, vector updates and reductions
    const bool sweeper = MODE == SYNC_CLUSTER || (a.hybrid && blockIdx.x < a.hybrid);
    if (MODE == SYNC_CLUSTER || a.hybrid) {
        const cg::cluster_group cl = cg::this_cluster();
        const int crank = (int)cl.block_rank(), csize = (int)cl.num_blocks();
        // the push tables and the hybrid split assume one cluster size; a launch
        // with another (the same in every block) reports an error and does nothing
        if (((a.dsmem || a.tile) && csize != a.cluster) ||
            (a.hybrid && (csize != a.hybrid || csize != a.gs.perCluster))) {
            if (crank == 0 && threadIdx.x == 0) a.st->code = GBFV_ERR_CUDA;
            return;
        }
        for (int k = 0; k < PUSH_BUFFERS; ++k) {
            ps.mb[k] = smemAddr(&mbar[k]);
            ps.ph[k] = 0;
        }
        ps.dep = smemAddr(dep);
        ps.lev = smemAddr(&mbar[PUSH_BUFFERS]);
        ps.levPh = 0;
        if (a.dsmem && sweeper) {
            for (int j = threadIdx.x; j <= a.numLev; j += NT) psm.lev[j] = a.levPtr[j];
            for (int j = threadIdx.x; j < 2 * a.numLev; j += NT) psm.nval[j] = a.levVals[crank * 2 * a.numLev + j];
        }
        if (a.dsmem && sweeper && threadIdx.x == 0) {
            // one arrival per phase (thread 0, carrying the expected bytes)
            for (int k = 0; k < PUSH_BUFFERS; ++k) mbarInit(ps.mb[k], 1);
            mbarInit(ps.lev, csize);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        if (a.tile && sweeper) {
            // this block's per-level table and one halo mbarrier per level
            for (int j = threadIdx.x; j < a.numLev; j += NT) {
                tsm.info[j] = a.tinfo[crank * a.numLev + j];
                mbarInit(smemAddr(&tsm.mb[j]), 1);
            }
            if (threadIdx.x == 0) {
                *tsm.bad = 0;
            }
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        cl.sync();
    }
    const double eps = 2.2250738585072014e-308 * 1e10;  // numeric_limits<double>::min()*1e10
    PhaseClock pc(a.prof, gt);
    if (a.factor) {
        if (MODE == SYNC_GRID && a.hybrid) {
            if (sweeper) {
                const Team<SYNC_CLUSTER> tc;
                phaseFactor<T, B, SYNC_CLUSTER>(a, tc);
            }
            if (!teamSync<MODE>(a.gs)) goto timeout;
        }
        else if (!phaseFactor<T, B, MODE>(a, tm))
            goto timeout;
        pc.tick(0);
        if (*(volatile int*)&a.st->code == GBFV_ERR_SINGULAR) goto done;
    }
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
        blockPartials<1, MODE>(mx, isMax1, a.partial, tm);
        if (!teamSync<MODE>(a.gs)) goto timeout;
        double tot[1];
        allCombine<1, MODE>(a.partial, isMax1, tot, tm);
        double resErr = fmax(tot[0], eps);
        const double initErr = resErr;
        auto converged = [&](double re) { return re / fmax(1e-20, initErr) <= a.redTol || re <= a.absTol; };
        if (converged(resErr)) {
            if (gt == 0) { a.st->converged = 1; a.st->iterations = 0; a.st->resid = resErr; a.st->resid0 = initErr; }
            goto done;
        }
        double rho = 1.0, alpha = 1.0, omega = 1.0;
        {
            // partials of the next reduction go to the second half of the buffer so the
            // combine above cannot race with them
            double dd[1] = {0.0};
            const bool isSum1[1] = {false};
            for (int i = gt; i < N; i += gs) {
                double t = 0.0;
#pragma unroll
                for (int e = 0; e < B; ++e) t += (double)(a.rhs[i * B + e] * a.rhs[i * B + e]);
                dd[0] += t;
            }
            blockPartials<1, MODE>(dd, isSum1, a.partial + 2 * tm.nblk, tm);
            if (!teamSync<MODE>(a.gs)) goto timeout;
        }
        int it = 0;
        int buf = 1;  // which half of the partial buffer holds (b, r)
        for (; it < a.maxIter; ++it) {
            double rho_i;
            {
                const bool isSum1[1] = {false};
                double tot1[1];
                allCombine<1, MODE>(a.partial + 2 * tm.nblk * buf, isSum1, tot1, tm);
                rho_i = tot1[0];
            }
            if (fabs(rho) <= eps || fabs(omega) <= eps) {
                if (gt == 0) a.st->code = GBFV_ERR_BREAKDOWN;
                break;
            }
            const double beta = (rho_i / rho) * (alpha / omega);
            rho = rho_i;
            pc.tick(5);
            if constexpr (MODE == SYNC_CLUSTER) {
                if (a.tile) {
                    sweepLowerTile<T, B, NT>(a, nullptr, a.y, true, (T)beta, (T)omega, tm, tsm, ps);
                    pc.tick(1);
                    sweepUpperTile<T, B, NT>(a, a.y, tm, tsm, ps);
                    pc.tick(2);
                }
                else if (a.dsmem) {
                    sweepLowerPush<T, B, NT>(a, nullptr, a.y, true, (T)beta, (T)omega, tm, dep, ps, psm);
                    pc.tick(1);
                    sweepUpperPush<T, B, NT>(a, a.y, tm, dep, ps, psm);
                    pc.tick(2);
                }
                else {
                    sweepLower<T, B, MODE>(a, nullptr, a.y, true, (T)beta, (T)omega, tm);
                    sweepUpper<T, B, MODE>(a, a.y, tm);
                }
            }
            else if (a.hybrid) {
                if (sweeper) {
                    const Team<SYNC_CLUSTER> tc;
                    if (a.tile) {
                        sweepLowerTile<T, B, NT>(a, nullptr, a.y, true, (T)beta, (T)omega, tc, tsm, ps);
                        sweepUpperTile<T, B, NT>(a, a.y, tc, tsm, ps);
                    }
                    else {
                        sweepLowerPush<T, B, NT>(a, nullptr, a.y, true, (T)beta, (T)omega, tc, dep, ps, psm);
                        sweepUpperPush<T, B, NT>(a, a.y, tc, dep, ps, psm);
                    }
                }
                if (!teamSync<MODE>(a.gs)) goto timeout;
            }
            else {
                if (!sweepLower<T, B, MODE>(a, nullptr, a.y, true, (T)beta, (T)omega, tm)) goto timeout;
                if (!sweepUpper<T, B, MODE>(a, a.y, tm)) goto timeout;
            }
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
                blockPartials<1, MODE>(dd, isSum1, a.partial + 2 * tm.nblk * buf, tm);
                if (!teamSync<MODE>(a.gs)) goto timeout;
                double tot1[1];
                allCombine<1, MODE>(a.partial + 2 * tm.nblk * buf, isSum1, tot1, tm);
                pc.tick(3);
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
                blockPartials<2, MODE>(red, kinds, a.partial + 2 * tm.nblk * buf, tm);
                if (!teamSync<MODE>(a.gs)) goto timeout;
                double tot2[2];
                allCombine<2, MODE>(a.partial + 2 * tm.nblk * buf, kinds, tot2, tm);
                resErr = tot2[0];
                const bool stag = tot2[1] == 0.0;
                if (converged(resErr)) {
                    if (gt == 0) a.st->converged = 1;
                    break;
                }
                if (stag || resErr > a.maxRes) break;
            }
            pc.tick(4);
            if constexpr (MODE == SYNC_CLUSTER) {
                if (a.tile) {
                    sweepLowerTile<T, B, NT>(a, a.r, a.z, false, T(0), T(0), tm, tsm, ps);
                    pc.tick(1);
                    sweepUpperTile<T, B, NT>(a, a.z, tm, tsm, ps);
                    pc.tick(2);
                }
                else if (a.dsmem) {
                    sweepLowerPush<T, B, NT>(a, a.r, a.z, false, T(0), T(0), tm, dep, ps, psm);
                    pc.tick(1);
                    sweepUpperPush<T, B, NT>(a, a.z, tm, dep, ps, psm);
                    pc.tick(2);
                }
                else {
                    sweepLower<T, B, MODE>(a, a.r, a.z, false, T(0), T(0), tm);
                    sweepUpper<T, B, MODE>(a, a.z, tm);
                }
            }
            else if (a.hybrid) {
                if (sweeper) {
                    const Team<SYNC_CLUSTER> tc;
                    if (a.tile) {
                        sweepLowerTile<T, B, NT>(a, a.r, a.z, false, T(0), T(0), tc, tsm, ps);
                        sweepUpperTile<T, B, NT>(a, a.z, tc, tsm, ps);
                    }
                    else {
                        sweepLowerPush<T, B, NT>(a, a.r, a.z, false, T(0), T(0), tc, dep, ps, psm);
                        sweepUpperPush<T, B, NT>(a, a.z, tc, dep, ps, psm);
                    }
                }
                if (!teamSync<MODE>(a.gs)) goto timeout;
            }
            else {
                if (!sweepLower<T, B, MODE>(a, a.r, a.z, false, T(0), T(0), tm)) goto timeout;
                if (!sweepUpper<T, B, MODE>(a, a.z, tm)) goto timeout;
            }
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
                blockPartials<2, MODE>(dd, isSum2, a.partial + 2 * tm.nblk * buf, tm);
                if (!teamSync<MODE>(a.gs)) goto timeout;
                double tot2[2];
                allCombine<2, MODE>(a.partial + 2 * tm.nblk * buf, isSum2, tot2, tm);
                pc.tick(3);
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
                blockPartials<2, MODE>(red, kinds, a.partial + 2 * tm.nblk * buf, tm);
                if (!teamSync<MODE>(a.gs)) goto timeout;
                // z == 0 everywhere is stagnation (the residual of this check is still s)
                const bool kindMax[2] = {false, true};
                double tot2[2];
                allCombine<2, MODE>(a.partial + 2 * tm.nblk * buf, kindMax, tot2, tm);
                if (tot2[1] == 0.0) break;
            }
        }
        if (gt == 0) {
            a.st->iterations = it;
            a.st->resid = resErr;
            a.st->resid0 = initErr;
        }
        if (!ps.ok) atomicExch(&a.st->code, GBFV_ERR_TIMEOUT);
    }
done:
    return;
timeout:
    if (gt == 0) a.st->code = GBFV_ERR_TIMEOUT;
}

// one linear solve in one launch: Dune::SeqILU<...,0> set-up
// (istlpreconditionerwrappers.hh:151-190) and BiCGStabSolver::apply
// (bicgstabsolver.hh:120-330) with CombinedCriterion (combinedcriterion.hh:116-144)
template <class T, int B, int MODE, int NT>
__global__ void __launch_bounds__(NT, 1) kBicgstab(KArgs<T> a)
{
    __shared__ __align__(8) unsigned long long mbar[PUSH_BUFFERS + 1];
    extern __shared__ __align__(16) unsigned char dynSmem[];
    const Team<MODE> tm;
    bicgstabBody<T, B, MODE, NT>(a, tm, mbar, dynSmem);
}

// Batched solve: every cluster of the grid takes systems from a work queue
// (order[0..count), largest first) and solves each with the same body as the
// single-system kernel, so a system's result does not depend on the batch.
template <class T, int B, int NT>
__global__ void __launch_bounds__(NT, 1) kBicgstabBatch(const KArgs<T>* __restrict__ args,
                                                        const int* __restrict__ order, const int* count, int* queue)
{
    __shared__ __align__(8) unsigned long long mbar[PUSH_BUFFERS + 1];
    __shared__ int sNext;
    extern __shared__ __align__(16) unsigned char dynSmem[];
    cg::cluster_group cl = cg::this_cluster();
    const Team<SYNC_CLUSTER> tm;
    for (;;) {
        if (tm.rank == 0 && threadIdx.x == 0) sNext = atomicAdd(queue, 1);
        cl.sync();
        const int q = *cl.map_shared_rank(&sNext, 0);
        cl.sync();  // every block has read the index before block 0 takes the next one
        if (q >= *count) break;
        const KArgs<T> a = args[order[q]];
        bicgstabBody<T, B, SYNC_CLUSTER, NT>(a, tm, mbar, dynSmem);
        cl.sync();
        if (a.dsmem && threadIdx.x == 0)
            for (int k = 0; k < PUSH_BUFFERS + 1; ++k)
                asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smemAddr(&mbar[k])) : "memory");
        cl.sync();
    }
}

// ------------------------------------------------ bounded-wait self-test --
// One block waits, with the sweeps' bounded wait, on an mbarrier phase that
// nothing completes; the wait gives up and the kernel reports
// GBFV_ERR_TIMEOUT, as a solve whose data never arrives would.
__global__ void kWaitTimeoutProbe(DevStatus* st)
{
    __shared__ __align__(8) unsigned long long mb;
    if (threadIdx.x == 0) mbarInit(smemAddr(&mb), 1);
    __syncthreads();
    const bool ok = mbarWait(smemAddr(&mb), 0u);
    __syncthreads();
    if (threadIdx.x == 0) {
        st->code = ok ? GBFV_OK : GBFV_ERR_TIMEOUT;
        st->iterations = 1;
    }
}

void launchWaitTimeoutProbe(DevStatus* st, cudaStream_t s)
{
    kWaitTimeoutProbe<<<1, 32, 0, s>>>(st);
    countLaunch();
}

// ------------------------------------------------- launch + FP64 helpers --
template <class T, int B, int MODE, int NT>
static int launchOne(const KArgs<T>& a, int nblocks, cudaStream_t s)
{
    void* args[] = {(void*)&a};
    cudaError_t e;
    auto fn = kBicgstab<T, B, MODE, NT>;
    if (MODE == SYNC_GRID) {
        e = cudaLaunchCooperativeKernel((void*)fn, nblocks, NT, args, 0, s);
    }
    else {
        static bool attrSet = false;
        if (!attrSet) {
            cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
            cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)PushSmem<T, B, NT>::bytes(MAX_PUSH_LEVELS));
            attrSet = true;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(nblocks, 1, 1);
        cfg.blockDim = dim3(NT, 1, 1);
        cfg.dynamicSmemBytes = a.tile    ? TileSmem<T, B, NT>::bytes(a.numLev, a.thalo, a.twidth, a.dim)
                               : a.dsmem ? PushSmem<T, B, NT>::bytes(a.numLev)
                                         : 0;
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = nblocks;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        e = cudaLaunchKernelEx(&cfg, fn, a);
    }
    countLaunch();
    return e == cudaSuccess ? GBFV_OK : GBFV_ERR_CUDA;
}

// hybrid: the grid kernel over nblocks blocks in clusters of HYBRID_CLUSTER,
// cooperative (every block resident, for the software grid barrier)
template <class T, int B, int NT>
static int launchHybrid(const KArgs<T>& a, int nblocks, cudaStream_t s)
{
    auto fn = kBicgstab<T, B, SYNC_GRID, NT>;
    static bool attrSet = false;
    if (!attrSet) {
        cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)PushSmem<T, B, NT>::bytes(MAX_PUSH_LEVELS));
        attrSet = true;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nblocks, 1, 1);
    cfg.blockDim = dim3(NT, 1, 1);
    cfg.dynamicSmemBytes = a.tile    ? TileSmem<T, B, NT>::bytes(a.numLev, a.thalo, a.twidth, a.dim)
                           : a.dsmem ? PushSmem<T, B, NT>::bytes(a.numLev)
                                     : 0;
    cfg.stream = s;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = HYBRID_CLUSTER;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    at[1].id = cudaLaunchAttributeCooperative;
    at[1].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 2;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, fn, a);
    countLaunch();
    return e == cudaSuccess ? GBFV_OK : GBFV_ERR_CUDA;
}

// how many blocks a hybrid launch may have (whole clusters that are resident at once)
template <class T, int NT>
static int maxHybridBlocksNT(int b)
{
    const void* fn = b == 2 ? (const void*)kBicgstab<T, 2, SYNC_GRID, NT> : (const void*)kBicgstab<T, 3, SYNC_GRID, NT>;
    const size_t dyn = b == 2 ? PushSmem<T, 2, NT>::bytes(MAX_PUSH_LEVELS) : PushSmem<T, 3, NT>::bytes(MAX_PUSH_LEVELS);
    cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(NT, 1, 1);
    cfg.gridDim = dim3(HYBRID_CLUSTER, 1, 1);
    cfg.dynamicSmemBytes = dyn;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = HYBRID_CLUSTER;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, fn, &cfg) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    return n * HYBRID_CLUSTER;
}

template <class T>
int maxHybridBlocks(int b, bool narrow)
{
    return narrow ? maxHybridBlocksNT<T, SOLVER_THREADS>(b) : maxHybridBlocksNT<T, clusterThreads<T>()>(b);
}

template <class T>
int launchBicgstab(const KArgs<T>& a, int b, int mode, int nblocks, cudaStream_t s)
{
    constexpr int NTC = clusterThreads<T>();
    const bool narrow = (mode & SYNC_NARROW) != 0;
    mode &= ~SYNC_NARROW;
    if (mode == SYNC_HYBRID && narrow)
        return b == 2 ? launchHybrid<T, 2, SOLVER_THREADS>(a, nblocks, s)
                      : launchHybrid<T, 3, SOLVER_THREADS>(a, nblocks, s);
    if (mode == SYNC_HYBRID)
        return b == 2 ? launchHybrid<T, 2, NTC>(a, nblocks, s) : launchHybrid<T, 3, NTC>(a, nblocks, s);
    if (mode == SYNC_GRID)
        return b == 2 ? launchOne<T, 2, SYNC_GRID, SOLVER_THREADS>(a, nblocks, s)
                      : launchOne<T, 3, SYNC_GRID, SOLVER_THREADS>(a, nblocks, s);
    return b == 2 ? launchOne<T, 2, SYNC_CLUSTER, NTC>(a, nblocks, s)
                  : launchOne<T, 3, SYNC_CLUSTER, NTC>(a, nblocks, s);
}

template <class T, int B>
static int launchBatchB(const KArgs<T>* args, const int* order, const int* count, int* queue, int clusterSize,
                        int numClusters, int maxLev, cudaStream_t s)
{
    constexpr int NT = clusterThreads<T>();
    auto fn = kBicgstabBatch<T, B, NT>;
    static bool attrSet = false;
    if (!attrSet) {
        cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)PushSmem<T, B, NT>::bytes(MAX_PUSH_LEVELS));
        attrSet = true;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(clusterSize * numClusters, 1, 1);
    cfg.blockDim = dim3(NT, 1, 1);
    cfg.dynamicSmemBytes = PushSmem<T, B, NT>::bytes(maxLev);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = clusterSize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, fn, args, order, count, queue);
    countLaunch();
    return e == cudaSuccess ? GBFV_OK : GBFV_ERR_CUDA;
}

template <class T>
int launchBicgstabBatch(const KArgs<T>* args, const int* order, const int* count, int* queue, int b,
                        int clusterSize, int numClusters, int maxLev, cudaStream_t s)
{
    return b == 2 ? launchBatchB<T, 2>(args, order, count, queue, clusterSize, numClusters, maxLev, s)
                  : launchBatchB<T, 3>(args, order, count, queue, clusterSize, numClusters, maxLev, s);
}

// how many clusters of the given size fit on the device at once
template <class T>
int maxActiveClusters(int b, int clusterSize)
{
    constexpr int NT = clusterThreads<T>();
    const void* fn = b == 2 ? (const void*)kBicgstabBatch<T, 2, NT> : (const void*)kBicgstabBatch<T, 3, NT>;
    const size_t dyn = b == 2 ? PushSmem<T, 2, NT>::bytes(MAX_PUSH_LEVELS) : PushSmem<T, 3, NT>::bytes(MAX_PUSH_LEVELS);
    cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(NT, 1, 1);
    cfg.gridDim = dim3(clusterSize, 1, 1);
    cfg.dynamicSmemBytes = dyn;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = clusterSize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, fn, &cfg) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    return n;
}

template <class T>
int maxSolverBlocks(int b)
{
    int dev = 0, nsm = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (b == 2)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kBicgstab<T, 2, SYNC_GRID, SOLVER_THREADS>,
                                                      SOLVER_THREADS, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kBicgstab<T, 3, SYNC_GRID, SOLVER_THREADS>,
                                                      SOLVER_THREADS, 0);
    return nsm * (occ > 0 ? occ : 1);
}

template <class T>
int maxClusterBlocks(int b)
{
    constexpr int NTC = clusterThreads<T>();
    int n = 0;
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(NTC, 1, 1);
    cfg.gridDim = dim3(16, 1, 1);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 16;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const void* fn = b == 2 ? (const void*)kBicgstab<T, 2, SYNC_CLUSTER, NTC>
                            : (const void*)kBicgstab<T, 3, SYNC_CLUSTER, NTC>;
    const size_t dyn = b == 2 ? PushSmem<T, 2, NTC>::bytes(MAX_PUSH_LEVELS) : PushSmem<T, 3, NTC>::bytes(MAX_PUSH_LEVELS);
    cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    cfg.dynamicSmemBytes = dyn;
    if (cudaOccupancyMaxPotentialClusterSize(&n, fn, &cfg) != cudaSuccess) {
        cudaGetLastError();
        n = 8;
    }
    return n > 0 ? n : 1;
}

template <class T>
size_t tileSmemBytes(int b, int numLev, int haloSlots, int width, int dim)
{
    constexpr int NT = clusterThreads<T>();
    return b == 2 ? TileSmem<T, 2, NT>::bytes(numLev, haloSlots, width, dim)
                  : TileSmem<T, 3, NT>::bytes(numLev, haloSlots, width, dim);
}

template <class T>
size_t solverSmemLimit(int b)
{
    constexpr int NT = clusterThreads<T>();
    return b == 2 ? PushSmem<T, 2, NT>::bytes(MAX_PUSH_LEVELS) : PushSmem<T, 3, NT>::bytes(MAX_PUSH_LEVELS);
}

template size_t tileSmemBytes<double>(int, int, int, int, int);
template size_t tileSmemBytes<float>(int, int, int, int, int);
template size_t solverSmemLimit<double>(int);
template size_t solverSmemLimit<float>(int);
template int launchBicgstab<double>(const KArgs<double>&, int, int, int, cudaStream_t);
template int launchBicgstab<float>(const KArgs<float>&, int, int, int, cudaStream_t);
template int maxSolverBlocks<double>(int);
template int maxSolverBlocks<float>(int);
template int maxClusterBlocks<double>(int);
template int maxClusterBlocks<float>(int);
template int maxHybridBlocks<double>(int, bool);
template int maxHybridBlocks<float>(int, bool);
template int launchBicgstabBatch<double>(const KArgs<double>*, const int*, const int*, int*, int, int, int, int,
                                         cudaStream_t);
template int launchBicgstabBatch<float>(const KArgs<float>*, const int*, const int*, int*, int, int, int, int,
                                        cudaStream_t);
template int maxActiveClusters<double>(int, int);
template int maxActiveClusters<float>(int, int);

// A32 = (float) A64 over all slots: ParallelBaseBackend::setMatrix's copy of
// the Jacobian into the solver's own matrix (parallelbasebackend.hh:241-250),
// in the mixed form's FP32 solver scalar
__global__ void kCastMatrix(const double* __restrict__ src, float* __restrict__ dst, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

void launchCastMatrix(const double* src, float* dst, long n, cudaStream_t s)
{
    int nb = (int)((n + 255) / 256);
    if (nb > 4096) nb = 4096;
    kCastMatrix<<<nb, 256, 0, s>>>(src, dst, n);
    countLaunch();
}

// x64 += d32: a step of the mixed form's outer iterative refinement (this
// project's; the reference solves in one precision)
__global__ void kAccumulate(int n, double* __restrict__ x, const float* __restrict__ d)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] += (double)d[i];
}

void launchAccumulate(int n, double* x, const float* d, cudaStream_t s)
{
    int nb = (n + 255) / 256;
    if (nb > 4096) nb = 4096;
    kAccumulate<<<nb, 256, 0, s>>>(n, x, d);
    countLaunch();
}

// FP64 true residual of the refinement: r = b - A x, r32 = (float) r,
// max|r| into st->resid (as ordered bits in errorBits)
template <int B>
__device__ __forceinline__ double residual64Row(int i, int ld, int nslot, const int* __restrict__ col,
                                                const double* __restrict__ A, const double* __restrict__ b,
                                                const double* __restrict__ x, double* __restrict__ r,
                                                float* __restrict__ r32, double mx)
{
    double acc[B];
#pragma unroll
    for (int e = 0; e < B; ++e) acc[e] = 0.0;
    for (int s = 0; s < nslot; ++s) {
        const int k = col[s * ld + i];
        if (k < 0) continue;
#pragma unroll
        for (int rr = 0; rr < B; ++rr)
#pragma unroll
            for (int c = 0; c < B; ++c) acc[rr] += A[(s * B * B + rr * B + c) * ld + i] * x[k * B + c];
    }
#pragma unroll
    for (int e = 0; e < B; ++e) {
        const double ri = b[i * B + e] - acc[e];
        r[i * B + e] = ri;
        r32[i * B + e] = (float)ri;
        mx = fmax(mx, fabs(ri));
    }
    return mx;
}

__device__ __forceinline__ void warpMaxToStatus(double mx, DevStatus* st)
{
    unsigned long long bits = __double_as_longlong(mx);
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ob = __shfl_down_sync(0xffffffffu, bits, o);
        bits = ob > bits ? ob : bits;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(&st->errorBits, bits);
}

// FP64 true residual b - A x of the outer refinement, with the max-norm the
// refinement's stop test uses (the same norm as CombinedCriterion's,
// combinedcriterion.hh:116-144)
template <int B>
__global__ void kResidual64(int N, int ld, int nslot, const int* __restrict__ col,
                            const double* __restrict__ A, const double* __restrict__ b,
                            const double* __restrict__ x, double* __restrict__ r,
                            float* __restrict__ r32, DevStatus* st)
{
    double mx = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
        mx = residual64Row<B>(i, ld, nslot, col, A, b, x, r, r32, mx);
    warpMaxToStatus(mx, st);
}

void launchResidual64(int N, int ld, int nslot, int b, const int* col, const double* A, const double* rhs,
                      const double* x, double* r, float* r32, DevStatus* st, cudaStream_t s)
{
    int nb = (N + 255) / 256;
    if (nb > 2048) nb = 2048;
    if (b == 2)
        kResidual64<2><<<nb, 256, 0, s>>>(N, ld, nslot, col, A, rhs, x, r, r32, st);
    else
        kResidual64<3><<<nb, 256, 0, s>>>(N, ld, nslot, col, A, rhs, x, r, r32, st);
    countLaunch();
}

// ------------------------------------------- batched refinement helpers --
// Grid (gx, K): blockIdx.y is the system, blocks of a system stride over its
// rows; systems with active[k] == 0 are skipped.
__global__ void kBatchCast(const SolveJob* __restrict__ jobs, const int* __restrict__ active)
{
    const SolveJob& j = jobs[blockIdx.y];
    if (!active[blockIdx.y]) return;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < j.nval; i += (long)gridDim.x * blockDim.x)
        j.A32[i] = (float)j.A64[i];
}

__global__ void kBatchZeroX(const SolveJob* __restrict__ jobs, const int* __restrict__ active)
{
    const SolveJob& j = jobs[blockIdx.y];
    if (!active[blockIdx.y]) return;
    const int n = j.N * j.b;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) j.xref[i] = 0.0;
}

__global__ void kBatchAccumulate(const SolveJob* __restrict__ jobs, const int* __restrict__ active)
{
    const SolveJob& j = jobs[blockIdx.y];
    if (!active[blockIdx.y]) return;
    const int n = j.N * j.b;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        j.xref[i] += (double)j.dx32[i];
}

template <int B>
__global__ void kBatchResidual64(const SolveJob* __restrict__ jobs, const int* __restrict__ active)
{
    const SolveJob& j = jobs[blockIdx.y];
    if (!active[blockIdx.y] || j.b != B) return;
    double mx = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < j.N; i += gridDim.x * blockDim.x)
        mx = residual64Row<B>(i, j.ld, j.nslot, j.col, j.A64, j.rhs, j.xref, j.rref, j.r32, mx);
    warpMaxToStatus(mx, j.st);
}

void launchBatchCast(const SolveJob* jobs, const int* active, int K, int gx, cudaStream_t s)
{
    kBatchCast<<<dim3(gx, K), 256, 0, s>>>(jobs, active);
    countLaunch();
}
void launchBatchZeroX(const SolveJob* jobs, const int* active, int K, int gx, cudaStream_t s)
{
    kBatchZeroX<<<dim3(gx, K), 256, 0, s>>>(jobs, active);
    countLaunch();
}
void launchBatchAccumulate(const SolveJob* jobs, const int* active, int K, int gx, cudaStream_t s)
{
    kBatchAccumulate<<<dim3(gx, K), 256, 0, s>>>(jobs, active);
    countLaunch();
}
void launchBatchResidual64(const SolveJob* jobs, const int* active, int K, int gx, int b, cudaStream_t s)
{
    if (b == 2) kBatchResidual64<2><<<dim3(gx, K), 256, 0, s>>>(jobs, active);
    else kBatchResidual64<3><<<dim3(gx, K), 256, 0, s>>>(jobs, active);
    countLaunch();
}

}  // namespace gbfv
