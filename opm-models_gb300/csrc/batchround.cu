// Device-side decisions of a batched Newton round.
//
// A round of a batch advances every active system by one Newton iteration:
// linearize, Newton error, (mixed precision: FP64 residual, refinement
// rounds of FP32 BiCGStab), update guard, Newton update.  Between those
// phases each system takes the decisions gbfv_newton_apply and solveMixed
// take on the host for a single system -- the proceed rule of
// NewtonMethod::proceed_ (newtonmethod.hh:788-806), the maximum-error check
// of preSolve_ (:600-606), the refinement loop's convergence, divergence and
// stagnation rules, the inner tolerance of the next FP32 solve -- here made
// by one thread per system in small single-block kernels, so the whole round
// is one captured CUDA graph with no host decision inside it.  The time-step
// bookkeeping (step completed, dt halving after a failure, the next dt) stays
// on the host between rounds.
//
// This unit is compiled with -fmad=false: the decisions' double arithmetic
// (inner tolerance, convergence ratios) is the host's, operation for
// operation, so a system's result stays bit-identical to its run alone.
#include <cuda_runtime.h>

#include "../../include/gbfv.h"
#include "gbfv_internal.cuh"
#include "solver.cuh"

namespace gbfv {

namespace {

constexpr int ROUND_THREADS = 256;

__device__ __forceinline__ double bitsToDouble(unsigned long long b) { return __longlong_as_double((long long)b); }

__device__ __forceinline__ void clearStatus(DevStatus& s)
{
    s.code = 0;
    s.where = 0;
    s.iterations = 0;
    s.converged = 0;
    s.refinements = 0;
    s.nonfinite = 0;
    s.switched = 0;
    s.pad = 0;
    s.errorBits = 0ull;
    s.resid = 0.0;
    s.resid0 = 0.0;
}

__device__ __forceinline__ void failSys(RoundSys& y, int status)
{
    y.phase = RS_FAIL;
    y.status = status;
    y.kry = 0;
}

// NewtonMethod::proceed_ (newtonmethod.hh:788-806)
__device__ __forceinline__ bool proceed(const RoundSys& y, const RoundParams& p)
{
    if (y.numIterations < 1) return true;
    if (y.error <= p.newtonTol) return false;
    if (y.numIterations >= p.newtonMaxIt) return y.error * 4.0 < y.lastError;
    return true;
}

// the Newton loop has ended: converged or not (the tail of gbfv_newton_apply)
__device__ __forceinline__ void newtonEnd(RoundSys& y, const RoundParams& p)
{
    if (y.error <= p.newtonTol) y.phase = RS_END_OK;
    else failSys(y, GBFV_ERR_NOT_CONVERGED);
}

// mixed precision: the inner tolerance of the next FP32 solve (solveMixed)
__device__ __forceinline__ double innerTolerance(const RoundSys& y, const RoundParams& p)
{
    const double target = fmax(p.linTol * y.resErr0, p.absTol);
    const double need = target / y.resErr;
    return fmin(0.5, fmax(0.5 * need, p.innerTol));
}

// the Krylov queue: systems with kry set, largest first (stable by index),
// as the host's stable_sort by cell count orders them
__device__ void buildOrder(const RoundSys* __restrict__ ys, const SolveJob* __restrict__ sj, int K, int* order,
                           int* queue)
{
    __shared__ int sCount;
    if (threadIdx.x == 0) sCount = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < K; i += blockDim.x) {
        if (!ys[i].kry) continue;
        int rank = 0;
        for (int j = 0; j < K; ++j)
            if (ys[j].kry && (sj[j].N > sj[i].N || (sj[j].N == sj[i].N && j < i))) ++rank;
        order[rank] = i;
        atomicAdd(&sCount, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        order[K] = sCount;
        *queue = 0;
    }
}

// system i takes part in the next Krylov launch, with this reduction target
// and (first launch of a solve) the ILU(0) factorization
template <class T>
__device__ __forceinline__ void armKrylov(RoundSys& y, KArgs<T>* ka, int i, double redTol, int factor)
{
    y.kry = 1;
    y.factorNext = factor;
    ka[i].redTol = redTol;
    ka[i].factor = factor;
}

// ------------------------------------------------------------ kernels -----
// start of the round: which systems linearize, their dt and storage flag
__global__ void __launch_bounds__(ROUND_THREADS) kRoundBegin(RoundSys* ys, JobState* js, DevStatus* st, int K)
{
    for (int i = threadIdx.x; i < K; i += blockDim.x) {
        RoundSys& y = ys[i];
        const int act = y.phase == RS_LIN;
        js[i].active = act;
        js[i].dt = y.dt;
        js[i].iter0 = y.numIterations == 0;
        if (act) y.lastError = y.error;
        y.kry = 0;
        y.kryLaunches = y.kryFactors = y.kryIters = 0;
        clearStatus(st[i]);
    }
}

// after the linearization and the Newton error (batchRound's first block)
template <class T>
__global__ void __launch_bounds__(ROUND_THREADS)
    kRoundAfterLin(RoundSys* ys, const JobState* js, DevStatus* st, int* act, KArgs<T>* ka, const SolveJob* sj,
                   int* order, int* queue, RoundParams p, int K)
{
    for (int i = threadIdx.x; i < K; i += blockDim.x) {
        RoundSys& y = ys[i];
        act[i] = 0;
        if (js[i].active) {
            y.linearizations++;
            const DevStatus& h = st[i];
            y.error = bitsToDouble(h.errorBits);
            if (h.nonfinite) failSys(y, GBFV_ERR_NONFINITE);
            else if (y.error > p.newtonMaxError) failSys(y, GBFV_ERR_NUMERICAL);
            else if (!proceed(y, p)) {
                y.numIterations++;
                newtonEnd(y, p);
            }
            else y.phase = RS_SOLVE;
        }
        if (y.phase == RS_SOLVE) {
            if (p.mixed) act[i] = 1;  // FP32 matrix, x = 0, FP64 residual first
            else
                armKrylov(y, ka, i, p.linTol, 1);  // plain FP64: one launch to the linear tolerance
        }
        clearStatus(st[i]);
    }
    __syncthreads();
    if (!p.mixed) buildOrder(ys, sj, K, order, queue);
}

// mixed: after r = b - A*0 (solveMixed's first residual)
__global__ void __launch_bounds__(ROUND_THREADS)
    kRoundAfterRes0(RoundSys* ys, DevStatus* st, int* act, KArgs<float>* ka, const SolveJob* sj, int* order,
                    int* queue, RoundParams p, int K)
{
    const double eps = 2.2250738585072014e-308 * 1e10;  // numeric_limits<double>::min() * 1e10
    for (int i = threadIdx.x; i < K; i += blockDim.x) {
        RoundSys& y = ys[i];
        if (act[i]) {
            y.resErr = fmax(bitsToDouble(st[i].errorBits), eps);
            y.resErr0 = y.resErr;
            y.refs = 0;
            if (y.resErr / fmax(1e-20, y.resErr0) <= p.linTol || y.resErr <= p.absTol) y.phase = RS_UPDATE;
            else
                armKrylov(y, ka, i, innerTolerance(y, p), 1);
        }
        act[i] = 0;
        clearStatus(st[i]);
    }
    __syncthreads();
    buildOrder(ys, sj, K, order, queue);
}

// after a Krylov launch: iterations and the launch's status per system
__global__ void __launch_bounds__(ROUND_THREADS)
    kRoundAfterKrylov(RoundSys* ys, DevStatus* st, int* act, RoundParams p, int K)
{
    for (int i = threadIdx.x; i < K; i += blockDim.x) {
        RoundSys& y = ys[i];
        act[i] = 0;
        if (y.kry) {
            const DevStatus& h = st[i];
            y.kryLaunches++;
            y.kryFactors += y.factorNext;
            y.kryIters += h.iterations;
            y.lastIt = h.iterations;
            y.linItStep += h.iterations;
            y.refs++;
            y.lastKs = h.code ? h.code : (h.converged ? GBFV_OK : GBFV_ERR_NOT_CONVERGED);
            y.kry = 0;
            if (!p.mixed) {
                if (y.lastKs != GBFV_OK) failSys(y, y.lastKs);
                else y.phase = RS_UPDATE;
            }
            else if (y.lastKs != GBFV_OK && y.lastKs != GBFV_ERR_NOT_CONVERGED)
                failSys(y, y.lastKs);
            else
                act[i] = 1;  // accumulate the inner solution, new FP64 residual
        }
        clearStatus(st[i]);
    }
}

// mixed: after x += dx and the new FP64 residual -- converged, failed, or the
// next refinement with its inner tolerance (the loop of solveMixed)
__global__ void __launch_bounds__(ROUND_THREADS)
    kRoundAfterRefine(RoundSys* ys, DevStatus* st, int* act, KArgs<float>* ka, const SolveJob* sj, int* order,
                      int* queue, RoundParams p, int K, int lastRefinement)
{
    for (int i = threadIdx.x; i < K; i += blockDim.x) {
        RoundSys& y = ys[i];
        if (act[i]) {
            y.resErr = bitsToDouble(st[i].errorBits);
            if (!isfinite(y.resErr)) failSys(y, GBFV_ERR_NONFINITE);
            else if (y.resErr / fmax(1e-20, y.resErr0) <= p.linTol || y.resErr <= p.absTol) y.phase = RS_UPDATE;
            else if (y.resErr > p.linMaxError * y.resErr0) failSys(y, GBFV_ERR_NOT_CONVERGED);
            else if (y.lastKs == GBFV_ERR_NOT_CONVERGED && y.lastIt >= p.linMaxIt)
                failSys(y, GBFV_ERR_NOT_CONVERGED);
            else if (lastRefinement)
                failSys(y, GBFV_ERR_NOT_CONVERGED);
            else
                armKrylov(y, ka, i, innerTolerance(y, p), 0);
        }
        act[i] = 0;
        clearStatus(st[i]);
    }
    __syncthreads();
    buildOrder(ys, sj, K, order, queue);
}

// before the update guard: the systems whose solve succeeded
__global__ void __launch_bounds__(ROUND_THREADS) kRoundBeforeCheck(RoundSys* ys, JobState* js, DevStatus* st, int K)
{
    for (int i = threadIdx.x; i < K; i += blockDim.x) {
        js[i].active = ys[i].phase == RS_UPDATE;
        clearStatus(st[i]);
    }
}

// after the update guard: a non-finite update fails the step
__global__ void __launch_bounds__(ROUND_THREADS) kRoundAfterCheck(RoundSys* ys, JobState* js, DevStatus* st, int K)
{
    for (int i = threadIdx.x; i < K; i += blockDim.x) {
        if (js[i].active && st[i].nonfinite) {
            js[i].active = 0;
            failSys(ys[i], GBFV_ERR_NONFINITE);
        }
        clearStatus(st[i]);
    }
}

// after the Newton update: another iteration or the end of the Newton loop
__global__ void __launch_bounds__(ROUND_THREADS)
    kRoundAfterUpdate(RoundSys* ys, const JobState* js, RoundParams p, int K)
{
    for (int i = threadIdx.x; i < K; i += blockDim.x) {
        RoundSys& y = ys[i];
        if (!js[i].active) continue;
        y.numIterations++;
        if (proceed(y, p)) y.phase = RS_LIN;
        else newtonEnd(y, p);
    }
}

// end of the round: a completed step advances the time level (solution(1)
// = solution(0)); a failed attempt goes back to it (updateFailed,
// fvbasediscretization.hh:1362-1367, and the retry of gbfv_time_integration)
__global__ void __launch_bounds__(256) kRoundTimeLevel(const RoundSys* __restrict__ ys, const LinJob* __restrict__ jobs)
{
    const int i = blockIdx.y;
    const int ph = ys[i].phase;
    if (ph != RS_END_OK && ph != RS_FAIL) return;
    const LinJob& j = jobs[i];
    const int n = j.m.N * j.m.b;
    const bool advance = ph == RS_END_OK;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        if (advance) j.xOld[q] = j.x[q];
        else j.x[q] = j.xOld[q];
    }
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < j.m.N; q += gridDim.x * blockDim.x) {
        if (advance) j.meaningOld[q] = j.meaning[q];
        else j.meaning[q] = j.meaningOld[q];
    }
}

}  // namespace

void launchRoundBegin(RoundSys* ys, JobState* js, DevStatus* st, int K, cudaStream_t s)
{
    kRoundBegin<<<1, ROUND_THREADS, 0, s>>>(ys, js, st, K);
    countLaunch();
}

void launchRoundAfterLin(RoundSys* ys, const JobState* js, DevStatus* st, int* act, KArgs<float>* ka32,
                         KArgs<double>* ka64, const SolveJob* sj, int* order, int* queue, const RoundParams& p, int K,
                         cudaStream_t s)
{
    if (p.mixed)
        kRoundAfterLin<float><<<1, ROUND_THREADS, 0, s>>>(ys, js, st, act, ka32, sj, order, queue, p, K);
    else
        kRoundAfterLin<double><<<1, ROUND_THREADS, 0, s>>>(ys, js, st, act, ka64, sj, order, queue, p, K);
    countLaunch();
}

void launchRoundAfterRes0(RoundSys* ys, DevStatus* st, int* act, KArgs<float>* ka, const SolveJob* sj, int* order,
                          int* queue, const RoundParams& p, int K, cudaStream_t s)
{
    kRoundAfterRes0<<<1, ROUND_THREADS, 0, s>>>(ys, st, act, ka, sj, order, queue, p, K);
    countLaunch();
}

void launchRoundAfterKrylov(RoundSys* ys, DevStatus* st, int* act, const RoundParams& p, int K, cudaStream_t s)
{
    kRoundAfterKrylov<<<1, ROUND_THREADS, 0, s>>>(ys, st, act, p, K);
    countLaunch();
}

void launchRoundAfterRefine(RoundSys* ys, DevStatus* st, int* act, KArgs<float>* ka, const SolveJob* sj, int* order,
                            int* queue, const RoundParams& p, int K, int lastRefinement, cudaStream_t s)
{
    kRoundAfterRefine<<<1, ROUND_THREADS, 0, s>>>(ys, st, act, ka, sj, order, queue, p, K, lastRefinement);
    countLaunch();
}

void launchRoundBeforeCheck(RoundSys* ys, JobState* js, DevStatus* st, int K, cudaStream_t s)
{
    kRoundBeforeCheck<<<1, ROUND_THREADS, 0, s>>>(ys, js, st, K);
    countLaunch();
}

void launchRoundAfterCheck(RoundSys* ys, JobState* js, DevStatus* st, int K, cudaStream_t s)
{
    kRoundAfterCheck<<<1, ROUND_THREADS, 0, s>>>(ys, js, st, K);
    countLaunch();
}

void launchRoundAfterUpdate(RoundSys* ys, const JobState* js, const RoundParams& p, int K, cudaStream_t s)
{
    kRoundAfterUpdate<<<1, ROUND_THREADS, 0, s>>>(ys, js, p, K);
    countLaunch();
}

void launchRoundTimeLevel(const RoundSys* ys, const LinJob* jobs, int K, int gx, cudaStream_t s)
{
    kRoundTimeLevel<<<dim3(gx, K), 256, 0, s>>>(ys, jobs);
    countLaunch();
}

}  // namespace gbfv
