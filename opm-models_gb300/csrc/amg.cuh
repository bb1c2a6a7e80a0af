// Algebraic multigrid preconditioner for BiCGStab (the reference's
// ParallelAmgBackend, parallelamgbackend.hh:85-330): host interface.
#pragma once

#include <cuda_runtime.h>

#include "gbfv_internal.cuh"

namespace gbfv {

constexpr int AMG_MAX_LEVELS = 15;   // CoarsenCriterion(maxLevel = 15)
constexpr int AMG_MAX_COLORS = 64;   // colours of one level's sweep order

// The system matrix as the ILU(0) path stores it: block-ELL slots (ascending
// natural column order) in the solver's internal row order.
struct AmgSystem {
    int N, b, nslot, ld;
    const int* colHost;   // [s*ld + p] internal column of slot s of internal row p, or -1
    const int* natural;   // [p] natural row of internal row p
};

struct AmgData;

// The hierarchy's structure (aggregates, coarse patterns, colours, sweep
// orders) from the FP64 matrix A64 (device, solver layout) of the first
// solve.  NULL with *status set on failure.
AmgData* amgCreate(const AmgSystem& sys, const double* A64, int coarsenTarget, cudaStream_t s, int* status);
void amgDestroy(AmgData* d);

// Rows of each level (up to AMG_MAX_LEVELS); returns the level count.
int amgLevelSizes(const AmgData* d, int* sizes);
// Colours of each level; returns the level count.
int amgLevelColors(const AmgData* d, int* colors);

// BiCGStab + one V-cycle per preconditioner application, one persistent
// launch: coarse values and inverted diagonals from A (solver layout, T
// precision), then the iteration on rhs (internal order) into x (internal
// order).  iterations, time of the kernels (ms) and algorithmic bytes out.
template <class T>
int amgSolve(AmgData* d, const T* A, const T* rhs, T* x, double redTol, double absTol, double maxRes, int maxIter,
             cudaStream_t s, DevStatus* st, DevStatus* hst, int& iters, float* ms, double* bytes);

// One V-cycle v = M^-1 d in FP64 (vectors in internal order) with the
// values of A: compared with the oracle's V-cycle in the tests.
int amgApply64(AmgData* d, const double* A, const double* dv, double* v, cudaStream_t s, DevStatus* st,
               DevStatus* hst);

}  // namespace gbfv
