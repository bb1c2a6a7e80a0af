// Block ILU(0) + BiCGStab for a general block-ELL pattern (the 9-point
// Jacobian of the vertex-centred discretization): host interface.
#pragma once

#include <vector>

#include <cuda_runtime.h>

#include "gbfv_internal.cuh"

namespace gbfv {

constexpr int GILU_MAX_SLOTS = 27;  // the 3 x 3 x 3 vertex neighbourhood

struct GiluData;

// The matrix layout of the context: nslot slots per row in ascending
// natural column order with the diagonal in slot nslot / 2 (slots below it
// lower, above it upper; -1 = no entry), rows in the level-major internal
// order given by levPtr (every row's lower entries in earlier levels, upper
// entries in later ones).  colDev is the device copy of colHost.  NULL with
// *status set on failure.
GiluData* giluCreate(int N, int b, int nslot, int ld, const std::vector<int>& colHost, const int* colDev,
                     const std::vector<int>& levPtr, int* status);
void giluDestroy(GiluData* d);
// whether the solves of a precision sweep with tagged words (no barrier per
// level), and the blocks of the launch
int giluTagged(const GiluData* d, int fp64);
int giluBlocks(const GiluData* d);

// BiCGStab + block ILU(0) (the reference's ParallelBiCGStabSolverBackend
// with Dune::SeqILU<..., 0> in natural order) in one persistent launch: the
// factorization of A (T precision, solver layout) when factor != 0, then the
// iteration on rhs into x (internal order).
template <class T>
int giluSolve(GiluData* d, const T* A, const T* rhs, T* x, int factor, double redTol, double absTol, double maxRes,
              int maxIter, cudaStream_t s, DevStatus* st, DevStatus* hst, int& iters, float* ms, double* bytes);

// v = (LU)^-1 dv in FP64 after factoring A (internal order), for tests
int giluApply64(GiluData* d, const double* A, const double* dv, double* v, cudaStream_t s, DevStatus* st,
                DevStatus* hst);

}  // namespace gbfv
