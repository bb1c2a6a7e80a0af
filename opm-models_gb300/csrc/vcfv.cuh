// Vertex-centred finite volumes (VcfvDiscretization): host set-up of the
// stencils and the device linearization of the immiscible model on them.
#pragma once

#include <vector>

#include <cuda_runtime.h>

#include "../../include/gbfv.h"
#include "gbfv_internal.cuh"

namespace gbfv {

constexpr int VCFV_SLOTS = 9;  // 3 x 3 vertex neighbourhood, slot (dy+1)*3 + (dx+1)
constexpr int VCFV_DIAG = 4;

// Natural-order description derived from the problem: the sub-control-volume
// totals of every vertex and its neighbour in each slot.
struct VcfvSetup {
    int N = 0, E = 0;
    std::vector<double> totalVolume;  // [N] dofTotalVolume
    std::vector<int> nbr;             // [N*9] natural neighbour per slot, -1 none
};

// Checks the grid (axis-aligned quadrilaterals whose corners form a 3 x 3
// vertex neighbourhood) and fills s; GBFV_OK or an error with the reason set.
int vcfvSetup(const gbfv_problem* P, VcfvSetup& s);

struct VcfvDev;

// Element geometry, boundary faces, incidence lists and scratch on the
// device; perm maps natural vertex -> internal row, ld the row stride.
VcfvDev* vcfvUpload(const gbfv_problem* P, const VcfvSetup& s, const DevPhysics& ph, const std::vector<int>& perm,
                    int ld, int* status);
void vcfvDestroy(VcfvDev* d);
// algorithmic bytes of one linearization (element and gather passes)
double vcfvLinearizeBytes(const VcfvDev* d);

// Residual and Jacobian (block-ELL, VCFV_SLOTS slots) of the current
// intensive quantities: the element pass (one thread per element and focus
// corner) and the per-vertex gather in element order.
void launchVcfvAssemble(const VcfvDev* d, const DevMesh& m, IqBuffers iq, double* storageOld, int iter0, double dt,
                        double* residual, double* jval, cudaStream_t s);

// The same with the finite-difference local linearizer: iq0 the state's
// intensive quantities, fd those of the per-vertex deflected states
// (launchFdDeflect + launchIq), method the numeric difference method.
void launchVcfvAssembleFd(const VcfvDev* d, const DevMesh& m, IqBuffers iq0, const FdIq& fd, const double* refP,
                          int method, double* storageOld, int iter0, double dt, double* residual, double* jval,
                          cudaStream_t s);

}  // namespace gbfv
