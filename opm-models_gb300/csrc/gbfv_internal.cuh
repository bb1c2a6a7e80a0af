// Internal device layouts and kernel launchers of libgbfv.
//
// Cell ordering on the device: "wavefront-major".  Cells are sorted by ILU(0)
// level (level = 1 + max level of the lower-index neighbours; i+j+k on a
// structured grid), and by natural index inside a level.  Every kernel --
// linearization, SpMV, the level-scheduled ILU(0) sweeps -- works in this
// order: a level is a contiguous index range, and the neighbours of a run of
// consecutive cells are runs of consecutive cells in the adjacent levels.
//
// Matrix layout: block-ELL, structure-of-arrays.  Each row has S = 2*dim+1
// slots sorted by the natural column index (the order dune's BCRSMatrix keeps
// and ILU(0) walks): slots [0, dim) lower (-z,-y,-x), slot dim diagonal,
// slots (dim, 2dim] upper (+x,+y,+z).  Entry e of slot s of row p lives at
// val[(s*b*b + e)*ldN + p], so a warp touching consecutive rows reads
// consecutive addresses.  Missing neighbours have col = -1 and zero blocks.
//
// Vectors (solution, residual, Krylov vectors) are block vectors in the same
// cell order: entry e of cell p at [p*b + e].
#pragma once
#include <atomic>
#include <cuda_runtime.h>

#include <cstdint>

#include "gbfv_physics.cuh"

namespace gbfv {

constexpr int MAX_DIM = 3;
constexpr int MAX_SLOTS = 7;
constexpr int MAX_MATERIALS = 16;

// per-boundary-intersection record (built on the host, axis-aligned faces)
struct BFace {
    int p;          // internal cell index
    int type;       // enum gbfv_bc
    int axis;       // 0..2
    double nrm;     // +1 / -1 along axis
    double tmpA;    // x_face - x_cell along axis (gradient direction)
    double dInA;    // x_cell - x_face along axis
    double gTimesDist;
    double area;
    double pb[2];   // boundary phase pressures (free flow)
    double mobb[2]; // kr/mu of the boundary state
    double rhob[2]; // boundary densities
    double rate[3]; // mass-rate boundary values per equation
    double transB;  // transmissibility flux module: boundary transmissibility
    double dzgB;    // and (z_cell - z_face) * g
};

// static description of one grid (or one batch of grids) on the device
struct DevMesh {
    int N;         // cells
    int ldN;       // leading dimension of SoA arrays
    int dim;       // 2 or 3
    int b;         // equations per cell
    int model;
    int nslot;     // 2*dim+1
    const int* nbr;       // [dir*ldN + p], dir = intersection index 0..2dim-1, -1 = none
    const double* dTot;   // [dir*ldN + p] x_J - x_I along the face axis
    const double* gIn;    // [dir*ldN + p] g . (x_I - x_face)
    const double* gEx;    // [dir*ldN + p] g . (x_J - x_face)
    const double* Kh;     // [dir*ldN + p] harmonic-mean permeability along axis
    const double* area;   // [dir*ldN + p]
    const double* volume; // [p]
    const double* porosity;
    const double* perm;   // [axis*ldN + p]
    const int* material;  // [p]
    const int* cflag;     // [p] constraint row index or -1
    const int* bfPtr;     // [p..p+1] range into bfaces, internal order
    const BFace* bfaces;
    const double* consPv;     // [k*3 + e]
    const int* consMeaning;   // [k]
    const int* consCells;     // internal index of each constrained cell
    const int* consOf;        // constraint record of each constrained cell
    int numConsCells;
    int slotOfDir[6];     // ELL slot of intersection direction
    const int* inst;      // [p] instance of the cell (batched systems)
    int fluxModule;       // enum gbfv_flux
    const double* trans;  // [dir*ldN + p] transmissibility flux module: face transmissibility
    const double* dzg;    // [dir*ldN + p] (z_I - z_J) * g
    const int* tieUpI;    // [dir*ldN + p] interior upstream when the pressure difference is zero
    int tpfa;             // TpfaLinearizer + BlackOilLocalResidualTPFA (rows not divided by the volume)
};

struct DevPhysics {
    int numMaterials;
    TwoPhaseLaw law[MAX_MATERIALS];
    double coreyN[MAX_MATERIALS];
    double rho[2], mu[2];
    BlackOilPvt pvt;
};

// Newton-update parameters (blackoilnewtonmethodparameters.hh)
struct UpdateParams {
    double dsMax, dpMaxRel, oscThreshold, pMin, pMax, swMax, waterOnly;
};

// intensive quantities written by the IQ pass and read by the assembly pass
//   immiscible: val 6 (p0,p1,rho0,rho1,lam0,lam1), der 6x2, sto 2x3
//   black-oil:  val 11 (p,rho0..2,lam0..2,invB0..2,Rs), der 10x3 (no p), sto 3x4
struct IqBuffers {
    double* val;   // [q*ldN + p]
    double* der;   // [(q*b + k)*ldN + p]
    double* sto;   // [(e*(b+1) + k)*ldN + p], k = 0 value, 1..b derivatives
};

// planes of each IqBuffers array for b equations: the immiscible IQ kernel
// writes 6 values and 6 quantities with 2 derivatives, the black-oil one
// 11 values and 10 quantities with 3 derivatives; storage is one value and
// b derivatives per equation
constexpr int iqValuePlanes(int b) { return b == 2 ? 6 : 11; }
constexpr int iqDerivPlanes(int b) { return b == 2 ? 12 : 30; }
constexpr int iqStoragePlanes(int b) { return b * (b + 1); }

// finite-difference linearizer: intensive quantities of the deflected
// states, per primary variable (+eps and the second, minus state)
struct FdIq {
    IqBuffers plus[3];
    IqBuffers minus[3];
};


// device-side status words (bounded waits report here instead of trapping)
struct DevStatus {
    int code;        // gbfv_status of the last device-side failure
    int where;
    int iterations;  // Krylov iterations
    int converged;
    int refinements;
    int nonfinite;
    int switched;
    int pad;
    unsigned long long errorBits;  // Newton error as ordered bits (max |r|)
    double resid;    // final residual max-norm
    double resid0;   // initial residual max-norm
};
// One system of a batch for the batched linearization / Newton kernels
// (grid (gx, K), blockIdx.y = system): the same per-cell code as the
// single-system kernels, with this system's buffers.
struct LinJob {
    DevMesh m;
    const DevPhysics* phys;
    double *x, *xOld;
    int *meaning, *meaningOld;
    IqBuffers iq;
    double* storageOld;
    double* residual;
    double* jval;
    const double* dx;
    int* wasSwitched;
    DevStatus* st;
};
// per-round state of a batched system
struct JobState {
    double dt;
    int iter0;   // Newton iteration 0: refresh the storage cache
    int active;
};

// Device-side state of a batched Newton round (batchround.cu): one entry
// per system, copied in before and out after every round.
enum RoundPhase {
    RS_LIN = 0,     // linearizes in this round
    RS_SOLVE = 1,   // (inside a round) solving
    RS_UPDATE = 2,  // (inside a round) solved, to be updated
    RS_END_OK = 3,  // the Newton loop converged in this round: the step is complete
    RS_FAIL = 4,    // failed in this round (status): back to the old time level
    RS_IDLE = 5     // not taking part
};
struct RoundParams {
    double newtonTol, newtonMaxError, linTol, absTol, innerTol, linMaxError;
    int newtonMaxIt, linMaxIt, mixed, pad;
};
struct RoundSys {
    int phase, status, numIterations, linearizations;
    int linItStep, kry, refs, lastKs;
    int lastIt, factorNext, kryLaunches, kryFactors;
    int kryIters, pad;
    double dt, error, lastError, resErr, resErr0;
};

// kernel launches of this library (several host threads may launch: atomic);
// while a thread captures a CUDA graph its launches are counted for the
// graph instead and added to the total each time the graph is replayed
extern std::atomic<int64_t> g_launches;
extern thread_local int t_captureLaunches;
inline void countLaunch(int n = 1)
{
    if (t_captureLaunches >= 0) t_captureLaunches += n;
    else g_launches += n;
}

// ---------------------------------------------------- kernel launchers ----
void launchApplyConstraints(const DevMesh& m, double* x, double* xOld, int* meaning, int* meaningOld,
                            cudaStream_t s);
void launchIq(const DevMesh& m, const DevPhysics* phys, const double* x, const int* meaning,
              IqBuffers iq, cudaStream_t s);
// output quantities of the current state: out[plane*ldN + p], GBFV_OUTPUT_PLANES planes
void launchOutputFields(const DevMesh& m, const DevPhysics* phys, const double* x, const int* meaning,
                        IqBuffers iq, double* out, cudaStream_t s);
void launchAssemble(const DevMesh& m, const DevPhysics* phys, IqBuffers iq, double* storageOld,
                    int iter0, double dt, double* residual, double* jval, cudaStream_t s);
void launchSetRefPressure(const double* x, int idx, double* refP, cudaStream_t s);
void launchFdDeflect(const DevMesh& m, int b, const double* x, const int* meaning, const double* refP, int pv,
                     int dir, double* xd, cudaStream_t s);
void launchAssembleFd(const DevMesh& m, const DevPhysics* phys, IqBuffers iq0, const FdIq& fd, const int* meaning,
                      const double* refP, int method, double* storageOld, int iter0, double dt, double* residual,
                      double* jval, cudaStream_t s);
void launchNewtonError(const DevMesh& m, const double* residual, DevStatus* st, cudaStream_t s);
void launchCheckUpdate(int n, const double* dx, DevStatus* st, cudaStream_t s);
void launchNewtonUpdate(const DevMesh& m, const DevPhysics* phys, const double* dx, double* x,
                        int* meaning, int* wasSwitched, UpdateParams prm, DevStatus* st,
                        cudaStream_t s);
void launchBatchLinearize(const LinJob* jobs, const JobState* js, int K, int gx, cudaStream_t s);
void launchBatchNewtonError(const LinJob* jobs, const JobState* js, int K, int gx, cudaStream_t s);
void launchBatchCheckUpdate(const LinJob* jobs, const JobState* js, int K, int gx, cudaStream_t s);
void launchBatchNewtonUpdate(const LinJob* jobs, const JobState* js, int K, int gx, UpdateParams prm,
                             cudaStream_t s);
void launchBoundaryStates(const DevPhysics* phys, BFace* bf, const int* bfMaterial, int nbf,
                          cudaStream_t s);

}  // namespace gbfv
