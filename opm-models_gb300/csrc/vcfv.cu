// Vertex-centred finite volumes (VcfvDiscretization) on the device: the
// stencil geometry of 2D axis-aligned quadrilaterals and the AD
// linearization of the immiscible model on it.
//
// Reference: VcfvStencil (vcfvstencil.hh:466-1015: corners, edge centres,
// sub-control volumes as quadrilaterals, one sub-control-volume face per
// edge from the edge centre to the element centre, boundary faces half an
// intersection each), P1FeGradientCalculator (p1fegradientcalculator.hh:
// 83-290) and FvBaseGradientCalculator (fvbasegradientcalculator.hh:
// 200-318), the Darcy module (darcyfluxmodule.hh:183-525), the local
// residual (fvbaselocalresidual.hh:158-191, 299-348, 419-626) and
// FvBaseAdLocalLinearizer with one focus per element corner
// (fvbaseadlocallinearizer.hh:173-292), scattered by FvBaseLinearizer::
// linearizeElement_ (fvbaselinearizer.hh:595-626).
//
// GPU shape: the element pass runs one thread per (element, focus corner):
// it evaluates the element's four corner residuals with the derivatives of
// the focus corner's primary variables and writes them to a scratch buffer.
// The gather pass runs one thread per vertex: it adds its (at most four)
// elements' contributions in element order -- the reference's summation
// order -- into the residual row and the nine Jacobian blocks of the row.
// No atomics; the result does not depend on scheduling.  The geometry the
// element pass needs (sub-control volumes, face normals and areas, P1
// gradients at the integration points, mean permeabilities, gravity terms)
// is computed once on the host in the reference's operation order.
//
// The intensive quantities of the immiscible model have constant densities,
// so a corner's density carries no derivatives; every quantity of a corner
// other than the focus one enters with its value only.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/gbfv.h"
#include "gbfv_internal.cuh"
#include "vcfv.cuh"

namespace gbfv {

void setLastError(const std::string& s);

namespace {

using D2 = Dual<2>;

// corners of each edge of the 2D cube (dune-geometry numbering: corner c at
// ((c & 1), (c >> 1) & 1)), the edges' local centres, and the boundary
// intersections' corners
const int EDGE_CORNER[4][2] = {{0, 2}, {1, 3}, {0, 1}, {2, 3}};
const double EDGE_LOCAL[4][2] = {{0.0, 0.5}, {1.0, 0.5}, {0.5, 0.0}, {0.5, 1.0}};
// sub-control-volume face k separates corner FI[k] (interior) and FJ[k]
// (exterior): the edge's corners with corner 2 moved to the interior side
// (vcfvstencil.hh:904-907)
__constant__ int FI[4] = {2, 1, 0, 3};
__constant__ int FJ[4] = {0, 3, 1, 2};

struct ElemGeo {
    int v[4];              // internal row of each corner
    double scvVol[4];
    double fa[4];          // face areas
    double fn[4][2];       // unit normals, interior to exterior
    double Kh[4][2];       // entry-wise harmonic mean of the two corners' K
    double dTot[4][2];     // x_j - x_i
    double absTot2[4];     // |x_j - x_i|^2
    double gIn[4], gEx[4]; // g . (x_i - x_ip), g . (x_j - x_ip)
    double w2p[4][2];      // two-point gradient weights (x_j - x_i) / |x_j - x_i|^2
    double grad[4][4][2];  // P1: gradient of corner c's shape function at face k
};

struct BFaceV {
    int c, type;
    double area;
    double n[2];
    double w[2];           // (x_ip - x_scv) / |x_ip - x_scv|^2, the boundary gradient's weights
    double dIn[2];         // x_vertex - x_ip
    double gTimesDist, absDist2;
    double K[2];           // the vertex's permeability
    double pb[2], mobb[2], rhob[2];  // free-flow state
    double rate[3];        // mass rate per equation
};

struct VcfvArgs {
    int E, ld;
    const ElemGeo* geo;
    const int* bfPtr;
    const BFaceV* bf;
    const int* inc;        // [k*ld + p] element*4 + corner of vertex p's k-th element, -1 none
    const unsigned char* incSlot;  // [(k*4 + f)*ld + p] slot of the element's corner f in row p
    double* R;             // [(e*4 + f)*b + a] residual of corner f (focus f)
    double* J;             // [((e*4 + f)*4 + j)*b*b + a*b + pv] d res_j,a / d x_f,pv
    int p1;
    double rhoRef[3];      // black-oil surface densities (water, oil, gas)
};

double harmonicMeanV(double x, double y)
{
    if (x * y <= 0) return 0.0;
    return (2 * x * y) / (x + y);
}

double quadArea(const double* p0, const double* p1, const double* p2, const double* p3)
{
    return 0.5 * std::abs((p3[0] - p1[0]) * (p2[1] - p0[1]) - (p3[1] - p1[1]) * (p2[0] - p0[0]));
}

// the geometry of one element (VcfvStencil::update, vcfvstencil.hh:864-
// 1015), natural vertex indices; AxisAlignedCubeGeometry::global(x) =
// lower + x .* (upper - lower)
struct HostElem {
    double lower[2], upper[2];
    double vpos[4][2], scvVol[4], scvCenter[4][2];
    int fi[4], fj[4];
    double fn[4][2], fa[4], fip[4][2], grad[4][4][2];
};

HostElem hostElem(const gbfv_problem* P, const int* corner)
{
    HostElem E;
    for (int d = 0; d < 2; ++d) {
        E.lower[d] = P->center[3 * corner[0] + d];
        E.upper[d] = P->center[3 * corner[3] + d];
    }
    auto global = [&](const double* l, double* x) {
        for (int d = 0; d < 2; ++d) x[d] = E.lower[d] + l[d] * (E.upper[d] - E.lower[d]);
    };
    const double elemLocal[2] = {0.5, 0.5};
    double elemGlobal[2], edgeCoord[4][2];
    global(elemLocal, elemGlobal);
    for (int c = 0; c < 4; ++c) {
        const double l[2] = {double(c & 1), double((c >> 1) & 1)};
        global(l, E.vpos[c]);
    }
    for (int k = 0; k < 4; ++k) global(EDGE_LOCAL[k], edgeCoord[k]);
    E.scvVol[0] = quadArea(E.vpos[0], edgeCoord[2], elemGlobal, edgeCoord[0]);
    E.scvVol[1] = quadArea(E.vpos[1], edgeCoord[1], elemGlobal, edgeCoord[2]);
    E.scvVol[2] = quadArea(E.vpos[2], edgeCoord[0], elemGlobal, edgeCoord[3]);
    E.scvVol[3] = quadArea(E.vpos[3], edgeCoord[3], elemGlobal, edgeCoord[1]);
    // sub-control-volume centres: the mean of the local corners
    for (int c = 0; c < 4; ++c) {
        const double x0 = (c & 1) ? 0.5 : 0.0, y0 = ((c >> 1) & 1) ? 0.5 : 0.0;
        const double loc[4][2] = {{x0, y0}, {x0 + 0.5, y0}, {x0, y0 + 0.5}, {x0 + 0.5, y0 + 0.5}};
        double ctr[2] = {0.0, 0.0};
        for (int q = 0; q < 4; ++q)
            for (int d = 0; d < 2; ++d) ctr[d] += loc[q][d];
        for (int d = 0; d < 2; ++d) ctr[d] /= 4;
        global(ctr, E.scvCenter[c]);
    }
    const double jInv[2] = {1.0 / (E.upper[0] - E.lower[0]), 1.0 / (E.upper[1] - E.lower[1])};
    for (int k = 0; k < 4; ++k) {
        int i = EDGE_CORNER[k][0], j = EDGE_CORNER[k][1];
        if (i == 2 || j == 2) std::swap(i, j);
        E.fi[k] = i;
        E.fj[k] = j;
        const double ipLocal[2] = {(EDGE_LOCAL[k][0] + elemLocal[0]) * 0.5, (EDGE_LOCAL[k][1] + elemLocal[1]) * 0.5};
        double diff[2] = {elemGlobal[0] - edgeCoord[k][0], elemGlobal[1] - edgeCoord[k][1]};
        double n[2] = {diff[1], -diff[0]};
        for (int d = 0; d < 2; ++d) diff[d] = E.vpos[j][d] - E.vpos[i][d];
        if (n[0] * diff[0] + n[1] * diff[1] < 0) {
            n[0] *= -1;
            n[1] *= -1;
        }
        const double area = std::sqrt(n[0] * n[0] + n[1] * n[1]);
        E.fa[k] = area;
        E.fn[k][0] = n[0] / area;
        E.fn[k][1] = n[1] / area;
        global(ipLocal, E.fip[k]);
        for (int c = 0; c < 4; ++c) {
            const bool bx = c & 1, by = (c >> 1) & 1;
            const double gx = (bx ? 1.0 : -1.0) * (by ? ipLocal[1] : 1.0 - ipLocal[1]);
            const double gy = (bx ? ipLocal[0] : 1.0 - ipLocal[0]) * (by ? 1.0 : -1.0);
            E.grad[k][c][0] = jInv[0] * gx;
            E.grad[k][c][1] = jInv[1] * gy;
        }
    }
    return E;
}

int slotOf(const double* a, const double* b)
{
    const int dx = b[0] > a[0] ? 1 : (b[0] < a[0] ? -1 : 0);
    const int dy = b[1] > a[1] ? 1 : (b[1] < a[1] ? -1 : 0);
    return (dy + 1) * 3 + (dx + 1);
}

// ---------------------------------------------------------------- kernels --
using D3 = Dual<3>;
__device__ __forceinline__ double valueOf(double x) { return x; }
__device__ __forceinline__ double valueOf(const D2& x) { return x.v; }
__device__ __forceinline__ double valueOf(const D3& x) { return x.v; }

// Intensive-quantity value planes of the two models (the IQ pass's layout):
// two-phase p0 p1 rho0 rho1 lam0 lam1; black-oil p rho0..2 lam0..2
// invB0..2 Rs (one pressure: zero capillary pressure)
template <int B> struct Iq;
template <> struct Iq<2> {
    static constexpr int NV = 6;
    static __device__ __forceinline__ int p(int a) { return a; }
    static __device__ __forceinline__ int rho(int a) { return 2 + a; }
    static __device__ __forceinline__ int lam(int a) { return 4 + a; }
};
template <> struct Iq<3> {
    static constexpr int NV = 11;
    static __device__ __forceinline__ int p(int) { return 0; }
    static __device__ __forceinline__ int rho(int a) { return 1 + a; }
    static __device__ __forceinline__ int lam(int a) { return 4 + a; }
    static __device__ __forceinline__ int invB(int a) { return 7 + a; }
    static __device__ __forceinline__ int rs() { return 10; }
};

// FvBaseLocalResidual::eval of one element (fvbaselocalresidual.hh:158-191)
// for the model with B equations (2: immiscible two-phase; 3: black-oil,
// blackoillocalresidual.hh:101-367) in the number type T (duals for
// automatic differentiation, double for finite differences).  Q(c, k):
// intensive-quantity value plane k of corner c; Sto(c, e): the storage of
// equation e in corner c; sto0: the storage values of the unperturbed state
// (the cache at iteration 0).
template <class T, int B, bool P1, class QF, class SF>
__device__ __forceinline__ void elementEval(const VcfvArgs& a, const DevMesh& m, int e, const QF& Q, const SF& Sto,
                                            const double* __restrict__ sto0, const double* __restrict__ storageOld,
                                            int iter0, double dt, T (&res)[4][B])
{
    using I = Iq<B>;
    constexpr int NP = B;  // phases
    const ElemGeo& G = a.geo[e];
    const int ld = m.ldN;
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int q = 0; q < B; ++q) res[c][q] = T(0.0);
    // evalFluxes: the four sub-control-volume faces
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        const int i = FI[k], j = FJ[k];
        T pg[NP][2];
#pragma unroll
        for (int ph = 0; ph < NP; ++ph) {
            if (P1) {
                pg[ph][0] = T(0.0);
                pg[ph][1] = T(0.0);
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const T dv = Q(c, I::p(ph));
                    pg[ph][0] = pg[ph][0] + dv * G.grad[k][c][0];
                    pg[ph][1] = pg[ph][1] + dv * G.grad[k][c][1];
                }
            }
            else {
                const T deltay = Q(j, I::p(ph)) - Q(i, I::p(ph));
                pg[ph][0] = deltay * G.w2p[k][0];
                pg[ph][1] = deltay * G.w2p[k][1];
            }
            // gravity correction (darcyfluxmodule.hh:214-283)
            const T pStatIn = -(Q(i, I::rho(ph)) * G.gIn[k]);
            const T pStatEx = -(Q(j, I::rho(ph)) * G.gEx[k]);
            const T fs = (pStatEx - pStatIn) / G.absTot2[k];
            pg[ph][0] = pg[ph][0] + G.dTot[k][0] * fs;
            pg[ph][1] = pg[ph][1] + G.dTot[k][1] * fs;
        }
        T flux[B];
#pragma unroll
        for (int q = 0; q < B; ++q) flux[q] = T(0.0);
#pragma unroll
        for (int ph = 0; ph < NP; ++ph) {
            T tmp(0.0);
            tmp = tmp + pg[ph][0] * G.fn[k][0];
            tmp = tmp + pg[ph][1] * G.fn[k][1];
            const int up = valueOf(tmp) > 0 ? j : i;
            const T mob = Q(up, I::lam(ph));
            T vf(0.0);
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                T fv = G.Kh[k][d] * pg[ph][d];
                fv = fv * (-mob);
                vf = vf + fv * G.fn[k][d];
            }
            if constexpr (B == 2) {
                flux[ph] = T(0.0) + vf * Q(up, I::rho(ph));
            }
            else {
                // component fluxes of the phase: water -> 1, oil -> 0 (and
                // the gas dissolved in it -> 2), gas -> 2
                const int comp = ph == 0 ? 1 : (ph == 1 ? 0 : 2);
                const T svf = Q(up, Iq<3>::invB(ph)) * vf;
                flux[comp] = flux[comp] + svf * a.rhoRef[ph];
                if (ph == 1) flux[2] = flux[2] + Q(up, Iq<3>::rs()) * svf * a.rhoRef[2];
            }
        }
#pragma unroll
        for (int q = 0; q < B; ++q) {
            flux[q] = flux[q] * (1.0 * G.fa[k]);
            res[i][q] = res[i][q] + flux[q];
            res[j][q] = res[j][q] - flux[q];
        }
    }
    // evalVolumeTerms_: storage of the four sub-control volumes
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const double scvVolume = G.scvVol[c] * 1.0;
#pragma unroll
        for (int q = 0; q < B; ++q) {
            T tmp = Sto(c, q);
            const double tmp2 = iter0 ? sto0[q * (B + 1) * ld + G.v[c]] : storageOld[q * ld + G.v[c]];
            tmp = tmp - tmp2;
            tmp = tmp * (scvVolume / dt);
            res[c][q] = res[c][q] + tmp;
            res[c][q] = res[c][q] - 0.0 * scvVolume;
        }
    }
    // evalBoundary_: this element's boundary sub-control-volume faces
    for (int bf = a.bfPtr[e]; bf < a.bfPtr[e + 1]; ++bf) {
        const BFaceV Bf = a.bf[bf];
        T values[B];
#pragma unroll
        for (int q = 0; q < B; ++q) values[q] = T(0.0);
        if (Bf.type == GBFV_BC_MASSRATE) {
#pragma unroll
            for (int q = 0; q < B; ++q) values[q] = T(Bf.rate[q]);
        }
        else if (B == 2 && Bf.type == GBFV_BC_FREEFLOW) {
#pragma unroll
            for (int ph = 0; ph < 2; ++ph) {
                const T pIn = Q(Bf.c, I::p(ph));
                const T deltay = T(Bf.pb[ph]) - pIn;
                T pg[2];
                pg[0] = deltay * Bf.w[0];
                pg[1] = deltay * Bf.w[1];
                const T pStatIn = (-Bf.gTimesDist) * Q(Bf.c, I::rho(ph));
                const T fsc = pStatIn / Bf.absDist2;
                pg[0] = pg[0] + Bf.dIn[0] * fsc;
                pg[1] = pg[1] + Bf.dIn[1] * fsc;
                T tmp(0.0);
                tmp = tmp + pg[0] * Bf.n[0];
                tmp = tmp + pg[1] * Bf.n[1];
                const T mob = valueOf(tmp) > 0.0 ? T(Bf.mobb[ph]) : Q(Bf.c, I::lam(ph));
                T vf(0.0);
#pragma unroll
                for (int d = 0; d < 2; ++d) {
                    T fv = Bf.K[d] * pg[d];
                    fv = fv * (-mob);
                    vf = vf + fv * Bf.n[d];
                }
                const T dens = Bf.pb[ph] > valueOf(pIn) ? T(Bf.rhob[ph]) : Q(Bf.c, I::rho(ph));
                values[ph] = values[ph] + vf * dens;
            }
        }
        const double aa = Bf.area * 1.0;
#pragma unroll
        for (int q = 0; q < B; ++q) res[Bf.c][q] = res[Bf.c][q] + values[q] * aa;
    }
    // volumetric residual
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const double V = m.volume[G.v[c]];
#pragma unroll
        for (int q = 0; q < B; ++q) res[c][q] = res[c][q] / V;
    }
}

// Element pass (automatic differentiation): thread (e, f) evaluates element
// e with the derivatives of corner f (fvbaseadlocallinearizer.hh:173-292).
template <int B, bool P1>
__global__ void __launch_bounds__(128) kVcfvElement(VcfvArgs a, DevMesh m, IqBuffers iq,
                                                    const double* __restrict__ storageOld, int iter0, double dt)
{
    using D = Dual<B>;
    constexpr int NV = Iq<B>::NV;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.E * 4) return;
    const int e = t >> 2, f = t & 3;
    const ElemGeo& G = a.geo[e];
    const int ld = m.ldN;
    double cv[4][NV];  // the corners' intensive-quantity values
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int k = 0; k < NV; ++k) cv[c][k] = iq.val[k * ld + G.v[c]];
    const int vf = G.v[f];
    double fd[NV][B];  // the focus corner's derivatives
#pragma unroll
    for (int k = 0; k < NV; ++k)
#pragma unroll
        for (int d = 0; d < B; ++d) {
            if (B == 2) fd[k][d] = iq.der[(k * 2 + d) * ld + vf];
            else fd[k][d] = k == 0 ? (d == 1 ? 1.0 : 0.0) : iq.der[((k - 1) * 3 + d) * ld + vf];
        }
    auto Q = [&](int c, int k) {
        D r(cv[c][k]);
        if (c == f)
#pragma unroll
            for (int d = 0; d < B; ++d) r.d[d] = fd[k][d];
        return r;
    };
    auto Sto = [&](int c, int q) {
        const int v = G.v[c];
        D r(iq.sto[(q * (B + 1) + 0) * ld + v]);
        if (c == f)
#pragma unroll
            for (int d = 0; d < B; ++d) r.d[d] = iq.sto[(q * (B + 1) + 1 + d) * ld + v];
        return r;
    };
    D res[4][B];
    elementEval<D, B, P1>(a, m, e, Q, Sto, iq.sto, storageOld, iter0, dt, res);
    const size_t ef = (size_t)e * 4 + f;
#pragma unroll
    for (int q = 0; q < B; ++q) a.R[ef * B + q] = res[f][q].v;
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int q = 0; q < B; ++q)
#pragma unroll
            for (int pv = 0; pv < B; ++pv) a.J[(ef * 4 + j) * B * B + q * B + pv] = res[j][q].d[pv];
}

// Element pass (finite differences, fvbasefdlocallinearizer.hh:236-510; the
// two-phase model): thread (e, f) evaluates element e unperturbed and with
// corner f's primary variable pv deflected (the deflected states' intensive
// quantities come from the per-vertex deflection passes, plus[pv] at
// x + eps, minus[pv] at the second state), the columns of corner f being
// the differences divided by the total deflection.
template <bool P1>
__global__ void __launch_bounds__(128) kVcfvElementFd(VcfvArgs a, DevMesh m, IqBuffers iq0, FdIq fdq,
                                                      const double* __restrict__ refP, int method,
                                                      const double* __restrict__ storageOld, int iter0, double dt)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.E * 4) return;
    const int e = t >> 2, f = t & 3;
    const ElemGeo& G = a.geo[e];
    const int ld = m.ldN;
    double cv[4][6];
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int k = 0; k < 6; ++k) cv[c][k] = iq0.val[k * ld + G.v[c]];
    const int vf = G.v[f];
    auto eval = [&](const IqBuffers* dq, int it0, double (&res)[4][2]) {
        auto Q = [&](int c, int k) { return (dq && c == f) ? dq->val[k * ld + vf] : cv[c][k]; };
        auto Sto = [&](int c, int ph) {
            return (dq && c == f) ? dq->sto[(ph * 3) * ld + vf] : iq0.sto[(ph * 3) * ld + G.v[c]];
        };
        elementEval<double, 2, P1>(a, m, e, Q, Sto, iq0.sto, storageOld, it0, dt, res);
    };
    double res0[4][2];
    eval(nullptr, iter0, res0);
    const size_t ef = (size_t)e * 4 + f;
    a.R[ef * 2 + 0] = res0[f][0];
    a.R[ef * 2 + 1] = res0[f][1];
    // the deflection of this vertex's primary variable (the immiscible
    // model's primaryVarWeight: 10 / reference pressure for the pressure)
    const double baseEps = fmax(0.9123e-10, 2.220446049250313e-16 * 1.23e3);
#pragma unroll 1
    for (int pv = 0; pv < 2; ++pv) {
        const double w = pv == 0 ? 10 / *refP : 1.0;
        const double eps = baseEps / w;
        double delta = 0.0;
        double d[4][2], r1[4][2];
        // the stashed state reads the storage cache: the unperturbed storage
        if (method >= 0) {
            delta += eps;
            eval(&fdq.plus[pv], iter0, r1);
#pragma unroll
            for (int c = 0; c < 4; ++c) d[c][0] = r1[c][0], d[c][1] = r1[c][1];
        }
        else {
#pragma unroll
            for (int c = 0; c < 4; ++c) d[c][0] = res0[c][0], d[c][1] = res0[c][1];
        }
        if (method <= 0) {
            delta += eps;
            eval(&fdq.minus[pv], iter0, r1);
#pragma unroll
            for (int c = 0; c < 4; ++c) d[c][0] -= r1[c][0], d[c][1] -= r1[c][1];
        }
        else {
#pragma unroll
            for (int c = 0; c < 4; ++c) d[c][0] -= res0[c][0], d[c][1] -= res0[c][1];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int ph = 0; ph < 2; ++ph) a.J[(ef * 4 + j) * 4 + ph * 2 + pv] = d[j][ph] / delta;
    }
}

// Gather pass: vertex p's residual and Jacobian row, its elements' records
// added in element order (residual_[globI] += ..., addToBlock(globJ, globI,
// ...), fvbaselinearizer.hh:609-621); a constrained vertex's row becomes the
// identity with a zero residual (applyConstraintsToLinearization_,
// fvbaselinearizer.hh:649-666); the storage cache at iteration 0.
template <int B>
__global__ void __launch_bounds__(128) kVcfvGather(VcfvArgs a, DevMesh m, IqBuffers iq, double* __restrict__ storageOld,
                                                   int iter0, double* __restrict__ residual, double* __restrict__ jval)
{
    constexpr int BB = B * B;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m.N) return;
    const int ld = m.ldN;
    double r[B];
#pragma unroll
    for (int q = 0; q < B; ++q) r[q] = 0.0;
    double Jb[VCFV_SLOTS][BB];
#pragma unroll
    for (int s = 0; s < VCFV_SLOTS; ++s)
#pragma unroll
        for (int q = 0; q < BB; ++q) Jb[s][q] = 0.0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int ec = a.inc[k * ld + p];
        if (ec < 0) break;
        const size_t e = ec >> 2;
        const int c = ec & 3;
#pragma unroll
        for (int q = 0; q < B; ++q) r[q] += a.R[(e * 4 + c) * B + q];
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            const int s = a.incSlot[(k * 4 + f) * ld + p];
            const double* src = &a.J[((e * 4 + f) * 4 + c) * BB];
#pragma unroll
            for (int sl = 0; sl < VCFV_SLOTS; ++sl)
                if (sl == s)
#pragma unroll
                    for (int q = 0; q < BB; ++q) Jb[sl][q] += src[q];
        }
    }
    if (m.cflag[p] >= 0) {
#pragma unroll
        for (int q = 0; q < B; ++q) r[q] = 0.0;
#pragma unroll
        for (int s = 0; s < VCFV_SLOTS; ++s)
#pragma unroll
            for (int q = 0; q < BB; ++q) Jb[s][q] = (s == VCFV_DIAG && q % (B + 1) == 0) ? 1.0 : 0.0;
    }
#pragma unroll
    for (int q = 0; q < B; ++q) residual[B * p + q] = r[q];
#pragma unroll
    for (int s = 0; s < VCFV_SLOTS; ++s)
#pragma unroll
        for (int q = 0; q < BB; ++q) jval[((size_t)s * BB + q) * ld + p] = Jb[s][q];
    if (iter0)
#pragma unroll
        for (int q = 0; q < B; ++q) storageOld[q * ld + p] = iq.sto[(q * (B + 1) + 0) * ld + p];
}

}  // namespace

struct VcfvDev {
    int E = 0, N = 0, ld = 0, p1 = 1, nbf = 0, b = 2;
    double rhoRef[3] = {0, 0, 0};
    ElemGeo* geo = nullptr;
    int* bfPtr = nullptr;
    BFaceV* bf = nullptr;
    int* inc = nullptr;
    unsigned char* incSlot = nullptr;
    double* R = nullptr;
    double* J = nullptr;
};

int vcfvSetup(const gbfv_problem* P, VcfvSetup& s)
{
    auto fail = [](const std::string& w, int code) {
        setLastError("vertex-centred grid: " + w);
        return code;
    };
    if (P->flux_module != GBFV_FLUX_DARCY) return fail("the Darcy flux module only", GBFV_ERR_UNSUPPORTED);
    const int N = P->num_cells, E = P->num_elements;
    if (P->model == GBFV_MODEL_BLACKOIL_3P && P->bface_type)
        for (int f = 0; f < P->num_bfaces; ++f)
            if (P->bface_type[f] == GBFV_BC_FREEFLOW)
                return fail("free-flow boundaries are the two-phase model's", GBFV_ERR_UNSUPPORTED);
    for (int i = 0; i < N; ++i)
        if (P->center[3 * i + 2] != 0.0) return fail("2D grids only (vertex z = 0)", GBFV_ERR_UNSUPPORTED);
    s.N = N;
    s.E = E;
    s.totalVolume.assign(N, 0.0);
    s.nbr.assign((size_t)N * VCFV_SLOTS, -1);
    std::vector<char> used(N, 0);
    for (int e = 0; e < E; ++e) {
        const int* cn = &P->elem_corner[4 * e];
        const double* x0 = &P->center[3 * cn[0]];
        const double* x3 = &P->center[3 * cn[3]];
        const double* x1 = &P->center[3 * cn[1]];
        const double* x2 = &P->center[3 * cn[2]];
        if (!(x3[0] > x0[0] && x3[1] > x0[1]) || x1[0] != x3[0] || x1[1] != x0[1] || x2[0] != x0[0] ||
            x2[1] != x3[1])
            return fail("element " + std::to_string(e) + " is not an axis-aligned box in corner order",
                        GBFV_ERR_UNSUPPORTED);
        const HostElem H = hostElem(P, cn);
        for (int c = 0; c < 4; ++c) {
            s.totalVolume[cn[c]] += H.scvVol[c];
            used[cn[c]] = 1;
        }
        for (int a = 0; a < 4; ++a)
            for (int c = 0; c < 4; ++c) {
                const int sl = slotOf(&P->center[3 * cn[a]], &P->center[3 * cn[c]]);
                int& q = s.nbr[(size_t)cn[a] * VCFV_SLOTS + sl];
                if (q >= 0 && q != cn[c])
                    return fail("two vertices in one neighbour direction of vertex " + std::to_string(cn[a]),
                                GBFV_ERR_UNSUPPORTED);
                q = cn[c];
            }
    }
    for (int i = 0; i < N; ++i) {
        if (!used[i]) return fail("vertex " + std::to_string(i) + " belongs to no element", GBFV_ERR_ARG);
        int prev = -1;
        for (int sl = 0; sl < VCFV_SLOTS; ++sl) {
            const int q = s.nbr[(size_t)i * VCFV_SLOTS + sl];
            if (q < 0) continue;
            if (q <= prev)
                return fail("vertex numbering is not the grid's natural order (x fastest)", GBFV_ERR_UNSUPPORTED);
            prev = q;
        }
    }
    return GBFV_OK;
}

VcfvDev* vcfvUpload(const gbfv_problem* P, const VcfvSetup& s, const DevPhysics& ph, const std::vector<int>& perm,
                    int ld, int* status)
{
    VcfvDev* d = new VcfvDev();
    auto fail = [&](int st) -> VcfvDev* {
        if (status) *status = st;
        vcfvDestroy(d);
        return nullptr;
    };
    const int N = s.N, E = s.E;
    d->E = E;
    d->N = N;
    d->ld = ld;
    d->p1 = P->p1_gradients ? 1 : 0;
    d->b = P->model == GBFV_MODEL_BLACKOIL_3P ? 3 : 2;
    d->rhoRef[0] = ph.pvt.rhoRefW;
    d->rhoRef[1] = ph.pvt.rhoRefO;
    d->rhoRef[2] = ph.pvt.rhoRefG;
    std::vector<ElemGeo> geo(E);
    std::vector<int> bfPtr(E + 1, 0);
    std::vector<BFaceV> bf;
    const double* g = P->gravity;
    for (int e = 0; e < E; ++e) {
        const int* cn = &P->elem_corner[4 * e];
        const HostElem H = hostElem(P, cn);
        ElemGeo& G = geo[e];
        std::memset(&G, 0, sizeof(G));
        for (int c = 0; c < 4; ++c) {
            G.v[c] = perm[cn[c]];
            G.scvVol[c] = H.scvVol[c];
        }
        for (int k = 0; k < 4; ++k) {
            const int i = H.fi[k], j = H.fj[k];
            if (i != (k == 0 ? 2 : k == 1 ? 1 : k == 2 ? 0 : 3) || j != (k == 0 ? 0 : k == 1 ? 3 : k == 2 ? 1 : 2)) {
                setLastError("vertex-centred grid: face corner table mismatch");
                return fail(GBFV_ERR_UNSUPPORTED);
            }
            G.fa[k] = H.fa[k];
            double distSq = 0.0;
            for (int dd = 0; dd < 2; ++dd) {
                G.fn[k][dd] = H.fn[k][dd];
                G.Kh[k][dd] = harmonicMeanV(P->perm[3 * cn[i] + dd], P->perm[3 * cn[j] + dd]);
                const double t = H.vpos[j][dd] - H.vpos[i][dd];
                distSq += t * t;
            }
            double dIn[2], dEx[2];
            for (int dd = 0; dd < 2; ++dd) {
                dIn[dd] = H.vpos[i][dd] - H.fip[k][dd];
                dEx[dd] = H.vpos[j][dd] - H.fip[k][dd];
                G.dTot[k][dd] = H.vpos[j][dd] - H.vpos[i][dd];
            }
            G.absTot2[k] = G.dTot[k][0] * G.dTot[k][0] + G.dTot[k][1] * G.dTot[k][1];
            double gIn = 0.0, gEx = 0.0;
            for (int dd = 0; dd < 2; ++dd) gIn += g[dd] * dIn[dd];
            for (int dd = 0; dd < 2; ++dd) gEx += g[dd] * dEx[dd];
            G.gIn[k] = gIn;
            G.gEx[k] = gEx;
            for (int dd = 0; dd < 2; ++dd) G.w2p[k][dd] = (H.vpos[j][dd] - H.vpos[i][dd]) / distSq;
            for (int c = 0; c < 4; ++c)
                for (int dd = 0; dd < 2; ++dd) G.grad[k][c][dd] = H.grad[k][c][dd];
        }
        // boundary sub-control-volume faces, the free-flow states on the host
        for (int b = P->bface_ptr[e]; b < P->bface_ptr[e + 1]; ++b) {
            BFaceV B;
            std::memset(&B, 0, sizeof(B));
            const int c = P->bface_corner[b];
            const int vn = cn[c];
            B.c = c;
            B.type = P->bface_type ? P->bface_type[b] : GBFV_BC_NOFLOW;
            B.area = P->bface_area[b];
            const double* xf = &P->bface_center[3 * b];
            const double* xc = H.scvCenter[c];
            double distSq = 0.0;
            for (int dd = 0; dd < 2; ++dd) {
                const double t = xf[dd] - xc[dd];
                distSq += t * t;
            }
            for (int dd = 0; dd < 2; ++dd) {
                B.n[dd] = P->bface_normal[3 * b + dd];
                B.w[dd] = (xf[dd] - xc[dd]) / distSq;
                B.dIn[dd] = H.vpos[c][dd] - xf[dd];
                B.K[dd] = P->perm[3 * vn + dd];
            }
            double absDist2 = 0.0, gTimesDist = 0.0;
            for (int dd = 0; dd < 2; ++dd) absDist2 += B.dIn[dd] * B.dIn[dd];
            for (int dd = 0; dd < 2; ++dd) gTimesDist += g[dd] * B.dIn[dd];
            B.absDist2 = absDist2;
            B.gTimesDist = gTimesDist;
            const double* val = &P->bface_value[4 * b];
            if (B.type == GBFV_BC_MASSRATE) {
                for (int q = 0; q < d->b; ++q) B.rate[q] = val[q];
            }
            else if (B.type == GBFV_BC_FREEFLOW) {
                const TwoPhaseLaw& L = ph.law[P->material[vn]];
                const double pw = val[0], Swb = val[1];
                const double sumRes = L.Swr + L.Snr;
                const double SwE = (Swb - L.Swr) / (1.0 - sumRes);
                const double SnE = ((1 - Swb) - L.Snr) / (1.0 - sumRes);
                const double pcn = pcnw(L, SwE);
                B.pb[0] = pw;
                B.pb[1] = pw + pcn - 0.0;
                const double krb[2] = {krw(L, SwE), krn(L, 1.0 - SnE)};
                for (int a = 0; a < 2; ++a) {
                    B.mobb[a] = krb[a] / P->mu[a];
                    B.rhob[a] = P->rho[a];
                }
            }
            else if (B.type != GBFV_BC_NOFLOW) {
                setLastError("vertex-centred grid: unknown boundary type");
                return fail(GBFV_ERR_ARG);
            }
            bf.push_back(B);
        }
        bfPtr[e + 1] = (int)bf.size();
    }
    // vertex -> (element, corner) in element order, and the slot of each of
    // the element's corners in the vertex's row
    std::vector<int> inc((size_t)4 * ld, -1);
    std::vector<unsigned char> incSlot((size_t)16 * ld, 0);
    std::vector<int> cnt(N, 0);
    for (int e = 0; e < E; ++e) {
        const int* cn = &P->elem_corner[4 * e];
        for (int c = 0; c < 4; ++c) {
            const int vn = cn[c], p = perm[vn];
            const int k = cnt[vn]++;
            if (k >= 4) {
                setLastError("vertex-centred grid: a vertex in more than four elements");
                return fail(GBFV_ERR_UNSUPPORTED);
            }
            inc[(size_t)k * ld + p] = e * 4 + c;
            for (int f = 0; f < 4; ++f)
                incSlot[((size_t)k * 4 + f) * ld + p] =
                    (unsigned char)slotOf(&P->center[3 * vn], &P->center[3 * cn[f]]);
        }
    }
    auto upload = [&](auto** dst, const auto& vec) -> bool {
        using T = typename std::decay<decltype(vec)>::type::value_type;
        const size_t bytes = sizeof(T) * std::max<size_t>(1, vec.size());
        if (cudaMalloc((void**)dst, bytes) != cudaSuccess) return false;
        return vec.empty() || cudaMemcpy(*dst, vec.data(), sizeof(T) * vec.size(), cudaMemcpyHostToDevice) == cudaSuccess;
    };
    if (!upload(&d->geo, geo) || !upload(&d->bfPtr, bfPtr) || !upload(&d->bf, bf) || !upload(&d->inc, inc) ||
        !upload(&d->incSlot, incSlot))
        return fail(GBFV_ERR_OOM);
    d->nbf = (int)bf.size();
    if (cudaMalloc((void**)&d->R, sizeof(double) * (size_t)E * 4 * d->b) != cudaSuccess ||
        cudaMalloc((void**)&d->J, sizeof(double) * (size_t)E * 16 * d->b * d->b) != cudaSuccess)
        return fail(GBFV_ERR_OOM);
    if (status) *status = GBFV_OK;
    return d;
}

void vcfvDestroy(VcfvDev* d)
{
    if (!d) return;
    cudaFree(d->geo);
    cudaFree(d->bfPtr);
    cudaFree(d->bf);
    cudaFree(d->inc);
    cudaFree(d->incSlot);
    cudaFree(d->R);
    cudaFree(d->J);
    delete d;
}

double vcfvLinearizeBytes(const VcfvDev* d)
{
    // element pass: geometry, 4 corners' values, the focus derivatives and
    // storage, the scratch records; gather: incidence, scratch, the row
    const double E = d->E, N = d->N;
    const double elem = E * 4 * (sizeof(ElemGeo) / 4.0 + 4 * 6 * 8 + 12 * 8 + 4 * 6 * 8 + 72 * 8 / 4.0);
    const double bnd = (double)d->nbf * sizeof(BFaceV) * 4;
    const double gather = N * (4 * 4 + 16 + 4 * (8 * 2 + 4 * 32) + VCFV_SLOTS * 32 + 16);
    return elem + bnd + gather;
}

namespace {
VcfvArgs vcfvArgs(const VcfvDev* d)
{
    VcfvArgs a;
    a.E = d->E;
    a.ld = d->ld;
    a.geo = d->geo;
    a.bfPtr = d->bfPtr;
    a.bf = d->bf;
    a.inc = d->inc;
    a.incSlot = d->incSlot;
    a.R = d->R;
    a.J = d->J;
    a.p1 = d->p1;
    for (int k = 0; k < 3; ++k) a.rhoRef[k] = d->rhoRef[k];
    return a;
}
}  // namespace

void launchVcfvAssembleFd(const VcfvDev* d, const DevMesh& m, IqBuffers iq0, const FdIq& fd, const double* refP,
                          int method, double* storageOld, int iter0, double dt, double* residual, double* jval,
                          cudaStream_t s)
{
    const VcfvArgs a = vcfvArgs(d);
    const int nt = 4 * d->E;
    if (d->p1) kVcfvElementFd<true><<<(nt + 127) / 128, 128, 0, s>>>(a, m, iq0, fd, refP, method, storageOld, iter0, dt);
    else kVcfvElementFd<false><<<(nt + 127) / 128, 128, 0, s>>>(a, m, iq0, fd, refP, method, storageOld, iter0, dt);
    kVcfvGather<2><<<(m.N + 127) / 128, 128, 0, s>>>(a, m, iq0, storageOld, iter0, residual, jval);
    countLaunch(2);
}

void launchVcfvAssemble(const VcfvDev* d, const DevMesh& m, IqBuffers iq, double* storageOld, int iter0, double dt,
                        double* residual, double* jval, cudaStream_t s)
{
    const VcfvArgs a = vcfvArgs(d);
    const int nt = 4 * d->E;
    const int nb = (nt + 127) / 128, ng = (m.N + 127) / 128;
    if (d->b == 3) {
        if (d->p1) kVcfvElement<3, true><<<nb, 128, 0, s>>>(a, m, iq, storageOld, iter0, dt);
        else kVcfvElement<3, false><<<nb, 128, 0, s>>>(a, m, iq, storageOld, iter0, dt);
        kVcfvGather<3><<<ng, 128, 0, s>>>(a, m, iq, storageOld, iter0, residual, jval);
    }
    else {
        if (d->p1) kVcfvElement<2, true><<<nb, 128, 0, s>>>(a, m, iq, storageOld, iter0, dt);
        else kVcfvElement<2, false><<<nb, 128, 0, s>>>(a, m, iq, storageOld, iter0, dt);
        kVcfvGather<2><<<ng, 128, 0, s>>>(a, m, iq, storageOld, iter0, residual, jval);
    }
    countLaunch(2);
}

}  // namespace gbfv
