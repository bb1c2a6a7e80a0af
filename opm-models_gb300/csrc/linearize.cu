// Linearization kernels: intensive quantities (K1), cell-centric TPFA
// assembly (K2), constraints, Newton error and Newton update (K7).
//
// This translation unit is compiled with -fmad=false: the FP64 residual and
// Jacobian follow the reference's operation order term by term, so they can
// be compared with the CPU restatement at the 1e-12 level.
//
// K2 mirrors the reference's element loop (fvbaselinearizer.hh:510-626 with
// FvBaseAdLocalLinearizer, fvbaseadlocallinearizer.hh:173-292): cell I's
// faces are evaluated with derivatives with respect to x_I only, giving the
// residual row I, the diagonal block (I,I) and the column blocks (J,I) of
// its neighbours.  The single-system AD path runs it face-parallel: a group
// of 2*dim lanes per cell, one lane per intersection, the cell's own dual
// quantities staged in shared memory, the faces summed in intersection
// order from warp shuffles.  The batched and finite-difference paths run
// one thread per cell.  Each block has exactly one writer, so there are no
// atomics and the summation order inside a row is the reference's:
// interior faces in intersection order, storage, boundary faces.  The
// expensive intensive quantities (pow-heavy material laws, PVT tables) are
// computed once per cell by K1 and read back -- FP64 arithmetic is the scarce
// resource on this GPU, bytes are cheap.
#include <cstdlib>

#include "../../include/gbfv.h"
#include "gbfv_internal.cuh"

namespace gbfv {

using D2 = Dual<2>;
using D3 = Dual<3>;

// ------------------------------------------------------- constraints -----
// FvBaseLinearizer::applyConstraintsToSolution_ (fvbaselinearizer.hh:630-645)
__device__ __forceinline__ void kApplyConstraintsBody(const DevMesh& m, double* __restrict__ x, double* __restrict__ xOld,
                                  int* __restrict__ meaning, int* __restrict__ meaningOld, const int k)
{
    if (k >= m.numConsCells) return;
    const int p = m.consCells[k];
    const int c = m.consOf[k];
    for (int e = 0; e < m.b; ++e) {
        x[p * m.b + e] = m.consPv[3 * c + e];
        xOld[p * m.b + e] = m.consPv[3 * c + e];
    }
    meaning[p] = m.consMeaning[c];
    meaningOld[p] = m.consMeaning[c];
}

// FvBaseLinearizer::applyConstraintsToSolution_ (fvbaselinearizer.hh:630-645)
__global__ void kApplyConstraints(DevMesh m, double* __restrict__ x, double* __restrict__ xOld,
                                  int* __restrict__ meaning, int* __restrict__ meaningOld)
{
    kApplyConstraintsBody(m, x, xOld, meaning, meaningOld, blockIdx.x * blockDim.x + threadIdx.x);
}

void launchApplyConstraints(const DevMesh& m, double* x, double* xOld, int* meaning, int* meaningOld,
                            cudaStream_t s)
{
    if (m.numConsCells == 0) return;
    kApplyConstraints<<<(m.numConsCells + 127) / 128, 128, 0, s>>>(m, x, xOld, meaning, meaningOld);
    countLaunch();
}

// ------------------------------------------------------------- K1 --------
// ImmiscibleIntensiveQuantities::update (immiscibleintensivequantities.hh:93-151)
// and ImmiscibleLocalResidual::computeStorage (immisciblelocalresidual.hh:75-109)
// out (output fields, see launchOutputFields): nullptr in the linearization
__device__ __forceinline__ void kIqImmiscibleBody(const DevMesh& m, const DevPhysics* __restrict__ phys,
                                                     const double* __restrict__ x, IqBuffers iq, const int p,
                                                     double* __restrict__ out = nullptr)
{
    if (p >= m.N) return;
    const int ld = m.ldN;
    const TwoPhaseLaw L = phys->law[m.material[p]];
    const double pv0 = x[2 * p + 0], pv1 = x[2 * p + 1];
    D2 sumSat(0.0);
    D2 Sw = D2::var(pv1, 1);
    D2 S[2];
    S[0] = Sw;
    sumSat = sumSat + Sw;
    S[1] = 1.0 - sumSat;
    const double sumRes = L.Swr + L.Snr;
    D2 SwE = (S[0] - L.Swr) / (1.0 - sumRes);
    D2 SnE = (S[1] - L.Snr) / (1.0 - sumRes);
    D2 pc[2];
    pc[0] = D2(0.0);
    pc[1] = pcnw(L, SwE);
    D2 kr[2];
    kr[0] = krw(L, SwE);
    kr[1] = krn(L, 1.0 - SnE);
    D2 p0 = D2::var(pv0, 0);
    D2 pr[2], rho[2], lam[2];
    for (int a = 0; a < 2; ++a) pr[a] = p0 + (pc[a] - pc[0]);
    for (int a = 0; a < 2; ++a) {
        D2 mu(phys->mu[a]);
        rho[a] = D2(phys->rho[a]);
        lam[a] = kr[a] / mu;
    }
    const double phi = m.porosity[p];
    const D2* q[6] = {&pr[0], &pr[1], &rho[0], &rho[1], &lam[0], &lam[1]};
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        iq.val[k * ld + p] = q[k]->v;
        iq.der[(k * 2 + 0) * ld + p] = q[k]->d[0];
        iq.der[(k * 2 + 1) * ld + p] = q[k]->d[1];
    }
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        D2 st = (D2(phi) * S[a]) * rho[a];
        iq.sto[(a * 3 + 0) * ld + p] = st.v;
        iq.sto[(a * 3 + 1) * ld + p] = st.d[0];
        iq.sto[(a * 3 + 2) * ld + p] = st.d[1];
    }
    if (out) {
        for (int a = 0; a < 2; ++a) {
            out[(0 * 3 + a) * ld + p] = pr[a].v;
            out[(1 * 3 + a) * ld + p] = rho[a].v;
            out[(2 * 3 + a) * ld + p] = S[a].v;
            out[(3 * 3 + a) * ld + p] = lam[a].v;
            out[(4 * 3 + a) * ld + p] = kr[a].v;
            out[(5 * 3 + a) * ld + p] = phys->mu[a];
        }
        for (int q = 0; q < 6; ++q) out[(q * 3 + 2) * ld + p] = 0.0;
        out[18 * ld + p] = phi;
    }
}

// ImmiscibleIntensiveQuantities::update (immiscibleintensivequantities.hh:93-151)
// and the storage term (immisciblelocalresidual.hh:99-109), once per cell
__global__ void __launch_bounds__(256) kIqImmiscible(DevMesh m, const DevPhysics* __restrict__ phys,
                                                     const double* __restrict__ x, IqBuffers iq)
{
    kIqImmiscibleBody(m, phys, x, iq, blockIdx.x * blockDim.x + threadIdx.x);
}

// BlackOilIntensiveQuantities::update (blackoilintensivequantities.hh:179-462)
// for water meaning Sw, pressure meaning Po, gas meaning Sg / Rs, zero p_c,
// Corey relperm via updateRelperms; storage per blackoillocalresidual.hh:101-188
__device__ __forceinline__ void kIqBlackoilBody(const DevMesh& m, const DevPhysics* __restrict__ phys,
                                                   const double* __restrict__ x,
                                                   const int* __restrict__ meaning, IqBuffers iq, const int p,
                                                   double* __restrict__ out = nullptr)
{
    if (p >= m.N) return;
    const int ld = m.ldN;
    const BlackOilPvt& T = phys->pvt;
    const double pv0 = x[3 * p + 0], pv1 = x[3 * p + 1], pv2 = x[3 * p + 2];
    const int gm = meaning[p];
    D3 Sw = D3::var(pv0, 0);
    D3 Sg(0.0);
    if (gm == GBFV_GAS_SG) Sg = D3::var(pv2, 2);
    D3 So = 1.0 - Sw - Sg;
    D3 S[3] = {Sw, So, Sg};
    const double n = phys->coreyN[m.material[p]];
    D3 kr[3];
    for (int a = 0; a < 3; ++a) kr[a] = corey(S[a], n);
    D3 po = D3::var(pv1, 1) * 1.0;
    D3 pr = po + (D3(0.0) - D3(0.0));
    D3 RsSat = tableEval(T.rsSat, pr);
    D3 Rs = gm == GBFV_GAS_RS ? D3::var(pv2, 2) : RsSat;
    D3 invB[3], mu[3];
    invB[0] = waterInvB(T, pr);
    mu[0] = D3(T.muw);
    const bool sat = S[2].v > 0.0 && Rs.v >= (1.0 - 1e-10) * RsSat.v;
    if (sat) {
        invB[1] = tableEval(T.invBoSat, pr);
        mu[1] = tableEval(T.muoSat, pr);
    }
    else {
        D3 pb = tableEval(T.pBubble, Rs);
        D3 ib = tableEval(T.invBoSat, pb);
        invB[1] = ib * (1.0 + T.oilComp * (pr - pb));
        mu[1] = tableEval(T.muoSat, pb);
    }
    invB[2] = tableEval(T.invBg, pr);
    mu[2] = tableEval(T.mug, pr);
    D3 lam[3], rho[3];
    for (int a = 0; a < 3; ++a) lam[a] = kr[a] / mu[a];
    rho[0] = invB[0] * T.rhoRefW;
    rho[2] = invB[2] * T.rhoRefG;
    rho[1] = invB[1] * T.rhoRefO;
    rho[1] = rho[1] + invB[1] * Rs * T.rhoRefG;
    const double phi = m.porosity[p];
    // values: p, rho0..2, lam0..2, invB0..2, Rs ; derivatives for all but p
    iq.val[0 * ld + p] = pr.v;
    const D3* q[10] = {&rho[0], &rho[1], &rho[2], &lam[0], &lam[1], &lam[2],
                       &invB[0], &invB[1], &invB[2], &Rs};
#pragma unroll
    for (int k = 0; k < 10; ++k) {
        iq.val[(k + 1) * ld + p] = q[k]->v;
#pragma unroll
        for (int j = 0; j < 3; ++j) iq.der[(k * 3 + j) * ld + p] = q[k]->d[j];
    }
    D3 tmp[3] = {D3(0.0), D3(0.0), D3(0.0)};
    const int comp[3] = {1, 0, 2};
    D3 dphi(phi);
    for (int a = 0; a < 3; ++a) {
        D3 sv = S[a] * invB[a] * dphi;
        tmp[comp[a]] = tmp[comp[a]] + sv;
        if (a == 1) tmp[2] = tmp[2] + Rs * sv;
    }
    tmp[1] = tmp[1] * T.rhoRefW;
    tmp[2] = tmp[2] * T.rhoRefG;
    tmp[0] = tmp[0] * T.rhoRefO;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        iq.sto[(e * 4 + 0) * ld + p] = tmp[e].v;
#pragma unroll
        for (int j = 0; j < 3; ++j) iq.sto[(e * 4 + 1 + j) * ld + p] = tmp[e].d[j];
    }
    if (out) {
        for (int a = 0; a < 3; ++a) {
            out[(0 * 3 + a) * ld + p] = pr.v;
            out[(1 * 3 + a) * ld + p] = rho[a].v;
            out[(2 * 3 + a) * ld + p] = S[a].v;
            out[(3 * 3 + a) * ld + p] = lam[a].v;
            out[(4 * 3 + a) * ld + p] = kr[a].v;
            out[(5 * 3 + a) * ld + p] = mu[a].v;
        }
        out[18 * ld + p] = phi;
    }
}

// BlackOilIntensiveQuantities::update (blackoilintensivequantities.hh:179-470)
// and the storage term (blackoillocalresidual.hh:102-188), once per cell
__global__ void __launch_bounds__(256) kIqBlackoil(DevMesh m, const DevPhysics* __restrict__ phys,
                                                   const double* __restrict__ x,
                                                   const int* __restrict__ meaning, IqBuffers iq)
{
    kIqBlackoilBody(m, phys, x, meaning, iq, blockIdx.x * blockDim.x + threadIdx.x);
}

// The output quantities of the current state (the values the reference's
// VtkMultiPhaseModule reads from the intensive quantities,
// vtkmultiphasemodule.hh:195-260): the intensive-quantity pass with its
// values also written to out[plane*ldN + p], planes [q*3 + phase] for q =
// pressure, density, saturation, mobility, relative permeability, viscosity,
// and plane 18 the porosity
__global__ void __launch_bounds__(256) kOutputFields(DevMesh m, const DevPhysics* __restrict__ phys,
                                                     const double* __restrict__ x, const int* __restrict__ meaning,
                                                     IqBuffers iq, double* __restrict__ out)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (m.model == GBFV_MODEL_IMMISCIBLE_2P) kIqImmiscibleBody(m, phys, x, iq, p, out);
    else kIqBlackoilBody(m, phys, x, meaning, iq, p, out);
}

void launchOutputFields(const DevMesh& m, const DevPhysics* phys, const double* x, const int* meaning,
                        IqBuffers iq, double* out, cudaStream_t s)
{
    const int bs = 256, nb = (m.N + bs - 1) / bs;
    kOutputFields<<<nb, bs, 0, s>>>(m, phys, x, meaning, iq, out);
    countLaunch();
}

void launchIq(const DevMesh& m, const DevPhysics* phys, const double* x, const int* meaning,
              IqBuffers iq, cudaStream_t s)
{
    const int bs = 256, nb = (m.N + bs - 1) / bs;
    if (m.model == GBFV_MODEL_IMMISCIBLE_2P)
        kIqImmiscible<<<nb, bs, 0, s>>>(m, phys, x, iq);
    else
        kIqBlackoil<<<nb, bs, 0, s>>>(m, phys, x, meaning, iq);
    countLaunch();
}

// ------------------------------------------------------------- K2 --------
// load a dual from the IQ buffers
template <int B>
__device__ __forceinline__ Dual<B> ldDual(const IqBuffers& iq, int ld, int qv, int qd, int p)
{
    Dual<B> r;
    r.v = iq.val[qv * ld + p];
#pragma unroll
    for (int j = 0; j < B; ++j) r.d[j] = iq.der[(qd * B + j) * ld + p];
    return r;
}

// write block (row q, slot s) = -flux.d / V_q (zero in constraint rows)
template <int B>
__device__ __forceinline__ void writeOffBlock(double* __restrict__ jval, int ld, int slot, int q,
                                              const Dual<B>* flux, double Vq, bool zero)
{
    const double iv = 1.0 / Vq;  // Jacobian entries only: one reciprocal per block
#pragma unroll
    for (int e = 0; e < B; ++e)
#pragma unroll
        for (int v = 0; v < B; ++v) {
            const double d = zero ? 0.0 : (0.0 - flux[e].d[v]) * iv;
            jval[(slot * B * B + e * B + v) * ld + q] = d;
        }
}

// Axis-aligned Darcy flux of one phase, focus = interior cell
// (darcyfluxmodule.hh:183-322, 459-525).  Components of the gradient off the
// face axis are exact zeros, so only the axis component is carried.
template <int B>
__device__ __forceinline__ Dual<B> darcyPhase(const Dual<B>& pI, double pJ, const Dual<B>& rhoI,
                                              double rhoJ, const Dual<B>& lamI, double lamJ,
                                              double dTot, double gIn, double gEx, double Kh,
                                              double nrm, bool& upI)
{
    const double distSq = dTot * dTot;
    Dual<B> deltay = pJ - pI;
    Dual<B> pg = deltay * (dTot / distSq);
    Dual<B> pStatIn = (-rhoI) * gIn;
    const double pStatEx = (-rhoJ) * gEx;
    Dual<B> fs = (pStatEx - pStatIn) / distSq;
    pg = pg + dTot * fs;
    const double t = pg.v * nrm;
    upI = !(t > 0.0);
    Dual<B> mob = upI ? lamI : Dual<B>(lamJ);
    Dual<B> fv = Kh * pg;
    fv = fv * (-mob);
    return fv * nrm;
}

// Transmissibility flux of one phase, focus = interior cell
// (transfluxmodule.hh:201-318): hydrostatic correction with the average
// density, upwind by the sign of the pressure difference, ties decided on the
// host (larger volume, then lower global index), q = dp * lambda_up * (-T).
__device__ __forceinline__ D2 transPhase(const D2& pI, double pJ, const D2& rhoI, double rhoJ, const D2& lamI,
                                         double lamJ, double T, double dzg, bool tieUpI, bool& upI)
{
    if (lamI.v <= 0.0 && lamJ <= 0.0) {
        upI = true;
        return D2(0.0);
    }
    D2 rhoAvg = (rhoI + rhoJ) / 2.0;
    D2 pEx(pJ);
    pEx = pEx + rhoAvg * dzg;
    D2 pd = pEx - pI;
    upI = pd.v > 0.0 ? false : (pd.v < 0.0 ? true : tieUpI);
    if (upI) return (pd * lamI) * (-T);
    return pd * (lamJ * (-T));
}

// One phase's flux of BlackOilLocalResidualTPFA::calculateFluxes_
// (blackoillocalresidualtpfa.hh:334-385), focus = interior cell: darcy =
// dp * mob_up * transMult * (-T / A).  The pressure difference and the
// upstream choice are the transmissibility module's (transfluxmodule.hh:
// 201-318: the average density times the depth term, the sign of the
// difference, ties by volume then global index), which the reference's
// TPFA path takes from its flux module.  transMult, the rock-compaction
// multiplier average, is 1 here (no rock compaction) and multiplying by it
// changes no bit, so it is left out.
template <int B>
__device__ __forceinline__ Dual<B> tpfaPhase(const Dual<B>& pI, double pJ, const Dual<B>& rhoI, double rhoJ,
                                             const Dual<B>& lamI, double lamJ, double T, double area, double dzg,
                                             bool tieUpI, bool& upI)
{
    Dual<B> rhoAvg = (rhoI + rhoJ) / 2.0;
    Dual<B> pEx(pJ);
    pEx = pEx + rhoAvg * dzg;
    Dual<B> pd = pEx - pI;
    upI = pd.v > 0.0 ? false : (pd.v < 0.0 ? true : tieUpI);
    const double f = -T / area;
    if (upI) return (pd * lamI) * f;
    return pd * (lamJ * f);
}

// The local residual of element p (FvBaseLocalResidual::eval,
// fvbaselocalresidual.hh:158-191) divided by its volume, in three parts so
// that a cell-parallel and a face-parallel kernel run the same operations:
// the element's own intensive quantities as duals, one interior face's flux
// (times the face area), and the terms after the faces (storage, boundary
// faces, the division by the volume).
struct OwnImmiscible {
    D2 pI[2], rhoI[2], lamI[2];
};

__device__ __forceinline__ void ownImmiscible(const DevMesh& m, const IqBuffers& iq, const int p, OwnImmiscible& o)
{
    const int ld = m.ldN;
    for (int a = 0; a < 2; ++a) {
        o.pI[a] = ldDual<2>(iq, ld, a, a, p);
        o.rhoI[a] = ldDual<2>(iq, ld, 2 + a, 2 + a, p);
        o.lamI[a] = ldDual<2>(iq, ld, 4 + a, 4 + a, p);
    }
}

// interior face `dir` of element p with the neighbour's values from `nbr`:
// false when the cell has no neighbour there
__device__ __forceinline__ bool faceImmiscible(const DevMesh& m, const OwnImmiscible& o, const IqBuffers& nbr,
                                               const int p, const int dir, int& q, D2 (&flux)[2])
{
    const int ld = m.ldN;
    q = m.nbr[dir * ld + p];
    if (q < 0) return false;
    const double dTot = m.dTot[dir * ld + p];
    const double gIn = m.gIn[dir * ld + p];
    const double gEx = m.gEx[dir * ld + p];
    const double Kh = m.Kh[dir * ld + p];
    const double area = m.area[dir * ld + p];
    const double nrm = (dir & 1) ? 1.0 : -1.0;
    for (int a = 0; a < 2; ++a) {
        const double pJ = nbr.val[a * ld + q];
        const double rhoJ = nbr.val[(2 + a) * ld + q];
        const double lamJ = nbr.val[(4 + a) * ld + q];
        bool upI;
        D2 vf = m.fluxModule == GBFV_FLUX_TRANS
                    ? transPhase(o.pI[a], pJ, o.rhoI[a], rhoJ, o.lamI[a], lamJ, m.trans[dir * ld + p],
                                 m.dzg[dir * ld + p], m.tieUpI[dir * ld + p] != 0, upI)
                    : darcyPhase<2>(o.pI[a], pJ, o.rhoI[a], rhoJ, o.lamI[a], lamJ, dTot, gIn, gEx, Kh, nrm, upI);
        flux[a] = D2(0.0) + (upI ? vf * o.rhoI[a] : vf * rhoJ);
    }
    double alpha = 1.0;
    alpha *= area;
    for (int e = 0; e < 2; ++e) flux[e] = flux[e] * alpha;
    return true;
}

// the terms after the interior faces for equation e (storage, boundary
// faces, / V); the equations do not mix, so a lane per equation gives the
// same results as one thread for all
__device__ __forceinline__ void tailImmiscibleEq(const DevMesh& m, const OwnImmiscible& o, const IqBuffers& iq,
                                                 double* __restrict__ storageOld, int iter0, double dt, const int p,
                                                 const int e, D2& r)
{
    const int ld = m.ldN;
    const double V = m.volume[p];
    const double scvVolume = V * 1.0;
    {
        D2 tmp;
        tmp.v = iq.sto[(e * 3 + 0) * ld + p];
        tmp.d[0] = iq.sto[(e * 3 + 1) * ld + p];
        tmp.d[1] = iq.sto[(e * 3 + 2) * ld + p];
        double tmp2;
        if (iter0) {
            tmp2 = tmp.v;
            storageOld[e * ld + p] = tmp2;
        }
        else
            tmp2 = storageOld[e * ld + p];
        tmp = tmp - tmp2;
        tmp = tmp * (scvVolume / dt);
        r = r + tmp;
    }
    r = r - 0.0 * scvVolume;
    const int a = e;  // equation e is phase e's conservation
    for (int f = m.bfPtr[p]; f < m.bfPtr[p + 1]; ++f) {
        const BFace bf = m.bfaces[f];
        D2 value(0.0);
        if (bf.type == GBFV_BC_MASSRATE) {
            value = D2(bf.rate[e]);
        }
        else if (bf.type == GBFV_BC_FREEFLOW && m.fluxModule == GBFV_FLUX_TRANS) {
            // calculateBoundaryGradients_ of the transmissibility module (transfluxmodule.hh:324-415)
            D2 rhoAvg = (o.rhoI[a] + bf.rhob[a]) / 2.0;
            D2 pEx(bf.pb[a]);
            pEx = pEx + rhoAvg * bf.dzgB;
            D2 pd = pEx - o.pI[a];
            D2 vf = pd.v > 0.0 ? (pd * bf.mobb[a]) * (-bf.transB) : (pd * o.lamI[a]) * (-bf.transB);
            D2 dens = bf.pb[a] > o.pI[a].v ? D2(bf.rhob[a]) : o.rhoI[a];
            value = value + vf * dens;
        }
        else if (bf.type == GBFV_BC_FREEFLOW) {
            const double distSq = bf.tmpA * bf.tmpA;
            const double absDist2 = bf.dInA * bf.dInA;
            const double K = m.perm[bf.axis * ld + p];
            D2 deltay = bf.pb[a] - o.pI[a];
            D2 pg = deltay * (bf.tmpA / distSq);
            D2 pStatIn = (-bf.gTimesDist) * o.rhoI[a];
            D2 fsc = pStatIn / absDist2;
            pg = pg + bf.dInA * fsc;
            const double t = pg.v * bf.nrm;
            D2 mob = t > 0.0 ? D2(bf.mobb[a]) : o.lamI[a];
            D2 fv = K * pg;
            fv = fv * (-mob);
            D2 vf = fv * bf.nrm;
            D2 dens = bf.pb[a] > o.pI[a].v ? D2(bf.rhob[a]) : o.rhoI[a];
            value = value + vf * dens;
        }
        const double aa = bf.area * 1.0;
        value = value * aa;
        r = r + value;
    }
    r = r / V;
}

__device__ __forceinline__ void tailImmiscible(const DevMesh& m, const OwnImmiscible& o, const IqBuffers& iq,
                                               double* __restrict__ storageOld, int iter0, double dt, const int p,
                                               D2 (&res)[2])
{
    for (int e = 0; e < 2; ++e) tailImmiscibleEq(m, o, iq, storageOld, iter0, dt, p, e, res[e]);
}

// the whole local residual of element p, its faces in intersection order;
// each interior face's flux (times the face area) also goes to
// sink(dir, q, flux).  `iq`: the element's own intensive quantities, `nbr`:
// its neighbours' (the same buffers for AD; the deflected state of p for
// finite differences)
template <class Sink>
__device__ __forceinline__ void localImmiscible(const DevMesh& m, const IqBuffers& iq, const IqBuffers& nbr,
                                                double* __restrict__ storageOld, int iter0, double dt, const int p,
                                                D2 (&res)[2], Sink& sink)
{
    OwnImmiscible o;
    ownImmiscible(m, iq, p, o);
    res[0] = D2(0.0);
    res[1] = D2(0.0);
    const int ndir = 2 * m.dim;
    for (int dir = 0; dir < ndir; ++dir) {
        int q;
        D2 flux[2];
        if (!faceImmiscible(m, o, nbr, p, dir, q, flux)) continue;
        for (int e = 0; e < 2; ++e) res[e] = res[e] + flux[e];
        sink(dir, q, flux);
    }
    tailImmiscible(m, o, iq, storageOld, iter0, dt, p, res);
}

// AD: a face's flux derivatives are the off-diagonal block (q, p)
template <int B>
struct OffBlockSink {
    const DevMesh& m;
    double* jval;
    __device__ void operator()(int dir, int q, const Dual<B>* flux) const
    {
        // the TPFA linearizer's rows are not divided by the volume: V = 1 is exact
        writeOffBlock<B>(jval, m.ldN, m.slotOfDir[dir ^ 1], q, flux, m.tpfa ? 1.0 : m.volume[q], m.cflag[q] >= 0);
    }
};

// the residual row and diagonal block of element p (identity in constraint rows)
template <int B>
__device__ __forceinline__ void writeDiag(const DevMesh& m, const Dual<B> (&res)[B], double* __restrict__ residual,
                                          double* __restrict__ jval, const int p)
{
    const int ld = m.ldN;
    const bool cons = m.cflag[p] >= 0;
    const int ds = m.dim;  // diagonal slot
    for (int e = 0; e < B; ++e) {
        residual[B * p + e] = cons ? 0.0 : res[e].v;
        for (int v = 0; v < B; ++v)
            jval[(ds * B * B + e * B + v) * ld + p] = cons ? (e == v ? 1.0 : 0.0) : res[e].d[v];
    }
}

// row e of it
template <int B>
__device__ __forceinline__ void writeDiagRow(const DevMesh& m, const Dual<B>& r, const int e,
                                             double* __restrict__ residual, double* __restrict__ jval, const int p)
{
    const int ld = m.ldN;
    const bool cons = m.cflag[p] >= 0;
    const int ds = m.dim;
    residual[B * p + e] = cons ? 0.0 : r.v;
    for (int v = 0; v < B; ++v) jval[(ds * B * B + e * B + v) * ld + p] = cons ? (e == v ? 1.0 : 0.0) : r.d[v];
}

__device__ __forceinline__ void kAssembleImmiscibleBody(const DevMesh& m, const DevPhysics* __restrict__ phys,
                                                           IqBuffers iq, double* __restrict__ storageOld,
                                                           int iter0, double dt,
                                                           double* __restrict__ residual,
                                                           double* __restrict__ jval, const int p)
{
    if (p >= m.N) return;
    OffBlockSink<2> sink{m, jval};
    D2 res[2];
    localImmiscible(m, iq, iq, storageOld, iter0, dt, p, res, sink);
    writeDiag<2>(m, res, residual, jval, p);
}

// one element per thread: FvBaseAdLocalLinearizer::linearize
// (fvbaseadlocallinearizer.hh:173-292) and its scatter
// (FvBaseLinearizer::linearizeElement_, fvbaselinearizer.hh:595-626)
__global__ void __launch_bounds__(128) kAssembleImmiscible(DevMesh m, const DevPhysics* __restrict__ phys,
                                                           IqBuffers iq, double* __restrict__ storageOld,
                                                           int iter0, double dt,
                                                           double* __restrict__ residual,
                                                           double* __restrict__ jval)
{
    kAssembleImmiscibleBody(m, phys, iq, storageOld, iter0, dt, residual, jval, blockIdx.x * blockDim.x + threadIdx.x);
}

// The black-oil local residual in the same three parts: the element's own
// quantities (p as a seeded variable, the rest from K1), one interior
// face's flux, the terms after the faces.
struct OwnBlackoil {
    D3 pI, rhoI[3], lamI[3], invBI[3], RsI;
};

__device__ __forceinline__ void ownBlackoil(const DevMesh& m, const IqBuffers& iq, const int p, OwnBlackoil& o)
{
    const int ld = m.ldN;
    o.pI = D3::var(iq.val[0 * ld + p], 1);
    for (int a = 0; a < 3; ++a) {
        o.rhoI[a] = ldDual<3>(iq, ld, 1 + a, a, p);
        o.lamI[a] = ldDual<3>(iq, ld, 4 + a, 3 + a, p);
        o.invBI[a] = ldDual<3>(iq, ld, 7 + a, 6 + a, p);
    }
    o.RsI = ldDual<3>(iq, ld, 10, 9, p);
}

__device__ __forceinline__ bool faceBlackoil(const DevMesh& m, const DevPhysics* __restrict__ phys,
                                             const OwnBlackoil& o, const IqBuffers& nbr, const int p, const int dir,
                                             int& q, D3 (&flux)[3])
{
    const int ld = m.ldN;
    q = m.nbr[dir * ld + p];
    if (q < 0) return false;
    const BlackOilPvt& T = phys->pvt;
    const double rhoRef[3] = {T.rhoRefW, T.rhoRefO, T.rhoRefG};
    const int comp[3] = {1, 0, 2};
    const double dTot = m.dTot[dir * ld + p];
    const double gIn = m.gIn[dir * ld + p];
    const double gEx = m.gEx[dir * ld + p];
    const double Kh = m.Kh[dir * ld + p];
    const double area = m.area[dir * ld + p];
    const double nrm = (dir & 1) ? 1.0 : -1.0;
    const double pJ = nbr.val[0 * ld + q];
    for (int e = 0; e < 3; ++e) flux[e] = D3(0.0);
    for (int a = 0; a < 3; ++a) {
        const double rhoJ = nbr.val[(1 + a) * ld + q];
        const double lamJ = nbr.val[(4 + a) * ld + q];
        bool upI;
        const size_t oo = (size_t)dir * ld + p;
        D3 vf = m.tpfa ? tpfaPhase<3>(o.pI, pJ, o.rhoI[a], rhoJ, o.lamI[a], lamJ, m.trans[oo], area, m.dzg[oo],
                                      m.tieUpI[oo] != 0, upI)
                       : darcyPhase<3>(o.pI, pJ, o.rhoI[a], rhoJ, o.lamI[a], lamJ, dTot, gIn, gEx, Kh, nrm, upI);
        D3 invB = upI ? o.invBI[a] : D3(nbr.val[(7 + a) * ld + q]);
        D3 svf = invB * vf;
        flux[comp[a]] = flux[comp[a]] + svf * rhoRef[a];
        if (a == 1) {
            D3 Rs = upI ? o.RsI : D3(nbr.val[10 * ld + q]);
            flux[2] = flux[2] + Rs * svf * T.rhoRefG;
        }
    }
    double alpha = 1.0;
    alpha *= area;
    for (int e = 0; e < 3; ++e) flux[e] = flux[e] * alpha;
    return true;
}

__device__ __forceinline__ void tailBlackoilEq(const DevMesh& m, const IqBuffers& iq, double* __restrict__ storageOld,
                                               int iter0, double dt, const int p, const int e, D3& r)
{
    const int ld = m.ldN;
    const double V = m.volume[p];
    const double scvVolume = V * 1.0;
    {
        D3 tmp;
        tmp.v = iq.sto[(e * 4 + 0) * ld + p];
        for (int j = 0; j < 3; ++j) tmp.d[j] = iq.sto[(e * 4 + 1 + j) * ld + p];
        double tmp2;
        if (iter0) {
            tmp2 = tmp.v;
            storageOld[e * ld + p] = tmp2;
        }
        else
            tmp2 = storageOld[e * ld + p];
        tmp = tmp - tmp2;
        tmp = tmp * (scvVolume / dt);
        r = r + tmp;
    }
    r = r - 0.0 * scvVolume;
    for (int f = m.bfPtr[p]; f < m.bfPtr[p + 1]; ++f) {
        const BFace& bf = m.bfaces[f];
        if (bf.type != GBFV_BC_MASSRATE) continue;
        const double aa = bf.area * 1.0;
        r = r + D3(bf.rate[e]) * aa;
    }
    // FvBaseLinearizer divides each row by its volume; TpfaLinearizer
    // (tpfalinearizer.hh:711-866) keeps the fluxes times the face area and
    // the storage times volume / dt as they are
    if (!m.tpfa) r = r / V;
}

__device__ __forceinline__ void tailBlackoil(const DevMesh& m, const IqBuffers& iq, double* __restrict__ storageOld,
                                             int iter0, double dt, const int p, D3 (&res)[3])
{
    for (int e = 0; e < 3; ++e) tailBlackoilEq(m, iq, storageOld, iter0, dt, p, e, res[e]);
}

template <class Sink>
__device__ __forceinline__ void localBlackoil(const DevMesh& m, const DevPhysics* __restrict__ phys,
                                              const IqBuffers& iq, const IqBuffers& nbr,
                                              double* __restrict__ storageOld, int iter0, double dt, const int p,
                                              D3 (&res)[3], Sink& sink)
{
    OwnBlackoil o;
    ownBlackoil(m, iq, p, o);
    for (int e = 0; e < 3; ++e) res[e] = D3(0.0);
    for (int dir = 0; dir < 6; ++dir) {
        int q;
        D3 flux[3];
        if (!faceBlackoil(m, phys, o, nbr, p, dir, q, flux)) continue;
        for (int e = 0; e < 3; ++e) res[e] = res[e] + flux[e];
        sink(dir, q, flux);
    }
    tailBlackoil(m, iq, storageOld, iter0, dt, p, res);
}

__device__ __forceinline__ void kAssembleBlackoilBody(const DevMesh& m, const DevPhysics* __restrict__ phys,
                                                         IqBuffers iq, double* __restrict__ storageOld,
                                                         int iter0, double dt,
                                                         double* __restrict__ residual,
                                                         double* __restrict__ jval, const int p)
{
    if (p >= m.N) return;
    OffBlockSink<3> sink{m, jval};
    D3 res[3];
    localBlackoil(m, phys, iq, iq, storageOld, iter0, dt, p, res, sink);
    writeDiag<3>(m, res, residual, jval, p);
}

// the black-oil element (fvbaseadlocallinearizer.hh:173-292,
// fvbaselinearizer.hh:595-626)
__global__ void __launch_bounds__(128) kAssembleBlackoil(DevMesh m, const DevPhysics* __restrict__ phys,
                                                         IqBuffers iq, double* __restrict__ storageOld,
                                                         int iter0, double dt,
                                                         double* __restrict__ residual,
                                                         double* __restrict__ jval)
{
    kAssembleBlackoilBody(m, phys, iq, storageOld, iter0, dt, residual, jval, blockIdx.x * blockDim.x + threadIdx.x);
}

// ------------------------------------------- K2, face-parallel form -----
// The same element linearization with the faces in parallel: a group of G
// lanes of one warp per cell (G = 2*dim: one lane per intersection), the
// cell's own dual quantities staged once in shared memory for its group,
// each lane evaluating its face's flux and writing its off-diagonal block
// (row q, column p: one writer per block), then every lane of the group
// summing the G fluxes in intersection order from the group's shuffles and
// lane e adding equation e's storage and boundary terms -- the operations
// and their order of the cell-parallel kernel, so the results are the same
// to the bit.
template <int B>
__device__ __forceinline__ Dual<B> shflDualFrom(const Dual<B>& x, int src)
{
    Dual<B> r;
    r.v = __shfl_sync(0xffffffffu, x.v, src);
#pragma unroll
    for (int j = 0; j < B; ++j) r.d[j] = __shfl_sync(0xffffffffu, x.d[j], src);
    return r;
}

constexpr int FACE_THREADS = 256;
// the staged states are plain arrays of doubles in dual order
static_assert(sizeof(OwnImmiscible) == 6 * 3 * sizeof(double), "OwnImmiscible layout");
static_assert(sizeof(OwnBlackoil) == 11 * 4 * sizeof(double), "OwnBlackoil layout");

template <int G>
__global__ void __launch_bounds__(FACE_THREADS) kAssembleImmiscibleFaces(DevMesh m, IqBuffers iq,
                                                                         double* __restrict__ storageOld, int iter0,
                                                                         double dt, double* __restrict__ residual,
                                                                         double* __restrict__ jval)
{
    constexpr int GPW = 32 / G, CELLS = (FACE_THREADS / 32) * GPW;
    __shared__ __align__(16) unsigned char ownRaw[CELLS * sizeof(OwnImmiscible)];
    OwnImmiscible* own = reinterpret_cast<OwnImmiscible*>(ownRaw);
    const int lane = threadIdx.x & 31, grp = lane / G, g = lane - grp * G;
    const int c = (threadIdx.x >> 5) * GPW + grp;
    const int p = blockIdx.x * CELLS + c;
    const bool active = grp < GPW && p < m.N;
    if (active) {
        // the group stages the cell's 6 duals (ownImmiscible's loads, spread
        // over the lanes): dual k is value plane k with derivative plane k
        double* ow = reinterpret_cast<double*>(&own[c]);
        const int ld = m.ldN;
        for (int i = g; i < 6 * 3; i += G) {
            const int k = i / 3, comp = i - k * 3;
            ow[i] = comp == 0 ? iq.val[k * ld + p] : iq.der[(k * 2 + comp - 1) * ld + p];
        }
    }
    __syncthreads();
    D2 flux[2] = {D2(0.0), D2(0.0)};
    bool has = false;
    if (active && g < 2 * m.dim) {
        int q;
        has = faceImmiscible(m, own[c], iq, p, g, q, flux);
        if (has) {
            OffBlockSink<2> sink{m, jval};
            sink(g, q, flux);
        }
    }
    D2 res[2] = {D2(0.0), D2(0.0)};
    const int base = grp < GPW ? lane - g : lane;
    for (int d = 0; d < G; ++d) {
        const int src = grp < GPW ? base + d : lane;
        const bool hd = __shfl_sync(0xffffffffu, has, src);
        D2 fd[2];
        for (int e = 0; e < 2; ++e) fd[e] = shflDualFrom<2>(flux[e], src);
        if (hd)
            for (int e = 0; e < 2; ++e) res[e] = res[e] + fd[e];
    }
    // lane e of the group finishes equation e
    if (active && g < 2) {
        D2 r = g == 0 ? res[0] : res[1];
        tailImmiscibleEq(m, own[c], iq, storageOld, iter0, dt, p, g, r);
        writeDiagRow<2>(m, r, g, residual, jval, p);
    }
}

// Black-oil: the group's fluxes go through shared memory, and the 12
// components of the cell's three residual duals (value and 3 derivatives
// each) are summed and finished two per lane -- dual sums, dual minus or
// plus a scalar and dual divided by a scalar act component by component,
// so each component sees the cell-parallel kernel's operations in its order
__device__ __forceinline__ void tailBlackoilComponent(const DevMesh& m, const IqBuffers& iq,
                                                      double* __restrict__ storageOld, int iter0, double dt,
                                                      const int p, const int e, const int comp, double r,
                                                      double* __restrict__ residual, double* __restrict__ jval)
{
    const int ld = m.ldN;
    const double V = m.volume[p];
    const double scvVolume = V * 1.0;
    // storage: (S - S_old) * (V / dt); S_old only moves the value
    double t = iq.sto[(e * 4 + comp) * ld + p];
    if (comp == 0) {
        double tmp2;
        if (iter0) {
            tmp2 = t;
            storageOld[e * ld + p] = tmp2;
        }
        else
            tmp2 = storageOld[e * ld + p];
        t = t - tmp2;
    }
    t = t * (scvVolume / dt);
    r = r + t;
    if (comp == 0) r = r - 0.0 * scvVolume;
    for (int f = m.bfPtr[p]; f < m.bfPtr[p + 1]; ++f) {
        const BFace& bf = m.bfaces[f];
        if (bf.type != GBFV_BC_MASSRATE) continue;
        const double aa = bf.area * 1.0;
        r = r + (comp == 0 ? bf.rate[e] : 0.0) * aa;
    }
    if (!m.tpfa) r = comp == 0 ? r / V : r * (1.0 / V);
    const bool cons = m.cflag[p] >= 0;
    if (comp == 0) residual[3 * p + e] = cons ? 0.0 : r;
    else {
        const int v = comp - 1;
        jval[(m.dim * 9 + e * 3 + v) * ld + p] = cons ? (e == v ? 1.0 : 0.0) : r;
    }
}

__global__ void __launch_bounds__(FACE_THREADS) kAssembleBlackoilFaces(DevMesh m, const DevPhysics* __restrict__ phys,
                                                                       IqBuffers iq, double* __restrict__ storageOld,
                                                                       int iter0, double dt,
                                                                       double* __restrict__ residual,
                                                                       double* __restrict__ jval)
{
    constexpr int G = 6, GPW = 32 / G, CELLS = (FACE_THREADS / 32) * GPW;
    __shared__ __align__(16) unsigned char ownRaw[CELLS * sizeof(OwnBlackoil)];
    __shared__ double fsm[CELLS][G][12];
    __shared__ int hsm[CELLS][G];
    OwnBlackoil* own = reinterpret_cast<OwnBlackoil*>(ownRaw);
    const int lane = threadIdx.x & 31, grp = lane / G, g = lane - grp * G;
    const int c = (threadIdx.x >> 5) * GPW + grp;
    const int p = blockIdx.x * CELLS + c;
    const bool active = grp < GPW && p < m.N;
    if (active) {
        // the group stages the cell's 11 duals (ownBlackoil's loads, spread
        // over the lanes): dual 0 the pressure seeded as variable 1, dual
        // k >= 1 value plane k with derivative plane k - 1
        double* ow = reinterpret_cast<double*>(&own[c]);
        const int ld = m.ldN;
        for (int i = g; i < 11 * 4; i += G) {
            const int k = i / 4, comp = i - k * 4;
            double v;
            if (k == 0) v = comp == 0 ? iq.val[p] : (comp == 2 ? 1.0 : 0.0);
            else v = comp == 0 ? iq.val[k * ld + p] : iq.der[((k - 1) * 3 + comp - 1) * ld + p];
            ow[i] = v;
        }
    }
    __syncthreads();
    if (active) {
        int q;
        D3 flux[3];
        const bool has = faceBlackoil(m, phys, own[c], iq, p, g, q, flux);
        hsm[c][g] = has ? 1 : 0;
        if (has) {
            OffBlockSink<3> sink{m, jval};
            sink(g, q, flux);
            for (int e = 0; e < 3; ++e) {
                fsm[c][g][e * 4] = flux[e].v;
                for (int j = 0; j < 3; ++j) fsm[c][g][e * 4 + 1 + j] = flux[e].d[j];
            }
        }
    }
    __syncwarp();
    if (!active) return;
    // lane g: components g and g + 6 (equation k / 4, component k % 4)
    for (int k = g; k < 12; k += G) {
        double r = 0.0;
        for (int d = 0; d < G; ++d)
            if (hsm[c][d]) r = r + fsm[c][d][k];
        tailBlackoilComponent(m, iq, storageOld, iter0, dt, p, k / 4, k % 4, r, residual, jval);
    }
}

// The AD element linearization of one system: the face-parallel kernels
// (GBFV_CELL_ASSEMBLY=1 selects the cell-parallel ones, the same results)
void launchAssemble(const DevMesh& m, const DevPhysics* phys, IqBuffers iq, double* storageOld,
                    int iter0, double dt, double* residual, double* jval, cudaStream_t s)
{
    static const bool cellPath = getenv("GBFV_CELL_ASSEMBLY") != nullptr;
    if (cellPath) {
        const int bs = 128, nb = (m.N + bs - 1) / bs;
        if (m.model == GBFV_MODEL_IMMISCIBLE_2P)
            kAssembleImmiscible<<<nb, bs, 0, s>>>(m, phys, iq, storageOld, iter0, dt, residual, jval);
        else
            kAssembleBlackoil<<<nb, bs, 0, s>>>(m, phys, iq, storageOld, iter0, dt, residual, jval);
    }
    else if (m.model == GBFV_MODEL_IMMISCIBLE_2P && m.dim == 2) {
        constexpr int cells = (FACE_THREADS / 32) * (32 / 4);
        kAssembleImmiscibleFaces<4><<<(m.N + cells - 1) / cells, FACE_THREADS, 0, s>>>(m, iq, storageOld, iter0, dt,
                                                                                   residual, jval);
    }
    else if (m.model == GBFV_MODEL_IMMISCIBLE_2P) {
        constexpr int cells = (FACE_THREADS / 32) * (32 / 6);
        kAssembleImmiscibleFaces<6><<<(m.N + cells - 1) / cells, FACE_THREADS, 0, s>>>(m, iq, storageOld, iter0, dt,
                                                                                   residual, jval);
    }
    else {
        constexpr int cells = (FACE_THREADS / 32) * (32 / 6);
        kAssembleBlackoilFaces<<<(m.N + cells - 1) / cells, FACE_THREADS, 0, s>>>(m, phys, iq, storageOld, iter0,
                                                                                 dt, residual, jval);
    }
    countLaunch();
}

// ------------------------------------------ finite-difference linearizer --
// FvBaseFdLocalLinearizer (fvbasefdlocallinearizer.hh:222-510).  Element p's
// Jacobian column for primary variable pv is its local residual at a
// deflected state of p minus the one at another state, divided by the total
// deflection: forward (method +1) x + eps against x, central (0) x + eps
// against (x + eps) - (eps + eps), backward (-1) x against x - eps.  eps =
// BaseEpsilon / primaryVarWeight, BaseEpsilon = max(0.9123e-10, machine
// epsilon * 1.23e3) (fvbasefdlocallinearizer.hh:75-79, 272-283).  The
// neighbours keep their intensive quantities; the old time level's storage
// comes from the cache the unperturbed evaluation filled.
//
// The deflected intensive quantities of every cell are computed at once
// (one deflected copy of the state per primary variable and direction: a
// cell's quantities depend on its own variables only), then one thread per
// element evaluates its local residual at each deflected state.

// primaryVarWeight: immisciblemodel.hh:321-333 (pressure 10 / reference
// pressure), blackoilmodel.hh:395-440 (Sw 1, po 1/300e5, gas variable by its
// meaning: Sg 1, Rs 1/250, Rv 1/0.025)
__device__ __forceinline__ double fdEps(const DevMesh& m, int b, const int* __restrict__ meaning, double refP, int p,
                                        int pv)
{
    const double baseEps = fmax(0.9123e-10, 2.220446049250313e-16 * 1.23e3);
    double w;
    if (m.model == GBFV_MODEL_IMMISCIBLE_2P)
        w = pv == 0 ? 10 / refP : 1.0;
    else if (pv == 0)
        w = 1.0;
    else if (pv == 1)
        w = 1.0 / 300e5;
    else {
        const int g = meaning[p];
        w = g == GBFV_GAS_SG ? 1.0 : g == GBFV_GAS_RS ? 1.0 / 250. : 1.0 / 0.025;
    }
    return baseEps / w;
}

// the reference pressure: the pressure of the first cell (natural order) at
// the start of a time step (ImmiscibleModel::updateBegin, immisciblemodel.hh:301-316)
__global__ void kSetRefPressure(const double* __restrict__ x, int idx, double* refP) { *refP = x[idx]; }

void launchSetRefPressure(const double* x, int idx, double* refP, cudaStream_t s)
{
    kSetRefPressure<<<1, 1, 0, s>>>(x, idx, refP);
    countLaunch();
}

// deflected copy of the state: primary variable pv of every cell moved by
// +eps (dir > 0), from +eps back by eps + eps (dir == 0, central), or by
// -(0 + eps) (dir < 0, backward) -- FvBaseFdLocalLinearizer's deflections
// (fvbasefdlocallinearizer.hh:425-455) for all elements at once
__global__ void __launch_bounds__(256) kFdDeflect(DevMesh m, int b, const double* __restrict__ x,
                                                  const int* __restrict__ meaning, const double* __restrict__ refP,
                                                  int pv, int dir, double* __restrict__ xd)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m.N) return;
    for (int e = 0; e < b; ++e) xd[b * p + e] = x[b * p + e];
    const double eps = fdEps(m, b, meaning, *refP, p, pv);
    double v = x[b * p + pv];
    if (dir > 0)
        v += eps;
    else if (dir == 0) {
        v += eps;
        v -= eps + eps;
    }
    else
        v -= 0.0 + eps;
    xd[b * p + pv] = v;
}

void launchFdDeflect(const DevMesh& m, int b, const double* x, const int* meaning, const double* refP, int pv,
                     int dir, double* xd, cudaStream_t s)
{
    const int bs = 256, nb = (m.N + bs - 1) / bs;
    kFdDeflect<<<nb, bs, 0, s>>>(m, b, x, meaning, refP, pv, dir, xd);
    countLaunch();
}

// FD: a face's flux values (times the area)
template <int B>
struct FluxValueSink {
    double (*f)[B];
    __device__ void operator()(int dir, int q, const Dual<B>* flux) const
    {
        for (int e = 0; e < B; ++e) f[dir][e] = flux[e].v;
    }
};

template <int B, class Local>
__device__ __forceinline__ void fdElement(const DevMesh& m, const FdIq& fd, IqBuffers iq0,
                                          const int* __restrict__ meaning, const double* __restrict__ refP,
                                          int method, double* __restrict__ storageOld, int iter0,
                                          double* __restrict__ residual, double* __restrict__ jval, const int p,
                                          Local local)
{
    using D = Dual<B>;
    const int ld = m.ldN;
    const int ndir = 2 * m.dim;
    double f0[6][B], fd1[6][B];
    FluxValueSink<B> s0{f0}, s1{fd1};
    D res0[B], res1[B];
    local(iq0, iter0, res0, s0);  // localResidual_.eval(residual_, elemCtx)
    const bool cons = m.cflag[p] >= 0;
    const int ds = m.dim;
    for (int e = 0; e < B; ++e) residual[B * p + e] = cons ? 0.0 : res0[e].v;
    const double refPv = *refP;
    for (int pv = 0; pv < B; ++pv) {
        const double eps = fdEps(m, B, meaning, refPv, p, pv);
        double delta = 0.0;
        double dI[B], dJ[6][B];
        // the neighbours' residual in this element's context: (0 - flux) / V_q
        if (method >= 0) {
            delta += eps;
            local(fd.plus[pv], 0, res1, s1);
            for (int e = 0; e < B; ++e) dI[e] = res1[e].v;
            for (int dir = 0; dir < ndir; ++dir) {
                const int q = m.nbr[dir * ld + p];
                if (q < 0) continue;
                for (int e = 0; e < B; ++e) dJ[dir][e] = (0.0 - fd1[dir][e]) / m.volume[q];
            }
        }
        else {
            for (int e = 0; e < B; ++e) dI[e] = res0[e].v;
            for (int dir = 0; dir < ndir; ++dir) {
                const int q = m.nbr[dir * ld + p];
                if (q < 0) continue;
                for (int e = 0; e < B; ++e) dJ[dir][e] = (0.0 - f0[dir][e]) / m.volume[q];
            }
        }
        if (method <= 0) {
            delta += eps;
            local(fd.minus[pv], 0, res1, s1);
            for (int e = 0; e < B; ++e) dI[e] -= res1[e].v;
            for (int dir = 0; dir < ndir; ++dir) {
                const int q = m.nbr[dir * ld + p];
                if (q < 0) continue;
                for (int e = 0; e < B; ++e) dJ[dir][e] -= (0.0 - fd1[dir][e]) / m.volume[q];
            }
        }
        else {
            for (int e = 0; e < B; ++e) dI[e] -= res0[e].v;
            for (int dir = 0; dir < ndir; ++dir) {
                const int q = m.nbr[dir * ld + p];
                if (q < 0) continue;
                for (int e = 0; e < B; ++e) dJ[dir][e] -= (0.0 - f0[dir][e]) / m.volume[q];
            }
        }
        for (int e = 0; e < B; ++e)
            jval[(ds * B * B + e * B + pv) * ld + p] = cons ? (e == pv ? 1.0 : 0.0) : dI[e] / delta;
        for (int dir = 0; dir < ndir; ++dir) {
            const int q = m.nbr[dir * ld + p];
            if (q < 0) continue;
            const bool zq = m.cflag[q] >= 0;
            for (int e = 0; e < B; ++e)
                jval[(m.slotOfDir[dir ^ 1] * B * B + e * B + pv) * ld + q] = zq ? 0.0 : dJ[dir][e] / delta;
        }
    }
}

// one element per thread: FvBaseFdLocalLinearizer::linearize
// (fvbasefdlocallinearizer.hh:236-510) and the scatter (fvbaselinearizer.hh:595-626)
__global__ void __launch_bounds__(128) kAssembleFdImmiscible(DevMesh m, IqBuffers iq0, FdIq fd,
                                                             const int* __restrict__ meaning,
                                                             const double* __restrict__ refP, int method,
                                                             double* __restrict__ storageOld, int iter0, double dt,
                                                             double* __restrict__ residual, double* __restrict__ jval)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m.N) return;
    fdElement<2>(m, fd, iq0, meaning, refP, method, storageOld, iter0, residual, jval, p,
                 [&](const IqBuffers& own, int it0, D2 (&res)[2], FluxValueSink<2>& sink) {
                     localImmiscible(m, own, iq0, storageOld, it0, dt, p, res, sink);
                 });
}

__global__ void __launch_bounds__(128) kAssembleFdBlackoil(DevMesh m, const DevPhysics* __restrict__ phys,
                                                           IqBuffers iq0, FdIq fd, const int* __restrict__ meaning,
                                                           const double* __restrict__ refP, int method,
                                                           double* __restrict__ storageOld, int iter0, double dt,
                                                           double* __restrict__ residual, double* __restrict__ jval)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m.N) return;
    fdElement<3>(m, fd, iq0, meaning, refP, method, storageOld, iter0, residual, jval, p,
                 [&](const IqBuffers& own, int it0, D3 (&res)[3], FluxValueSink<3>& sink) {
                     localBlackoil(m, phys, own, iq0, storageOld, it0, dt, p, res, sink);
                 });
}

void launchAssembleFd(const DevMesh& m, const DevPhysics* phys, IqBuffers iq0, const FdIq& fd, const int* meaning,
                      const double* refP, int method, double* storageOld, int iter0, double dt, double* residual,
                      double* jval, cudaStream_t s)
{
    const int bs = 128, nb = (m.N + bs - 1) / bs;
    if (m.model == GBFV_MODEL_IMMISCIBLE_2P)
        kAssembleFdImmiscible<<<nb, bs, 0, s>>>(m, iq0, fd, meaning, refP, method, storageOld, iter0, dt, residual,
                                                jval);
    else
        kAssembleFdBlackoil<<<nb, bs, 0, s>>>(m, phys, iq0, fd, meaning, refP, method, storageOld, iter0, dt,
                                              residual, jval);
    countLaunch();
}

// ------------------------------------------------------- Newton error ----
// NewtonMethod::preSolve_ (newtonmethod.hh:572-607): max |r| over
// unconstrained cells; non-finite values are flagged.  The maximum of
// non-negative doubles is order independent, so an atomicMax on the bit
// pattern gives a deterministic result.
__global__ void kNewtonError(DevMesh m, const double* __restrict__ r, DevStatus* st)
{
    __shared__ unsigned long long smax[8];
    __shared__ int snf[8];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0;
    int nf = 0;
    if (p < m.N && m.cflag[p] < 0 && m.volume[p] > 0.0)
        for (int k = 0; k < m.b; ++k) {
            const double v = r[p * m.b + k];
            if (!isfinite(v)) nf = 1;
            else e = fmax(e, fabs(v));
        }
    unsigned long long bits = __double_as_longlong(e);
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ob = __shfl_down_sync(0xffffffffu, bits, o);
        bits = ob > bits ? ob : bits;
        nf |= __shfl_down_sync(0xffffffffu, nf, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { smax[w] = bits; snf[w] = nf; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long b = 0;
        int f = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { b = smax[i] > b ? smax[i] : b; f |= snf[i]; }
        atomicMax(&st->errorBits, b);
        if (f) atomicOr(&st->nonfinite, 1);
    }
}

void launchNewtonError(const DevMesh& m, const double* residual, DevStatus* st, cudaStream_t s)
{
    kNewtonError<<<(m.N + 255) / 256, 256, 0, s>>>(m, residual, st);
    countLaunch();
}

// NewtonMethod::update_ guard: a non-finite update aborts the step
// (newtonmethod.hh:677-678)
__global__ void kCheckUpdate(int n, const double* __restrict__ dx, DevStatus* st)
{
    int bad = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (!isfinite(dx[i])) bad = 1;
    bad = __syncthreads_or(bad);
    if (bad && threadIdx.x == 0) atomicOr(&st->nonfinite, 1);
}

void launchCheckUpdate(int n, const double* dx, DevStatus* st, cudaStream_t s)
{
    int nb = (n + 255) / 256;
    if (nb > 1024) nb = 1024;
    kCheckUpdate<<<nb, 256, 0, s>>>(n, dx, st);
    countLaunch();
}

// ----------------------------------------------------- Newton update -----
__device__ __forceinline__ double signum(double v) { return (double)((v > 0) - (v < 0)); }

// BlackOilPrimaryVariables::adaptPrimaryVariables (blackoilprimaryvariables.hh:549-910)
__device__ bool adaptPv(const BlackOilPvt& T, const UpdateParams& prm, double* pv, int& meaning, double eps)
{
    const double sw = pv[0];
    const double sg = meaning == GBFV_GAS_SG ? pv[2] : 0.0;
    const double rsMax = 8.98846567431158e307;  // numeric_limits<double>::max()/2
    if (sw >= prm.waterOnly) {
        pv[0] = fmin(prm.swMax, sw);
        pv[2] = 0.0;
        const bool changed = meaning != GBFV_GAS_SG;
        if (changed) meaning = GBFV_GAS_SG;
        return changed;
    }
    bool changed = false;
    if (meaning == GBFV_GAS_SG) {
        const double s = 1.0 - sw - 0.0;
        if (sg < -eps && s > 0.0) {
            const double po = pv[1];
            meaning = GBFV_GAS_RS;
            const double rsSat = tableEval(T.rsSat, po);
            pv[2] = fmin(rsMax, rsSat);
            changed = true;
        }
    }
    else if (meaning == GBFV_GAS_RS) {
        const double po = pv[1];
        const double rsSat = tableEval(T.rsSat, po);
        const double rs = pv[2];
        if (rs > fmin(rsMax, rsSat * (1.0 + eps))) {
            meaning = GBFV_GAS_SG;
            pv[2] = 0.0;
            changed = true;
        }
    }
    return changed;
}

// NewtonMethod::update_ / BlackOilNewtonMethod::updatePrimaryVariables_
// (newtonmethod.hh:665-731, blackoilnewtonmethod.hh:226-427)
__device__ __forceinline__ int kNewtonUpdateCell(const DevMesh& m, const DevPhysics* __restrict__ phys,
                                                 const double* __restrict__ dx, double* __restrict__ x,
                                                 int* __restrict__ meaning, int* __restrict__ wasSwitched,
                                                 const UpdateParams& prm, const int p)
{
    int sw = 0;
    if (p < m.N) {
        const int k = m.cflag[p];
        const int b = m.b;
        if (k >= 0) {
            for (int e = 0; e < b; ++e) x[p * b + e] = m.consPv[3 * k + e];
            meaning[p] = m.consMeaning[k];
        }
        else if (m.model == GBFV_MODEL_IMMISCIBLE_2P) {
            for (int e = 0; e < b; ++e) x[p * b + e] = x[p * b + e] - dx[p * b + e];
        }
        else {
            const double up[3] = {dx[3 * p], dx[3 * p + 1], dx[3 * p + 2]};
            const double cv[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
            const int mg = meaning[p];
            double dSw = 0, dSo = 0, dSg = 0;
            dSw = up[0];
            dSo -= dSw;
            if (mg == GBFV_GAS_SG) { dSg = up[2]; dSo -= dSg; }
            double maxSat = fmax(fabs(dSg), fabs(dSo));
            maxSat = fmax(maxSat, fabs(dSw));
            maxSat = fmax(maxSat, 0.0);
            double satAlpha = 1.0;
            if (maxSat > prm.dsMax) satAlpha = prm.dsMax / maxSat;
            double nv[3];
            for (int pvIdx = 0; pvIdx < 3; ++pvIdx) {
                double delta = up[pvIdx];
                if (pvIdx == 1) {
                    if (fabs(delta) > prm.dpMaxRel * cv[1]) delta = signum(delta) * prm.dpMaxRel * cv[1];
                }
                else if (pvIdx == 0)
                    delta *= satAlpha;
                else {
                    if (mg == GBFV_GAS_SG) delta *= satAlpha;
                    else if (delta > cv[2]) delta = cv[2];
                }
                nv[pvIdx] = cv[pvIdx] - delta;
                if (pvIdx == 1) nv[1] = fmin(fmax(nv[1], prm.pMin), prm.pMax);
            }
            int mm = mg;
            const double eps = wasSwitched[p] ? prm.oscThreshold : 0.0;
            const bool ch = adaptPv(phys->pvt, prm, nv, mm, eps);
            wasSwitched[p] = ch ? 1 : 0;
            sw = ch ? 1 : 0;
            for (int e = 0; e < 3; ++e) x[3 * p + e] = nv[e];
            meaning[p] = mm;
        }
    }
    return sw;
}

// NewtonMethod::updatePrimaryVariables_ (newtonmethod.hh:723-731) for the
// immiscible model; BlackOilNewtonMethod::updatePrimaryVariables_
// (blackoilnewtonmethod.hh:226-427) with chopping and switching for black-oil
__global__ void kNewtonUpdate(DevMesh m, const DevPhysics* __restrict__ phys, const double* __restrict__ dx,
                              double* __restrict__ x, int* __restrict__ meaning,
                              int* __restrict__ wasSwitched, UpdateParams prm, DevStatus* st)
{
    int sw = kNewtonUpdateCell(m, phys, dx, x, meaning, wasSwitched, prm, blockIdx.x * blockDim.x + threadIdx.x);
    sw = __syncthreads_count(sw);
    if (threadIdx.x == 0 && sw) atomicAdd(&st->switched, sw);
}

void launchNewtonUpdate(const DevMesh& m, const DevPhysics* phys, const double* dx, double* x,
                        int* meaning, int* wasSwitched, UpdateParams prm, DevStatus* st,
                        cudaStream_t s)
{
    kNewtonUpdate<<<(m.N + 255) / 256, 256, 0, s>>>(m, phys, dx, x, meaning, wasSwitched, prm, st);
    countLaunch();
}

// ------------------------------------------------------------ batched ----
// Grid (gx, K): blockIdx.y is the system, its blocks stride over its cells and
// run the same per-cell code as the single-system kernels above.
__global__ void __launch_bounds__(128) kBatchConstraints(const LinJob* __restrict__ jobs,
                                                         const JobState* __restrict__ js)
{
    if (!js[blockIdx.y].active) return;
    const LinJob& j = jobs[blockIdx.y];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < j.m.numConsCells; k += gridDim.x * blockDim.x)
        kApplyConstraintsBody(j.m, j.x, j.xOld, j.meaning, j.meaningOld, k);
}

__global__ void __launch_bounds__(128) kBatchIq(const LinJob* __restrict__ jobs, const JobState* __restrict__ js)
{
    if (!js[blockIdx.y].active) return;
    const LinJob& j = jobs[blockIdx.y];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < j.m.N; p += gridDim.x * blockDim.x) {
        if (j.m.model == GBFV_MODEL_IMMISCIBLE_2P)
            kIqImmiscibleBody(j.m, j.phys, j.x, j.iq, p);
        else
            kIqBlackoilBody(j.m, j.phys, j.x, j.meaning, j.iq, p);
    }
}

__global__ void __launch_bounds__(128) kBatchAssemble(const LinJob* __restrict__ jobs,
                                                      const JobState* __restrict__ js)
{
    const JobState st = js[blockIdx.y];
    if (!st.active) return;
    const LinJob& j = jobs[blockIdx.y];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < j.m.N; p += gridDim.x * blockDim.x) {
        if (j.m.model == GBFV_MODEL_IMMISCIBLE_2P)
            kAssembleImmiscibleBody(j.m, j.phys, j.iq, j.storageOld, st.iter0, st.dt, j.residual, j.jval, p);
        else
            kAssembleBlackoilBody(j.m, j.phys, j.iq, j.storageOld, st.iter0, st.dt, j.residual, j.jval, p);
    }
}

void launchBatchLinearize(const LinJob* jobs, const JobState* js, int K, int gx, cudaStream_t s)
{
    kBatchConstraints<<<dim3(gx, K), 128, 0, s>>>(jobs, js);
    kBatchIq<<<dim3(gx, K), 128, 0, s>>>(jobs, js);
    kBatchAssemble<<<dim3(gx, K), 128, 0, s>>>(jobs, js);
    countLaunch(3);
}

// max |r| over unconstrained cells of each system (as kNewtonError)
__global__ void __launch_bounds__(256) kBatchNewtonError(const LinJob* __restrict__ jobs,
                                                         const JobState* __restrict__ js)
{
    if (!js[blockIdx.y].active) return;
    const LinJob& j = jobs[blockIdx.y];
    __shared__ unsigned long long smax[8];
    __shared__ int snf[8];
    double e = 0.0;
    int nf = 0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < j.m.N; p += gridDim.x * blockDim.x)
        if (j.m.cflag[p] < 0 && j.m.volume[p] > 0.0)
            for (int k = 0; k < j.m.b; ++k) {
                const double v = j.residual[p * j.m.b + k];
                if (!isfinite(v)) nf = 1;
                else e = fmax(e, fabs(v));
            }
    unsigned long long bits = __double_as_longlong(e);
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ob = __shfl_down_sync(0xffffffffu, bits, o);
        bits = ob > bits ? ob : bits;
        nf |= __shfl_down_sync(0xffffffffu, nf, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { smax[w] = bits; snf[w] = nf; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long b = 0;
        int f = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { b = smax[i] > b ? smax[i] : b; f |= snf[i]; }
        atomicMax(&j.st->errorBits, b);
        if (f) atomicOr(&j.st->nonfinite, 1);
    }
}

void launchBatchNewtonError(const LinJob* jobs, const JobState* js, int K, int gx, cudaStream_t s)
{
    kBatchNewtonError<<<dim3(gx, K), 256, 0, s>>>(jobs, js);
    countLaunch();
}

__global__ void __launch_bounds__(256) kBatchCheckUpdate(const LinJob* __restrict__ jobs,
                                                         const JobState* __restrict__ js)
{
    if (!js[blockIdx.y].active) return;
    const LinJob& j = jobs[blockIdx.y];
    const int n = j.m.N * j.m.b;
    int bad = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (!isfinite(j.dx[i])) bad = 1;
    bad = __syncthreads_or(bad);
    if (bad && threadIdx.x == 0) atomicOr(&j.st->nonfinite, 1);
}

void launchBatchCheckUpdate(const LinJob* jobs, const JobState* js, int K, int gx, cudaStream_t s)
{
    kBatchCheckUpdate<<<dim3(gx, K), 256, 0, s>>>(jobs, js);
    countLaunch();
}

__global__ void __launch_bounds__(256) kBatchNewtonUpdate(const LinJob* __restrict__ jobs,
                                                          const JobState* __restrict__ js, UpdateParams prm)
{
    if (!js[blockIdx.y].active) return;
    const LinJob& j = jobs[blockIdx.y];
    int sw = 0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < j.m.N; p += gridDim.x * blockDim.x)
        sw += kNewtonUpdateCell(j.m, j.phys, j.dx, j.x, j.meaning, j.wasSwitched, prm, p);
    if (sw) atomicAdd(&j.st->switched, sw);
}

void launchBatchNewtonUpdate(const LinJob* jobs, const JobState* js, int K, int gx, UpdateParams prm,
                             cudaStream_t s)
{
    kBatchNewtonUpdate<<<dim3(gx, K), 256, 0, s>>>(jobs, js, prm);
    countLaunch();
}

}  // namespace gbfv
