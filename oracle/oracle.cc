// ORACLE -- test infrastructure only.  Only tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline / reference legs may load or run this
// library.  It checks the product; it is never the product path.
//
// CPU restatement (C++17, no dependencies) of the reference's hot path.
// Parity status: UNPINNED against the reference's own output -- the
// reference needs dune-* and opm-common, neither is installed, so it cannot
// be compiled here, and its tests pin no numbers.  The restatement follows
// the reference source line by line where the reference holds the code
// (citations below); the opm-common / dune-istl parts it relies on are
// restated from their published algorithms and listed in the oracle's table
// of unpinned choices.
//
// Followed files (paths inside OPM/opm-models):
//   element loop, scatter, constraints  fvbaselinearizer.hh:510-666
//   AD local linearization              fvbaseadlocallinearizer.hh:173-292
//   residual = fluxes + storage + bnd   fvbaselocalresidual.hh:158-191,
//                                       299-361, 419-484, 491-626
//   immiscible IQ / storage / flux      immiscibleintensivequantities.hh:93-151,
//                                       immisciblelocalresidual.hh:75-155
//   black-oil IQ / storage / flux       blackoilintensivequantities.hh:179-470,
//                                       blackoillocalresidual.hh:101-367
//   Darcy gradients + upwind            darcyfluxmodule.hh:183-525,
//                                       fvbasegradientcalculator.hh:200-318
//   free-flow boundary                  immiscibleboundaryratevector.hh:97-150
//   BiCGStab + criterion                bicgstabsolver.hh:120-330,
//                                       combinedcriterion.hh:116-209,
//                                       parallelbicgstabbackend.hh:131-166
//   Newton                              newtonmethod.hh:228-845
//   black-oil chop + switching          blackoilnewtonmethod.hh:226-427,
//                                       blackoilprimaryvariables.hh:549-910
//   time integration                    fvbaseproblem.hh:512-606,
//                                       simulator.hh:505-512, 780-802
#ifdef _OPENMP
#include <omp.h>
#endif

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <set>
#include <stdexcept>
#include <vector>

#include "../include/gbfv.h"
#include "physics.hh"

namespace oracle {

using D2 = Dual<2>;
using D3 = Dual<3>;

struct NumericalProblem : std::runtime_error {
    int code;
    NumericalProblem(const char* m, int c = GBFV_ERR_NUMERICAL) : std::runtime_error(m), code(c) {}
};

// entry-wise harmonic mean of the two cells' K
// (MultiPhaseBaseProblem::intersectionIntrinsicPermeability, multiphasebaseproblem.hh:109-125)
static double harmonicMean(double x, double y)
{
    if (x * y <= 0) return 0.0;
    return (2 * x * y) / (x + y);
}

// ----------------------------------------------------------- problem ------
struct Prob {
    int model = 0, N = 0, b = 2;
    std::vector<double> center, volume, porosity, perm;
    std::vector<int> material;
    std::vector<int> connPtr, connNbr;
    std::vector<double> connNormal, connCenter, connArea;
    std::vector<int> bfPtr, bfType;
    std::vector<double> bfNormal, bfCenter, bfArea, bfValue;
    std::vector<int> constraint;
    std::vector<double> consPv;
    std::vector<int> consMeaning;
    double g[3] = {0, 0, 0};
    std::vector<TwoPhaseLaw> laws;
    std::vector<double> coreyN;
    double rho[2] = {0, 0}, mu[2] = {0, 0};
    BlackOilPvt pvt;
    int fluxModule = GBFV_FLUX_DARCY;
    int dimWorld = 3;   // the highest coordinate axis the faces use, plus one
    // vertex-centred grids: the cells are the vertices
    int numElements = 0, p1Gradients = 0;
    std::vector<int> elemCorner, bfCorner;
};

template <class T>
static std::vector<T> cp(const T* p, size_t n)
{
    return p ? std::vector<T>(p, p + n) : std::vector<T>(n, T(0));
}

static Prob copyProblem(const gbfv_problem& q)
{
    Prob P;
    P.model = q.model;
    P.N = q.num_cells;
    P.b = q.model == GBFV_MODEL_BLACKOIL_3P ? 3 : 2;
    const size_t N = P.N;
    P.center = cp(q.center, 3 * N);
    P.volume = cp(q.volume, N);
    P.porosity = cp(q.porosity, N);
    P.perm = cp(q.perm, 3 * N);
    P.material = cp(q.material, N);
    P.connPtr = cp(q.conn_ptr, N + 1);
    P.connNbr = cp(q.conn_nbr, q.num_conn);
    P.connNormal = cp(q.conn_normal, 3 * (size_t)q.num_conn);
    P.connCenter = cp(q.conn_center, 3 * (size_t)q.num_conn);
    P.connArea = cp(q.conn_area, q.num_conn);
    P.fluxModule = q.flux_module;
    {
        int maxAxis = 0;
        for (int c = 0; c < q.num_conn; ++c)
            for (int d = 0; d < 3; ++d)
                if (q.conn_normal[3 * c + d] != 0.0) maxAxis = std::max(maxAxis, d);
        P.dimWorld = maxAxis + 1;
    }
    P.numElements = q.num_elements;
    if (P.numElements > 0) {
        P.elemCorner = cp(q.elem_corner, 4 * (size_t)P.numElements);
        P.bfCorner = cp(q.bface_corner, q.num_bfaces);
        P.p1Gradients = q.p1_gradients;
        P.dimWorld = 2;
    }
    P.bfPtr = cp(q.bface_ptr, (P.numElements > 0 ? P.numElements : N) + 1);
    P.bfType = cp(q.bface_type, q.num_bfaces);
    P.bfNormal = cp(q.bface_normal, 3 * (size_t)q.num_bfaces);
    P.bfCenter = cp(q.bface_center, 3 * (size_t)q.num_bfaces);
    P.bfArea = cp(q.bface_area, q.num_bfaces);
    P.bfValue = cp(q.bface_value, 4 * (size_t)q.num_bfaces);
    if (q.constraint)
        P.constraint = cp(q.constraint, N);
    else
        P.constraint.assign(N, -1);
    P.consPv = cp(q.constraint_pv, 3 * (size_t)q.num_constraints);
    P.consMeaning = cp(q.constraint_meaning, q.num_constraints);
    for (int d = 0; d < 3; ++d) P.g[d] = q.gravity[d];
    for (int m = 0; m < q.num_materials; ++m) {
        const double* mp = q.material_params + m * GBFV_MAT_STRIDE;
        const int law = (int)mp[0];
        TwoPhaseLaw L;
        if (law == GBFV_LAW_REG_VAN_GENUCHTEN || law == GBFV_LAW_REG_BROOKS_COREY) {
            L.law = law == GBFV_LAW_REG_VAN_GENUCHTEN ? 0 : 1;
            L.Swr = mp[1];
            L.Snr = mp[2];
            if (L.law == 0) { L.alpha = mp[3]; L.n = mp[4]; }
            else { L.pe = mp[3]; L.lambda = mp[4]; }
            L.finalize();
        }
        P.laws.push_back(L);
        P.coreyN.push_back(law == GBFV_LAW_COREY3P ? mp[4] : 2.0);
    }
    P.rho[0] = q.rho[0]; P.rho[1] = q.rho[1];
    P.mu[0] = q.mu[0]; P.mu[1] = q.mu[1];
    if (q.pvt) {
        const gbfv_blackoil_pvt& t = *q.pvt;
        BlackOilPvt& v = P.pvt;
        v.rhoRefO = t.rho_ref_oil; v.rhoRefW = t.rho_ref_water; v.rhoRefG = t.rho_ref_gas;
        for (int i = 0; i < t.n_oil; ++i) {
            v.rsSat.x.push_back(t.oil_p[i]); v.rsSat.y.push_back(t.oil_rs[i]);
            v.pBubble.x.push_back(t.oil_rs[i]); v.pBubble.y.push_back(t.oil_p[i]);
            v.invBoSat.x.push_back(t.oil_p[i]); v.invBoSat.y.push_back(1.0 / t.oil_bo[i]);
            v.muoSat.x.push_back(t.oil_p[i]); v.muoSat.y.push_back(t.oil_mu[i]);
        }
        v.oilComp = t.oil_compressibility;
        for (int i = 0; i < t.n_gas; ++i) {
            v.invBg.x.push_back(t.gas_p[i]); v.invBg.y.push_back(1.0 / t.gas_bg[i]);
            v.mug.x.push_back(t.gas_p[i]); v.mug.y.push_back(t.gas_mu[i]);
        }
        v.pwRef = t.water_p_ref; v.bwRef = t.water_bw_ref;
        v.cw = t.water_compressibility; v.muw = t.water_mu;
    }
    return P;
}

// ------------------------------------------------- intensive quantities ----
struct IQ2 {
    D2 S[2], p[2], rho[2], mu[2], kr[2], lam[2];
    double phi;
};

// ImmiscibleIntensiveQuantities::update (immiscibleintensivequantities.hh:93-151)
static IQ2 immiscibleIQ(const Prob& P, int c, const double* pv)
{
    IQ2 q;
    const TwoPhaseLaw& L = P.laws[P.material[c]];
    D2 sumSat(0.0);
    D2 Sw = D2::variable(pv[1], 1);
    q.S[0] = Sw;
    sumSat += Sw;
    q.S[1] = 1.0 - sumSat;
    // EffToAbsLaw: effective saturations, then the effective law
    const double sumRes = L.Swr + L.Snr;
    D2 SwE = (q.S[0] - L.Swr) / (1.0 - sumRes);
    D2 SnE = (q.S[1] - L.Snr) / (1.0 - sumRes);
    D2 pc[2];
    pc[0] = D2(0.0);
    pc[1] = L.pcnw(SwE);
    q.kr[0] = L.krw(SwE);
    q.kr[1] = L.krn(1.0 - SnE);
    D2 p0 = D2::variable(pv[0], 0);
    for (int a = 0; a < 2; ++a) q.p[a] = p0 + (pc[a] - pc[0]);
    for (int a = 0; a < 2; ++a) {
        q.mu[a] = D2(P.mu[a]);
        q.rho[a] = D2(P.rho[a]);
        q.lam[a] = q.kr[a] / q.mu[a];
    }
    q.phi = P.porosity[c];
    return q;
}

// phases: 0 water, 1 oil, 2 gas; PV: 0 Sw, 1 po, 2 Sg|Rs
struct IQ3 {
    D3 S[3], p[3], invB[3], rho[3], mu[3], lam[3], kr[3];
    D3 Rs;
    double phi;
};

// Corey k_r = S^n, supplied through the problem's updateRelperms hook
// (blackoilintensivequantities.hh:262, multiphasebaseproblem.hh:256-261)
template <class E>
static E corey(const E& S, double n)
{
    if (S <= 0.0) return E(0.0);
    if (S >= 1.0) return E(1.0);
    if (n == 2.0) return S * S;
    return pow(S, n);
}

// BlackOilIntensiveQuantities::update (blackoilintensivequantities.hh:179-462)
// with water meaning Sw, pressure meaning Po, gas meaning Sg or Rs, zero
// capillary pressure and Corey relperms from the updateRelperms hook.
static IQ3 blackoilIQ(const Prob& P, int c, const double* pv, int gasMeaning)
{
    IQ3 q;
    const BlackOilPvt& T = P.pvt;
    D3 Sw = D3::variable(pv[0], 0);
    D3 Sg(0.0);
    if (gasMeaning == GBFV_GAS_SG) Sg = D3::variable(pv[2], 2);
    D3 So = 1.0 - Sw - Sg;
    q.S[0] = Sw; q.S[1] = So; q.S[2] = Sg;
    const double n = P.coreyN[P.material[c]];
    D3 kr[3];
    for (int a = 0; a < 3; ++a) kr[a] = corey(q.S[a], n);
    D3 po = D3::variable(pv[1], 1) * 1.0;
    for (int a = 0; a < 3; ++a) q.p[a] = po + (D3(0.0) - D3(0.0));
    D3 RsSat = T.rsSat.eval(q.p[1]);
    if (gasMeaning == GBFV_GAS_RS)
        q.Rs = D3::variable(pv[2], 2);
    else
        q.Rs = RsSat;  // min(RsMax, RsSat) with RsMax unbounded
    // inverse formation volume factors and viscosities
    q.invB[0] = T.waterInvB(q.p[0]);
    q.mu[0] = D3(T.muw);
    const bool sat = q.S[2].v > 0.0 && q.Rs.v >= (1.0 - 1e-10) * RsSat.v;
    T.oil(q.p[1], q.Rs, sat, q.invB[1], q.mu[1]);
    q.invB[2] = T.invBg.eval(q.p[2]);
    q.mu[2] = T.mug.eval(q.p[2]);
    for (int a = 0; a < 3; ++a) q.lam[a] = kr[a] / q.mu[a];
    for (int a = 0; a < 3; ++a) q.kr[a] = kr[a];
    q.rho[0] = q.invB[0] * T.rhoRefW;
    q.rho[2] = q.invB[2] * T.rhoRefG;
    q.rho[1] = q.invB[1] * T.rhoRefO;
    q.rho[1] += q.invB[1] * q.Rs * T.rhoRefG;
    q.phi = P.porosity[c];
    return q;
}

// ------------------------------------------------------------ Darcy -------
// Interior-face potential gradient, upwind and volume flux for the focus
// element I (darcyfluxmodule.hh:183-322, 459-525; fvbasegradientcalculator.hh
// :200-246).  Returns the upstream flag per phase (true: interior upstream).
template <class D, int NP>
static void darcyInterior(const Prob& P, int I, int J, int c, const D* pI, const double* pJ,
                          const D* rhoI, const double* rhoJ, const D* lamI, const double* lamJ,
                          D* vflux, bool* upInterior)
{
    const double* xI = &P.center[3 * I];
    const double* xJ = &P.center[3 * J];
    const double* xf = &P.connCenter[3 * c];
    const double* n = &P.connNormal[3 * c];
    double distSq = 0.0;
    for (int d = 0; d < 3; ++d) {
        const double t = xJ[d] - xI[d];
        distSq += t * t;
    }
    double dIn[3], dEx[3], dTot[3];
    for (int d = 0; d < 3; ++d) {
        dIn[d] = xI[d] - xf[d];
        dEx[d] = xJ[d] - xf[d];
        dTot[d] = xJ[d] - xI[d];
    }
    double absTot2 = 0.0, gIn = 0.0, gEx = 0.0;
    for (int d = 0; d < 3; ++d) absTot2 += dTot[d] * dTot[d];
    for (int d = 0; d < 3; ++d) gIn += P.g[d] * dIn[d];
    for (int d = 0; d < 3; ++d) gEx += P.g[d] * dEx[d];
    double Kh[3];
    for (int d = 0; d < 3; ++d) Kh[d] = harmonicMean(P.perm[3 * I + d], P.perm[3 * J + d]);
    for (int a = 0; a < NP; ++a) {
        D deltay = pJ[a] - pI[a];
        D pg[3];
        for (int d = 0; d < 3; ++d) pg[d] = deltay * ((xJ[d] - xI[d]) / distSq);
        D pStatIn = (-rhoI[a]) * gIn;
        const double pStatEx = (-rhoJ[a]) * gEx;
        D fs = (pStatEx - pStatIn) / absTot2;
        for (int d = 0; d < 3; ++d) pg[d] += dTot[d] * fs;
        D tmp(0.0);
        for (int d = 0; d < 3; ++d) tmp += pg[d] * n[d];
        const bool upI = !(tmp > 0.0);
        upInterior[a] = upI;
        D mob = upI ? lamI[a] : D(lamJ[a]);
        D vf(0.0);
        for (int d = 0; d < 3; ++d) {
            D fv = Kh[d] * pg[d];
            fv *= -mob;
            vf += fv * n[d];
        }
        vflux[a] = vf;
    }
}

// ------------------------------------------------------ transmissibility --
// TransExtensiveQuantities::transmissibility_ (transfluxmodule.hh:425-456):
// T0 T1 / (T0 + T1), T_k = K_kk |n . d_k| / |d_k|^2, k the axis of n
static double transInteriorT(const Prob& P, int I, int J, int c)
{
    const double* n = &P.connNormal[3 * c];
    const double* xf = &P.connCenter[3 * c];
    double d0[3], d1[3];
    for (int d = 0; d < 3; ++d) {
        d0[d] = xf[d] - P.center[3 * I + d];
        d1[d] = xf[d] - P.center[3 * J + d];
    }
    double nd0 = 0, nd1 = 0, s0 = 0, s1 = 0;
    for (int d = 0; d < 3; ++d) {
        nd0 += n[d] * d0[d];
        nd1 += n[d] * d1[d];
        s0 += d0[d] * d0[d];
        s1 += d1[d] * d1[d];
    }
    nd0 = std::abs(nd0);
    nd1 = std::abs(nd1);
    int idx = 0;
    double val = 0.0;
    for (int d = 0; d < P.dimWorld; ++d)
        if (std::abs(n[d]) > val) { val = std::abs(n[d]); idx = d; }
    const double T0 = P.perm[3 * I + idx] * nd0 / s0;
    const double T1 = P.perm[3 * J + idx] * nd1 / s1;
    return T0 * T1 / (T0 + T1);
}

// transmissibilityBoundary_ (transfluxmodule.hh:457-480): the reference takes
// the geometry of the element's interior face with the boundary face's
// index (stencil.interiorFace(scvfIdx)); on square cells with a diagonal,
// axis-independent K that equals the boundary face's own half transmissibility
static double transBoundaryT(const Prob& P, int I, int k)
{
    const int c = P.connPtr[I] + k;
    if (c >= P.connPtr[I + 1]) return std::numeric_limits<double>::quiet_NaN();
    const double* n = &P.connNormal[3 * c];
    const double* xf = &P.connCenter[3 * c];
    double nd = 0, s0 = 0;
    for (int d = 0; d < 3; ++d) {
        const double t = xf[d] - P.center[3 * I + d];
        nd += n[d] * t;
        s0 += t * t;
    }
    int idx = 0;
    double val = 0.0;
    for (int d = 0; d < P.dimWorld; ++d)
        if (std::abs(n[d]) > val) { val = std::abs(n[d]); idx = d; }
    return P.perm[3 * I + idx] * nd / s0;
}

// calculateGradients_ of the transmissibility module for one phase, focus =
// interior element I (transfluxmodule.hh:201-318): hydrostatic correction
// with the average density, upwind by the sign of the pressure difference
// (ties: larger volume, then lower global index), q = dp * lambda_up * (-T)
template <class D>
static D transInterior(const Prob& P, int I, int J, double T, const D& pI, double pJ, const D& rhoI, double rhoJ,
                       const D& lamI, double lamJ, bool& upInterior)
{
    if (lamI.v <= 0.0 && lamJ <= 0.0) {
        upInterior = true;
        return D(0.0);
    }
    const double g = P.g[P.dimWorld - 1];
    const double distZ = P.center[3 * I + P.dimWorld - 1] - P.center[3 * J + P.dimWorld - 1];
    D rhoAvg = (rhoI + rhoJ) / 2.0;
    D pEx(pJ);
    pEx += rhoAvg * (distZ * g);
    D pd = pEx - pI;
    if (pd.v > 0.0) upInterior = false;
    else if (pd.v < 0.0) upInterior = true;
    else {
        const double Vin = P.volume[I], Vex = P.volume[J];
        upInterior = Vin > Vex ? true : (Vin < Vex ? false : I < J);
    }
    if (upInterior) return pd * lamI * (-T);
    return pd * (lamJ * (-T));
}

// ------------------------------------------------------ linearization -----
struct Bcrs {
    int n = 0, b = 2;
    std::vector<int> rowPtr, col;
    std::vector<double> val;  // nnz * b * b, row-major blocks
    int find(int r, int c) const
    {
        for (int k = rowPtr[r]; k < rowPtr[r + 1]; ++k)
            if (col[k] == c) return k;
        return -1;
    }
};

struct AmgHierarchy;  // amg.hh
struct VcfvGrid;      // vcfv.hh

struct Sim {
    Prob P;
    gbfv_params prm;
    int N, b;
    std::vector<double> x, xOld;          // N*b
    std::vector<int> meaning, meaningOld; // gas meaning per cell
    std::vector<char> wasSwitched;
    std::vector<double> storageOld;       // N*b
    std::vector<double> residual;         // N*b
    std::vector<double> rscale;           // N*b: sum of |terms| / V (parity scale)
    Bcrs J;
    std::vector<int> diagSlot, connSlot;  // block index of (I,I) and of (J,I) per connection
    double dt = 1.0;
    int newtonIter = 0;
    std::vector<double> dx;
    int lastLinIters = 0;
    double error = 0, lastError = 0;
    int numIterations = 0;
    double refPressure = 1.0;  // ImmiscibleModel::referencePressure_ (immisciblemodel.hh:301-316)
    std::shared_ptr<AmgHierarchy> amg;  // ParallelAmgBackend's hierarchy (structure kept across solves)
    std::shared_ptr<VcfvGrid> vcfv;  // vertex-centred stencils (vcfv.hh), else NULL
};

static void buildPattern(Sim& S)
{
    const Prob& P = S.P;
    S.J.n = S.N;
    S.J.b = S.b;
    S.J.rowPtr.assign(S.N + 1, 0);
    std::vector<std::vector<int>> rows(S.N);
    for (int I = 0; I < S.N; ++I) {
        rows[I].push_back(I);
        for (int c = P.connPtr[I]; c < P.connPtr[I + 1]; ++c) rows[I].push_back(P.connNbr[c]);
        std::sort(rows[I].begin(), rows[I].end());
        rows[I].erase(std::unique(rows[I].begin(), rows[I].end()), rows[I].end());
    }
    for (int I = 0; I < S.N; ++I) S.J.rowPtr[I + 1] = S.J.rowPtr[I] + (int)rows[I].size();
    S.J.col.resize(S.J.rowPtr[S.N]);
    for (int I = 0; I < S.N; ++I)
        std::copy(rows[I].begin(), rows[I].end(), S.J.col.begin() + S.J.rowPtr[I]);
    S.J.val.assign((size_t)S.J.rowPtr[S.N] * S.b * S.b, 0.0);
    S.diagSlot.resize(S.N);
    S.connSlot.resize(P.connNbr.size());
    for (int I = 0; I < S.N; ++I) {
        S.diagSlot[I] = S.J.find(I, I);
        for (int c = P.connPtr[I]; c < P.connPtr[I + 1]; ++c) S.connSlot[c] = S.J.find(P.connNbr[c], I);
    }
}

// constrained cells take their prescribed primary variables
// (FvBaseLinearizer::applyConstraintsToSolution_, fvbaselinearizer.hh:630-645)
static void applyConstraintsToSolution(Sim& S)
{
    for (int I = 0; I < S.N; ++I) {
        const int k = S.P.constraint[I];
        if (k < 0) continue;
        for (int e = 0; e < S.b; ++e) {
            S.x[I * S.b + e] = S.P.consPv[3 * k + e];
            S.xOld[I * S.b + e] = S.P.consPv[3 * k + e];
        }
        S.meaning[I] = S.P.consMeaning[k];
        S.meaningOld[I] = S.P.consMeaning[k];
    }
}

// an element's residual and derivative columns into the global system:
// residual_[globI] += ..., jacobian_->addToBlock(globJ, globI, ...)
// (FvBaseLinearizer::linearizeElement_, fvbaselinearizer.hh:595-626)
template <int B>
static void scatterElement(Sim& S, int I, const Dual<B>* resI, const std::vector<Dual<B>>& resJ)
{
    const Prob& P = S.P;
    for (int e = 0; e < B; ++e) S.residual[I * B + e] = resI[e].v;
    double* blk = &S.J.val[(size_t)S.diagSlot[I] * B * B];
    for (int e = 0; e < B; ++e)
        for (int v = 0; v < B; ++v) blk[e * B + v] = resI[e].d[v];
    int k = 0;
    for (int c = P.connPtr[I]; c < P.connPtr[I + 1]; ++c, ++k) {
        double* ob = &S.J.val[(size_t)S.connSlot[c] * B * B];
        for (int e = 0; e < B; ++e)
            for (int v = 0; v < B; ++v) ob[e * B + v] = resJ[k * B + e].d[v];
    }
}

// FvBaseLocalResidual::eval of element I (fvbaselocalresidual.hh:158-191):
// res = the element's own residual, resJ = its neighbours' (-flux / V_J, in
// connection order), sc = the parity scale (sum of |terms| / V).  qi is I's
// intensive quantities (perturbed ones for the finite-difference
// linearizer), iq every cell's unperturbed ones.  iter0: Newton iteration 0
// with no stashed intensive quantities -- the storage becomes the cached old
// time level (fvbaselocalresidual.hh:535-571); otherwise the cache is read.
static void elementImmiscible(Sim& S, int I, const IQ2& qi, const std::vector<IQ2>& iq, bool iter0, D2* res,
                              std::vector<D2>& resJ, double* sc)
{
    const Prob& P = S.P;
    for (int e = 0; e < 2; ++e) {
        res[e] = D2(0.0);
        sc[e] = 0.0;
    }
    const int nc = P.connPtr[I + 1] - P.connPtr[I];
    resJ.assign(2 * nc, D2(0.0));
    // evalFluxes
    int k = 0;
    for (int c = P.connPtr[I]; c < P.connPtr[I + 1]; ++c, ++k) {
        const int Jc = P.connNbr[c];
        const IQ2& qj = iq[Jc];
        double pJ[2], rhoJ[2], lamJ[2];
        for (int a = 0; a < 2; ++a) { pJ[a] = qj.p[a].v; rhoJ[a] = qj.rho[a].v; lamJ[a] = qj.lam[a].v; }
        D2 vf[2];
        bool upI[2];
        if (P.fluxModule == GBFV_FLUX_TRANS) {
            const double T = transInteriorT(P, I, Jc, c);
            for (int a = 0; a < 2; ++a)
                vf[a] = transInterior<D2>(P, I, Jc, T, qi.p[a], pJ[a], qi.rho[a], rhoJ[a], qi.lam[a], lamJ[a], upI[a]);
        }
        else
            darcyInterior<D2, 2>(P, I, Jc, c, qi.p, pJ, qi.rho, rhoJ, qi.lam, lamJ, vf, upI);
        D2 flux[2];
        for (int a = 0; a < 2; ++a) {
            flux[a] = D2(0.0);
            if (upI[a]) flux[a] += vf[a] * qi.rho[a];
            else flux[a] += vf[a] * rhoJ[a];
        }
        double alpha = 1.0;
        alpha *= P.connArea[c];
        for (int e = 0; e < 2; ++e) flux[e] *= alpha;
        for (int e = 0; e < 2; ++e) {
            res[e] += flux[e];
            resJ[k * 2 + e] -= flux[e];
            sc[e] += std::abs(flux[e].v);
        }
    }
    // evalVolumeTerms_
    {
        const double scvVolume = P.volume[I] * 1.0;
        D2 tmp[2];
        for (int a = 0; a < 2; ++a) tmp[a] = (D2(qi.phi) * qi.S[a]) * qi.rho[a];
        double tmp2[2];
        if (iter0) {
            for (int e = 0; e < 2; ++e) tmp2[e] = tmp[e].v;
            for (int e = 0; e < 2; ++e) S.storageOld[I * 2 + e] = tmp2[e];
        }
        else
            for (int e = 0; e < 2; ++e) tmp2[e] = S.storageOld[I * 2 + e];
        for (int e = 0; e < 2; ++e) {
            sc[e] += std::abs(tmp[e].v) * (scvVolume / S.dt) + std::abs(tmp2[e]) * (scvVolume / S.dt);
            tmp[e] -= tmp2[e];
            tmp[e] *= scvVolume / S.dt;
            res[e] += tmp[e];
        }
        for (int e = 0; e < 2; ++e) res[e] -= 0.0 * scvVolume;
    }
    // evalBoundary_
    for (int f = P.bfPtr[I]; f < P.bfPtr[I + 1]; ++f) {
        D2 values[2] = {D2(0.0), D2(0.0)};
        const int type = P.bfType[f];
        if (type == GBFV_BC_MASSRATE) {
            for (int e = 0; e < 2; ++e) values[e] = D2(P.bfValue[4 * f + e]);
        }
        else if (type == GBFV_BC_FREEFLOW) {
            const TwoPhaseLaw& L = P.laws[P.material[I]];
            const double pw = P.bfValue[4 * f + 0], Swb = P.bfValue[4 * f + 1];
            const double sumRes = L.Swr + L.Snr;
            const double SwE = (Swb - L.Swr) / (1.0 - sumRes);
            const double SnE = ((1 - Swb) - L.Snr) / (1.0 - sumRes);
            const double pcn = L.pcnw(SwE);
            const double pb[2] = {pw, pw + pcn - 0.0};
            const double krb[2] = {L.krw(SwE), L.krn(1.0 - SnE)};
            if (P.fluxModule == GBFV_FLUX_TRANS) {
                // calculateBoundaryGradients_ (transfluxmodule.hh:324-415)
                const double T = transBoundaryT(P, I, f - P.bfPtr[I]);
                const double g = P.g[P.dimWorld - 1];
                const double distZ = P.center[3 * I + P.dimWorld - 1] - P.bfCenter[3 * f + P.dimWorld - 1];
                for (int a = 0; a < 2; ++a) {
                    D2 rhoAvg = (qi.rho[a] + P.rho[a]) / 2.0;
                    D2 pEx(pb[a]);
                    pEx += rhoAvg * (distZ * g);
                    D2 pd = pEx - qi.p[a];
                    D2 vf = pd.v > 0.0 ? pd * (krb[a] / P.mu[a]) * (-T) : pd * qi.lam[a] * (-T);
                    D2 dens = pb[a] > qi.p[a].v ? D2(P.rho[a]) : qi.rho[a];
                    values[a] += vf * dens;
                }
            }
            else
            {
            const double* xI = &P.center[3 * I];
            const double* xf = &P.bfCenter[3 * f];
            const double* n = &P.bfNormal[3 * f];
            double distSq = 0;
            for (int d = 0; d < 3; ++d) { const double t = xf[d] - xI[d]; distSq += t * t; }
            double dIn[3];
            for (int d = 0; d < 3; ++d) dIn[d] = xI[d] - xf[d];
            double absDist2 = 0, gTimesDist = 0;
            for (int d = 0; d < 3; ++d) absDist2 += dIn[d] * dIn[d];
            for (int d = 0; d < 3; ++d) gTimesDist += P.g[d] * dIn[d];
            for (int a = 0; a < 2; ++a) {
                D2 deltay = pb[a] - qi.p[a];
                D2 pg[3];
                for (int d = 0; d < 3; ++d) pg[d] = deltay * ((xf[d] - xI[d]) / distSq);
                D2 pStatIn = (-gTimesDist) * qi.rho[a];
                D2 fsc = pStatIn / absDist2;
                for (int d = 0; d < 3; ++d) pg[d] += dIn[d] * fsc;
                D2 tmp(0.0);
                for (int d = 0; d < 3; ++d) tmp += pg[d] * n[d];
                D2 mob = tmp > 0.0 ? D2(krb[a] / P.mu[a]) : qi.lam[a];
                D2 vf(0.0);
                for (int d = 0; d < 3; ++d) {
                    D2 fv = P.perm[3 * I + d] * pg[d];
                    fv *= -mob;
                    vf += fv * n[d];
                }
                D2 dens = pb[a] > qi.p[a].v ? D2(P.rho[a]) : qi.rho[a];
                values[a] += vf * dens;
            }
            }
        }
        const double aa = P.bfArea[f] * 1.0;
        for (int e = 0; e < 2; ++e) values[e] *= aa;
        for (int e = 0; e < 2; ++e) res[e] += values[e];
        for (int e = 0; e < 2; ++e) sc[e] += std::abs(values[e].v);
    }
    // volumetric residual (fvbaselocalresidual.hh:174-190)
    for (int e = 0; e < 2; ++e) res[e] /= P.volume[I];
    k = 0;
    for (int c = P.connPtr[I]; c < P.connPtr[I + 1]; ++c, ++k)
        for (int e = 0; e < 2; ++e) resJ[k * 2 + e] /= P.volume[P.connNbr[c]];
}

static void elementBlackoil(Sim& S, int I, const IQ3& qi, const std::vector<IQ3>& iq, bool iter0, D3* res,
                            std::vector<D3>& resJ, double* sc)
{
    const Prob& P = S.P;
    const BlackOilPvt& T = P.pvt;
    const double rhoRef[3] = {T.rhoRefW, T.rhoRefO, T.rhoRefG};
    const int compOfPhase[3] = {1, 0, 2};
    for (int e = 0; e < 3; ++e) {
        res[e] = D3(0.0);
        sc[e] = 0.0;
    }
    const int nc = P.connPtr[I + 1] - P.connPtr[I];
    resJ.assign(3 * nc, D3(0.0));
    int k = 0;
    for (int c = P.connPtr[I]; c < P.connPtr[I + 1]; ++c, ++k) {
        const int Jc = P.connNbr[c];
        const IQ3& qj = iq[Jc];
        double pJ[3], rhoJ[3], lamJ[3];
        for (int a = 0; a < 3; ++a) { pJ[a] = qj.p[a].v; rhoJ[a] = qj.rho[a].v; lamJ[a] = qj.lam[a].v; }
        D3 vf[3];
        bool upI[3];
        darcyInterior<D3, 3>(P, I, Jc, c, qi.p, pJ, qi.rho, rhoJ, qi.lam, lamJ, vf, upI);
        D3 flux[3] = {D3(0.0), D3(0.0), D3(0.0)};
        // BlackOilLocalResidual::computeFlux / evalPhaseFluxes_
        for (int a = 0; a < 3; ++a) {
            D3 invB = upI[a] ? qi.invB[a] : D3(qj.invB[a].v);
            D3 svf = invB * vf[a];
            flux[compOfPhase[a]] += svf * rhoRef[a];
            if (a == 1) {
                D3 Rs = upI[a] ? qi.Rs : D3(qj.Rs.v);
                flux[2] += Rs * svf * T.rhoRefG;
            }
        }
        double alpha = 1.0;
        alpha *= P.connArea[c];
        for (int e = 0; e < 3; ++e) flux[e] *= alpha;
        for (int e = 0; e < 3; ++e) {
            res[e] += flux[e];
            resJ[k * 3 + e] -= flux[e];
            sc[e] += std::abs(flux[e].v);
        }
    }
    {
        const double scvVolume = P.volume[I] * 1.0;
        D3 tmp[3] = {D3(0.0), D3(0.0), D3(0.0)};
        // BlackOilLocalResidual::computeStorage
        D3 phi(qi.phi);
        for (int a = 0; a < 3; ++a) {
            D3 sv = qi.S[a] * qi.invB[a] * phi;
            tmp[compOfPhase[a]] += sv;
            if (a == 1) tmp[2] += qi.Rs * sv;
        }
        tmp[1] *= T.rhoRefW;
        tmp[2] *= T.rhoRefG;
        tmp[0] *= T.rhoRefO;
        double tmp2[3];
        if (iter0) {
            for (int e = 0; e < 3; ++e) tmp2[e] = tmp[e].v;
            for (int e = 0; e < 3; ++e) S.storageOld[I * 3 + e] = tmp2[e];
        }
        else
            for (int e = 0; e < 3; ++e) tmp2[e] = S.storageOld[I * 3 + e];
        for (int e = 0; e < 3; ++e) {
            sc[e] += std::abs(tmp[e].v) * (scvVolume / S.dt) + std::abs(tmp2[e]) * (scvVolume / S.dt);
            tmp[e] -= tmp2[e];
            tmp[e] *= scvVolume / S.dt;
            res[e] += tmp[e];
        }
        for (int e = 0; e < 3; ++e) res[e] -= 0.0 * scvVolume;
    }
    // black-oil problems here only have no-flow or mass-rate boundaries
    for (int f = P.bfPtr[I]; f < P.bfPtr[I + 1]; ++f) {
        if (P.bfType[f] != GBFV_BC_MASSRATE) continue;
        const double aa = P.bfArea[f] * 1.0;
        for (int e = 0; e < 3; ++e) res[e] += D3(P.bfValue[4 * f + e]) * aa;
    }
    for (int e = 0; e < 3; ++e) res[e] /= P.volume[I];
    k = 0;
    for (int c = P.connPtr[I]; c < P.connPtr[I + 1]; ++c, ++k)
        for (int e = 0; e < 3; ++e) resJ[k * 3 + e] /= P.volume[P.connNbr[c]];
}

// TpfaLinearizer::linearize_ for cell I (tpfalinearizer.hh:711-866) with
// BlackOilLocalResidualTPFA (blackoillocalresidualtpfa.hh:234-505): for
// each neighbour record (the cell's interior faces in intersection order)
// the flux of calculateFluxes_ times the face area into row I and, negated,
// into column I of the neighbour's row; then the storage term times
// volume / dt; rows are not divided by the volume.  The pressure difference
// and the upstream choice of calculateFluxes_ come from the reference's
// flux module (absent here) and are restated from the transmissibility
// module (transfluxmodule.hh:201-318): average density times the depth
// term, sign of the difference, ties by volume then global index.  The
// face transmissibility is the transmissibility module's too (harmonic of
// the half transmissibilities); transMult (rock compaction) is 1.
static void elementBlackoilTpfa(Sim& S, int I, const IQ3& qi, const std::vector<IQ3>& iq, bool iter0, D3* res,
                                std::vector<D3>& resJ, double* sc)
{
    const Prob& P = S.P;
    const BlackOilPvt& T = P.pvt;
    const double rhoRef[3] = {T.rhoRefW, T.rhoRefO, T.rhoRefG};
    const int compOfPhase[3] = {1, 0, 2};
    for (int e = 0; e < 3; ++e) {
        res[e] = D3(0.0);
        sc[e] = 0.0;
    }
    const int nc = P.connPtr[I + 1] - P.connPtr[I];
    resJ.assign(3 * nc, D3(0.0));
    const double g = P.g[P.dimWorld - 1];
    int k = 0;
    for (int c = P.connPtr[I]; c < P.connPtr[I + 1]; ++c, ++k) {
        const int Jc = P.connNbr[c];
        const IQ3& qj = iq[Jc];
        const double trans = transInteriorT(P, I, Jc, c);
        const double faceArea = P.connArea[c];
        const double distZ = P.center[3 * I + P.dimWorld - 1] - P.center[3 * Jc + P.dimWorld - 1];
        D3 flux[3] = {D3(0.0), D3(0.0), D3(0.0)};
        for (int a = 0; a < 3; ++a) {
            // calculatePhasePressureDiff_
            D3 rhoAvg = (qi.rho[a] + qj.rho[a].v) / 2.0;
            D3 pEx(qj.p[a].v);
            pEx += rhoAvg * (distZ * g);
            D3 pd = pEx - qi.p[a];
            bool upI;
            if (pd.v > 0.0) upI = false;
            else if (pd.v < 0.0) upI = true;
            else {
                const double Vin = P.volume[I], Vex = P.volume[Jc];
                upI = Vin > Vex ? true : (Vin < Vex ? false : I < Jc);
            }
            D3 darcyFlux = upI ? (pd * qi.lam[a]) * (-trans / faceArea) : pd * (qj.lam[a].v * (-trans / faceArea));
            // evalPhaseFluxes_
            D3 invB = upI ? qi.invB[a] : D3(qj.invB[a].v);
            D3 svf = invB * darcyFlux;
            flux[compOfPhase[a]] += svf * rhoRef[a];
            if (a == 1) {
                D3 Rs = upI ? qi.Rs : D3(qj.Rs.v);
                flux[2] += Rs * svf * T.rhoRefG;
            }
        }
        for (int e = 0; e < 3; ++e) flux[e] *= faceArea;
        for (int e = 0; e < 3; ++e) {
            res[e] += flux[e];
            resJ[k * 3 + e] -= flux[e];
            sc[e] += std::abs(flux[e].v);
        }
    }
    {
        const double storefac = P.volume[I] / S.dt;
        D3 tmp[3] = {D3(0.0), D3(0.0), D3(0.0)};
        D3 phi(qi.phi);
        for (int a = 0; a < 3; ++a) {
            D3 sv = qi.S[a] * qi.invB[a] * phi;
            tmp[compOfPhase[a]] += sv;
            if (a == 1) tmp[2] += qi.Rs * sv;
        }
        tmp[1] *= T.rhoRefW;
        tmp[2] *= T.rhoRefG;
        tmp[0] *= T.rhoRefO;
        double tmp2[3];
        if (iter0) {
            for (int e = 0; e < 3; ++e) tmp2[e] = tmp[e].v;
            for (int e = 0; e < 3; ++e) S.storageOld[I * 3 + e] = tmp2[e];
        }
        else
            for (int e = 0; e < 3; ++e) tmp2[e] = S.storageOld[I * 3 + e];
        for (int e = 0; e < 3; ++e) {
            sc[e] += std::abs(tmp[e].v) * storefac + std::abs(tmp2[e]) * storefac;
            tmp[e] -= tmp2[e];
            tmp[e] *= storefac;
            res[e] += tmp[e];
        }
    }
    // boundary terms (mass rate; no-flow adds nothing), after the cell terms
    for (int f = P.bfPtr[I]; f < P.bfPtr[I + 1]; ++f) {
        if (P.bfType[f] != GBFV_BC_MASSRATE) continue;
        const double aa = P.bfArea[f] * 1.0;
        for (int e = 0; e < 3; ++e) res[e] += D3(P.bfValue[4 * f + e]) * aa;
    }
}

// the TPFA linearizer's cell loop (tpfalinearizer.hh:711-866)
static void linearizeBlackoilTpfa(Sim& S, const std::vector<IQ3>& iq)
{
    const bool iter0 = S.newtonIter == 0;
#pragma omp parallel for schedule(static)
    for (int I = 0; I < S.N; ++I) {
        D3 res[3];
        double sc[3];
        std::vector<D3> resJ;
        elementBlackoilTpfa(S, I, iq[I], iq, iter0, res, resJ, sc);
        for (int e = 0; e < 3; ++e) S.rscale[I * 3 + e] = sc[e];
        scatterElement<3>(S, I, res, resJ);
    }
}

// one element of FvBaseAdLocalLinearizer::linearize + scatter, per model
// (fvbaseadlocallinearizer.hh:173-292, fvbaselinearizer.hh:510-593)
static void linearizeImmiscible(Sim& S, const std::vector<IQ2>& iq)
{
    const bool iter0 = S.newtonIter == 0;
#pragma omp parallel for schedule(static)
    for (int I = 0; I < S.N; ++I) {
        D2 res[2];
        double sc[2];
        std::vector<D2> resJ;
        elementImmiscible(S, I, iq[I], iq, iter0, res, resJ, sc);
        for (int e = 0; e < 2; ++e) S.rscale[I * 2 + e] = sc[e] / S.P.volume[I];
        scatterElement<2>(S, I, res, resJ);
    }
}

// the black-oil element loop (fvbaseadlocallinearizer.hh:173-292,
// fvbaselinearizer.hh:510-593)
static void linearizeBlackoil(Sim& S, const std::vector<IQ3>& iq)
{
    const bool iter0 = S.newtonIter == 0;
#pragma omp parallel for schedule(static)
    for (int I = 0; I < S.N; ++I) {
        D3 res[3];
        double sc[3];
        std::vector<D3> resJ;
        elementBlackoil(S, I, iq[I], iq, iter0, res, resJ, sc);
        for (int e = 0; e < 3; ++e) S.rscale[I * 3 + e] = sc[e] / S.P.volume[I];
        scatterElement<3>(S, I, res, resJ);
    }
}

// ------------------------------------------ finite-difference linearizer --
// primaryVarWeight: immisciblemodel.hh:321-333 (pressure 10 / reference
// pressure, else 1), blackoilmodel.hh:395-440 (Sw 1, po 1/300e5, the gas
// variable by its meaning: Sg 1, Rs 1/250, Rv 1/0.025)
static double pvWeight(const Sim& S, int I, int pv)
{
    if (S.P.model == GBFV_MODEL_IMMISCIBLE_2P) return pv == 0 ? 10 / S.refPressure : 1.0;
    if (pv == 0) return 1.0;
    if (pv == 1) return 1.0 / 300e5;
    const int m = S.meaning[I];
    return m == GBFV_GAS_SG ? 1.0 : m == GBFV_GAS_RS ? 1.0 / 250. : 1.0 / 0.025;
}

// FvBaseFdLocalLinearizer::linearize / evalPartialDerivative_ /
// updateLocalJacobian_ (fvbasefdlocallinearizer.hh:222-240, 414-510): the
// element's local residual, then per primary variable of the element the
// residual at the deflected state(s) -- +eps (method >= 0), then
// -(delta + eps) from there (method <= 0) -- their difference divided by
// the total deflection delta.  eps = BaseEpsilon / primaryVarWeight with
// BaseEpsilon = max(0.9123e-10, machine epsilon * 1.23e3)
// (fvbasefdlocallinearizer.hh:75-79, 272-283).  The neighbours keep their
// unperturbed intensive quantities; the storage of the old time level comes
// from the cache the unperturbed evaluation filled (stashed quantities,
// fvbaselocalresidual.hh:537-564).
template <int B, class IQ, class IqFn, class ElemFn>
static void linearizeFd(Sim& S, const std::vector<IQ>& iq, IqFn iqOf, ElemFn elem)
{
    using D = Dual<B>;
    const Prob& P = S.P;
    const bool iter0 = S.newtonIter == 0;
    const int method = S.prm.numeric_difference_method;
    const double baseEps = std::max(0.9123e-10, std::numeric_limits<double>::epsilon() * 1.23e3);
#pragma omp parallel for schedule(static)
    for (int I = 0; I < S.N; ++I) {
        D res0[B], resD[B];
        double sc[B], scD[B];
        std::vector<D> resJ0, resJD;
        elem(S, I, iq[I], iq, iter0, res0, resJ0, sc);
        for (int e = 0; e < B; ++e) S.rscale[I * B + e] = sc[e] / P.volume[I];
        for (int e = 0; e < B; ++e) S.residual[I * B + e] = res0[e].v;
        const int nc = P.connPtr[I + 1] - P.connPtr[I];
        std::vector<double> dJ((size_t)B * nc);
        double* diag = &S.J.val[(size_t)S.diagSlot[I] * B * B];
        for (int pv = 0; pv < B; ++pv) {
            double xs[B];
            for (int e = 0; e < B; ++e) xs[e] = S.x[(size_t)I * B + e];
            const double eps = baseEps / pvWeight(S, I, pv);
            double delta = 0.0;
            double dI[B];
            if (method >= 0) {
                xs[pv] += eps;
                delta += eps;
                elem(S, I, iqOf(S, I, xs), iq, false, resD, resJD, scD);
                for (int e = 0; e < B; ++e) dI[e] = resD[e].v;
                for (int k = 0; k < B * nc; ++k) dJ[k] = resJD[k].v;
            }
            else {
                for (int e = 0; e < B; ++e) dI[e] = res0[e].v;
                for (int k = 0; k < B * nc; ++k) dJ[k] = resJ0[k].v;
            }
            if (method <= 0) {
                xs[pv] -= delta + eps;
                delta += eps;
                elem(S, I, iqOf(S, I, xs), iq, false, resD, resJD, scD);
                for (int e = 0; e < B; ++e) dI[e] -= resD[e].v;
                for (int k = 0; k < B * nc; ++k) dJ[k] -= resJD[k].v;
            }
            else {
                for (int e = 0; e < B; ++e) dI[e] -= res0[e].v;
                for (int k = 0; k < B * nc; ++k) dJ[k] -= resJ0[k].v;
            }
            for (int e = 0; e < B; ++e) diag[e * B + pv] = dI[e] / delta;
            int k = 0;
            for (int c = P.connPtr[I]; c < P.connPtr[I + 1]; ++c, ++k) {
                double* ob = &S.J.val[(size_t)S.connSlot[c] * B * B];
                for (int e = 0; e < B; ++e) ob[e * B + pv] = dJ[(size_t)k * B + e] / delta;
            }
        }
    }
}

// constrained rows: zero residual, identity diagonal, no off-diagonal blocks
// (FvBaseLinearizer::applyConstraintsToLinearization_, fvbaselinearizer.hh:649-666)
static void applyConstraintsToLinearization(Sim& S)
{
    const int b = S.b;
    for (int I = 0; I < S.N; ++I) {
        if (S.P.constraint[I] < 0) continue;
        for (int k = S.J.rowPtr[I]; k < S.J.rowPtr[I + 1]; ++k) {
            double* blk = &S.J.val[(size_t)k * b * b];
            for (int e = 0; e < b * b; ++e) blk[e] = 0.0;
            if (S.J.col[k] == I)
                for (int e = 0; e < b; ++e) blk[e * b + e] = 1.0;
        }
        for (int e = 0; e < b; ++e) S.residual[I * b + e] = 0.0;
    }
}

#include "vcfv.hh"

// FvBaseLinearizer::linearizeDomain / linearize_ (fvbaselinearizer.hh:201-241,
// 510-593): constraints, intensive quantities, element loop, constraints
static void linearize(Sim& S)
{
    applyConstraintsToSolution(S);
    std::fill(S.J.val.begin(), S.J.val.end(), 0.0);
    std::fill(S.residual.begin(), S.residual.end(), 0.0);
    const bool fd = S.prm.local_linearizer == GBFV_LIN_FD;
    if (S.vcfv && S.P.model == GBFV_MODEL_BLACKOIL_3P) {
        if (fd) throw NumericalProblem("vertex-centred black-oil grids take the AD local linearizer", GBFV_ERR_UNSUPPORTED);
        std::vector<IQ3> iq(S.N);
#pragma omp parallel for schedule(static)
        for (int I = 0; I < S.N; ++I) iq[I] = blackoilIQ(S.P, I, &S.x[I * 3], S.meaning[I]);
        linearizeBlackoilVcfv(S, iq);
    }
    else if (S.vcfv) {
        std::vector<IQ2> iq(S.N);
#pragma omp parallel for schedule(static)
        for (int I = 0; I < S.N; ++I) iq[I] = immiscibleIQ(S.P, I, &S.x[I * 2]);
        if (fd)
            linearizeImmiscibleVcfvFd(S, iq);
        else
            linearizeImmiscibleVcfv(S, iq);
    }
    else if (S.P.model == GBFV_MODEL_IMMISCIBLE_2P) {
        std::vector<IQ2> iq(S.N);
#pragma omp parallel for schedule(static)
        for (int I = 0; I < S.N; ++I) iq[I] = immiscibleIQ(S.P, I, &S.x[I * 2]);
        if (fd)
            linearizeFd<2>(S, iq, [](const Sim& s, int I, const double* x) { return immiscibleIQ(s.P, I, x); },
                           elementImmiscible);
        else
            linearizeImmiscible(S, iq);
    }
    else {
        std::vector<IQ3> iq(S.N);
#pragma omp parallel for schedule(static)
        for (int I = 0; I < S.N; ++I) iq[I] = blackoilIQ(S.P, I, &S.x[I * 3], S.meaning[I]);
        if (S.prm.linearizer == GBFV_LINEARIZER_TPFA)
            linearizeBlackoilTpfa(S, iq);
        else if (fd)
            linearizeFd<3>(S, iq,
                           [](const Sim& s, int I, const double* x) { return blackoilIQ(s.P, I, x, s.meaning[I]); },
                           elementBlackoil);
        else
            linearizeBlackoil(S, iq);
    }
    for (double v : S.residual)
        if (!std::isfinite(v)) throw NumericalProblem("non-finite residual", GBFV_ERR_NONFINITE);
    applyConstraintsToLinearization(S);
}

// ------------------------------------------------------ linear solver -----
// block helpers (row-major b x b)
// pivot inverse: MatrixBlock's invertMatrix (matrixblock.hh:40-66), which
// calls dune-common's FMatrixHelp::invertMatrix for 2x2 and 3x3 blocks
// (not vendored; the cofactor formula restated)
static void blockInvert(int b, double* A)
{
    // adjugate / determinant
    if (b == 2) {
        const double a = A[0], bb = A[1], c = A[2], d = A[3];
        const double det = a * d - bb * c;
        if (det == 0.0 || !std::isfinite(det)) throw NumericalProblem("singular ILU pivot", GBFV_ERR_SINGULAR);
        const double id = 1.0 / det;
        A[0] = d * id; A[1] = -bb * id; A[2] = -c * id; A[3] = a * id;
        return;
    }
    const double a00 = A[0], a01 = A[1], a02 = A[2];
    const double a10 = A[3], a11 = A[4], a12 = A[5];
    const double a20 = A[6], a21 = A[7], a22 = A[8];
    const double c00 = a11 * a22 - a12 * a21;
    const double c01 = a12 * a20 - a10 * a22;
    const double c02 = a10 * a21 - a11 * a20;
    const double det = a00 * c00 + a01 * c01 + a02 * c02;
    if (det == 0.0 || !std::isfinite(det)) throw NumericalProblem("singular ILU pivot", GBFV_ERR_SINGULAR);
    const double id = 1.0 / det;
    A[0] = c00 * id;
    A[1] = (a02 * a21 - a01 * a22) * id;
    A[2] = (a01 * a12 - a02 * a11) * id;
    A[3] = c01 * id;
    A[4] = (a00 * a22 - a02 * a20) * id;
    A[5] = (a02 * a10 - a00 * a12) * id;
    A[6] = c02 * id;
    A[7] = (a01 * a20 - a00 * a21) * id;
    A[8] = (a00 * a11 - a01 * a10) * id;
}
// A = A * M (dune-common FieldMatrix::rightmultiply, used by dune-istl's
// block ILU(0) on the blocks istlpreconditionerwrappers.hh:161 hands it)
static void rightMultiply(int b, double* A, const double* M)
{
    double C[9];
    std::memcpy(C, A, sizeof(double) * b * b);
    for (int i = 0; i < b; ++i)
        for (int j = 0; j < b; ++j) {
            double s = 0;
            for (int k = 0; k < b; ++k) s += C[i * b + k] * M[k * b + j];
            A[i * b + j] = s;
        }
}
// y -= A x (dune-common FieldMatrix::mmv, as dune-istl's ILU back-solve
// uses it on the same blocks)
static void mmv(int b, const double* A, const double* x, double* y)
{
    for (int i = 0; i < b; ++i)
        for (int j = 0; j < b; ++j) y[i] -= A[i * b + j] * x[j];
}

// block ILU(0), natural order, inverse pivots stored on the diagonal
// (dune-istl blockILU0Decomposition, called through Dune::SeqILU from
// istlpreconditionerwrappers.hh:161-180)
static void ilu0Factor(const Bcrs& A, std::vector<double>& F)
{
    const int b = A.b, bb = b * b;
    F = A.val;
    for (int i = 0; i < A.n; ++i) {
        int ij = A.rowPtr[i];
        for (; ij < A.rowPtr[i + 1] && A.col[ij] < i; ++ij) {
            const int j = A.col[ij];
            const int jj = A.find(j, j);
            rightMultiply(b, &F[(size_t)ij * bb], &F[(size_t)jj * bb]);
            int ik = ij + 1, jk = jj + 1;
            while (ik < A.rowPtr[i + 1] && jk < A.rowPtr[j + 1]) {
                if (A.col[ik] == A.col[jk]) {
                    // B = L_ij * U_jk ; A_ik -= B
                    double B[9];
                    for (int r = 0; r < b; ++r)
                        for (int s = 0; s < b; ++s) {
                            double t = 0;
                            for (int q = 0; q < b; ++q) t += F[(size_t)ij * bb + r * b + q] * F[(size_t)jk * bb + q * b + s];
                            B[r * b + s] = t;
                        }
                    for (int e = 0; e < bb; ++e) F[(size_t)ik * bb + e] -= B[e];
                    ++ik; ++jk;
                }
                else if (A.col[ik] < A.col[jk]) ++ik;
                else ++jk;
            }
        }
        if (ij >= A.rowPtr[i + 1] || A.col[ij] != i) throw NumericalProblem("diagonal entry missing", GBFV_ERR_ARG);
        blockInvert(b, &F[(size_t)ij * bb]);
    }
}

// dune-istl blockILUBacksolve: v = (LU)^-1 d, the apply of Dune::SeqILU that
// PreconditionerWrapperILU wraps (istlpreconditionerwrappers.hh:149-180)
static void ilu0Apply(const Bcrs& A, const std::vector<double>& F, std::vector<double>& v, const std::vector<double>& d)
{
    const int b = A.b, bb = b * b;
    for (int i = 0; i < A.n; ++i) {
        double rhs[3];
        for (int e = 0; e < b; ++e) rhs[e] = d[i * b + e];
        for (int k = A.rowPtr[i]; k < A.rowPtr[i + 1] && A.col[k] < i; ++k)
            mmv(b, &F[(size_t)k * bb], &v[A.col[k] * b], rhs);
        for (int e = 0; e < b; ++e) v[i * b + e] = rhs[e];
    }
    for (int i = A.n - 1; i >= 0; --i) {
        double rhs[3];
        for (int e = 0; e < b; ++e) rhs[e] = v[i * b + e];
        int k = A.rowPtr[i + 1] - 1;
        for (; A.col[k] > i; --k) mmv(b, &F[(size_t)k * bb], &v[A.col[k] * b], rhs);
        const double* Di = &F[(size_t)k * bb];
        for (int r = 0; r < b; ++r) {
            double s = 0;
            for (int c = 0; c < b; ++c) s += Di[r * b + c] * rhs[c];
            v[i * b + r] = s;
        }
    }
}

// y = A x (BCRSMatrix::mv through OverlappingOperator::apply,
// overlappingoperator.hh:58-63)
static void spmv(const Bcrs& A, const std::vector<double>& x, std::vector<double>& y)
{
    const int b = A.b, bb = b * b;
    for (int i = 0; i < A.n; ++i) {
        double yi[3] = {0, 0, 0};
        for (int k = A.rowPtr[i]; k < A.rowPtr[i + 1]; ++k) {
            const double* blk = &A.val[(size_t)k * bb];
            const double* xj = &x[A.col[k] * b];
            for (int r = 0; r < b; ++r)
                for (int c = 0; c < b; ++c) yi[r] += blk[r * b + c] * xj[c];
        }
        for (int e = 0; e < b; ++e) y[i * b + e] = yi[e];
    }
}

#include "amg.hh"

// Summation order of the scalar products (a test switch, process-wide):
// 0 = the reference's sequential loop; L > 0 = another correct order, the
// one a parallel machine uses: L strided partial sums (lane t takes blocks
// t, t + L, ...), combined by a pairwise tree.  Only the rounding of the
// dot products changes; every other operation stays as it is.
static int g_dotLanes = 0;

// OverlappingScalarProduct::dot (overlappingscalarproduct.hh:58-70) on one
// rank: the plain sum over all entries
static double dot(const std::vector<double>& a, const std::vector<double>& b, int bs)
{
    const size_t n = a.size() / bs;
    if (g_dotLanes <= 0) {
        double s = 0;
        for (size_t i = 0; i < n; ++i) {
            double t = 0;
            for (int e = 0; e < bs; ++e) t += a[i * bs + e] * b[i * bs + e];
            s += t;
        }
        return s;
    }
    const size_t L = (size_t)g_dotLanes;
    std::vector<double> part(L, 0.0);
    for (size_t i = 0; i < n; ++i) {
        double t = 0;
        for (int e = 0; e < bs; ++e) t += a[i * bs + e] * b[i * bs + e];
        part[i % L] += t;
    }
    for (size_t w = 1; w < L; w *= 2)
        for (size_t j = 0; j + w < L; j += 2 * w) part[j] += part[j + w];
    return part[0];
}

// CombinedCriterion (combinedcriterion.hh:55-209): max-norm residual
// reduction or absolute residual, divergence above maxRes; setInitial
// :116-129, update :131-135, converged :137-144
struct Criterion {
    double redTol, absTol, maxRes;
    double resErr = 0, initErr = 0, lastErr = 0;
    bool stagnates = false;
    void updateErrors(const std::vector<double>& change, const std::vector<double>& r)
    {
        lastErr = resErr;
        resErr = 0;
        stagnates = true;
        for (size_t i = 0; i < r.size(); ++i) {
            resErr = std::max(resErr, std::abs(r[i]));
            if (stagnates && change[i] != 0.0) stagnates = false;
        }
    }
    void setInitial(const std::vector<double>& x, const std::vector<double>& r)
    {
        updateErrors(x, r);
        stagnates = false;
        resErr = std::max(resErr, std::numeric_limits<double>::min() * 1e10);
        initErr = resErr;
        lastErr = resErr;
    }
    bool converged() const
    {
        return resErr / std::max(1e-20, initErr) <= redTol || resErr <= absTol;
    }
    bool failed() const { return !converged() && (stagnates || resErr > maxRes); }
};

// the preconditioner application v = M^-1 d (v is written in full)
using Precond = std::function<void(std::vector<double>&, const std::vector<double>&)>;

// BiCGStabSolver::apply (bicgstabsolver.hh:120-330) with the preconditioner
// of the backend: SeqILU(0) (ParallelBiCGStabSolverBackend) or the AMG
// V-cycle (ParallelAmgBackend)
static bool bicgstab(const Bcrs& A, const Precond& prec, const std::vector<double>& b, std::vector<double>& x,
                     Criterion& crit, int maxIter, int& iters)
{
    const double eps = std::numeric_limits<double>::min() * 1e10;
    const int bs = A.b;
    const size_t n = b.size();
    x.assign(n, 0.0);
    std::vector<double> r = b;
    crit.setInitial(x, r);
    iters = 0;
    if (crit.converged()) return true;
    const std::vector<double>& r0hat = b;
    double rho = 1.0, alpha = 1.0, omega = 1.0;
    std::vector<double> v(n, 0.0), p(n, 0.0), y(n, 0.0), z(n, 0.0);
    std::vector<double>& h = x;
    std::vector<double>& s = r;
    std::vector<double>& t = y;
    for (; iters < maxIter; ++iters) {
        const double rho_i = dot(r0hat, r, bs);
        if (std::abs(rho) <= eps || std::abs(omega) <= eps) throw NumericalProblem("BiCGStab breakdown", GBFV_ERR_BREAKDOWN);
        const double beta = (rho_i / rho) * (alpha / omega);
        rho = rho_i;
        for (size_t i = 0; i < n; ++i) {
            double tmp = v[i];
            tmp *= omega;
            tmp -= p[i];
            tmp *= -beta;
            p[i] = r[i];
            p[i] += tmp;
        }
        prec(y, p);
        spmv(A, y, v);
        double denom = dot(r0hat, v, bs);
        if (std::abs(denom) <= eps) throw NumericalProblem("BiCGStab breakdown", GBFV_ERR_BREAKDOWN);
        alpha = rho_i / denom;
        if (std::abs(alpha) <= eps) throw NumericalProblem("BiCGStab stagnation", GBFV_ERR_BREAKDOWN);
        for (size_t i = 0; i < n; ++i) {
            double tmp = y[i];
            tmp *= alpha;
            tmp += x[i];
            h[i] = tmp;
            tmp = v[i];
            tmp *= alpha;
            s[i] -= tmp;
        }
        crit.updateErrors(y, s);
        if (crit.converged()) return true;
        if (crit.failed()) return false;
        z = s;
        prec(z, s);
        spmv(A, z, t);
        denom = dot(t, t, bs);
        if (std::abs(denom) <= eps) throw NumericalProblem("BiCGStab breakdown", GBFV_ERR_BREAKDOWN);
        omega = dot(t, s, bs) / denom;
        if (std::abs(omega) <= eps) throw NumericalProblem("BiCGStab stagnation", GBFV_ERR_BREAKDOWN);
        for (size_t i = 0; i < n; ++i) x[i] += omega * z[i];
        crit.updateErrors(z, r);
        if (crit.converged()) return true;
        if (crit.failed()) return false;
        for (size_t i = 0; i < n; ++i) r[i] += -omega * t[i];
    }
    return false;
}

// the criterion's parameters as ParallelBiCGStabSolverBackend::prepareSolver_
// sets them (parallelbicgstabbackend.hh:136-146): an absolute tolerance
// below 0 becomes the Newton tolerance / 100
static Criterion makeCriterion(const gbfv_params& prm)
{
    Criterion c;
    c.redTol = prm.linear_tolerance;
    c.absTol = prm.linear_abs_tolerance < 0 ? prm.newton_tolerance / 100.0 : prm.linear_abs_tolerance;
    c.maxRes = prm.linear_max_error;
    return c;
}

// ------------------------------------------------------------ Newton ------
// NewtonMethod::preSolve_ (newtonmethod.hh:572-607): max |r| over the
// unconstrained cells of positive volume
static double newtonError(const Sim& S)
{
    double err = 0;
    for (int I = 0; I < S.N; ++I) {
        if (S.P.volume[I] <= 0.0) continue;
        if (S.P.constraint[I] >= 0) continue;
        for (int e = 0; e < S.b; ++e) err = std::max(std::abs(S.residual[I * S.b + e] * 1.0), err);
    }
    return err;
}

static double signum(double v) { return (v > 0) - (v < 0); }

// BlackOilPrimaryVariables::adaptPrimaryVariables for Sw / Po / {Sg, Rs}
// (blackoilprimaryvariables.hh:549-909)
static bool adaptPrimaryVariables(const Sim& S, double* pv, int& meaning, double eps)
{
    const gbfv_params& prm = S.prm;
    double sw = pv[0];
    double sg = meaning == GBFV_GAS_SG ? pv[2] : 0.0;
    if (sw >= prm.water_only_threshold) {
        pv[0] = std::min(prm.max_water_saturation, sw);
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
            const double rsSat = S.P.pvt.rsSat.eval(po);
            pv[2] = std::min(std::numeric_limits<double>::max() / 2, rsSat);
            changed = true;
        }
    }
    else if (meaning == GBFV_GAS_RS) {
        const double po = pv[1];
        const double rsSat = S.P.pvt.rsSat.eval(po);
        const double rs = pv[2];
        if (rs > std::min(std::numeric_limits<double>::max() / 2, rsSat * (1.0 + eps))) {
            meaning = GBFV_GAS_SG;
            pv[2] = 0.0;
            changed = true;
        }
    }
    return changed;
}

// NewtonMethod::update_ (newtonmethod.hh:665-731) and
// BlackOilNewtonMethod::updatePrimaryVariables_ (blackoilnewtonmethod.hh:226-427)
static int newtonUpdate(Sim& S, const std::vector<double>& cur, const std::vector<int>& curMeaning)
{
    double onenorm = 0;
    for (double v : S.dx) onenorm += std::abs(v);
    if (!std::isfinite(onenorm)) throw NumericalProblem("Non-finite update!", GBFV_ERR_NONFINITE);
    const int b = S.b;
    int switched = 0;
    for (int I = 0; I < S.N; ++I) {
        const int k = S.P.constraint[I];
        if (k >= 0) {
            for (int e = 0; e < b; ++e) S.x[I * b + e] = S.P.consPv[3 * k + e];
            S.meaning[I] = S.P.consMeaning[k];
            continue;
        }
        if (S.P.model == GBFV_MODEL_IMMISCIBLE_2P) {
            for (int e = 0; e < b; ++e) {
                S.x[I * b + e] = cur[I * b + e];
                S.x[I * b + e] -= S.dx[I * b + e];
            }
            continue;
        }
        const double* up = &S.dx[I * 3];
        const double* cv = &cur[I * 3];
        const int mg = curMeaning[I];
        double dSw = 0, dSo = 0, dSg = 0;
        dSw = up[0];
        dSo -= dSw;
        if (mg == GBFV_GAS_SG) { dSg = up[2]; dSo -= dSg; }
        double maxSat = std::max(std::abs(dSg), std::abs(dSo));
        maxSat = std::max(maxSat, std::abs(dSw));
        maxSat = std::max(maxSat, 0.0);
        double satAlpha = 1.0;
        if (maxSat > S.prm.ds_max) satAlpha = S.prm.ds_max / maxSat;
        double nv[3];
        for (int pvIdx = 0; pvIdx < 3; ++pvIdx) {
            double delta = up[pvIdx];
            if (pvIdx == 1) {
                if (std::abs(delta) > S.prm.dp_max_rel * cv[pvIdx]) delta = signum(delta) * S.prm.dp_max_rel * cv[pvIdx];
            }
            else if (pvIdx == 0) {
                delta *= satAlpha;
            }
            else {
                if (mg == GBFV_GAS_SG) delta *= satAlpha;
                else if (delta > cv[2]) delta = cv[2];
            }
            nv[pvIdx] = cv[pvIdx] - delta;
            if (pvIdx == 1) nv[pvIdx] = std::min(std::max(nv[pvIdx], S.prm.pressure_min), S.prm.pressure_max);
        }
        int m = mg;
        const double eps = S.wasSwitched[I] ? S.prm.pv_oscillation_threshold : 0.0;
        S.wasSwitched[I] = adaptPrimaryVariables(S, nv, m, eps);
        if (S.wasSwitched[I]) ++switched;
        for (int e = 0; e < 3; ++e) S.x[I * 3 + e] = nv[e];
        S.meaning[I] = m;
    }
    return switched;
}

// ParallelBaseBackend::prepare / setResidual / setMatrix / solve
// (parallelbasebackend.hh:182-284): the system copied into the solver's
// own storage, then the BiCGStab loop below on it
static int solveLinear(Sim& S, int& iters)
{
    std::vector<double> F;
    Precond prec;
    if (S.prm.linear_solver == GBFV_LINSOLVER_AMG) {
        if (!S.amg) S.amg = std::make_shared<AmgHierarchy>();
        amgSetup(*S.amg, S.J, S.prm.amg_coarsen_target);
        const AmgHierarchy* H = S.amg.get();
        prec = [H](std::vector<double>& v, const std::vector<double>& d) { amgApply(*H, v, d); };
    }
    else {
        ilu0Factor(S.J, F);
        const Bcrs* A = &S.J;
        const std::vector<double>* Fp = &F;
        prec = [A, Fp](std::vector<double>& v, const std::vector<double>& d) { ilu0Apply(*A, *Fp, v, d); };
    }
    Criterion crit = makeCriterion(S.prm);
    std::vector<double> xsol;
    const bool ok = bicgstab(S.J, prec, S.residual, xsol, crit, S.prm.linear_max_iterations, iters);
    S.dx = xsol;
    return ok ? GBFV_OK : GBFV_ERR_NOT_CONVERGED;
}

// NewtonMethod::apply (newtonmethod.hh:228-438)
static bool newtonApply(Sim& S, double dt, gbfv_newton_report& rep)
{
    S.dt = dt;
    S.refPressure = S.x[0];  // updateBegin (immisciblemodel.hh:301-316), before NewtonMethod::apply
    std::memset(&rep, 0, sizeof(rep));
    S.numIterations = 0;
    S.error = 0;
    S.lastError = 0;
    const int maxIt = S.prm.newton_max_iterations;
    auto converged = [&]() { return S.error <= S.prm.newton_tolerance; };
    auto proceed = [&]() {
        if (S.numIterations < 1) return true;
        if (converged()) return false;
        if (S.numIterations >= maxIt) return S.error * 4.0 < S.lastError;
        return true;
    };
    try {
        while (proceed()) {
            S.lastError = S.error;  // beginIteration_
            std::vector<double> cur = S.x;
            std::vector<int> curM = S.meaning;
            S.newtonIter = S.numIterations;
            linearize(S);
            rep.linearizations++;
            S.lastError = S.error;  // preSolve_
            S.error = newtonError(S);
            if (S.error > S.prm.newton_max_error) throw NumericalProblem("Newton error too large");
            if (!proceed()) { S.numIterations++; break; }
            int it = 0;
            const int st = solveLinear(S, it);
            rep.linear_iterations += it;
            if (st != GBFV_OK) {
                S.numIterations = S.prm.newton_target_iterations * 2;
                rep.status = st;
                rep.iterations = S.numIterations;
                rep.error = S.error;
                return false;
            }
            // applyConstraintsToSolution has already set the current constraint values
            cur = S.x;
            curM = S.meaning;
            newtonUpdate(S, cur, curM);
            S.numIterations++;
        }
    }
    catch (const NumericalProblem& e) {
        S.numIterations = S.prm.newton_target_iterations * 2;
        rep.status = e.code;
        rep.iterations = S.numIterations;
        rep.error = S.error;
        return false;
    }
    rep.iterations = S.numIterations;
    rep.error = S.error;
    if (!converged()) {
        S.numIterations = S.prm.newton_target_iterations * 2;
        rep.iterations = S.numIterations;
        rep.status = GBFV_ERR_NOT_CONVERGED;
        return false;
    }
    rep.converged = 1;
    return true;
}

// NewtonMethod::suggestTimeStepSize (newtonmethod.hh:448-465): grow or
// shrink towards the target iteration count, damped
static double suggestTimeStep(const Sim& S, double oldDt)
{
    const int target = S.prm.newton_target_iterations;
    const int n = S.numIterations;
    if (n > target) {
        const double percent = double(n - target) / target;
        return std::max(S.prm.min_time_step, oldDt / (1.0 + percent));
    }
    const double percent = double(target - n) / target;
    return std::max(S.prm.min_time_step, oldDt * (1.0 + percent / 1.2));
}

}  // namespace oracle

using namespace oracle;

// C ABI of the oracle: the entry points of include/gbfv.h with an oracle_
// prefix; the header's comments name the reference function each mirrors
extern "C" {

void oracle_default_params(gbfv_params* p)
{
    std::memset(p, 0, sizeof(*p));
    p->newton_tolerance = 1e-8;
    p->newton_max_iterations = 20;
    p->newton_target_iterations = 10;
    p->newton_max_error = 1e100;
    p->linear_tolerance = 1e-3;
    p->linear_abs_tolerance = -1.0;
    p->linear_max_iterations = 1000;
    p->linear_max_error = 1e7;
    p->precision = GBFV_PREC_FP64;
    p->inner_tolerance = 1e-3;
    p->max_refinements = 20;
    p->dp_max_rel = 0.3;
    p->ds_max = 0.2;
    p->pv_oscillation_threshold = 1e-5;
    p->pressure_min = -1e99;
    p->pressure_max = 1e99;
    p->max_water_saturation = 1.0;
    p->water_only_threshold = 1.0;
    p->min_time_step = 0.0;
    p->max_time_step = std::numeric_limits<double>::infinity();
    p->max_time_step_divisions = 10;
    p->local_linearizer = GBFV_LIN_AD;
    p->numeric_difference_method = 1;
    p->linear_solver = GBFV_LINSOLVER_ILU0;
    p->amg_coarsen_target = 5000;
    p->linearizer = GBFV_LINEARIZER_ELEMENT;
}

void* oracle_create(const gbfv_problem* prob, const gbfv_params* prm)
{
    try {
        auto* S = new Sim();
        S->P = copyProblem(*prob);
        S->prm = *prm;
        S->N = S->P.N;
        S->b = S->P.b;
        S->x.assign(S->N * S->b, 0.0);
        S->xOld = S->x;
        S->meaning.assign(S->N, 0);
        S->meaningOld = S->meaning;
        S->wasSwitched.assign(S->N, 0);
        S->storageOld.assign(S->N * S->b, 0.0);
        S->residual.assign(S->N * S->b, 0.0);
        S->rscale.assign(S->N * S->b, 0.0);
        if (S->P.numElements > 0) {
            // the vertex-centred discretization takes the immiscible model
            // with the Darcy flux module and the element linearizer
            if (S->P.fluxModule != GBFV_FLUX_DARCY || prm->linearizer != GBFV_LINEARIZER_ELEMENT) {
                delete S;
                return nullptr;
            }
            S->vcfv = vcfvGrid(S->P);
            S->P.volume = S->vcfv->totalVolume;
            S->vcfv->bfPtr = S->P.bfPtr;
            S->vcfv->bfCorner = S->P.bfCorner;
            buildPatternVcfv(*S);
        }
        else
            buildPattern(*S);
        return S;
    }
    catch (...) {
        return nullptr;
    }
}

void oracle_destroy(void* h) { delete static_cast<Sim*>(h); }

// The quantities the reference's VtkMultiPhaseModule writes
// (vtkmultiphasemodule.hh:195-260), from the intensive quantities of the
// current solution: out[(3*k + phase)*N + cell], k = 0 pressure, 1 density,
// 2 saturation, 3 mobility, 4 relative permeability, 5 viscosity, and
// out[18*N + cell] the porosity (the layout of gbfv_output_fields)
int oracle_output_fields(void* h, double* out)
{
    auto* S = static_cast<Sim*>(h);
    const int N = S->N, b = S->b;
    std::fill(out, out + (size_t)19 * N, 0.0);
    for (int c = 0; c < N; ++c) {
        const double* pv = &S->x[(size_t)c * b];
        auto put = [&](int k, int a, double v) { out[(size_t)(3 * k + a) * N + c] = v; };
        if (b == 2) {
            const IQ2 q = immiscibleIQ(S->P, c, pv);
            for (int a = 0; a < 2; ++a) {
                put(0, a, q.p[a].v);
                put(1, a, q.rho[a].v);
                put(2, a, q.S[a].v);
                put(3, a, q.lam[a].v);
                put(4, a, q.kr[a].v);
                put(5, a, q.mu[a].v);
            }
            out[(size_t)18 * N + c] = q.phi;
        }
        else {
            const IQ3 q = blackoilIQ(S->P, c, pv, S->meaning[c]);
            for (int a = 0; a < 3; ++a) {
                put(0, a, q.p[a].v);
                put(1, a, q.rho[a].v);
                put(2, a, q.S[a].v);
                put(3, a, q.lam[a].v);
                put(4, a, q.kr[a].v);
                put(5, a, q.mu[a].v);
            }
            out[(size_t)18 * N + c] = q.phi;
        }
    }
    return GBFV_OK;
}

// summation order of the BiCGStab scalar products: 0 the reference's
// sequential sum, L > 0 L strided partial sums combined pairwise (test switch)
void oracle_set_dot_lanes(int lanes) { g_dotLanes = lanes > 0 ? lanes : 0; }

#ifdef _OPENMP
void oracle_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }
int oracle_get_threads(void) { return omp_get_max_threads(); }
#else  // serial build (the sanitizer target)
void oracle_set_threads(int) {}
int oracle_get_threads(void) { return 1; }
#endif

int oracle_set_params(void* h, const gbfv_params* prm)
{
    static_cast<Sim*>(h)->prm = *prm;
    return GBFV_OK;
}

int oracle_set_solution(void* h, const double* pv, const int32_t* meaning)
{
    Sim& S = *static_cast<Sim*>(h);
    std::memcpy(S.x.data(), pv, sizeof(double) * S.N * S.b);
    S.xOld = S.x;
    S.refPressure = S.x[0];
    if (meaning)
        for (int I = 0; I < S.N; ++I) S.meaning[I] = meaning[I];
    S.meaningOld = S.meaning;
    return GBFV_OK;
}

int oracle_get_solution(void* h, double* pv, int32_t* meaning)
{
    Sim& S = *static_cast<Sim*>(h);
    std::memcpy(pv, S.x.data(), sizeof(double) * S.N * S.b);
    if (meaning)
        for (int I = 0; I < S.N; ++I) meaning[I] = S.meaning[I];
    return GBFV_OK;
}

int oracle_nnz(void* h) { return static_cast<Sim*>(h)->J.rowPtr.back(); }

int oracle_linearize(void* h, double dt, int newton_iter)
{
    Sim& S = *static_cast<Sim*>(h);
    S.dt = dt;
    S.newtonIter = newton_iter;
    try {
        linearize(S);
    }
    catch (const NumericalProblem& e) {
        return e.code;
    }
    return GBFV_OK;
}

int oracle_get_residual(void* h, double* r)
{
    Sim& S = *static_cast<Sim*>(h);
    std::memcpy(r, S.residual.data(), sizeof(double) * S.N * S.b);
    return GBFV_OK;
}

int oracle_get_residual_scale(void* h, double* r)
{
    Sim& S = *static_cast<Sim*>(h);
    std::memcpy(r, S.rscale.data(), sizeof(double) * S.N * S.b);
    return GBFV_OK;
}

int oracle_get_storage_old(void* h, double* s)
{
    Sim& S = *static_cast<Sim*>(h);
    std::memcpy(s, S.storageOld.data(), sizeof(double) * S.N * S.b);
    return GBFV_OK;
}

int oracle_get_jacobian(void* h, int32_t* rowPtr, int32_t* col, double* blocks)
{
    Sim& S = *static_cast<Sim*>(h);
    std::copy(S.J.rowPtr.begin(), S.J.rowPtr.end(), rowPtr);
    std::copy(S.J.col.begin(), S.J.col.end(), col);
    std::memcpy(blocks, S.J.val.data(), sizeof(double) * S.J.val.size());
    return GBFV_OK;
}

int oracle_newton_error(void* h, double* err)
{
    *err = newtonError(*static_cast<Sim*>(h));
    return GBFV_OK;
}

int oracle_solve(void* h, double* dx, int* iters)
{
    Sim& S = *static_cast<Sim*>(h);
    int it = 0, st;
    try {
        st = solveLinear(S, it);
    }
    catch (const NumericalProblem& e) {
        st = e.code;
    }
    if (iters) *iters = it;
    if (dx && S.dx.size() == S.x.size()) std::memcpy(dx, S.dx.data(), sizeof(double) * S.dx.size());
    return st;
}

int oracle_newton_update(void* h, int* switched)
{
    Sim& S = *static_cast<Sim*>(h);
    try {
        std::vector<double> cur = S.x;
        std::vector<int> curM = S.meaning;
        const int sw = newtonUpdate(S, cur, curM);
        if (switched) *switched = sw;
    }
    catch (const NumericalProblem& e) {
        return e.code;
    }
    return GBFV_OK;
}

int oracle_newton_apply(void* h, double dt, gbfv_newton_report* rep)
{
    Sim& S = *static_cast<Sim*>(h);
    gbfv_newton_report r;
    const bool ok = newtonApply(S, dt, r);
    if (!ok) {
        S.x = S.xOld;  // updateFailed: solution(0) = solution(1)
        S.meaning = S.meaningOld;
    }
    if (rep) *rep = r;
    return ok ? GBFV_OK : (r.status ? r.status : GBFV_ERR_NOT_CONVERGED);
}

// FvBaseProblem::timeIntegration + Simulator::run time-step control
int oracle_time_integration(void* h, int numSteps, double dt0, double endTime, int fixedDt,
                            double* stepDt, int32_t* stepNewton, int32_t* stepLinear,
                            int32_t* totalLin)
{
    Sim& S = *static_cast<Sim*>(h);
    double dt = dt0, t = 0.0;
    int lin = 0;
    for (int step = 0; step < numSteps; ++step) {
        if (t >= endTime) break;
        bool ok = false;
        gbfv_newton_report rep;
        int linIt = 0;
        const unsigned maxFails = S.prm.max_time_step_divisions;
        for (unsigned i = 0; i < maxFails; ++i) {
            ok = oracle_newton_apply(h, dt, &rep) == GBFV_OK;
            linIt += rep.linear_iterations;
            lin += rep.linearizations;
            if (ok) break;
            double nextDt = dt / 2.0;
            if (dt < S.prm.min_time_step * (1 + 1e-9)) return GBFV_ERR_NOT_CONVERGED;
            if (nextDt < S.prm.min_time_step) nextDt = S.prm.min_time_step;
            dt = nextDt;
        }
        if (!ok) return GBFV_ERR_NOT_CONVERGED;
        if (stepDt) stepDt[step] = dt;
        if (stepNewton) stepNewton[step] = S.numIterations;
        if (stepLinear) stepLinear[step] = linIt;
        // advanceTimeLevel
        S.xOld = S.x;
        S.meaningOld = S.meaning;
        t += dt;
        if (fixedDt) { dt = dt0; continue; }
        const double maxTs = std::max(0.0, endTime - t);
        double dtNext = std::min(S.prm.max_time_step, suggestTimeStep(S, dt));
        if (dtNext < maxTs && maxTs < dtNext * 2) dtNext = maxTs / 2 * 1.01;
        dt = std::min(maxTs, dtNext);
    }
    if (totalLin) *totalLin = lin;
    return GBFV_OK;
}

// stand-alone BCRS solve (prepare + setMatrix + setResidual + solve)
int oracle_bcrs_solve(int n, int b, const int32_t* rowPtr, const int32_t* col, const double* blocks,
                      const double* rhs, double* x, const gbfv_params* prm, int* iters)
{
    Bcrs A;
    A.n = n;
    A.b = b;
    A.rowPtr.assign(rowPtr, rowPtr + n + 1);
    A.col.assign(col, col + rowPtr[n]);
    A.val.assign(blocks, blocks + (size_t)rowPtr[n] * b * b);
    std::vector<double> F, xs, r(rhs, rhs + (size_t)n * b);
    int it = 0;
    try {
        AmgHierarchy H;
        Precond prec;
        if (prm->linear_solver == GBFV_LINSOLVER_AMG) {
            amgSetup(H, A, prm->amg_coarsen_target);
            prec = [&H](std::vector<double>& v, const std::vector<double>& d) { amgApply(H, v, d); };
        }
        else {
            ilu0Factor(A, F);
            prec = [&A, &F](std::vector<double>& v, const std::vector<double>& d) { ilu0Apply(A, F, v, d); };
        }
        Criterion crit = makeCriterion(*prm);
        const bool ok = bicgstab(A, prec, r, xs, crit, prm->linear_max_iterations, it);
        std::memcpy(x, xs.data(), sizeof(double) * xs.size());
        if (iters) *iters = it;
        return ok ? GBFV_OK : GBFV_ERR_NOT_CONVERGED;
    }
    catch (const NumericalProblem& e) {
        if (iters) *iters = it;
        return e.code;
    }
}

// The AMG hierarchy of a BCRS matrix and one V-cycle, for unit tests of the
// GPU form: sizes[l] = rows of level l (AMG_MAX_LEVELS entries); agg0 (n
// entries), colors0 (n entries), d / v (n*b) may each be NULL: the
// aggregate and the colour of every row of level 0, v = V-cycle(d).
// Returns the number of levels, or a negative status.
int oracle_amg(int n, int b, const int32_t* rowPtr, const int32_t* col, const double* blocks, int coarsenTarget,
               int32_t* sizes, int32_t* agg0, int32_t* colors0, const double* d, double* v)
{
    Bcrs A;
    A.n = n;
    A.b = b;
    A.rowPtr.assign(rowPtr, rowPtr + n + 1);
    A.col.assign(col, col + rowPtr[n]);
    A.val.assign(blocks, blocks + (size_t)rowPtr[n] * b * b);
    AmgHierarchy H;
    try {
        amgSetup(H, A, coarsenTarget);
    }
    catch (const NumericalProblem& e) {
        return -e.code;
    }
    const int L = (int)H.lv.size();
    for (int l = 0; l < AMG_MAX_LEVELS; ++l) sizes[l] = l < L ? H.lv[l].A.n : 0;
    if (agg0)
        for (int i = 0; i < n; ++i) agg0[i] = L > 1 ? H.lv[0].agg[i] : -1;
    if (colors0)
        for (int i = 0; i < n; ++i) colors0[i] = H.lv[0].color[i];
    if (d && v) {
        std::vector<double> dv(d, d + (size_t)n * b), vv;
        amgApply(H, vv, dv);
        std::memcpy(v, vv.data(), sizeof(double) * vv.size());
    }
    return L;
}

// ILU(0) factors and one application, for unit tests of the GPU kernels
int oracle_ilu0(int n, int b, const int32_t* rowPtr, const int32_t* col, const double* blocks,
                double* factors, const double* d, double* v)
{
    Bcrs A;
    A.n = n;
    A.b = b;
    A.rowPtr.assign(rowPtr, rowPtr + n + 1);
    A.col.assign(col, col + rowPtr[n]);
    A.val.assign(blocks, blocks + (size_t)rowPtr[n] * b * b);
    std::vector<double> F;
    try {
        ilu0Factor(A, F);
    }
    catch (const NumericalProblem& e) {
        return e.code;
    }
    if (factors) std::memcpy(factors, F.data(), sizeof(double) * F.size());
    if (d && v) {
        std::vector<double> dv(d, d + (size_t)n * b), vv((size_t)n * b, 0.0);
        ilu0Apply(A, F, vv, dv);
        std::memcpy(v, vv.data(), sizeof(double) * vv.size());
    }
    return GBFV_OK;
}

}  // extern "C"
