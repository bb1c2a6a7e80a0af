// ORACLE -- test infrastructure only.  Only tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline / reference legs may load or run anything
// under oracle/.  It checks the product; it is never the product path.
//
// Vertex-centred finite volumes (VcfvDiscretization) for 2D axis-aligned
// quadrilaterals and the immiscible model, restated from
//   the stencil             vcfvstencil.hh:466-501 (quadrilateralArea),
//                           836-1015 (update: corners, edges, sub-control
//                           volumes, faces, boundary faces), 1040-1060,
//                           1107-1150 (sub-control-volume volumes);
//                           quadraturegeometries.hh:51-79 (sub-control-
//                           volume centres)
//   gradients               p1fegradientcalculator.hh:83-290 (P1 / Q1
//                           shape-function gradients at the face
//                           integration points), fvbasegradientcalculator.hh
//                           :200-318 (two-point and boundary gradients)
//   fluxes                  darcyfluxmodule.hh:183-525
//   local residual          fvbaselocalresidual.hh:158-191, 299-348,
//                           419-484, 491-626; immisciblelocalresidual.hh:
//                           75-155; immiscibleboundaryratevector.hh:97-150
//   AD linearization        fvbaseadlocallinearizer.hh:173-292 (every
//                           degree of freedom of a VCFV stencil is primary:
//                           one focus per corner)
//   element loop / scatter  fvbaselinearizer.hh:595-626
//
// dune-geometry's reference element for the cube (corner c at
// ((c & 1), (c >> 1) & 1); edge k between EDGE_CORNER[k]) and dune-
// localfunctions' Q1 basis (N_c = prod_d (bit_d(c) ? x_d : 1 - x_d)) are not
// vendored under the reference tree; their published numbering and
// formulas are restated here.  Every intensive quantity carries the
// derivatives of its own vertex's primary variables, as the reference's
// do; the focus rules strip them exactly where the reference does.
// Included by oracle.cc inside namespace oracle.
#pragma once

// corners of each edge (referenceElement.subEntity(k, 1, 0|1, 2)) and the
// local centres of edges / faces of the 2D cube
static const int EDGE_CORNER[4][2] = {{0, 2}, {1, 3}, {0, 1}, {2, 3}};
static const double EDGE_LOCAL[4][2] = {{0.0, 0.5}, {1.0, 0.5}, {0.5, 0.0}, {0.5, 1.0}};

struct VcfvElement {
    int v[4];                   // vertex (degree of freedom) of each corner
    double lower[2], upper[2];  // the axis-aligned box
    double vpos[4][2];          // subContVol[c].global
    double scvVol[4];
    double scvCenter[4][2];     // ScvGeometry::center()
    int fi[4], fj[4];           // face k separates corners fi[k] -> fj[k]
    double fn[4][2], fa[4], fip[4][2];  // unit normal (i to j), area, integration point
    double grad[4][4][2];       // P1: gradient of corner c's shape function at face k
    double global0(double l) const { return lower[0] + l * (upper[0] - lower[0]); }
    double global1(double l) const { return lower[1] + l * (upper[1] - lower[1]); }
};

struct VcfvGrid {
    std::vector<VcfvElement> el;
    std::vector<double> totalVolume;  // dofTotalVolume per vertex
    std::vector<int> bfPtr, bfCorner;
    bool p1 = true;
};

// VcfvStencil::quadrilateralArea (vcfvstencil.hh:495-501)
static double quadArea(const double* p0, const double* p1, const double* p2, const double* p3)
{
    return 0.5 * std::abs((p3[0] - p1[0]) * (p2[1] - p0[1]) - (p3[1] - p1[1]) * (p2[0] - p0[0]));
}

// VcfvStencil::update for one quadrilateral (vcfvstencil.hh:864-1015),
// AxisAlignedCubeGeometry::global(x) = lower + x .* (upper - lower)
static VcfvElement vcfvElement(const Prob& P, const int* corner)
{
    VcfvElement E;
    for (int c = 0; c < 4; ++c) E.v[c] = corner[c];
    for (int d = 0; d < 2; ++d) {
        E.lower[d] = P.center[3 * corner[0] + d];
        E.upper[d] = P.center[3 * corner[3] + d];
    }
    auto global = [&](const double* l, double* x) {
        x[0] = E.global0(l[0]);
        x[1] = E.global1(l[1]);
    };
    const double elemLocal[2] = {0.5, 0.5};
    double elemGlobal[2], edgeCoord[4][2];
    global(elemLocal, elemGlobal);
    for (int c = 0; c < 4; ++c) {
        const double l[2] = {double(c & 1), double((c >> 1) & 1)};
        global(l, E.vpos[c]);
    }
    for (int k = 0; k < 4; ++k) global(EDGE_LOCAL[k], edgeCoord[k]);
    // fillSubContVolData_ (vcfvstencil.hh:1127-1148)
    E.scvVol[0] = quadArea(E.vpos[0], edgeCoord[2], elemGlobal, edgeCoord[0]);
    E.scvVol[1] = quadArea(E.vpos[1], edgeCoord[1], elemGlobal, edgeCoord[2]);
    E.scvVol[2] = quadArea(E.vpos[2], edgeCoord[0], elemGlobal, edgeCoord[3]);
    E.scvVol[3] = quadArea(E.vpos[3], edgeCoord[3], elemGlobal, edgeCoord[1]);
    // sub-control volume c: the box between corner c, the two edge centres
    // next to it and the element centre; its centre is the mean of its local
    // corners (QuadrialteralQuadratureGeometry::setCorners)
    for (int c = 0; c < 4; ++c) {
        const double x0 = (c & 1) ? 0.5 : 0.0, y0 = ((c >> 1) & 1) ? 0.5 : 0.0;
        const double loc[4][2] = {{x0, y0}, {x0 + 0.5, y0}, {x0, y0 + 0.5}, {x0 + 0.5, y0 + 0.5}};
        double ctr[2] = {0.0, 0.0};
        for (int q = 0; q < 4; ++q)
            for (int d = 0; d < 2; ++d) ctr[d] += loc[q][d];
        for (int d = 0; d < 2; ++d) ctr[d] /= 4;
        global(ctr, E.scvCenter[c]);
    }
    // sub-control-volume faces: one per edge, from the edge centre to the
    // element centre (vcfvstencil.hh:900-958)
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
        // Q1 shape functions' local gradients at the integration point,
        // mapped by the inverse transposed Jacobian (diagonal for boxes)
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

static std::shared_ptr<VcfvGrid> vcfvGrid(const Prob& P)
{
    auto G = std::make_shared<VcfvGrid>();
    G->p1 = P.p1Gradients != 0;
    G->totalVolume.assign(P.N, 0.0);
    for (int e = 0; e < P.numElements; ++e) {
        G->el.push_back(vcfvElement(P, &P.elemCorner[4 * e]));
        const VcfvElement& E = G->el.back();
        // dofTotalVolume: the element loop's sum of sub-control volumes
        for (int c = 0; c < 4; ++c) G->totalVolume[E.v[c]] += E.scvVol[c];
    }
    return G;
}

template <int N> static inline Dual<N> valueOnly(const Dual<N>& x) { return Dual<N>(x.v); }

// The Darcy volume fluxes of sub-control-volume face k for NP phases
// (darcyfluxmodule.hh:183-322, 459-525 on the vertex-centred stencil): the
// phase pressure gradients at the face's integration point (P1 or
// two-point), the gravity correction from the two vertices, upwinding by
// the sign of the potential gradient along the normal, the upstream
// mobility; vf[a] the volume flux per unit area, up[a] the upstream corner.
// f: the focus corner (-1: none).
template <int NB, class IQ, int NP>
static void vcfvPhaseFluxes(const Prob& P, const VcfvGrid& G, const VcfvElement& E, int k, int f,
                            const IQ* const (&q)[4], Dual<NB> (&vf)[NP], int (&up)[NP])
{
    using D = Dual<NB>;
    auto focus = [&](int c, const D& x) { return c == f ? x : valueOnly(x); };
    const int i = E.fi[k], j = E.fj[k];
    const double* n = E.fn[k];
    D pg[NP][2];  // [phase][dim]
    for (int a = 0; a < NP; ++a) {
        if (G.p1) {
            // P1FeGradientCalculator::calculateGradient
            pg[a][0] = D(0.0);
            pg[a][1] = D(0.0);
            for (int c = 0; c < 4; ++c) {
                const D dofVal = focus(c, q[c]->p[a]);
                for (int d = 0; d < 2; ++d) pg[a][d] += dofVal * E.grad[k][c][d];
            }
        }
        else {
            // FvBaseGradientCalculator::calculateGradient (two-point)
            D deltay;
            if (i == f) deltay = valueOnly(q[j]->p[a]) - q[i]->p[a];
            else if (j == f) deltay = q[j]->p[a] - valueOnly(q[i]->p[a]);
            else deltay = valueOnly(q[j]->p[a]) - valueOnly(q[i]->p[a]);
            double distSq = 0.0;
            for (int d = 0; d < 2; ++d) {
                const double t = E.vpos[j][d] - E.vpos[i][d];
                distSq += t * t;
            }
            for (int d = 0; d < 2; ++d) pg[a][d] = deltay * ((E.vpos[j][d] - E.vpos[i][d]) / distSq);
        }
    }
    // gravity (darcyfluxmodule.hh:214-283): posIn / posEx the vertices
    double dIn[2], dEx[2], dTot[2];
    for (int d = 0; d < 2; ++d) {
        dIn[d] = E.vpos[i][d] - E.fip[k][d];
        dEx[d] = E.vpos[j][d] - E.fip[k][d];
        dTot[d] = E.vpos[j][d] - E.vpos[i][d];
    }
    const double absTot2 = dTot[0] * dTot[0] + dTot[1] * dTot[1];
    double gIn = 0.0, gEx = 0.0;
    for (int d = 0; d < 2; ++d) gIn += P.g[d] * dIn[d];
    for (int d = 0; d < 2; ++d) gEx += P.g[d] * dEx[d];
    for (int a = 0; a < NP; ++a) {
        const D pStatIn = -(focus(i, q[i]->rho[a]) * gIn);
        const D pStatEx = -(focus(j, q[j]->rho[a]) * gEx);
        const D fs = (pStatEx - pStatIn) / absTot2;
        for (int d = 0; d < 2; ++d) pg[a][d] += dTot[d] * fs;
    }
    double Kh[2];
    for (int d = 0; d < 2; ++d) Kh[d] = harmonicMean(P.perm[3 * E.v[i] + d], P.perm[3 * E.v[j] + d]);
    for (int a = 0; a < NP; ++a) {
        D tmp(0.0);
        for (int d = 0; d < 2; ++d) tmp += pg[a][d] * n[d];
        up[a] = tmp > 0 ? j : i;
        const D mob = focus(up[a], q[up[a]]->lam[a]);
        vf[a] = D(0.0);
        for (int d = 0; d < 2; ++d) {
            D fv = Kh[d] * pg[a][d];
            fv *= -mob;
            vf[a] += fv * n[d];
        }
    }
}

// FvBaseLocalResidual::eval of element e with focus corner f: res[c][eq]
// the corners' residuals (divided by their total volumes), derivatives
// with respect to corner f's primary variables; sc[c][eq] the parity scale
// (sum of |terms| / V).  q: the corners' intensive quantities, each with
// the derivatives of its own primary variables (f = -1: no focus, the
// values only, as the finite-difference linearizer evaluates).
static void elementImmiscibleVcfv(Sim& S, const VcfvGrid& G, int e, int f, const IQ2* const (&q)[4], bool iter0,
                                  D2 (&res)[4][2], double (&sc)[4][2])
{
    const Prob& P = S.P;
    const VcfvElement& E = G.el[e];
    for (int c = 0; c < 4; ++c)
        for (int a = 0; a < 2; ++a) {
            res[c][a] = D2(0.0);
            sc[c][a] = 0.0;
        }
    auto focus = [&](int c, const D2& x) { return c == f ? x : valueOnly(x); };
    // evalFluxes
    for (int k = 0; k < 4; ++k) {
        const int i = E.fi[k], j = E.fj[k];
        D2 vf[2];
        int up[2];
        vcfvPhaseFluxes<2, IQ2, 2>(P, G, E, k, f, q, vf, up);
        D2 flux[2];
        for (int a = 0; a < 2; ++a) {
            flux[a] = D2(0.0);
            flux[a] += vf[a] * focus(up[a], q[up[a]]->rho[a]);
        }
        const double alpha = 1.0 * E.fa[k];
        for (int a = 0; a < 2; ++a) flux[a] *= alpha;
        for (int a = 0; a < 2; ++a) {
            res[i][a] += flux[a];
            res[j][a] -= flux[a];
            sc[i][a] += std::abs(flux[a].v);
            sc[j][a] += std::abs(flux[a].v);
        }
    }
    // evalVolumeTerms_
    for (int c = 0; c < 4; ++c) {
        const double scvVolume = E.scvVol[c] * 1.0;
        const int v = E.v[c];
        D2 tmp[2];
        for (int a = 0; a < 2; ++a) {
            tmp[a] = (D2(q[c]->phi) * q[c]->S[a]) * q[c]->rho[a];
            if (c != f) tmp[a] = valueOnly(tmp[a]);
        }
        double tmp2[2];
        if (iter0) {
            for (int a = 0; a < 2; ++a) tmp2[a] = tmp[a].v;
            for (int a = 0; a < 2; ++a) S.storageOld[v * 2 + a] = tmp2[a];
        }
        else
            for (int a = 0; a < 2; ++a) tmp2[a] = S.storageOld[v * 2 + a];
        for (int a = 0; a < 2; ++a) {
            sc[c][a] += std::abs(tmp[a].v) * (scvVolume / S.dt) + std::abs(tmp2[a]) * (scvVolume / S.dt);
            tmp[a] -= tmp2[a];
            tmp[a] *= scvVolume / S.dt;
            res[c][a] += tmp[a];
        }
        for (int a = 0; a < 2; ++a) res[c][a] -= 0.0 * scvVolume;
    }
    // evalBoundary_: boundary sub-control-volume faces of this element
    for (int b = G.bfPtr[e]; b < G.bfPtr[e + 1]; ++b) {
        const int c = G.bfCorner[b];
        const IQ2& qi = *q[c];
        D2 values[2] = {D2(0.0), D2(0.0)};
        const int type = P.bfType[b];
        if (type == GBFV_BC_MASSRATE) {
            for (int a = 0; a < 2; ++a) values[a] = D2(P.bfValue[4 * b + a]);
        }
        else if (type == GBFV_BC_FREEFLOW) {
            const TwoPhaseLaw& L = P.laws[P.material[E.v[c]]];
            const double pw = P.bfValue[4 * b + 0], Swb = P.bfValue[4 * b + 1];
            const double sumRes = L.Swr + L.Snr;
            const double SwE = (Swb - L.Swr) / (1.0 - sumRes);
            const double SnE = ((1 - Swb) - L.Snr) / (1.0 - sumRes);
            const double pcn = L.pcnw(SwE);
            const double pb[2] = {pw, pw + pcn - 0.0};
            const double krb[2] = {L.krw(SwE), L.krn(1.0 - SnE)};
            const double* xf = &P.bfCenter[3 * b];
            const double* n = &P.bfNormal[3 * b];
            // the gradient from the sub-control volume's centre, gravity
            // from the vertex (darcyfluxmodule.hh:332-449)
            const double* xc = E.scvCenter[c];
            double distSq = 0;
            for (int d = 0; d < 2; ++d) { const double t = xf[d] - xc[d]; distSq += t * t; }
            double dIn[2];
            for (int d = 0; d < 2; ++d) dIn[d] = E.vpos[c][d] - xf[d];
            double absDist2 = 0, gTimesDist = 0;
            for (int d = 0; d < 2; ++d) absDist2 += dIn[d] * dIn[d];
            for (int d = 0; d < 2; ++d) gTimesDist += P.g[d] * dIn[d];
            for (int a = 0; a < 2; ++a) {
                const D2 deltay = c == f ? pb[a] - qi.p[a] : D2(pb[a] - qi.p[a].v);
                D2 pg[2];
                for (int d = 0; d < 2; ++d) pg[d] = deltay * ((xf[d] - xc[d]) / distSq);
                const D2 pStatIn = (-gTimesDist) * qi.rho[a];
                const D2 fsc = pStatIn / absDist2;
                for (int d = 0; d < 2; ++d) pg[d] += dIn[d] * fsc;
                D2 tmp(0.0);
                for (int d = 0; d < 2; ++d) tmp += pg[d] * n[d];
                const D2 mob = tmp > 0.0 ? D2(krb[a] / P.mu[a]) : focus(c, qi.lam[a]);
                D2 vf(0.0);
                for (int d = 0; d < 2; ++d) {
                    D2 fv = P.perm[3 * E.v[c] + d] * pg[d];
                    fv *= -mob;
                    vf += fv * n[d];
                }
                const D2 dens = pb[a] > qi.p[a].v ? D2(P.rho[a]) : focus(c, qi.rho[a]);
                values[a] += vf * dens;
            }
        }
        const double aa = P.bfArea[b] * 1.0;
        for (int a = 0; a < 2; ++a) values[a] *= aa;
        for (int a = 0; a < 2; ++a) {
            res[c][a] += values[a];
            sc[c][a] += std::abs(values[a].v);
        }
    }
    // volumetric residual
    for (int c = 0; c < 4; ++c)
        for (int a = 0; a < 2; ++a) {
            res[c][a] /= G.totalVolume[E.v[c]];
            sc[c][a] /= G.totalVolume[E.v[c]];
        }
}

// The black-oil model on the vertex-centred stencil (blackoillocalresidual.hh:
// 101-367: component storage phi S invB (+ Rs for the gas dissolved in oil),
// component fluxes of the upstream invB (and Rs) times the phase volume
// flux, both scaled by the surface densities); boundaries are no-flow or
// mass rate.  Same conventions as elementImmiscibleVcfv.
static void elementBlackoilVcfv(Sim& S, const VcfvGrid& G, int e, int f, const IQ3* const (&q)[4], bool iter0,
                                D3 (&res)[4][3], double (&sc)[4][3])
{
    const Prob& P = S.P;
    const BlackOilPvt& T = P.pvt;
    const double rhoRef[3] = {T.rhoRefW, T.rhoRefO, T.rhoRefG};
    const int compOfPhase[3] = {1, 0, 2};
    const VcfvElement& E = G.el[e];
    for (int c = 0; c < 4; ++c)
        for (int a = 0; a < 3; ++a) {
            res[c][a] = D3(0.0);
            sc[c][a] = 0.0;
        }
    auto focus = [&](int c, const D3& x) { return c == f ? x : valueOnly(x); };
    // evalFluxes
    for (int k = 0; k < 4; ++k) {
        const int i = E.fi[k], j = E.fj[k];
        D3 vf[3];
        int up[3];
        vcfvPhaseFluxes<3, IQ3, 3>(P, G, E, k, f, q, vf, up);
        D3 flux[3] = {D3(0.0), D3(0.0), D3(0.0)};
        for (int a = 0; a < 3; ++a) {
            D3 invB = focus(up[a], q[up[a]]->invB[a]);
            D3 svf = invB * vf[a];
            flux[compOfPhase[a]] += svf * rhoRef[a];
            if (a == 1) {
                D3 Rs = focus(up[a], q[up[a]]->Rs);
                flux[2] += Rs * svf * T.rhoRefG;
            }
        }
        const double alpha = 1.0 * E.fa[k];
        for (int a = 0; a < 3; ++a) flux[a] *= alpha;
        for (int a = 0; a < 3; ++a) {
            res[i][a] += flux[a];
            res[j][a] -= flux[a];
            sc[i][a] += std::abs(flux[a].v);
            sc[j][a] += std::abs(flux[a].v);
        }
    }
    // evalVolumeTerms_
    for (int c = 0; c < 4; ++c) {
        const double scvVolume = E.scvVol[c] * 1.0;
        const int v = E.v[c];
        const IQ3& qc = *q[c];
        D3 tmp[3] = {D3(0.0), D3(0.0), D3(0.0)};
        D3 phi(qc.phi);
        for (int a = 0; a < 3; ++a) {
            D3 sv = qc.S[a] * qc.invB[a] * phi;
            tmp[compOfPhase[a]] += sv;
            if (a == 1) tmp[2] += qc.Rs * sv;
        }
        tmp[1] *= T.rhoRefW;
        tmp[2] *= T.rhoRefG;
        tmp[0] *= T.rhoRefO;
        if (c != f)
            for (int a = 0; a < 3; ++a) tmp[a] = valueOnly(tmp[a]);
        double tmp2[3];
        if (iter0) {
            for (int a = 0; a < 3; ++a) tmp2[a] = tmp[a].v;
            for (int a = 0; a < 3; ++a) S.storageOld[v * 3 + a] = tmp2[a];
        }
        else
            for (int a = 0; a < 3; ++a) tmp2[a] = S.storageOld[v * 3 + a];
        for (int a = 0; a < 3; ++a) {
            sc[c][a] += std::abs(tmp[a].v) * (scvVolume / S.dt) + std::abs(tmp2[a]) * (scvVolume / S.dt);
            tmp[a] -= tmp2[a];
            tmp[a] *= scvVolume / S.dt;
            res[c][a] += tmp[a];
        }
        for (int a = 0; a < 3; ++a) res[c][a] -= 0.0 * scvVolume;
    }
    // evalBoundary_: mass-rate boundary faces (no-flow adds nothing)
    for (int b = G.bfPtr[e]; b < G.bfPtr[e + 1]; ++b) {
        if (P.bfType[b] != GBFV_BC_MASSRATE) continue;
        const int c = G.bfCorner[b];
        const double aa = P.bfArea[b] * 1.0;
        for (int a = 0; a < 3; ++a) {
            const D3 val = D3(P.bfValue[4 * b + a]) * aa;
            res[c][a] += val;
            sc[c][a] += std::abs(val.v);
        }
    }
    for (int c = 0; c < 4; ++c)
        for (int a = 0; a < 3; ++a) {
            res[c][a] /= G.totalVolume[E.v[c]];
            sc[c][a] /= G.totalVolume[E.v[c]];
        }
}

static void linearizeBlackoilVcfv(Sim& S, const std::vector<IQ3>& iq)
{
    const VcfvGrid& G = *S.vcfv;
    const bool iter0 = S.newtonIter == 0;
    std::fill(S.rscale.begin(), S.rscale.end(), 0.0);
    for (int e = 0; e < (int)G.el.size(); ++e) {
        const VcfvElement& E = G.el[e];
        D3 res[4][4][3];
        double sc[4][4][3];
        const IQ3* q[4] = {&iq[E.v[0]], &iq[E.v[1]], &iq[E.v[2]], &iq[E.v[3]]};
        for (int f = 0; f < 4; ++f) elementBlackoilVcfv(S, G, e, f, q, iter0, res[f], sc[f]);
        for (int f = 0; f < 4; ++f) {
            const int gf = E.v[f];
            for (int a = 0; a < 3; ++a) {
                S.residual[gf * 3 + a] += res[f][f][a].v;
                S.rscale[gf * 3 + a] += sc[f][f][a];
            }
            for (int j = 0; j < 4; ++j) {
                double* blk = &S.J.val[(size_t)S.J.find(E.v[j], gf) * 9];
                for (int a = 0; a < 3; ++a)
                    for (int pv = 0; pv < 3; ++pv) blk[a * 3 + pv] += res[f][j][a].d[pv];
            }
        }
    }
}

// FvBaseLinearizer::linearizeElement_ over all elements in grid order
// (fvbaselinearizer.hh:595-626) with the AD local linearizer: one local
// evaluation per focus corner; residual_[corner f] += its residual, block
// (corner j, corner f) += d res_j / d x_f
static void linearizeImmiscibleVcfv(Sim& S, const std::vector<IQ2>& iq)
{
    const VcfvGrid& G = *S.vcfv;
    const bool iter0 = S.newtonIter == 0;
    std::fill(S.rscale.begin(), S.rscale.end(), 0.0);
    for (int e = 0; e < (int)G.el.size(); ++e) {
        const VcfvElement& E = G.el[e];
        D2 res[4][4][2];
        double sc[4][4][2];
        const IQ2* q[4] = {&iq[E.v[0]], &iq[E.v[1]], &iq[E.v[2]], &iq[E.v[3]]};
        for (int f = 0; f < 4; ++f) elementImmiscibleVcfv(S, G, e, f, q, iter0, res[f], sc[f]);
        for (int f = 0; f < 4; ++f) {
            const int gf = E.v[f];
            for (int a = 0; a < 2; ++a) {
                S.residual[gf * 2 + a] += res[f][f][a].v;
                S.rscale[gf * 2 + a] += sc[f][f][a];
            }
            for (int j = 0; j < 4; ++j) {
                double* blk = &S.J.val[(size_t)S.J.find(E.v[j], gf) * 4];
                for (int a = 0; a < 2; ++a)
                    for (int pv = 0; pv < 2; ++pv) blk[a * 2 + pv] += res[f][j][a].d[pv];
            }
        }
    }
}

// FvBaseFdLocalLinearizer on the vertex-centred stencil
// (fvbasefdlocallinearizer.hh:236-510): the element's four corner residuals
// unperturbed, then per corner f and primary variable the residuals with
// f's intensive quantities at the deflected state(s) -- the other corners
// keep theirs, the storage of the old time level comes from the cache the
// unperturbed evaluation filled -- their difference over the deflection
// being column (., f) of the element's local Jacobian.
static void linearizeImmiscibleVcfvFd(Sim& S, const std::vector<IQ2>& iq)
{
    const VcfvGrid& G = *S.vcfv;
    const bool iter0 = S.newtonIter == 0;
    const int method = S.prm.numeric_difference_method;
    const double baseEps = std::max(0.9123e-10, std::numeric_limits<double>::epsilon() * 1.23e3);
    std::fill(S.rscale.begin(), S.rscale.end(), 0.0);
    for (int e = 0; e < (int)G.el.size(); ++e) {
        const VcfvElement& E = G.el[e];
        const IQ2* q[4] = {&iq[E.v[0]], &iq[E.v[1]], &iq[E.v[2]], &iq[E.v[3]]};
        D2 res0[4][2], resD[4][2];
        double sc[4][2], scD[4][2];
        elementImmiscibleVcfv(S, G, e, -1, q, iter0, res0, sc);
        for (int c = 0; c < 4; ++c)
            for (int a = 0; a < 2; ++a) {
                S.residual[E.v[c] * 2 + a] += res0[c][a].v;
                S.rscale[E.v[c] * 2 + a] += sc[c][a];
            }
        for (int f = 0; f < 4; ++f) {
            const int gf = E.v[f];
            for (int pv = 0; pv < 2; ++pv) {
                double xs[2] = {S.x[gf * 2], S.x[gf * 2 + 1]};
                const double eps = baseEps / pvWeight(S, gf, pv);
                double delta = 0.0, d[4][2];
                const IQ2* qd[4] = {q[0], q[1], q[2], q[3]};
                if (method >= 0) {
                    xs[pv] += eps;
                    delta += eps;
                    const IQ2 dq = immiscibleIQ(S.P, gf, xs);
                    qd[f] = &dq;
                    elementImmiscibleVcfv(S, G, e, -1, qd, false, resD, scD);
                    for (int c = 0; c < 4; ++c)
                        for (int a = 0; a < 2; ++a) d[c][a] = resD[c][a].v;
                }
                else
                    for (int c = 0; c < 4; ++c)
                        for (int a = 0; a < 2; ++a) d[c][a] = res0[c][a].v;
                if (method <= 0) {
                    xs[pv] -= delta + eps;
                    delta += eps;
                    const IQ2 dq = immiscibleIQ(S.P, gf, xs);
                    qd[f] = &dq;
                    elementImmiscibleVcfv(S, G, e, -1, qd, false, resD, scD);
                    for (int c = 0; c < 4; ++c)
                        for (int a = 0; a < 2; ++a) d[c][a] -= resD[c][a].v;
                }
                else
                    for (int c = 0; c < 4; ++c)
                        for (int a = 0; a < 2; ++a) d[c][a] -= res0[c][a].v;
                for (int j = 0; j < 4; ++j) {
                    double* blk = &S.J.val[(size_t)S.J.find(E.v[j], gf) * 4];
                    for (int a = 0; a < 2; ++a) blk[a * 2 + pv] += d[j][a] / delta;
                }
            }
        }
    }
}

// the Jacobian's pattern: every pair of vertices sharing an element
static void buildPatternVcfv(Sim& S)
{
    const VcfvGrid& G = *S.vcfv;
    std::vector<std::vector<int>> rows(S.N);
    for (int I = 0; I < S.N; ++I) rows[I].push_back(I);
    for (const VcfvElement& E : G.el)
        for (int a = 0; a < 4; ++a)
            for (int c = 0; c < 4; ++c) rows[E.v[a]].push_back(E.v[c]);
    S.J.n = S.N;
    S.J.b = S.b;
    S.J.rowPtr.assign(S.N + 1, 0);
    for (int I = 0; I < S.N; ++I) {
        std::sort(rows[I].begin(), rows[I].end());
        rows[I].erase(std::unique(rows[I].begin(), rows[I].end()), rows[I].end());
        S.J.rowPtr[I + 1] = S.J.rowPtr[I] + (int)rows[I].size();
    }
    S.J.col.clear();
    for (int I = 0; I < S.N; ++I) S.J.col.insert(S.J.col.end(), rows[I].begin(), rows[I].end());
    S.J.val.assign((size_t)S.J.rowPtr[S.N] * S.b * S.b, 0.0);
}

