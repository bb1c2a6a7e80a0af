// ORACLE -- test infrastructure only (see dual.hh for who may use it).
//
// Material laws and PVT restated from their published mathematics.  The
// reference takes them from opm-common, which is not vendored under the
// reference tree; every choice below that could not be read from the
// reference is listed in the oracle's table of unpinned choices.
//   - EffToAbsLaw<RegularizedVanGenuchten>: lensproblem.hh:111-121 (law),
//     lensproblem.hh:245-258 (parameters)
//   - 3-phase Corey relperm through the updateRelperms hook:
//     blackoilintensivequantities.hh:262, multiphasebaseproblem.hh:256-261
//   - LiveOil / DryGas / ConstantCompressibilityWater PVT:
//     reservoirproblem.hh:223-327
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>

#include "dual.hh"

namespace oracle {

// ---------------------------------------------------------------- VG ------
struct TwoPhaseLaw {
    int law = 0;  // 0 = regularized van Genuchten, 1 = regularized Brooks-Corey
    double Swr = 0, Snr = 0;
    // van Genuchten
    double alpha = 1, n = 2, m = 0.5;
    // Brooks-Corey
    double pe = 1, lambda = 2;
    // regularisation thresholds (effective saturation)
    double pcLowSw = 0.01, pcHighSw = 0.99;
    double pcLow = 0, pcSlopeLow = 0, pcHigh = 0, pcSlopeHigh = 0;
    double splineM0 = 0;  // slope of the VG curve at pcHighSw
    double bcSlopeHigh = 0;

    double vgPc(double Sw) const { return std::pow(std::pow(Sw, -1.0 / m) - 1, 1.0 / n) / alpha; }
    double vgDPc(double Sw) const
    {
        const double powSw = std::pow(Sw, -1 / m);
        return -1.0 / alpha * std::pow(powSw - 1, 1.0 / n - 1) / n * powSw / Sw / m;
    }
    double bcPc(double Sw) const { return pe * std::pow(Sw, -1.0 / lambda); }
    double bcDPc(double Sw) const { return -pe / lambda * std::pow(Sw, -1.0 / lambda - 1.0); }

    void finalize()
    {
        if (law == 0) {
            m = 1.0 - 1.0 / n;
            pcLow = vgPc(pcLowSw);
            pcSlopeLow = vgDPc(pcLowSw);
            pcHigh = vgPc(pcHighSw);
            pcSlopeHigh = 2 * (0.0 - pcHigh) / (1.0 - pcHighSw);
            splineM0 = vgDPc(pcHighSw);
        }
        else {
            pcLow = bcPc(pcLowSw);
            pcSlopeLow = bcDPc(pcLowSw);
            bcSlopeHigh = bcDPc(1.0);
        }
    }

    // cubic Hermite segment on [x0, x1] with end values and end slopes
    template <class E>
    static E hermite(const E& x, double x0, double x1, double y0, double y1, double m0, double m1)
    {
        const double h = x1 - x0;
        E t = (x - x0) / h;
        E t2 = t * t;
        E t3 = t2 * t;
        E h00 = 2.0 * t3 - 3.0 * t2 + 1.0;
        E h10 = t3 - 2.0 * t2 + t;
        E h01 = -2.0 * t3 + 3.0 * t2;
        E h11 = t3 - t2;
        return h00 * y0 + h10 * (h * m0) + h01 * y1 + h11 * (h * m1);
    }

    // p_c,nw as a function of the effective wetting saturation
    // (opm-common RegularizedVanGenuchten / RegularizedBrooksCorey ::
    // twoPhaseSatPcnw; the law and its parameters: lensproblem.hh:111-121,
    // 245-258)
    template <class E>
    E pcnw(const E& Sw) const
    {
        if (law == 0) {
            if (Sw < pcLowSw) return pcLow + pcSlopeLow * (Sw - pcLowSw);
            if (Sw > pcHighSw) {
                const double yTh = pcHigh;
                const double m1 = (0.0 - yTh) / (1.0 - pcHighSw) * 2;
                if (Sw < 1.0) return hermite(Sw, pcHighSw, 1.0, pcHigh, 0.0, splineM0, pcSlopeHigh);
                return m1 * (Sw - 1.0) + 0.0;
            }
            return pow(pow(Sw, -1.0 / m) - 1, 1.0 / n) / alpha;
        }
        if (Sw <= pcLowSw) return pcLow + pcSlopeLow * (Sw - pcLowSw);
        if (Sw >= 1.0) return pe + bcSlopeHigh * (Sw - 1.0);
        return pe * pow(Sw, -1.0 / lambda);
    }
    // wetting relative permeability: Mualem (van Genuchten) or Burdine
    // (Brooks-Corey), opm-common's twoPhaseSatKrw, clamped outside (0, 1)
    template <class E>
    E krw(const E& Sw) const
    {
        if (Sw <= 0.0) return E(0.0);
        if (Sw >= 1.0) return E(1.0);
        if (law == 0) {
            E r = 1.0 - pow(1.0 - pow(Sw, 1 / m), m);
            return sqrt(Sw) * r * r;
        }
        return pow(Sw, 2.0 / lambda + 3.0);
    }
    // non-wetting relative permeability (opm-common twoPhaseSatKrn);
    // argument: 1 - S_n,eff (the reference evaluates krn through Sw = 1 - Sn)
    template <class E>
    E krn(const E& Sw) const
    {
        if (Sw <= 0.0) return E(1.0);
        if (Sw >= 1.0) return E(0.0);
        if (law == 0) return pow(1 - Sw, 1.0 / 3) * pow(1 - pow(Sw, 1 / m), 2 * m);
        E Sn = 1.0 - Sw;
        return Sn * Sn * (1.0 - pow(Sw, 2.0 / lambda + 1.0));
    }
};

// ----------------------------------------------------------- tables ------
// piecewise-linear table with linear extrapolation on the end segments
// (opm-common Tabulated1DFunction::eval with extrapolation, as the live-oil
// and dry-gas PVT of reservoirproblem.hh:223-305 use it)
struct Table1D {
    std::vector<double> x, y;
    int segment(double xv) const
    {
        const int n = (int)x.size();
        if (xv <= x[0]) return 0;
        if (xv >= x[n - 1]) return n - 2;
        int lo = 0, hi = n - 1;
        while (hi - lo > 1) {
            const int mid = (lo + hi) / 2;
            if (x[mid] <= xv) lo = mid; else hi = mid;
        }
        return lo;
    }
    template <class E>
    E eval(const E& xv) const
    {
        const int i = segment(value(xv));
        const double s = (y[i + 1] - y[i]) / (x[i + 1] - x[i]);
        return y[i] + s * (xv - x[i]);
    }
};

struct BlackOilPvt {
    double rhoRefO = 786, rhoRefW = 1037, rhoRefG = 0.97;
    Table1D rsSat;      // p -> Rs_sat
    Table1D pBubble;    // Rs -> p_b (inverse of rsSat)
    Table1D invBoSat;   // p -> 1/B_o (saturated)
    Table1D muoSat;     // p -> mu_o (saturated)
    double oilComp = 0;
    Table1D invBg;      // p -> 1/B_g
    Table1D mug;        // p -> mu_g
    double pwRef = 1.01325e5, bwRef = 1.0, cw = 0, muw = 1e-3;

    // ConstantCompressibilityWaterPvt::inverseFormationVolumeFactor, the
    // second-order expansion of exp(X) (reservoirproblem.hh:306-312)
    template <class E>
    E waterInvB(const E& p) const
    {
        E X = cw * (p - pwRef);
        return (1.0 + X * (1.0 + X * 0.5)) / bwRef;
    }
    // saturated branch when gas is present and Rs is at saturation
    // (BlackOilFluidSystem::inverseFormationVolumeFactor), else the
    // undersaturated extension through the bubble-point pressure (LiveOilPvt
    // set up from saturated tables only, reservoirproblem.hh:297-304; the
    // extension's form is a row of the oracle's table of unpinned choices)
    template <class E>
    void oil(const E& p, const E& Rs, bool saturated, E& invB, E& mu) const
    {
        if (saturated) {
            invB = invBoSat.eval(p);
            mu = muoSat.eval(p);
            return;
        }
        E pb = pBubble.eval(Rs);
        E ib = invBoSat.eval(pb);
        invB = ib * (1.0 + oilComp * (p - pb));
        mu = muoSat.eval(pb);
    }
};

}  // namespace oracle
