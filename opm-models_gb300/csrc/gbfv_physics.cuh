// Device physics of the ECFV/TPFA linearization: forward-mode duals,
// two-phase material laws, three-phase Corey relperm and black-oil PVT.
//
// Everything here is __host__ __device__ so that host-side set-up (material
// thresholds, boundary fluid states) evaluates exactly the same expressions
// as the kernels.  Operation order follows the reference's (see citations);
// translation units that include this header for parity-critical kernels are
// compiled without FMA contraction.
//
// Reference semantics:
//   DenseAd::Evaluation (opm-common, used via fvbaseadlocallinearizer.hh:62-72)
//   EffToAbsLaw<RegularizedVanGenuchten> (lensproblem.hh:111-121)
//   BlackOilFluidSystem PVT (reservoirproblem.hh:223-327) and the Corey
//   updateRelperms hook (blackoilintensivequantities.hh:262)
#pragma once
#include <cmath>
#include <cstdint>

#define GB_HD __host__ __device__ __forceinline__

namespace gbfv {

// ------------------------------------------------------------- duals -----
template <int N>
struct Dual {
    double v;
    double d[N];
    GB_HD Dual() {}
    GB_HD explicit Dual(double x) : v(x)
    {
#pragma unroll
        for (int i = 0; i < N; ++i) d[i] = 0.0;
    }
    static GB_HD Dual var(double x, int idx)
    {
        Dual r(x);
        r.d[idx] = 1.0;
        return r;
    }
};

template <int N> GB_HD Dual<N> operator+(const Dual<N>& a, const Dual<N>& b)
{ Dual<N> r; r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
template <int N> GB_HD Dual<N> operator-(const Dual<N>& a, const Dual<N>& b)
{ Dual<N> r; r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
template <int N> GB_HD Dual<N> operator+(const Dual<N>& a, double s)
{ Dual<N> r = a; r.v = a.v + s; return r; }
template <int N> GB_HD Dual<N> operator+(double s, const Dual<N>& a)
{ Dual<N> r = a; r.v = a.v + s; return r; }
template <int N> GB_HD Dual<N> operator-(const Dual<N>& a, double s)
{ Dual<N> r = a; r.v = a.v - s; return r; }
template <int N> GB_HD Dual<N> operator-(double s, const Dual<N>& a)
{ Dual<N> r; r.v = s - a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i]; return r; }
template <int N> GB_HD Dual<N> operator-(const Dual<N>& a)
{ Dual<N> r; r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i]; return r; }
// Values follow the reference's operation order exactly (they decide upwind
// directions and saturation branches); derivatives may round differently by
// an ulp, so they use fused multiply-adds and one reciprocal per division
// instead of a division per derivative -- FP64 issue is this GPU's scarce
// resource.
// (u w)' = u' w + w' u
template <int N> GB_HD Dual<N> operator*(const Dual<N>& a, const Dual<N>& b)
{ Dual<N> r; r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = fma(a.d[i], b.v, b.d[i] * a.v); return r; }
template <int N> GB_HD Dual<N> operator*(const Dual<N>& a, double s)
{ Dual<N> r; r.v = a.v * s;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * s; return r; }
template <int N> GB_HD Dual<N> operator*(double s, const Dual<N>& a) { return a * s; }
// (u / w)' = (w u' - u w') / w^2
template <int N> GB_HD Dual<N> operator/(const Dual<N>& a, const Dual<N>& b)
{ Dual<N> r; const double u = a.v, w = b.v, iw2 = 1.0 / (w * w);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = fma(w, a.d[i], -(u * b.d[i])) * iw2;
  r.v = u / w; return r; }
template <int N> GB_HD Dual<N> operator/(const Dual<N>& a, double s)
{ Dual<N> r; r.v = a.v / s; const double is = 1.0 / s;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * is; return r; }
// s / w: -s/w^2 w'
template <int N> GB_HD Dual<N> operator/(double s, const Dual<N>& a)
{ Dual<N> r; r.v = s / a.v; const double df = -s / (a.v * a.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = df * a.d[i]; return r; }

template <int N> GB_HD Dual<N> dpow(const Dual<N>& x, double e)
{
    if (x.v == 0.0) return Dual<N>(0.0);
    Dual<N> r;
    const double px = pow(x.v, e);
    r.v = px;
    const double df = px / x.v * e;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = df * x.d[i];
    return r;
}
template <int N> GB_HD Dual<N> dsqrt(const Dual<N>& x)
{
    Dual<N> r;
    const double sx = sqrt(x.v);
    r.v = sx;
    const double df = 0.5 / sx;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = df * x.d[i];
    return r;
}
GB_HD double dpow(double x, double e) { return pow(x, e); }
GB_HD double dsqrt(double x) { return sqrt(x); }
GB_HD double val(double x) { return x; }
template <int N> GB_HD double val(const Dual<N>& x) { return x.v; }
template <class E> GB_HD E konst(double x) { return E(x); }
template <> GB_HD double konst<double>(double x) { return x; }

// ----------------------------------------------------- material laws -----
// Parameter record of one two-phase material (effective-saturation law).
struct TwoPhaseLaw {
    int law;  // 0 regularized van Genuchten, 1 regularized Brooks-Corey
    double Swr, Snr;
    double alpha, n, m;
    double pe, lambda;
    double pcLowSw, pcHighSw;
    double pcLow, pcSlopeLow, pcHigh, pcSlopeHigh, splineM0, bcSlopeHigh;
};

GB_HD double vgPc(const TwoPhaseLaw& L, double Sw)
{ return pow(pow(Sw, -1.0 / L.m) - 1, 1.0 / L.n) / L.alpha; }
GB_HD double vgDPc(const TwoPhaseLaw& L, double Sw)
{
    const double powSw = pow(Sw, -1 / L.m);
    return -1.0 / L.alpha * pow(powSw - 1, 1.0 / L.n - 1) / L.n * powSw / Sw / L.m;
}

// thresholds of the regularisation (RegularizedVanGenuchtenParams::finalize)
inline void finalizeLaw(TwoPhaseLaw& L)
{
    L.pcLowSw = 0.01;
    L.pcHighSw = 0.99;
    if (L.law == 0) {
        L.m = 1.0 - 1.0 / L.n;
        L.pcLow = vgPc(L, L.pcLowSw);
        L.pcSlopeLow = vgDPc(L, L.pcLowSw);
        L.pcHigh = vgPc(L, L.pcHighSw);
        L.pcSlopeHigh = 2 * (0.0 - L.pcHigh) / (1.0 - L.pcHighSw);
        L.splineM0 = vgDPc(L, L.pcHighSw);
    }
    else {
        L.pcLow = L.pe * pow(L.pcLowSw, -1.0 / L.lambda);
        L.pcSlopeLow = -L.pe / L.lambda * pow(L.pcLowSw, -1.0 / L.lambda - 1.0);
        L.bcSlopeHigh = -L.pe / L.lambda * pow(1.0, -1.0 / L.lambda - 1.0);
    }
}

template <class E>
GB_HD E hermite(const E& x, double x0, double x1, double y0, double y1, double m0, double m1)
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

template <class E>
GB_HD E pcnw(const TwoPhaseLaw& L, const E& Sw)
{
    const double s = val(Sw);
    if (L.law == 0) {
        if (s < L.pcLowSw) return L.pcLow + L.pcSlopeLow * (Sw - L.pcLowSw);
        if (s > L.pcHighSw) {
            const double yTh = L.pcHigh;
            const double m1 = (0.0 - yTh) / (1.0 - L.pcHighSw) * 2;
            if (s < 1.0) return hermite(Sw, L.pcHighSw, 1.0, L.pcHigh, 0.0, L.splineM0, L.pcSlopeHigh);
            return m1 * (Sw - 1.0) + 0.0;
        }
        return dpow(dpow(Sw, -1.0 / L.m) - 1, 1.0 / L.n) / L.alpha;
    }
    if (s <= L.pcLowSw) return L.pcLow + L.pcSlopeLow * (Sw - L.pcLowSw);
    if (s >= 1.0) return L.pe + L.bcSlopeHigh * (Sw - 1.0);
    return L.pe * dpow(Sw, -1.0 / L.lambda);
}

template <class E>
GB_HD E krw(const TwoPhaseLaw& L, const E& Sw)
{
    const double s = val(Sw);
    if (s <= 0.0) return konst<E>(0.0);
    if (s >= 1.0) return konst<E>(1.0);
    if (L.law == 0) {
        E r = 1.0 - dpow(1.0 - dpow(Sw, 1 / L.m), L.m);
        return dsqrt(Sw) * r * r;
    }
    return dpow(Sw, 2.0 / L.lambda + 3.0);
}

// argument: 1 - S_n,eff
template <class E>
GB_HD E krn(const TwoPhaseLaw& L, const E& Sw)
{
    const double s = val(Sw);
    if (s <= 0.0) return konst<E>(1.0);
    if (s >= 1.0) return konst<E>(0.0);
    if (L.law == 0) return dpow(1 - Sw, 1.0 / 3) * dpow(1 - dpow(Sw, 1 / L.m), 2 * L.m);
    E Sn = 1.0 - Sw;
    return Sn * Sn * (1.0 - dpow(Sw, 2.0 / L.lambda + 1.0));
}

template <class E>
GB_HD E corey(const E& S, double n)
{
    const double s = val(S);
    if (s <= 0.0) return konst<E>(0.0);
    if (s >= 1.0) return konst<E>(1.0);
    if (n == 2.0) return S * S;
    return dpow(S, n);
}

// --------------------------------------------------------------- PVT -----
#define GBFV_MAX_TABLE 32
struct Table1D {
    int n;
    double x[GBFV_MAX_TABLE];
    double y[GBFV_MAX_TABLE];
};

GB_HD int tableSegment(const Table1D& t, double xv)
{
    const int n = t.n;
    if (xv <= t.x[0]) return 0;
    if (xv >= t.x[n - 1]) return n - 2;
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (t.x[mid] <= xv) lo = mid;
        else hi = mid;
    }
    return lo;
}

// piecewise linear with linear extrapolation on the end segments
template <class E>
GB_HD E tableEval(const Table1D& t, const E& xv)
{
    const int i = tableSegment(t, val(xv));
    const double s = (t.y[i + 1] - t.y[i]) / (t.x[i + 1] - t.x[i]);
    return t.y[i] + s * (xv - t.x[i]);
}

struct BlackOilPvt {
    double rhoRefO, rhoRefW, rhoRefG;
    Table1D rsSat, pBubble, invBoSat, muoSat, invBg, mug;
    double oilComp;
    double pwRef, bwRef, cw, muw;
};

template <class E>
GB_HD E waterInvB(const BlackOilPvt& T, const E& p)
{
    E X = T.cw * (p - T.pwRef);
    return (1.0 + X * (1.0 + X * 0.5)) / T.bwRef;
}

}  // namespace gbfv
