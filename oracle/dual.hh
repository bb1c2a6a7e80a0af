// ORACLE -- test infrastructure only.  Only tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline / reference legs may load or run anything
// under oracle/.  It checks the product; it is never the product path.
//
// Forward-mode dual numbers restating the semantics of opm-common's
// DenseAd::Evaluation (used by the reference through
// opm/models/discretization/common/fvbaseadlocallinearizer.hh:62-72):
// a value plus N partial derivatives, product/quotient rules, comparisons
// on the value only.  opm-common is not vendored under the reference tree,
// so these rules are restated from the published forward-mode AD algebra.
#pragma once
#include <cmath>

namespace oracle {

template <int N>
struct Dual {
    double v;
    double d[N];

    Dual() : v(0.0) { for (int i = 0; i < N; ++i) d[i] = 0.0; }
    Dual(double x) : v(x) { for (int i = 0; i < N; ++i) d[i] = 0.0; }
    static Dual variable(double x, int idx)
    {
        Dual r(x);
        r.d[idx] = 1.0;
        return r;
    }
    Dual& operator+=(const Dual& o) { v += o.v; for (int i = 0; i < N; ++i) d[i] += o.d[i]; return *this; }
    Dual& operator-=(const Dual& o) { v -= o.v; for (int i = 0; i < N; ++i) d[i] -= o.d[i]; return *this; }
    Dual& operator+=(double s) { v += s; return *this; }
    Dual& operator-=(double s) { v -= s; return *this; }
    // (u v)' = u' v + v' u
    Dual& operator*=(const Dual& o)
    {
        const double u = v, w = o.v;
        v *= w;
        for (int i = 0; i < N; ++i) d[i] = d[i] * w + o.d[i] * u;
        return *this;
    }
    Dual& operator*=(double s) { v *= s; for (int i = 0; i < N; ++i) d[i] *= s; return *this; }
    // (u / w)' = (w u' - u w') / w^2
    Dual& operator/=(const Dual& o)
    {
        const double u = v, w = o.v;
        for (int i = 0; i < N; ++i) d[i] = (w * d[i] - u * o.d[i]) / (w * w);
        v = u / w;
        return *this;
    }
    Dual& operator/=(double s) { v /= s; for (int i = 0; i < N; ++i) d[i] /= s; return *this; }
    Dual operator-() const { Dual r; r.v = -v; for (int i = 0; i < N; ++i) r.d[i] = -d[i]; return r; }
};

template <int N> inline Dual<N> operator+(Dual<N> a, const Dual<N>& b) { return a += b; }
template <int N> inline Dual<N> operator-(Dual<N> a, const Dual<N>& b) { return a -= b; }
template <int N> inline Dual<N> operator*(Dual<N> a, const Dual<N>& b) { return a *= b; }
template <int N> inline Dual<N> operator/(Dual<N> a, const Dual<N>& b) { return a /= b; }
template <int N> inline Dual<N> operator+(Dual<N> a, double s) { return a += s; }
template <int N> inline Dual<N> operator-(Dual<N> a, double s) { return a -= s; }
template <int N> inline Dual<N> operator*(Dual<N> a, double s) { return a *= s; }
template <int N> inline Dual<N> operator/(Dual<N> a, double s) { return a /= s; }
template <int N> inline Dual<N> operator+(double s, Dual<N> a) { return a += s; }
template <int N> inline Dual<N> operator*(double s, Dual<N> a) { return a *= s; }
template <int N> inline Dual<N> operator-(double s, const Dual<N>& a)
{
    Dual<N> r;
    r.v = s - a.v;
    for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
    return r;
}
// s / w: value s/w, derivative -s/w^2 * w'
template <int N> inline Dual<N> operator/(double s, const Dual<N>& a)
{
    Dual<N> r;
    r.v = s / a.v;
    const double df = -s / (a.v * a.v);
    for (int i = 0; i < N; ++i) r.d[i] = df * a.d[i];
    return r;
}
template <int N> inline bool operator<(const Dual<N>& a, double s) { return a.v < s; }
template <int N> inline bool operator>(const Dual<N>& a, double s) { return a.v > s; }
template <int N> inline bool operator<=(const Dual<N>& a, double s) { return a.v <= s; }
template <int N> inline bool operator>=(const Dual<N>& a, double s) { return a.v >= s; }
template <int N> inline bool operator>(const Dual<N>& a, const Dual<N>& b) { return a.v > b.v; }
template <int N> inline bool operator<(const Dual<N>& a, const Dual<N>& b) { return a.v < b.v; }

// pow with a constant exponent: (f^g)' = f^g * g / f * f'; base 0 -> 0
template <int N> inline Dual<N> pow(const Dual<N>& x, double e)
{
    Dual<N> r;
    const double px = std::pow(x.v, e);
    if (x.v == 0.0) return Dual<N>(0.0);
    r.v = px;
    const double df = px / x.v * e;
    for (int i = 0; i < N; ++i) r.d[i] = df * x.d[i];
    return r;
}
template <int N> inline Dual<N> sqrt(const Dual<N>& x)
{
    Dual<N> r;
    const double sx = std::sqrt(x.v);
    r.v = sx;
    const double df = 0.5 / sx;
    for (int i = 0; i < N; ++i) r.d[i] = df * x.d[i];
    return r;
}
template <int N> inline Dual<N> max(const Dual<N>& a, const Dual<N>& b) { return a.v > b.v ? a : b; }
template <int N> inline Dual<N> min(const Dual<N>& a, const Dual<N>& b) { return a.v < b.v ? a : b; }

// scalar overloads so the same templated physics compiles for double
inline double pow(double x, double e) { return std::pow(x, e); }
inline double sqrt(double x) { return std::sqrt(x); }

inline double value(double x) { return x; }
template <int N> inline double value(const Dual<N>& x) { return x.v; }

}  // namespace oracle
