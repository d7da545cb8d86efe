// ORACLE -- TEST INFRASTRUCTURE ONLY (see orc_core.h).
//
// The oracle's floating-point type.  The default build uses plain double.
// Built with -DORC_DUAL=K, `real` is a forward-mode dual number carrying K
// tangent lanes next to its value: the oracle then computes, in one run, the
// value of every quantity (bit for bit the double build's: every value
// operation is the same IEEE operation in the same order, and -ffp-contract=off
// keeps it unfused) and its directional derivatives along K seeded input
// directions -- an FP64 tangent-linear model of the whole restated time step,
// including the moving geometry.  Branches, comparisons, index arithmetic and
// stop tests use the value only, so the discrete decisions (tags, brackets,
// upwind switches, iteration counts) are those of the double build and the
// tangents are the derivative of that branch of the program.
#pragma once
#include <cmath>

namespace orc {

using std::atan;
using std::cos;
using std::fabs;
using std::floor;
using std::fmax;
using std::fmin;
using std::pow;
using std::sin;
using std::sqrt;

#ifndef ORC_DUAL

using real = double;
constexpr int kLanes = 0;
inline double val(double x) { return x; }

#else

constexpr int kLanes = ORC_DUAL;

struct Dual {
  double v;
  double d[kLanes];
  Dual() : v(0.0) {
    for (double& x : d) x = 0.0;
  }
  Dual(double x) : v(x) {  // NOLINT: implicit, constants enter as dual numbers
    for (double& y : d) y = 0.0;
  }
  explicit operator double() const { return v; }

  Dual& operator+=(const Dual& b) {
    v += b.v;
    for (int l = 0; l < kLanes; ++l) d[l] += b.d[l];
    return *this;
  }
  Dual& operator-=(const Dual& b) {
    v -= b.v;
    for (int l = 0; l < kLanes; ++l) d[l] -= b.d[l];
    return *this;
  }
  Dual& operator*=(const Dual& b) {
    for (int l = 0; l < kLanes; ++l) d[l] = d[l] * b.v + v * b.d[l];
    v *= b.v;
    return *this;
  }
  Dual& operator/=(const Dual& b) {
    const double q = v / b.v;
    for (int l = 0; l < kLanes; ++l) d[l] = (d[l] - q * b.d[l]) / b.v;
    v = q;
    return *this;
  }
};

using real = Dual;
inline double val(double x) { return x; }
inline double val(const Dual& x) { return x.v; }

inline Dual operator-(const Dual& a) {
  Dual r;
  r.v = -a.v;
  for (int l = 0; l < kLanes; ++l) r.d[l] = -a.d[l];
  return r;
}
inline Dual operator+(const Dual& a) { return a; }

inline Dual operator+(Dual a, const Dual& b) { return a += b; }
inline Dual operator-(Dual a, const Dual& b) { return a -= b; }
inline Dual operator*(Dual a, const Dual& b) { return a *= b; }
inline Dual operator/(Dual a, const Dual& b) { return a /= b; }
inline Dual operator+(Dual a, double b) { return a += Dual(b); }
inline Dual operator-(Dual a, double b) { return a -= Dual(b); }
inline Dual operator*(Dual a, double b) { return a *= Dual(b); }
inline Dual operator/(Dual a, double b) { return a /= Dual(b); }
inline Dual operator+(double a, const Dual& b) { return Dual(a) += b; }
inline Dual operator-(double a, const Dual& b) { return Dual(a) -= b; }
inline Dual operator*(double a, const Dual& b) { return Dual(a) *= b; }
inline Dual operator/(double a, const Dual& b) { return Dual(a) /= b; }

#define ORC_DUAL_CMP(op)                                                   \
  inline bool operator op(const Dual& a, const Dual& b) { return a.v op b.v; } \
  inline bool operator op(const Dual& a, double b) { return a.v op b; }       \
  inline bool operator op(double a, const Dual& b) { return a op b.v; }
ORC_DUAL_CMP(<)
ORC_DUAL_CMP(<=)
ORC_DUAL_CMP(>)
ORC_DUAL_CMP(>=)
ORC_DUAL_CMP(==)
ORC_DUAL_CMP(!=)
#undef ORC_DUAL_CMP

// f(a) with f'(a) = s: value f(a.v), tangents s * a.d
inline Dual chain(double fv, double s, const Dual& a) {
  Dual r(fv);
  for (int l = 0; l < kLanes; ++l) r.d[l] = s * a.d[l];
  return r;
}

inline Dual fabs(const Dual& a) { return chain(std::fabs(a.v), a.v < 0.0 ? -1.0 : 1.0, a); }
inline Dual sqrt(const Dual& a) {
  const double s = std::sqrt(a.v);
  return chain(s, s > 0.0 ? 0.5 / s : 0.0, a);
}
inline Dual sin(const Dual& a) { return chain(std::sin(a.v), std::cos(a.v), a); }
inline Dual cos(const Dual& a) { return chain(std::cos(a.v), -std::sin(a.v), a); }
inline Dual atan(const Dual& a) { return chain(std::atan(a.v), 1.0 / (1.0 + a.v * a.v), a); }
inline Dual floor(const Dual& a) { return chain(std::floor(a.v), 0.0, a); }
inline Dual pow(const Dual& a, double e) {
  return chain(std::pow(a.v, e), a.v != 0.0 ? e * std::pow(a.v, e - 1.0) : 0.0, a);
}
// std::fmax / std::fmin pick an operand (the other one where one is NaN);
// the tangent is the picked operand's
inline Dual fmax(const Dual& a, const Dual& b) { return (b.v > a.v || a.v != a.v) ? b : a; }
inline Dual fmin(const Dual& a, const Dual& b) { return (b.v < a.v || a.v != a.v) ? b : a; }
inline Dual fmax(const Dual& a, double b) { return fmax(a, Dual(b)); }
inline Dual fmax(double a, const Dual& b) { return fmax(Dual(a), b); }
inline Dual fmin(const Dual& a, double b) { return fmin(a, Dual(b)); }
inline Dual fmin(double a, const Dual& b) { return fmin(Dual(a), b); }

#endif

}  // namespace orc
