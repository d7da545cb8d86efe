// ORACLE -- TEST INFRASTRUCTURE ONLY (see orc_core.h).
// Immersed-boundary forcing routines of src/Forcing.f90, restated serially.
#include <algorithm>
#include <cmath>
#include "orc_core.h"

namespace orc {

// src/Interpolation.f90:16-22
real linear_interpolation(real x, real x0, real x1, real y0, real y1) {
  return y0 + (x - x0) * (y1 - y0) / (x1 - x0);
}

// src/Interpolation.f90:27-42; f = values at (x1,y1),(x2,y1),(x1,y2),(x2,y2)
real bilinear_interpolation(real x, real y, real x1, real x2, real y1, real y2,
                              const real f[4]) {
  const real numer = f[0] * (x2 - x) * (y2 - y) + f[2] * (x2 - x) * (y - y1) +
                       f[1] * (x - x1) * (y2 - y) + f[3] * (x - x1) * (y - y1);
  const real denom = (x2 - x1) * (y2 - y1);
  return numer / denom;
}

namespace {

// compute_derivative, src/Forcing.f90:1080-1089
real compute_derivative(real x, real x2, real x1, real p_x, real p_x2, real p_x1) {
  const real h2 = fabs(x2 - x);
  const real h1 = fabs(x1 - x);
  return (h1 * h1 * p_x2 - h2 * h2 * p_x1 + (h2 * h2 - h1 * h1) * p_x) /
         (h1 * h2 * (h1 + h2) + 1e-16);
}

// compute_value_and_derivatives, src/Forcing.f90:1091-1161
// The reference reads outside `var` when a stencil corner falls off the array
// (a probe with no bracket, or the staggered offset at index 1); the oracle
// records ORC_E_NOTFOUND in *err and clamps the corner into the array, as the
// GPU library does.
void value_and_derivatives(real x, real y, real z, int64_t i, int64_t j, int64_t k,
                           const F1& xg, const F1& yg, const F1& zg, int offset_axis,
                           const F3& var, real& val, real der[3], int* err) {
  int64_t ii = i, jj = j, kk = k;
  if (offset_axis == 1) ii = i - 1;
  if (offset_axis == 2) jj = j - 1;
  if (offset_axis == 3) kk = k - 1;
  if (ii < 1 || ii + 1 > var.n1 || jj < 1 || jj + 1 > var.n2 || kk < 1 || kk + 1 > var.n3) {
    if (*err == 0) *err = ORC_E_NOTFOUND;
    ii = std::max<int64_t>(1, std::min<int64_t>(ii, var.n1 - 1));
    jj = std::max<int64_t>(1, std::min<int64_t>(jj, var.n2 - 1));
    kk = std::max<int64_t>(1, std::min<int64_t>(kk, var.n3 - 1));
  }
  real f[4];
  f[0] = var(ii, jj, kk); f[1] = var(ii, jj + 1, kk); f[2] = var(ii, jj, kk + 1); f[3] = var(ii, jj + 1, kk + 1);
  const real t11 = bilinear_interpolation(y, z, yg(j), yg(j + 1), zg(k), zg(k + 1), f);
  f[0] = var(ii + 1, jj, kk); f[1] = var(ii + 1, jj + 1, kk); f[2] = var(ii + 1, jj, kk + 1); f[3] = var(ii + 1, jj + 1, kk + 1);
  const real t12 = bilinear_interpolation(y, z, yg(j), yg(j + 1), zg(k), zg(k + 1), f);
  f[0] = var(ii, jj, kk); f[1] = var(ii + 1, jj, kk); f[2] = var(ii, jj, kk + 1); f[3] = var(ii + 1, jj, kk + 1);
  const real t21 = bilinear_interpolation(x, z, xg(i), xg(i + 1), zg(k), zg(k + 1), f);
  f[0] = var(ii, jj + 1, kk); f[1] = var(ii + 1, jj + 1, kk); f[2] = var(ii, jj + 1, kk + 1); f[3] = var(ii + 1, jj + 1, kk + 1);
  const real t22 = bilinear_interpolation(x, z, xg(i), xg(i + 1), zg(k), zg(k + 1), f);
  f[0] = var(ii, jj, kk); f[1] = var(ii + 1, jj, kk); f[2] = var(ii, jj + 1, kk); f[3] = var(ii + 1, jj + 1, kk);
  const real t31 = bilinear_interpolation(x, y, xg(i), xg(i + 1), yg(j), yg(j + 1), f);
  f[0] = var(ii, jj, kk + 1); f[1] = var(ii + 1, jj, kk + 1); f[2] = var(ii, jj + 1, kk + 1); f[3] = var(ii + 1, jj + 1, kk + 1);
  const real t32 = bilinear_interpolation(x, y, xg(i), xg(i + 1), yg(j), yg(j + 1), f);
  val = linear_interpolation(x, xg(i), xg(i + 1), t11, t12);
  der[0] = compute_derivative(x, xg(i + 1), xg(i), val, t12, t11);
  der[1] = compute_derivative(y, yg(j + 1), yg(j), val, t22, t21);
  der[2] = compute_derivative(z, zg(k + 1), zg(k), val, t32, t31);
}

// find_index_in_array, src/Forcing.f90:1165-1183.  The reference leaves the
// result undefined when no bracket exists; the oracle records an error and
// returns the start index so that the caller stays in bounds.
int64_t find_index(Block& b, real value, const F1& a, int64_t start, int64_t finish) {
  for (int64_t i = start; i <= finish; ++i) {
    if (i < 1 || i + 1 > a.size()) continue;
    if (value >= a(i) && value < a(i + 1)) return i;
  }
  if (b.err == 0) b.err = ORC_E_NOTFOUND;
  int64_t s = start < 1 ? 1 : start;
  if (s + 1 > a.size()) s = a.size() - 1;
  return s;
}

inline real pt1_of(Block& b, int64_t i, int64_t j, int64_t k, real s2n) {
  return 1.5 * sqrt(b.deltax(i) * b.deltax(i) + b.deltay(j) * b.deltay(j) +
                         b.deltaz(k) * b.deltaz(k)) +
         (fabs(s2n) - s2n) * 0.5;
}

// The quadratic velocity reconstruction shared by every velocity variant.
inline real vel_quad(real pos_val, real surf, real dndn_e, real n1, real s2n) {
  const real cval = surf;
  const real bval = 2.0 / n1 * (pos_val - surf) - dndn_e;
  const real aval = dndn_e / n1 - (pos_val - surf) / (n1 * n1);
  return aval * (s2n * s2n) + bval * s2n + cval;
}

inline real dotn(Block& b, int64_t e, const real d[3]) {
  return d[0] * b.cosAlpha(e) + d[1] * b.cosBeta(e) + d[2] * b.cosGamma(e);
}

// dpdn of the rigid-body acceleration, src/Forcing.f90:29-52
void accel_terms(Block& b, int64_t e, real& ac_y, real& ac_z, real& at_y, real& at_z) {
  const int64_t sid = b.ibSurfId(e);
  if (sid == 50) {
    ac_z = ac_y = at_z = at_y = 0.0;
  } else if (sid == 51 || sid == 52) {
    b.thetaDot = sid == 51 ? b.thetaDot1 : b.thetaDot2;
    b.thetaDDot = sid == 51 ? b.thetaDDot1 : b.thetaDDot2;
    ac_z = -(b.thetaDot * b.thetaDot) * (b.zcent(e) - b.piv_z);
    ac_y = -(b.thetaDot * b.thetaDot) * (b.ycent(e) - b.piv_y);
    at_z = b.thetaDDot * (b.ycent(e) - b.piv_y);
    at_y = -b.thetaDDot * (b.zcent(e) - b.piv_z);
  }
}

// one pressure reconstruction (…1 and …Field variants), writes p(i,j,k)
void p_recon(Block& b, int64_t n, bool field) {
  const int64_t e = b.nelp(n);
  real ac_y = 0, ac_z = 0, at_y = 0, at_z = 0;
  accel_terms(b, e, ac_y, ac_z, at_y, at_z);
  const real dpdn = -((ac_z + at_z) * b.cosGamma(e) + (ac_y + at_y) * b.cosBeta(e)) -
                      b.yddot * b.cosBeta(e);
  const int64_t i = b.interceptedIndexPtr(n, 1), j = b.interceptedIndexPtr(n, 2),
                k = b.interceptedIndexPtr(n, 3);
  const real s2n = b.pNormDis(n);
  const real pt1 = pt1_of(b, i, j, k, s2n);
  const real px = b.xp(i) + pt1 * b.cosAlpha(e);
  const real py = b.yp(j) + pt1 * b.cosBeta(e);
  const real pz = b.zp(k) + pt1 * b.cosGamma(e);
  int64_t ix, iy, iz;
  if (!field) {
    ix = find_index(b, px, b.xp, 1, b.nx + 1);
    iy = find_index(b, py, b.yp, 1, b.ny + 1);
    iz = find_index(b, pz, b.zp, 1, b.nz + 1);
  } else {
    ix = find_index(b, px, b.xp, i - 7, i + 7);
    iy = find_index(b, py, b.yp, j - 7, j + 7);
    iz = find_index(b, pz, b.zp, k - 7, k + 7);
  }
  real val, der[3];
  value_and_derivatives(px, py, pz, ix, iy, iz, b.xp, b.yp, b.zp, 0, b.p, val, der, &b.err);
  const real dpdn_e = dotn(b, e, der);
  const real n1 = pt1 + s2n;
  const real bval = dpdn;
  const real aval = (dpdn_e - dpdn) / (2.0 * n1);
  const real cval = val - (dpdn_e + dpdn) * n1 * 0.5;
  b.p(i, j, k) = aval * (s2n * s2n) + bval * s2n + cval;
}

enum Comp { CU2 = 0, CU1, CV2, CV1, CW2, CW1 };

// surface velocity of one sample, src/Forcing.f90:112-118,156-162,194-204,
// 236-246,278-286,317-326 (…1); :910-922 etc. (…Field / …Ghost add alphaDot)
// mode: 0 = velocityForcing1, 1 = velocityForcingField, 2 = velocityForcingGhost.
// The reference writes the surface-50 v sample as `0 + ydot` in two places
// (Forcing.f90:237, :551); that form is kept because it maps -0.0 to +0.0.
real surf_velocity(Block& b, int64_t e, int comp, int mode) {
  const int64_t sid = b.ibSurfId(e);
  const bool with_alpha = mode != 0;
  if (comp == CU2 || comp == CU1) return b.xdot;
  if (comp == CV2 || comp == CV1) {
    if (sid == 50) {
      const bool plus0 = (comp == CV1 && mode == 0) || (comp == CV2 && mode == 2);
      return plus0 ? 0.0 + b.ydot : b.ydot;
    }
    b.thetaDot = sid == 51 ? b.thetaDot1 : b.thetaDot2;
    if (!with_alpha) return -b.thetaDot * (b.zcent(e) - b.piv_z) + b.ydot;
    return -b.thetaDot * (b.zcent(e) - b.piv_z) + (-b.alphaDot) * (b.xcent(e) - b.piv_x) + b.ydot;
  }
  if (sid == 50) return 0.0;
  b.thetaDot = sid == 51 ? b.thetaDot1 : b.thetaDot2;
  return b.thetaDot * (b.ycent(e) - b.piv_y);
}

struct CompGeo {
  const F1 *xg, *yg, *zg;
  int axis;
  const I1* nel;
  const F1* nd;
};

CompGeo comp_geo(Block& b, int c) {
  switch (c) {
    case CU2: return {&b.xu, &b.yu, &b.zu, 1, &b.nelu2, &b.u2NormDis};
    case CU1: return {&b.xu, &b.yu, &b.zu, 1, &b.nelu1, &b.u1NormDis};
    case CV2: return {&b.xv, &b.yv, &b.zv, 2, &b.nelv2, &b.v2NormDis};
    case CV1: return {&b.xv, &b.yv, &b.zv, 2, &b.nelv1, &b.v1NormDis};
    case CW2: return {&b.xw, &b.yw, &b.zw, 3, &b.nelw2, &b.w2NormDis};
    default: return {&b.xw, &b.yw, &b.zw, 3, &b.nelw1, &b.w1NormDis};
  }
}

// node position of the velocity sample of component c at IB cell (i,j,k)
void sample_pos(Block& b, int c, int64_t i, int64_t j, int64_t k, real q[3]) {
  const CompGeo g = comp_geo(b, c);
  q[0] = (*g.xg)(c == CU2 ? i + 1 : i);
  q[1] = (*g.yg)(c == CV2 ? j + 1 : j);
  q[2] = (*g.zg)(c == CW2 ? k + 1 : k);
}

// velocityForcing1 (mode 0), velocityForcingField (mode 1): one component of
// IB cell n.  Reads `src`, writes `dst` at the sample's own index.
void v_recon(Block& b, int64_t n, int c, int mode) {
  const CompGeo g = comp_geo(b, c);
  const int64_t e = (*g.nel)(n);
  const real surf = surf_velocity(b, e, c, mode);
  const int64_t i = b.interceptedIndexPtr(n, 1), j = b.interceptedIndexPtr(n, 2),
                k = b.interceptedIndexPtr(n, 3);
  const real s2n = (*g.nd)(n);
  const real pt1 = pt1_of(b, i, j, k, s2n);
  real q[3];
  sample_pos(b, c, i, j, k, q);
  const real px = q[0] + pt1 * b.cosAlpha(e);
  const real py = q[1] + pt1 * b.cosBeta(e);
  const real pz = q[2] + pt1 * b.cosGamma(e);
  int64_t ix, iy, iz;
  if (mode == 0) {
    ix = find_index(b, px, *g.xg, 1, b.nx + (c == CU2 ? 2 : 1));
    iy = find_index(b, py, *g.yg, 1, b.ny + (c == CV2 ? 2 : 1));
    iz = find_index(b, pz, *g.zg, 1, b.nz + (c == CW2 ? 2 : 1));
    if (c == CU2 && ix == b.nx + 2) ix = b.nx + 1;
    if (c == CU1 && ix == 1) ix = 2;
    if (c == CV2 && iy == b.ny + 2) iy = b.ny + 1;
    if (c == CV1 && iy == 1) iy = 2;
    if (c == CW2 && iz == b.nz + 2) iz = b.nz + 1;
    if (c == CW1 && iz == 1) iz = 2;
  } else {
    ix = find_index(b, px, *g.xg, i - 7, i + 7);
    iy = find_index(b, py, *g.yg, j - 7, j + 7);
    iz = find_index(b, pz, *g.zg, k - 7, k + 7);
  }
  F3& src = g.axis == 1 ? b.ut : (g.axis == 2 ? b.vt : b.wt);
  F3& dst = mode == 0 ? src : (g.axis == 1 ? b.u : (g.axis == 2 ? b.v : b.w));
  real val, der[3];
  value_and_derivatives(px, py, pz, ix, iy, iz, *g.xg, *g.yg, *g.zg, g.axis, src, val, der, &b.err);
  const real dn = dotn(b, e, der);
  const real n1 = pt1 + s2n;
  const real r = vel_quad(val, surf, dn, n1, s2n);
  int64_t ti = i, tj = j, tk = k;
  if (c == CU1) ti = i - 1;
  if (c == CV1) tj = j - 1;
  if (c == CW1) tk = k - 1;
  dst(ti, tj, tk) = r;
}

}  // namespace

// velocityForcing1, src/Forcing.f90:92-360
void velocity_forcing1(Block& b) {
  for (int64_t n = 1; n <= b.ibCellCount; ++n)
    for (int c = 0; c < 6; ++c) v_recon(b, n, c, 0);
}

// pressureForcing1, src/Forcing.f90:14-90
void pressure_forcing1(Block& b) {
  for (int64_t n = 1; n <= b.ibCellCount; ++n) p_recon(b, n, false);
}

// velocityForcingField, src/Forcing.f90:813-1075
void velocity_forcing_field(Block& b) {
  for (int64_t n = 1; n <= b.ibCellCount; ++n)
    for (int c = 0; c < 6; ++c) v_recon(b, n, c, 1);
}

// pressureForcingField, src/Forcing.f90:737-811
void pressure_forcing_field(Block& b) {
  for (int64_t n = 1; n <= b.ibCellCount; ++n) p_recon(b, n, true);
}

// pressureForcingGhost, src/Forcing.f90:362-448
void pressure_forcing_ghost(Block& b) {
  for (int64_t n = 1; n <= b.TSCellCount; ++n) {
    const int64_t i = b.TSIndexPtr(n, 1), j = b.TSIndexPtr(n, 2), k = b.TSIndexPtr(n, 3);
    const int64_t it = b.index_ts(n);
    const int64_t e = b.nelp(it);
    real ac_y = 0, ac_z = 0, at_y = 0, at_z = 0;
    accel_terms(b, e, ac_y, ac_z, at_y, at_z);
    const real dpdn = ((ac_z + at_z) * b.cosGamma(e) + (ac_y + at_y) * b.cosBeta(e)) +
                        (b.yddot * (b.cosBeta(e)));
    const real s2n = -b.pNormDis(it);
    const real pt1 = pt1_of(b, i, j, k, s2n);
    const real px = b.xp(i) - pt1 * b.cosAlpha(e);
    const real py = b.yp(j) - pt1 * b.cosBeta(e);
    const real pz = b.zp(k) - pt1 * b.cosGamma(e);
    const int64_t ix = find_index(b, px, b.xp, i - 7, i + 7);
    const int64_t iy = find_index(b, py, b.yp, j - 7, j + 7);
    const int64_t iz = find_index(b, pz, b.zp, k - 7, k + 7);
    real val, der[3];
    value_and_derivatives(px, py, pz, ix, iy, iz, b.xp, b.yp, b.zp, 0, b.p, val, der, &b.err);
    const real dpdn_e = -1.0 * dotn(b, e, der);
    const real n1 = pt1 + s2n;
    const real bval = dpdn;
    const real aval = (dpdn_e - dpdn) / (2.0 * n1);
    const real cval = val - (dpdn_e + dpdn) * n1 * 0.5;
    b.p_ghost(n) = aval * (s2n * s2n) + bval * s2n + cval;
    b.pt_ghost(n) = b.p(i, j, k);
  }
}

// velocityForcingGhost, src/Forcing.f90:450-734
void velocity_forcing_ghost(Block& b) {
  F1* ghost[6] = {&b.u2_ghost, &b.u1_ghost, &b.v2_ghost, &b.v1_ghost, &b.w2_ghost, &b.w1_ghost};
  F1* tghost[6] = {&b.u2t_ghost, &b.u1t_ghost, &b.v2t_ghost, &b.v1t_ghost, &b.w2t_ghost,
                   &b.w1t_ghost};
  for (int64_t n = 1; n <= b.TSCellCount; ++n) {
    const int64_t i = b.TSIndexPtr(n, 1), j = b.TSIndexPtr(n, 2), k = b.TSIndexPtr(n, 3);
    const int64_t it = b.index_ts(n);
    for (int c = 0; c < 6; ++c) {
      const CompGeo g = comp_geo(b, c);
      const int64_t e = (*g.nel)(it);
      const real surf = surf_velocity(b, e, c, 2);
      const real s2n = -(*g.nd)(it);
      const real pt1 = pt1_of(b, i, j, k, s2n);
      real q[3];
      sample_pos(b, c, i, j, k, q);
      const real px = q[0] - pt1 * b.cosAlpha(e);
      const real py = q[1] - pt1 * b.cosBeta(e);
      const real pz = q[2] - pt1 * b.cosGamma(e);
      const int64_t ix = find_index(b, px, *g.xg, i - 7, i + 7);
      const int64_t iy = find_index(b, py, *g.yg, j - 7, j + 7);
      const int64_t iz = find_index(b, pz, *g.zg, k - 7, k + 7);
      F3& src = g.axis == 1 ? b.ut : (g.axis == 2 ? b.vt : b.wt);
      F3& cur = g.axis == 1 ? b.u : (g.axis == 2 ? b.v : b.w);
      real val, der[3];
      value_and_derivatives(px, py, pz, ix, iy, iz, *g.xg, *g.yg, *g.zg, g.axis, src, val, der, &b.err);
      const real dn = -1.0 * dotn(b, e, der);
      const real n1 = pt1 + s2n;
      (*ghost[c])(n) = vel_quad(val, surf, dn, n1, s2n);
      int64_t ti = i, tj = j, tk = k;
      if (c == CU1) ti = i - 1;
      if (c == CV1) tj = j - 1;
      if (c == CW1) tk = k - 1;
      (*tghost[c])(n) = cur(ti, tj, tk);
    }
  }
}

}  // namespace orc
