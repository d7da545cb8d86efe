// ORACLE -- TEST INFRASTRUCTURE ONLY (see orc_core.h).
// Drag / lift integration over the IB elements, src/StressCalc.f90:14-208,
// summed serially in element order.
#include <cmath>
#include "orc_core.h"

namespace orc {

namespace {
real deriv(real x, real x2, real x1, real p_x, real p_x2, real p_x1) {
  const real h2 = fabs(x2 - x), h1 = fabs(x1 - x);
  return (h1 * h1 * p_x2 - h2 * h2 * p_x1 + (h2 * h2 - h1 * h1) * p_x) /
         (h1 * h2 * (h1 + h2) + 1e-16);
}
void vad(real x, real y, real z, int64_t i, int64_t j, int64_t k, const F1& xg,
         const F1& yg, const F1& zg, int off, const F3& var, real& val, real der[3]) {
  int64_t ii = i, jj = j, kk = k;
  if (off == 1) ii = i - 1;
  if (off == 2) jj = j - 1;
  if (off == 3) kk = k - 1;
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
  der[0] = deriv(x, xg(i + 1), xg(i), val, t12, t11);
  der[1] = deriv(y, yg(j + 1), yg(j), val, t22, t21);
  der[2] = deriv(z, zg(k + 1), zg(k), val, t32, t31);
}
int64_t fidx(Block& b, real v, const F1& a, int64_t s, int64_t f) {
  for (int64_t i = s; i <= f; ++i)
    if (v >= a(i) && v < a(i + 1)) return i;
  if (b.err == 0) b.err = ORC_E_NOTFOUND;
  return s;
}
}  // namespace

void stress_calculation(Block& b, real mu_f, real rho_f) {
  real vD = 0, pD = 0, vL = 0, pL = 0, sa = 0, aSx = 0, aSy = 0;
  for (int64_t e = 1; e <= b.ibElems; ++e) {
    const real nrm[3] = {b.cosAlpha(e), b.cosBeta(e), b.cosGamma(e)};
    const int64_t ic = fidx(b, b.xcent(e), b.x1, 2, b.nx + 1);
    const int64_t jc = fidx(b, b.ycent(e), b.y1, 2, b.ny + 1);
    const int64_t kc = fidx(b, b.zcent(e), b.z1, 2, b.nz + 1);
    const real dX = b.x1(ic + 1) - b.x1(ic), dY = b.y1(jc + 1) - b.y1(jc),
                 dZ = b.z1(kc + 1) - b.z1(kc);
    const real diag = sqrt(dX * dX + dY * dY + dZ * dZ);
    const real nd = diag;
    const real px = b.xcent(e) + nd * nrm[0], py = b.ycent(e) + nd * nrm[1],
                 pz = b.zcent(e) + nd * nrm[2];
    const int64_t sid = b.ibSurfId(e);
    if (sid == 50) {
      b.thetaDot = 0.0;
      b.thetaDDot = 0.0;
    } else if (sid == 51) {
      b.thetaDot = b.thetaDot1;
      b.thetaDDot = b.thetaDDot1;
    } else if (sid == 52) {
      b.thetaDot = b.thetaDot2;
      b.thetaDDot = b.thetaDDot2;
    }
    const real us = b.xdot;
    const real vs = -b.thetaDot * (b.zcent(e) - b.piv_z) + b.ydot;
    const real ws = b.thetaDot * (b.ycent(e) - b.piv_y);
    const real ac_z = -(b.thetaDot * b.thetaDot) * (b.zcent(e) - b.piv_z);
    const real ac_y = -(b.thetaDot * b.thetaDot) * (b.ycent(e) - b.piv_y);
    const real at_z = b.thetaDDot * (b.ycent(e) - b.piv_y);
    const real at_y = -b.thetaDDot * (b.zcent(e) - b.piv_z);
    const real dpdn = -((ac_z + at_z) * b.cosGamma(e) + (ac_y + at_y) * b.cosBeta(e)) -
                        b.yddot * b.cosBeta(e);
    real val, der[3], ddn[3];
    auto dotp = [&](const real a[3]) { return a[0] * nrm[0] + a[1] * nrm[1] + a[2] * nrm[2]; };
    vad(px, py, pz, fidx(b, px, b.xu, 2, b.nx + 1), fidx(b, py, b.yu, 2, b.ny + 1),
        fidx(b, pz, b.zu, 2, b.nz + 1), b.xu, b.yu, b.zu, 1, b.u, val, der);
    ddn[0] = (2.0 / nd) * (val - us) - dotp(der);
    vad(px, py, pz, fidx(b, px, b.xv, 2, b.nx + 1), fidx(b, py, b.yv, 2, b.ny + 1),
        fidx(b, pz, b.zv, 2, b.nz + 1), b.xv, b.yv, b.zv, 2, b.v, val, der);
    ddn[1] = (2.0 / nd) * (val - vs) - dotp(der);
    vad(px, py, pz, fidx(b, px, b.xw, 2, b.nx + 1), fidx(b, py, b.yw, 2, b.ny + 1),
        fidx(b, pz, b.zw, 2, b.nz + 1), b.xw, b.yw, b.zw, 3, b.w, val, der);
    ddn[2] = (2.0 / nd) * (val - ws) - dotp(der);
    const real alen = b.element_length(e);
    const real area = alen / 2.0;
    const real a_yz = 0.5 * fabs(alen * nrm[0]);
    const real a_xz = 0.5 * fabs(alen * nrm[1]);
    const real dd = dotp(ddn);
    real shear[3];
    for (int c = 0; c < 3; ++c) shear[c] = (ddn[c] - dd * nrm[c]) * mu_f * area;
    vad(px, py, pz, fidx(b, px, b.xp, 2, b.nx + 1), fidx(b, py, b.yp, 2, b.ny + 1),
        fidx(b, pz, b.zp, 2, b.nz + 1), b.xp, b.yp, b.zp, 0, b.p, val, der);
    const real dpdn_e = dotp(der);
    const real cval = val - (dpdn_e + dpdn) * diag * 0.5;
    real fs[3];
    for (int c = 0; c < 3; ++c) fs[c] = -cval * area * nrm[c] * rho_f;
    vD = vD + shear[0];
    pD = pD + fs[0];
    vL = vL + shear[1];
    pL = pL + fs[1];
    sa = sa + area;
    aSx = aSx + a_xz;
    aSy = aSy + a_yz;
  }
  aSx = 0.5 * aSx;
  aSy = 0.5 * aSy;
  b.viscous_drag = 2.0 * (vD / aSx);
  b.pressure_drag = 2.0 * (pD / aSy);
  b.viscous_lift = 2.0 * (vL / aSx);
  b.pressure_lift = 2.0 * (pL / aSy);
}

}  // namespace orc
