// ORACLE -- TEST INFRASTRUCTURE ONLY (see orc_core.h).
// Drag / lift integration over the IB elements, src/StressCalc.f90:14-208,
// summed serially in element order.
#include <cmath>
#include "orc_core.h"

namespace orc {

namespace {
double deriv(double x, double x2, double x1, double p_x, double p_x2, double p_x1) {
  const double h2 = std::fabs(x2 - x), h1 = std::fabs(x1 - x);
  return (h1 * h1 * p_x2 - h2 * h2 * p_x1 + (h2 * h2 - h1 * h1) * p_x) /
         (h1 * h2 * (h1 + h2) + 1e-16);
}
void vad(double x, double y, double z, int64_t i, int64_t j, int64_t k, const F1& xg,
         const F1& yg, const F1& zg, int off, const F3& var, double& val, double der[3]) {
  int64_t ii = i, jj = j, kk = k;
  if (off == 1) ii = i - 1;
  if (off == 2) jj = j - 1;
  if (off == 3) kk = k - 1;
  double f[4];
  f[0] = var(ii, jj, kk); f[1] = var(ii, jj + 1, kk); f[2] = var(ii, jj, kk + 1); f[3] = var(ii, jj + 1, kk + 1);
  const double t11 = bilinear_interpolation(y, z, yg(j), yg(j + 1), zg(k), zg(k + 1), f);
  f[0] = var(ii + 1, jj, kk); f[1] = var(ii + 1, jj + 1, kk); f[2] = var(ii + 1, jj, kk + 1); f[3] = var(ii + 1, jj + 1, kk + 1);
  const double t12 = bilinear_interpolation(y, z, yg(j), yg(j + 1), zg(k), zg(k + 1), f);
  f[0] = var(ii, jj, kk); f[1] = var(ii + 1, jj, kk); f[2] = var(ii, jj, kk + 1); f[3] = var(ii + 1, jj, kk + 1);
  const double t21 = bilinear_interpolation(x, z, xg(i), xg(i + 1), zg(k), zg(k + 1), f);
  f[0] = var(ii, jj + 1, kk); f[1] = var(ii + 1, jj + 1, kk); f[2] = var(ii, jj + 1, kk + 1); f[3] = var(ii + 1, jj + 1, kk + 1);
  const double t22 = bilinear_interpolation(x, z, xg(i), xg(i + 1), zg(k), zg(k + 1), f);
  f[0] = var(ii, jj, kk); f[1] = var(ii + 1, jj, kk); f[2] = var(ii, jj + 1, kk); f[3] = var(ii + 1, jj + 1, kk);
  const double t31 = bilinear_interpolation(x, y, xg(i), xg(i + 1), yg(j), yg(j + 1), f);
  f[0] = var(ii, jj, kk + 1); f[1] = var(ii + 1, jj, kk + 1); f[2] = var(ii, jj + 1, kk + 1); f[3] = var(ii + 1, jj + 1, kk + 1);
  const double t32 = bilinear_interpolation(x, y, xg(i), xg(i + 1), yg(j), yg(j + 1), f);
  val = linear_interpolation(x, xg(i), xg(i + 1), t11, t12);
  der[0] = deriv(x, xg(i + 1), xg(i), val, t12, t11);
  der[1] = deriv(y, yg(j + 1), yg(j), val, t22, t21);
  der[2] = deriv(z, zg(k + 1), zg(k), val, t32, t31);
}
int64_t fidx(Block& b, double v, const F1& a, int64_t s, int64_t f) {
  for (int64_t i = s; i <= f; ++i)
    if (v >= a(i) && v < a(i + 1)) return i;
  if (b.err == 0) b.err = ORC_E_NOTFOUND;
  return s;
}
}  // namespace

void stress_calculation(Block& b, double mu_f, double rho_f) {
  double vD = 0, pD = 0, vL = 0, pL = 0, sa = 0, aSx = 0, aSy = 0;
  for (int64_t e = 1; e <= b.ibElems; ++e) {
    const double nrm[3] = {b.cosAlpha(e), b.cosBeta(e), b.cosGamma(e)};
    const int64_t ic = fidx(b, b.xcent(e), b.x1, 2, b.nx + 1);
    const int64_t jc = fidx(b, b.ycent(e), b.y1, 2, b.ny + 1);
    const int64_t kc = fidx(b, b.zcent(e), b.z1, 2, b.nz + 1);
    const double dX = b.x1(ic + 1) - b.x1(ic), dY = b.y1(jc + 1) - b.y1(jc),
                 dZ = b.z1(kc + 1) - b.z1(kc);
    const double diag = std::sqrt(dX * dX + dY * dY + dZ * dZ);
    const double nd = diag;
    const double px = b.xcent(e) + nd * nrm[0], py = b.ycent(e) + nd * nrm[1],
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
    const double us = b.xdot;
    const double vs = -b.thetaDot * (b.zcent(e) - b.piv_z) + b.ydot;
    const double ws = b.thetaDot * (b.ycent(e) - b.piv_y);
    const double ac_z = -(b.thetaDot * b.thetaDot) * (b.zcent(e) - b.piv_z);
    const double ac_y = -(b.thetaDot * b.thetaDot) * (b.ycent(e) - b.piv_y);
    const double at_z = b.thetaDDot * (b.ycent(e) - b.piv_y);
    const double at_y = -b.thetaDDot * (b.zcent(e) - b.piv_z);
    const double dpdn = -((ac_z + at_z) * b.cosGamma(e) + (ac_y + at_y) * b.cosBeta(e)) -
                        b.yddot * b.cosBeta(e);
    double val, der[3], ddn[3];
    auto dotp = [&](const double a[3]) { return a[0] * nrm[0] + a[1] * nrm[1] + a[2] * nrm[2]; };
    vad(px, py, pz, fidx(b, px, b.xu, 2, b.nx + 1), fidx(b, py, b.yu, 2, b.ny + 1),
        fidx(b, pz, b.zu, 2, b.nz + 1), b.xu, b.yu, b.zu, 1, b.u, val, der);
    ddn[0] = (2.0 / nd) * (val - us) - dotp(der);
    vad(px, py, pz, fidx(b, px, b.xv, 2, b.nx + 1), fidx(b, py, b.yv, 2, b.ny + 1),
        fidx(b, pz, b.zv, 2, b.nz + 1), b.xv, b.yv, b.zv, 2, b.v, val, der);
    ddn[1] = (2.0 / nd) * (val - vs) - dotp(der);
    vad(px, py, pz, fidx(b, px, b.xw, 2, b.nx + 1), fidx(b, py, b.yw, 2, b.ny + 1),
        fidx(b, pz, b.zw, 2, b.nz + 1), b.xw, b.yw, b.zw, 3, b.w, val, der);
    ddn[2] = (2.0 / nd) * (val - ws) - dotp(der);
    const double alen = b.element_length(e);
    const double area = alen / 2.0;
    const double a_yz = 0.5 * std::fabs(alen * nrm[0]);
    const double a_xz = 0.5 * std::fabs(alen * nrm[1]);
    const double dd = dotp(ddn);
    double shear[3];
    for (int c = 0; c < 3; ++c) shear[c] = (ddn[c] - dd * nrm[c]) * mu_f * area;
    vad(px, py, pz, fidx(b, px, b.xp, 2, b.nx + 1), fidx(b, py, b.yp, 2, b.ny + 1),
        fidx(b, pz, b.zp, 2, b.nz + 1), b.xp, b.yp, b.zp, 0, b.p, val, der);
    const double dpdn_e = dotp(der);
    const double cval = val - (dpdn_e + dpdn) * diag * 0.5;
    double fs[3];
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
