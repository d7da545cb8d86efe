// ORACLE -- TEST INFRASTRUCTURE ONLY (see orc_core.h).
// Momentum predictor, its coefficient tables, Poisson coefficients and the
// domain / solid-cell boundary conditions, restated serially in FP64.
#include <cmath>
#include "orc_core.h"

namespace orc {

std::vector<Block*> g_blocks;
std::vector<Interface*> g_interfaces;

// src/AllocateArrays.f90:15-57 (+ the grid arrays of src/ReadInput.f90:206-225)
void allocate_arrays(Block& b) {
  const int64_t nx = b.nx, ny = b.ny, nz = b.nz;
  for (F3* f : {&b.u, &b.ut, &b.v, &b.vt, &b.w, &b.wt, &b.p, &b.b, &b.pc, &b.pco, &b.u_dum, &b.v_dum, &b.w_dum,
                &b.p_dum})
    f->alloc(nx + 2, ny + 2, nz + 2);
  b.cell.alloc(nx + 2, ny + 2, nz + 2);
  b.cell_n.alloc(nx + 2, ny + 2, nz + 2);
  b.cell2.alloc(nx + 3, ny + 3, nz + 3);
  b.cell_pr.alloc(nx + 3, ny + 3, nz + 3);
  b.nodeIdTag.alloc(nx + 3, ny + 3, nz + 3);
  b.Acx.alloc(nx, 3);
  b.Acy.alloc(ny, 3);
  b.Acz.alloc(nz, 3);
  b.x1.alloc(nx + 3);
  b.y1.alloc(ny + 3);
  b.z1.alloc(nz + 3);
  b.deltax.alloc(nx + 2);
  b.deltay.alloc(ny + 2);
  b.deltaz.alloc(nz + 2);
  b.xu.alloc(nx + 3);
  b.yu.alloc(ny + 2);
  b.zu.alloc(nz + 2);
  b.xv.alloc(nx + 2);
  b.yv.alloc(ny + 3);
  b.zv.alloc(nz + 2);
  b.xw.alloc(nx + 2);
  b.yw.alloc(ny + 2);
  b.zw.alloc(nz + 3);
  b.xp.alloc(nx + 2);
  b.yp.alloc(ny + 2);
  b.zp.alloc(nz + 2);
}

// src/ReadInput.f90:261-351: given x1(2..nx+2) (faces) fill the ghosts, the
// spacings and the staggered coordinate arrays.
void derive_grids(Block& b) {
  auto one = [](F1& c1, F1& d, int64_t n) {
    for (int64_t i = 2; i <= n + 1; ++i) d(i) = c1(i + 1) - c1(i);
    d(1) = d(2);
    d(n + 2) = d(n + 1);
    c1(1) = c1(2) - d(1);
    c1(n + 3) = c1(n + 2) + d(n + 2);
  };
  one(b.x1, b.deltax, b.nx);
  one(b.y1, b.deltay, b.ny);
  one(b.z1, b.deltaz, b.nz);
  for (int64_t i = 1; i <= b.nx + 3; ++i) b.xu(i) = b.x1(i);
  for (int64_t i = 1; i <= b.ny + 3; ++i) b.yv(i) = b.y1(i);
  for (int64_t i = 1; i <= b.nz + 3; ++i) b.zw(i) = b.z1(i);
  for (int64_t i = 1; i <= b.ny + 2; ++i) {
    b.yu(i) = 0.5 * (b.y1(i) + b.y1(i + 1));
    b.yw(i) = b.yu(i);
    b.yp(i) = b.yu(i);
  }
  for (int64_t i = 1; i <= b.nx + 2; ++i) {
    b.xv(i) = 0.5 * (b.x1(i) + b.x1(i + 1));
    b.xw(i) = b.xv(i);
    b.xp(i) = b.xv(i);
  }
  for (int64_t i = 1; i <= b.nz + 2; ++i) {
    b.zu(i) = 0.5 * (b.z1(i) + b.z1(i + 1));
    b.zv(i) = b.zu(i);
    b.zp(i) = b.zu(i);
  }
}

// ---------------------------------------------------------------------------
// Non-uniform third-order upwind coefficients, src/NavierStokes.f90:13-250 and
// compute_f / compute_s / compute_ak :915-996.  Fortran integer powers x**n
// are expanded by repeated multiplication ((x*x)*x, (x*x)*(x*x)); the real
// power x**2.0 folds to x*x and x**3.0 / x**4.0 call pow().
// ---------------------------------------------------------------------------
namespace {
inline real p2(real x) { return x * x; }
inline real p3(real x) { return (x * x) * x; }
inline real p4(real x) { real s = x * x; return s * s; }

void compute_f(const real t[3], real f[9]) {  // f[1..8]
  const real t1 = t[0], t2 = t[1], t3 = t[2];
  f[1] = t3;
  f[2] = 2.0 * t3 + p2(t3);
  f[3] = 3.0 * t3 + 3.0 * p2(t3) + p3(t3);
  f[4] = 4.0 * t3 + 6.0 * p2(t3) + 4.0 * p3(t3) + p4(t3);
  f[5] = 1.0 / (t1 * t2);
  f[6] = (2.0 * t1 + 1.0) / (p2(t1) * p2(t2));
  f[7] = (3.0 * p2(t1) + 3.0 * t1 + 1.0) / (p3(t1) * p3(t2));
  f[8] = (4.0 * p3(t1) + 6.0 * p2(t1) + 4.0 * t1 + 1.0) / (p4(t1) * p4(t2));
}

// s(5:10,1:7) stored as s[r][c] with r in 5..10, c in 1..7
struct S { real v[11][8]; };

S compute_s(real t2, const real f[9]) {
  S s{};
  auto& a = s.v;
  a[5][1] = -1.0 / p4(t2);
  a[5][2] = f[4];
  a[5][3] = f[4];
  a[5][4] = a[5][1];
  a[5][5] = -(f[1] / p4(t2) + f[4] / t2);
  a[5][6] = (f[4] / p2(t2) - f[2] / p4(t2));
  a[5][7] = -(f[3] / p4(t2) + f[4] / p3(t2));

  a[6][1] = -1.0;
  a[6][2] = f[8];
  a[6][3] = f[8];
  a[6][4] = -1.0;
  a[6][5] = (f[5] + f[8]);
  a[6][6] = (f[8] - f[6]);
  a[6][7] = (f[7] + f[8]);

  a[7][1] = -1.0;
  a[7][2] = (1.0 + f[4]);
  a[7][3] = f[4];
  a[7][4] = (f[4] - f[1]);
  a[7][5] = (f[4] - f[2]);
  a[7][6] = (f[4] - f[3]);

  const real r4 = pow(t2, 4.0), r2 = t2 * t2, r3 = pow(t2, 3.0);
  a[8][1] = -1.0 / r4;
  a[8][2] = (f[8] + (1.0 / r4));
  a[8][3] = f[8];
  a[8][4] = (f[5] / r4 - f[8] / t2);
  a[8][5] = (f[8] / r2 - f[6] / r4);
  a[8][6] = (f[7] / r4 - f[8] / r3);

  a[9][1] = -a[6][6] * a[5][1];
  a[9][2] = a[5][6] * a[6][1];
  a[9][3] = -(a[5][4] * a[6][6] + a[5][6] * a[6][2]);
  a[9][4] = (a[5][6] * a[6][4] + a[6][6] * a[5][2]);
  a[9][5] = (a[5][6] * a[6][3] - a[6][6] * a[5][3]);
  a[9][6] = (a[5][6] * a[6][5] - a[6][6] * a[5][5]);
  a[9][7] = (a[5][6] * a[6][7] - a[6][6] * a[5][7]);

  a[10][1] = -a[8][5] * a[7][1];
  a[10][2] = -a[8][5] * a[7][2];
  a[10][3] = a[7][5] * a[8][1];
  a[10][4] = a[7][5] * a[8][2];
  a[10][5] = (a[7][5] * a[8][3] - a[8][5] * a[7][3]);
  a[10][6] = (a[7][5] * a[8][4] - a[8][5] * a[7][4]);
  a[10][7] = (a[7][5] * a[8][6] - a[8][5] * a[7][6]);
  return s;
}

void compute_ak(const real t[3], real ak[8]) {
  const real t1 = t[0], t2 = t[1], t3 = t[2];
  ak[1] = (1.0 + 2.0 * t1) * (t3 + p2(t3)) * t2;
  ak[2] = (1.0 + t1) * (2.0 * t3 + p2(t3));
  ak[3] = (1.0 + t1);
  ak[4] = (1.0 + t1) * p2(1.0 + t3);
  ak[5] = p2(1.0 + t1) * (t3 + p2(t3)) * t2;
  ak[6] = p2(t1) * t2 * (t3 + p2(t3));
  ak[7] = (1.0 + t1) * (t3 + p2(t3)) * t2;
}

void fill_ca_ck(A2<real>& ca, A2<real>& ck, int64_t i, const real th[3]) {
  real f[9];
  compute_f(th, f);
  const S s = compute_s(th[1], f);
  const auto& a = s.v;
  ca(1, i) = a[9][7] * a[10][1] - a[10][7] * a[9][1];
  ca(2, i) = a[9][7] * a[10][2] + a[10][7] * a[9][3];
  ca(3, i) = a[9][5] * a[10][7] - a[10][5] * a[9][7];
  ca(4, i) = a[9][4] * a[10][7] + a[10][4] * a[9][7];
  ca(5, i) = a[9][7] * a[10][3] - a[10][7] * a[9][2];
  ca(6, i) = a[9][7] * a[10][6] - a[10][7] * a[9][6];
  real ak[8];
  compute_ak(th, ak);
  ck(1, i) = ak[3];
  ck(2, i) = -ak[4];
  ck(3, i) = ak[1] + ak[2];
  ck(4, i) = -ak[5];
  ck(5, i) = ak[6];
  ck(6, i) = ak[7];
}

void copy_col(A2<real>& dst, const A2<real>& src, int64_t i) {
  for (int64_t r = 1; r <= 6; ++r) dst(r, i) = src(r, i);
}
}  // namespace

void non_uni_coeff(Block& b) {
  const int64_t nx = b.nx, ny = b.ny, nz = b.nz;
  for (auto* a : {&b.ca_uu, &b.ck_uu, &b.ca_uv, &b.ck_uv, &b.ca_uw, &b.ck_uw}) a->alloc(6, nx + 2);
  for (auto* a : {&b.ca_vv, &b.ck_vv, &b.ca_vu, &b.ck_vu, &b.ca_vw, &b.ck_vw}) a->alloc(6, ny + 2);
  for (auto* a : {&b.ca_ww, &b.ck_ww, &b.ca_wu, &b.ck_wu, &b.ca_wv, &b.ck_wv}) a->alloc(6, nz + 2);

  // same-direction tables: theta = delta(i:i+2) / delta(i-1:i+1)
  auto same = [](F1& d, A2<real>& ca, A2<real>& ck, int64_t n) {
    for (int64_t i = 2; i <= n; ++i) {
      const real th[3] = {d(i) / d(i - 1), d(i + 1) / d(i), d(i + 2) / d(i + 1)};
      fill_ca_ck(ca, ck, i, th);
    }
  };
  same(b.deltax, b.ca_uu, b.ck_uu, nx);
  same(b.deltay, b.ca_vv, b.ck_vv, ny);
  same(b.deltaz, b.ca_ww, b.ck_ww, nz);

  // cross-direction tables on the staggered (mid-cell) spacing
  auto cross = [](F1& d, A2<real>& ca, A2<real>& ck, A2<real>& ca2, A2<real>& ck2,
                  int64_t n) {
    for (int64_t i = 2; i <= n; ++i) {
      real t1;
      if (i == 2)
        t1 = d(i - 1);
      else
        t1 = 0.5 * (d(i - 1) + d(i - 2));
      const real t2 = 0.5 * (d(i) + d(i - 1));
      const real t3 = 0.5 * (d(i) + d(i + 1));
      const real t4 = 0.5 * (d(i + 1) + d(i + 2));
      const real th[3] = {t2 / t1, t3 / t2, t4 / t3};
      fill_ca_ck(ca, ck, i, th);
      copy_col(ca2, ca, i);
      copy_col(ck2, ck, i);
    }
  };
  cross(b.deltax, b.ca_uv, b.ck_uv, b.ca_uw, b.ck_uw, nx);
  cross(b.deltay, b.ca_vu, b.ck_vu, b.ca_vw, b.ck_vw, ny);
  cross(b.deltaz, b.ca_wu, b.ck_wu, b.ca_wv, b.ck_wv, nz);
}

// src/CoefficientMatrix.f90:10-71
void coefficient_matrix(Block& b, bool is_coarse) {
  const int64_t nx = b.nx, ny = b.ny, nz = b.nz;
  for (int64_t j = 2; j <= ny + 1; ++j) {
    const real r1 = b.yp(j) - b.yp(j - 1), r2 = b.yp(j + 1) - b.yp(j), rs = r1 + r2;
    b.Acy(j - 1, 1) = 2.0 / (r1 * rs);
    b.Acy(j - 1, 2) = -2.0 / (r1 * r2);
    b.Acy(j - 1, 3) = 2.0 / (r2 * rs);
  }
  for (int64_t i = 2; i <= nx + 1; ++i) {
    const real r1 = b.xp(i) - b.xp(i - 1), r2 = b.xp(i + 1) - b.xp(i), rs = r1 + r2;
    b.Acx(i - 1, 1) = 2.0 / (r1 * rs);
    b.Acx(i - 1, 2) = -2.0 / (r1 * r2);
    b.Acx(i - 1, 3) = 2.0 / (r2 * rs);
  }
  for (int64_t i = 2; i <= nz + 1; ++i) {
    const real r1 = b.zp(i) - b.zp(i - 1), r2 = b.zp(i + 1) - b.zp(i), rs = r1 + r2;
    b.Acz(i - 1, 1) = 2.0 / (r1 * rs);
    b.Acz(i - 1, 2) = -2.0 / (r1 * r2);
    b.Acz(i - 1, 3) = 2.0 / (r2 * rs);
  }
  if (is_coarse) {
    b.Acx(1, 2) = b.Acx(1, 2) - b.Acx(1, 1);
    b.Acx(1, 1) = 0.0;
    b.Acx(nx, 2) = b.Acx(nx, 2) - b.Acx(nx, 3);
    b.Acx(nx, 3) = 0.0;
    b.Acy(1, 2) = b.Acy(1, 2) + b.Acy(1, 1);
    b.Acy(1, 1) = 0.0;
    b.Acy(ny, 2) = b.Acy(ny, 2) + b.Acy(ny, 3);
    b.Acy(ny, 3) = 0.0;
    b.Acz(1, 2) = b.Acz(1, 2) + b.Acz(1, 1);
    b.Acz(1, 1) = 0.0;
    b.Acz(nz, 2) = b.Acz(nz, 2) + b.Acz(nz, 3);
    b.Acz(nz, 3) = 0.0;
  }
}

// check_adjacent_cell, src/NavierStokes.f90:1002-1022
static bool check_adjacent(const I3& c, int64_t i, int64_t j, int64_t k, int64_t s) {
  if (c(i - s, j, k) == 2) return false;
  if (c(i + s, j, k) == 2) return false;
  if (c(i, j - s, k) == 2) return false;
  if (c(i, j + s, k) == 2) return false;
  if (c(i, j, k - s) == 2) return false;
  if (c(i, j, k + s) == 2) return false;
  return true;
}

// nsMomentum2order, src/NavierStokes.f90:252-912.  Serial loop over the
// fluid list in list order, including the in-place ghost substitution for
// cells next to a thin-surface (TS) cell and the restore with the t-ghosts
// of the last TS index.  Without TS cells (cell2 /= 2 everywhere) no cell
// writes u, v, w or p and each writes only its own ut, vt, wt, so the loop
// then runs in parallel (OpenMP) with the serial loop's results.
void ns_momentum_2order(Block& b, real deltat, real re) {
  const real alpha = 1.0;
  const int64_t nx_var = b.nx, ny_var = b.ny, nz_var = b.nz;
  F3 &u = b.u, &v = b.v, &w = b.w, &p = b.p;
  I3& c2 = b.cell2;
  const bool no_ts = b.TSCellCount == 0;
#pragma omp parallel for schedule(dynamic, 4096) if (no_ts)
  for (int64_t n = 1; n <= b.fluidCellCount; ++n) {
    const int64_t i = b.fluidIndexPtr(n, 1), j = b.fluidIndexPtr(n, 2), k = b.fluidIndexPtr(n, 3);
    int64_t index_ip1 = 0, index_im1 = 0, index_jp1 = 0, index_jm1 = 0, index_kp1 = 0,
            index_km1 = 0;
    if (c2(i + 1, j, k) == 2 || c2(i - 1, j, k) == 2 || c2(i, j + 1, k) == 2 ||
        c2(i, j - 1, k) == 2 || c2(i, j, k + 1) == 2 || c2(i, j, k - 1) == 2) {
      for (int64_t nn = 1; nn <= b.TSCellCount; ++nn) {
        const int64_t bt = b.index_ts(nn);
        auto dot = [&](int64_t idx, real px, real py, real pz) {
          return (px - b.xcent(idx)) * b.cosAlpha(idx) + (py - b.ycent(idx)) * b.cosBeta(idx) +
                 (pz - b.zcent(idx)) * b.cosGamma(idx);
        };
        const real u2 = dot(b.nelu2(bt), b.x1(i + 1), b.yp(j), b.zp(k));
        const real u1 = dot(b.nelu1(bt), b.x1(i), b.yp(j), b.zp(k));
        const real v2 = dot(b.nelv2(bt), b.xp(i), b.y1(j + 1), b.zp(k));
        const real v1 = dot(b.nelv1(bt), b.xp(i), b.y1(j), b.zp(k));
        const real w2 = dot(b.nelw2(bt), b.xp(i), b.yp(j), b.z1(k + 1));
        const real w1 = dot(b.nelw1(bt), b.xp(i), b.yp(j), b.z1(k));
        const real pd = dot(b.nelp(bt), b.xp(i), b.yp(j), b.zp(k));
        if (c2(i + 1, j, k) == 2) {
          index_ip1 = nn;
          if (u2 < 0) u(i + 1, j, k) = b.u2_ghost(nn);
          if (v2 < 0) v(i + 1, j, k) = b.v2_ghost(nn);
          if (v1 < 0) v(i + 1, j - 1, k) = b.v1_ghost(nn);
          if (w2 < 0) w(i + 1, j, k) = b.w2_ghost(nn);
          if (w1 < 0) w(i + 1, j, k - 1) = b.w1_ghost(nn);
          if (pd < 0) p(i + 1, j, k) = b.p_ghost(nn);
        }
        if (c2(i - 1, j, k) == 2) {
          index_im1 = nn;
          if (u1 < 0) u(i - 2, j, k) = b.u1_ghost(nn);
          if (v2 < 0) v(i - 1, j, k) = b.v2_ghost(nn);
          if (v1 < 0) v(i - 1, j - 1, k) = b.v1_ghost(nn);
          if (w2 < 0) w(i - 1, j, k) = b.w2_ghost(nn);
          if (w1 < 0) w(i - 1, j, k - 1) = b.w1_ghost(nn);
          if (pd < 0) p(i - 1, j, k) = b.p_ghost(nn);
        }
        if (c2(i, j + 1, k) == 2) {
          index_jp1 = nn;
          if (u2 < 0) u(i, j + 1, k) = b.u2_ghost(nn);
          if (u1 < 0) u(i - 1, j + 1, k) = b.u1_ghost(nn);
          if (v2 < 0) v(i, j + 1, k) = b.v2_ghost(nn);
          if (w2 < 0) w(i, j + 1, k) = b.w2_ghost(nn);
          if (w1 < 0) w(i, j + 1, k - 1) = b.w1_ghost(nn);
          if (pd < 0) p(i, j + 1, k) = b.p_ghost(nn);
        }
        if (c2(i, j - 1, k) == 2) {
          index_jm1 = nn;
          if (u2 < 0) u(i, j - 1, k) = b.u2_ghost(nn);
          if (u1 < 0) u(i - 1, j - 1, k) = b.u1_ghost(nn);
          if (v1 < 0) v(i, j - 2, k) = b.v1_ghost(nn);
          if (w2 < 0) w(i, j - 1, k) = b.w2_ghost(nn);
          if (w1 < 0) w(i, j - 1, k - 1) = b.w1_ghost(nn);
          if (pd < 0) p(i, j - 1, k) = b.p_ghost(nn);
        }
        if (c2(i, j, k + 1) == 2) {
          index_kp1 = nn;
          if (u2 < 0) u(i, j, k + 1) = b.u2_ghost(nn);
          if (u1 < 0) u(i - 1, j, k + 1) = b.u1_ghost(nn);
          if (v2 < 0) v(i, j, k + 1) = b.v2_ghost(nn);
          if (v1 < 0) v(i, j - 1, k + 1) = b.v1_ghost(nn);
          if (w2 < 0) w(i, j, k + 1) = b.w2_ghost(nn);
          if (pd < 0) p(i, j, k + 1) = b.p_ghost(nn);
        }
        if (c2(i, j, k - 1) == 2) {
          index_km1 = nn;
          if (u2 < 0) u(i, j, k - 1) = b.u2_ghost(nn);
          if (u1 < 0) u(i - 1, j, k - 1) = b.u1_ghost(nn);
          if (v2 < 0) v(i, j, k - 1) = b.v2_ghost(nn);
          if (v1 < 0) v(i, j - 1, k - 1) = b.v1_ghost(nn);
          if (w1 < 0) w(i, j, k - 2) = b.w1_ghost(nn);
          if (pd < 0) p(i, j, k - 1) = b.p_ghost(nn);
        }
      }
    }
    const real dxr = b.deltax(i + 1), dx = b.deltax(i), dxl = b.deltax(i - 1);
    const real dye = b.deltay(j + 1), dy = b.deltay(j), dyw = b.deltay(j - 1);
    const real dzt = b.deltaz(k + 1), dz = b.deltaz(k), dzb = b.deltaz(k - 1);

    const real u1a = u(i - 1, j, k) + u(i, j, k);
    const real u22 = u(i - 1, j, k) - u(i, j, k);
    const real u3 = u(i, j, k) + u(i + 1, j, k);
    const real u4 = u(i, j, k) - u(i + 1, j, k);
    const real u5 = u(i, j - 1, k) + u(i, j, k);
    const real u6 = u(i, j - 1, k) - u(i, j, k);
    const real u7 = u(i, j, k) + u(i, j + 1, k);
    const real u8 = u(i, j, k) - u(i, j + 1, k);
    const real u9 = u(i, j, k - 1) + u(i, j, k);
    const real u10 = u(i, j, k - 1) - u(i, j, k);
    const real u11 = u(i, j, k) + u(i, j, k + 1);
    const real u12 = u(i, j, k) - u(i, j, k + 1);
    const real u13 = u(i - 1, j, k) + u(i - 1, j + 1, k);
    const real u14 = u7;
    const real u15 = u(i - 1, j, k) + u(i - 1, j, k + 1);
    const real u16 = u11;

    const real v1a = v(i, j - 1, k) + v(i + 1, j - 1, k);
    const real v22 = v(i, j, k) + v(i + 1, j, k);
    const real v3 = v(i - 1, j, k) + v(i, j, k);
    const real v4 = v(i - 1, j, k) - v(i, j, k);
    const real v5 = v(i, j, k) + v(i + 1, j, k);
    const real v6 = v(i, j, k) - v(i + 1, j, k);
    const real v7 = v(i, j - 1, k) + v(i, j, k);
    const real v8 = v(i, j - 1, k) - v(i, j, k);
    const real v9 = v(i, j, k) + v(i, j + 1, k);
    const real v10 = v(i, j, k) - v(i, j + 1, k);
    const real v11 = v(i, j, k - 1) + v(i, j, k);
    const real v12 = v(i, j, k - 1) - v(i, j, k);
    const real v13 = v(i, j, k) + v(i, j, k + 1);
    const real v14 = v(i, j, k) - v(i, j, k + 1);
    const real v15 = v(i, j - 1, k) + v(i, j - 1, k + 1);
    const real v16 = v13;

    const real w1a = w(i, j, k - 1) + w(i + 1, j, k - 1);
    const real w22 = w(i, j, k) + w(i + 1, j, k);
    const real w3 = w(i, j, k - 1) + w(i, j + 1, k - 1);
    const real w4 = w(i, j, k) + w(i, j + 1, k);
    const real w5 = w(i - 1, j, k) + w(i, j, k);
    const real w6 = w(i - 1, j, k) - w(i, j, k);
    const real w7 = w(i, j, k) + w(i + 1, j, k);
    const real w8 = w(i, j, k) - w(i + 1, j, k);
    const real w9 = w(i, j - 1, k) + w(i, j, k);
    const real w10 = w(i, j - 1, k) - w(i, j, k);
    const real w11 = w(i, j, k) + w(i, j + 1, k);
    const real w12 = w(i, j, k) - w(i, j + 1, k);
    const real w13 = w(i, j, k - 1) + w(i, j, k);
    const real w14 = w(i, j, k - 1) - w(i, j, k);
    const real w15 = w(i, j, k) + w(i, j, k + 1);
    const real w16 = w(i, j, k) - w(i, j, k + 1);

    const real dpdx = (p(i, j, k) - p(i + 1, j, k)) / (0.5 * (dxr + dx));
    const real dpdy = (p(i, j, k) - p(i, j + 1, k)) / (0.5 * (dye + dy));
    const real dpdz = (p(i, j, k) - p(i, j, k + 1)) / (0.5 * (dzt + dz));

    const real dx2xr = dx + dxr, dx2xl = dx + dxl, dy2ye = dy + dye, dy2yw = dy + dyw,
                 dz2zt = dz + dzt, dz2zb = dz + dzb;

    // ---------------- U momentum ----------------
    const real vu_e = v(i + 1, j, k) + (dxr / (dx2xr)) * (v(i, j, k) - v(i + 1, j, k));
    const real vu_w =
        v(i + 1, j - 1, k) + (dxr / (dx2xr)) * (v(i, j - 1, k) - v(i + 1, j - 1, k));
    const real v_in_um = 0.5 * (vu_e + vu_w);
    const real wu_n = w(i + 1, j, k) + (dxr / (dx2xr)) * (w(i, j, k) - w(i + 1, j, k));
    const real wu_s =
        w(i + 1, j, k - 1) + (dxr / (dx2xr)) * (w(i, j, k - 1) - w(i + 1, j, k - 1));
    const real w_in_um = 0.5 * (wu_n + wu_s);

    real duudx, dvudy, dwudz;
    bool third = false;
    if (i > 2 && i < nx_var && j > 2 && j < ny_var + 1 && k > 2 && k < nz_var + 1)
      if (check_adjacent(b.cell, i, j, k, 1))
        if (check_adjacent(b.cell2, i, j, k, 2)) third = true;
    if (third) {
      const real ddy = 0.5 * (b.deltay(j) + b.deltay(j - 1));
      const real ddye = 0.5 * (b.deltay(j) + b.deltay(j + 1));
      const real ddz = 0.5 * (b.deltaz(k) + b.deltaz(k - 1));
      const real ddzr = 0.5 * (b.deltaz(k) + b.deltaz(k + 1));
      auto& ca = b.ca_uu;
      auto& ck = b.ck_uu;
      duudx = u(i, j, k) *
                  (ca(1, i) * u(i + 2, j, k) + ca(2, i) * u(i + 1, j, k) +
                   ca(3, i) * u(i, j, k) + ca(4, i) * u(i - 1, j, k) + ca(5, i) * u(i - 2, j, k)) /
                  (ca(6, i) * b.deltax(i + 1)) +
              fabs(u(i, j, k)) *
                  (ck(1, i) * u(i + 2, j, k) + ck(2, i) * u(i + 1, j, k) +
                   ck(3, i) * u(i, j, k) + ck(4, i) * u(i - 1, j, k) + ck(5, i) * u(i - 2, j, k)) /
                  (2.0 * ck(6, i) * b.deltax(i));
      auto& cav = b.ca_vu;
      auto& ckv = b.ck_vu;
      dvudy = v_in_um *
                  (cav(1, j) * u(i, j + 2, k) + cav(2, j) * u(i, j + 1, k) +
                   cav(3, j) * u(i, j, k) + cav(4, j) * u(i, j - 1, k) + cav(5, j) * u(i, j - 2, k)) /
                  (cav(6, j) * ddye) +
              fabs(v_in_um) *
                  (ckv(1, j) * u(i, j + 2, k) + ckv(2, j) * u(i, j + 1, k) +
                   ckv(3, j) * u(i, j, k) + ckv(4, j) * u(i, j - 1, k) + ckv(5, j) * u(i, j - 2, k)) /
                  (2.0 * ckv(6, j) * ddy);
      auto& caw = b.ca_wu;
      auto& ckw = b.ck_wu;
      dwudz = w_in_um *
                  (caw(1, k) * u(i, j, k + 2) + caw(2, k) * u(i, j, k + 1) +
                   caw(3, k) * u(i, j, k) + caw(4, k) * u(i, j, k - 1) + caw(5, k) * u(i, j, k - 2)) /
                  (caw(6, k) * ddzr) +
              fabs(w_in_um) *
                  (ckw(1, k) * u(i, j, k + 2) + ckw(2, k) * u(i, j, k + 1) +
                   ckw(3, k) * u(i, j, k) + ckw(4, k) * u(i, j, k - 1) + ckw(5, k) * u(i, j, k - 2)) /
                  (2.0 * ckw(6, k) * ddz);
    } else {
      duudx = -0.25 * (u1a * u1a + alpha * fabs(u1a) * u22 - u3 * u3 -
                       alpha * fabs(u3) * u4) /
              b.deltax(i);
      dvudy = -0.25 * (v1a * u5 + alpha * fabs(v1a) * u6 - v22 * u7 -
                       alpha * fabs(v22) * u8) /
              b.deltay(j);
      dwudz = -0.25 * (w1a * u9 + alpha * fabs(w1a) * u10 - w22 * u11 -
                       alpha * fabs(w22) * u12) /
              b.deltaz(k);
    }
    const real d2udx2 = (2.0 / dx2xr) * ((-u4 / dxr) + (u22 / dx));
    const real d2udy2 =
        (2.0 / (0.5 * (dy2ye + dy2yw))) * ((-u8 / (0.5 * dy2ye)) + (u6 / (0.5 * dy2yw)));
    const real d2udz2 =
        (2.0 / (0.5 * (dz2zt + dz2zb))) * ((-u12 / (0.5 * dz2zt)) + (u10 / (0.5 * dz2zb)));
    const real xtt2 = (d2udx2 + d2udy2 + d2udz2) / re;
    const real residu = (-duudx - dvudy - dwudz + xtt2);
    b.ut(i, j, k) = u(i, j, k) + deltat * (residu + dpdx);

    // ---------------- V momentum ----------------
    const real uv_e = u(i, j + 1, k) + (dye / (dy2ye)) * (u(i, j, k) - u(i, j + 1, k));
    const real uv_w =
        u(i - 1, j + 1, k) + (dye / (dy2ye)) * (u(i - 1, j, k) - u(i - 1, j + 1, k));
    const real u_in_vm = 0.5 * (uv_e + uv_w);
    const real wv_n = w(i, j + 1, k) + (dye / (dy2ye)) * (w(i, j, k) - w(i, j + 1, k));
    const real wv_s =
        w(i, j + 1, k - 1) + (dye / (dy2ye)) * (w(i, j, k - 1) - w(i, j + 1, k - 1));
    const real w_in_vm = 0.5 * (wv_n + wv_s);
    real duvdx, dvvdy, dwvdz;
    third = false;
    if (i > 2 && i < nx_var + 1 && j > 2 && j < ny_var && k > 2 && k < nz_var + 1)
      if (check_adjacent(b.cell, i, j, k, 1))
        if (check_adjacent(b.cell2, i, j, k, 2)) third = true;
    if (third) {
      const real ddx = 0.5 * (b.deltax(i) + b.deltax(i - 1));
      const real ddxr = 0.5 * (b.deltax(i) + b.deltax(i + 1));
      const real ddz = 0.5 * (b.deltaz(k) + b.deltaz(k - 1));
      const real ddzr = 0.5 * (b.deltaz(k) + b.deltaz(k + 1));
      auto& ca = b.ca_uw;
      auto& ck = b.ck_uw;
      duvdx = u_in_vm *
                  (ca(1, i) * v(i + 2, j, k) + ca(2, i) * v(i + 1, j, k) +
                   ca(3, i) * v(i, j, k) + ca(4, i) * v(i - 1, j, k) + ca(5, i) * v(i - 2, j, k)) /
                  (ca(6, i) * ddxr) +
              fabs(u_in_vm) *
                  (ck(1, i) * v(i + 2, j, k) + ck(2, i) * v(i + 1, j, k) +
                   ck(3, i) * v(i, j, k) + ck(4, i) * v(i - 1, j, k) + ck(5, i) * v(i - 2, j, k)) /
                  (2.0 * ck(6, i) * ddx);
      auto& cv = b.ca_vv;
      auto& kv = b.ck_vv;
      dvvdy = v(i, j, k) *
                  (cv(1, j) * v(i, j + 2, k) + cv(2, j) * v(i, j + 1, k) +
                   cv(3, j) * v(i, j, k) + cv(4, j) * v(i, j - 1, k) + cv(5, j) * v(i, j - 2, k)) /
                  (cv(6, j) * b.deltay(j + 1)) +
              fabs(v(i, j, k)) *
                  (kv(1, j) * v(i, j + 2, k) + kv(2, j) * v(i, j + 1, k) +
                   kv(3, j) * v(i, j, k) + kv(4, j) * v(i, j - 1, k) + kv(5, j) * v(i, j - 2, k)) /
                  (2.0 * kv(6, j) * b.deltay(j));
      auto& cw = b.ca_wu;
      auto& kw = b.ck_wu;
      dwvdz = w_in_vm *
                  (cw(1, k) * v(i, j, k + 2) + cw(2, k) * v(i, j, k + 1) +
                   cw(3, k) * v(i, j, k) + cw(4, k) * v(i, j, k - 1) + cw(5, k) * v(i, j, k - 2)) /
                  (cw(6, k) * ddzr) +
              fabs(w_in_vm) *
                  (kw(1, k) * v(i, j, k + 2) + kw(2, k) * v(i, j, k + 1) +
                   kw(3, k) * v(i, j, k) + kw(4, k) * v(i, j, k - 1) + kw(5, k) * v(i, j, k - 2)) /
                  (2.0 * kw(6, k) * ddz);
    } else {
      duvdx = -0.25 * (u13 * v3 + alpha * fabs(u13) * v4 - u14 * v5 -
                       alpha * fabs(u14) * v6) /
              b.deltax(i);
      dvvdy = -0.25 * (v7 * v7 + alpha * fabs(v7) * v8 - v9 * v9 -
                       alpha * fabs(v9) * v10) /
              b.deltay(j);
      dwvdz = -0.25 * (w3 * v11 + alpha * fabs(w3) * v12 - w4 * v13 -
                       alpha * fabs(w4) * v14) /
              b.deltaz(k);
    }
    const real d2vdx2 =
        (2.0 / (0.5 * (dx2xr + dx2xl))) * ((-v6 / (0.5 * dx2xr)) + (v4 / (0.5 * dx2xl)));
    const real d2vdy2 = (2.0 / dy2ye) * ((-v10 / dye) + (v8 / dy));
    const real d2vdz2 =
        (2.0 / (0.5 * (dz2zt + dz2zb))) * ((-v14 / (0.5 * dz2zt)) + (v12 / (0.5 * dz2zb)));
    const real ytt2 = (d2vdx2 + d2vdy2 + d2vdz2) / re;
    const real residv = (-duvdx - dvvdy - dwvdz + ytt2);
    b.vt(i, j, k) = v(i, j, k) + deltat * (residv + dpdy);

    // ---------------- W momentum ----------------
    const real uw_e = u(i, j, k + 1) + (dzt / (dz2zt)) * (u(i, j, k) - u(i, j, k + 1));
    const real uw_w =
        u(i - 1, j, k + 1) + (dzt / (dz2zt)) * (u(i - 1, j, k) - u(i - 1, j, k + 1));
    const real u_in_wm = 0.5 * (uw_e + uw_w);
    const real vw_n = v(i, j, k + 1) + (dzt / (dz2zt)) * (v(i, j, k) - v(i, j, k + 1));
    const real vw_s =
        v(i, j - 1, k + 1) + (dzt / (dz2zt)) * (v(i, j - 1, k) - v(i, j - 1, k + 1));
    const real v_in_wm = 0.5 * (vw_n + vw_s);
    real duwdx, dvwdy, dwwdz;
    third = false;
    if (i > 2 && i < nx_var + 1 && j > 2 && j < ny_var + 1 && k > 2 && k < nz_var)
      if (check_adjacent(b.cell, i, j, k, 1))
        if (check_adjacent(b.cell2, i, j, k, 2)) third = true;
    if (third) {
      const real ddx = 0.5 * (b.deltax(i) + b.deltax(i - 1));
      const real ddxr = 0.5 * (b.deltax(i) + b.deltax(i + 1));
      const real ddy = 0.5 * (b.deltay(j) + b.deltay(j - 1));
      const real ddye = 0.5 * (b.deltay(j) + b.deltay(j + 1));
      auto& ca = b.ca_uw;
      auto& ck = b.ck_uw;
      duwdx = u_in_wm *
                  (ca(1, i) * w(i + 2, j, k) + ca(2, i) * w(i + 1, j, k) +
                   ca(3, i) * w(i, j, k) + ca(4, i) * w(i - 1, j, k) + ca(5, i) * w(i - 2, j, k)) /
                  (ca(6, i) * ddxr) +
              fabs(u_in_wm) *
                  (ck(1, i) * w(i + 2, j, k) + ck(2, i) * w(i + 1, j, k) +
                   ck(3, i) * w(i, j, k) + ck(4, i) * w(i - 1, j, k) + ck(5, i) * w(i - 2, j, k)) /
                  (2.0 * ck(6, i) * ddx);
      auto& cv = b.ca_vw;
      auto& kv = b.ck_vw;
      dvwdy = v_in_wm *
                  (cv(1, j) * w(i, j + 2, k) + cv(2, j) * w(i, j + 1, k) +
                   cv(3, j) * w(i, j, k) + cv(4, j) * w(i, j - 1, k) + cv(5, j) * w(i, j - 2, k)) /
                  (cv(6, j) * ddye) +
              fabs(v_in_wm) *
                  (kv(1, j) * w(i, j + 2, k) + kv(2, j) * w(i, j + 1, k) +
                   kv(3, j) * w(i, j, k) + kv(4, j) * w(i, j - 1, k) + kv(5, j) * w(i, j - 2, k)) /
                  (2.0 * kv(6, j) * ddy);
      auto& cw = b.ca_ww;
      auto& kw = b.ck_ww;
      dwwdz = w(i, j, k) *
                  (cw(1, k) * w(i, j, k + 2) + cw(2, k) * w(i, j, k + 1) +
                   cw(3, k) * w(i, j, k) + cw(4, k) * w(i, j, k - 1) + cw(5, k) * w(i, j, k - 2)) /
                  (cw(6, k) * b.deltaz(k + 1)) +
              fabs(w(i, j, k)) *
                  (kw(1, k) * w(i, j, k + 2) + kw(2, k) * w(i, j, k + 1) +
                   kw(3, k) * w(i, j, k) + kw(4, k) * w(i, j, k - 1) + kw(5, k) * w(i, j, k - 2)) /
                  (2.0 * kw(6, k) * b.deltaz(k));
    } else {
      duwdx = -0.5 * (u15 * w5 + alpha * fabs(u15) * w6 - u16 * w7 -
                      alpha * fabs(u16) * w8) /
              b.deltax(i);
      dvwdy = -0.5 * (v15 * w9 + alpha * fabs(v15) * w10 - v16 * w11 -
                      alpha * fabs(v16) * w12) /
              b.deltay(j);
      dwwdz = -0.5 * (w13 * w13 + alpha * fabs(w13) * w14 - w15 * w15 -
                      alpha * fabs(w15) * w16) /
              b.deltaz(k);
    }
    const real d2wdx2 =
        (2.0 / (0.5 * (dx2xr + dx2xl))) * ((-w8 / (0.5 * dx2xr)) + (w6 / (0.5 * dx2xl)));
    const real d2wdy2 =
        (2.0 / (0.5 * (dy2ye + dy2yw))) * ((-w12 / (0.5 * dy2ye)) + (w10 / (0.5 * dy2yw)));
    const real d2wdz2 = (2.0 / dz2zt) * ((-w16 / dzt) + (w14 / dz));
    const real ztt2 = (d2wdx2 + d2wdy2 + d2wdz2) / re;
    const real residw = (-duwdx - dvwdy - dwwdz + ztt2);
    b.wt(i, j, k) = w(i, j, k) + deltat * (residw + dpdz);

    // restore with the t-ghosts of the last TS index (src/NavierStokes.f90:860-907)
    if (c2(i + 1, j, k) == 2) {
      u(i + 1, j, k) = b.u2t_ghost(index_ip1);
      v(i + 1, j, k) = b.v2t_ghost(index_ip1);
      v(i + 1, j - 1, k) = b.v1t_ghost(index_ip1);
      w(i + 1, j, k) = b.w2t_ghost(index_ip1);
      w(i + 1, j, k - 1) = b.w1t_ghost(index_ip1);
      p(i + 1, j, k) = b.pt_ghost(index_ip1);
    }
    if (c2(i - 1, j, k) == 2) {
      u(i - 2, j, k) = b.u1t_ghost(index_im1);
      v(i - 1, j, k) = b.v2t_ghost(index_im1);
      v(i - 1, j - 1, k) = b.v1t_ghost(index_im1);
      w(i - 1, j, k) = b.w2t_ghost(index_im1);
      w(i - 1, j, k - 1) = b.w1t_ghost(index_im1);
      p(i - 1, j, k) = b.pt_ghost(index_im1);
    }
    if (c2(i, j + 1, k) == 2) {
      u(i, j + 1, k) = b.u2t_ghost(index_jp1);
      u(i - 1, j + 1, k) = b.u1t_ghost(index_jp1);
      v(i, j + 1, k) = b.v2t_ghost(index_jp1);
      w(i, j + 1, k) = b.w2t_ghost(index_jp1);
      w(i, j + 1, k - 1) = b.w1t_ghost(index_jp1);
      p(i, j + 1, k) = b.pt_ghost(index_jp1);
    }
    if (c2(i, j - 1, k) == 2) {
      u(i, j - 1, k) = b.u2t_ghost(index_jm1);
      u(i - 1, j - 1, k) = b.u1t_ghost(index_jm1);
      v(i, j - 2, k) = b.v1t_ghost(index_jm1);
      w(i, j - 1, k) = b.w2t_ghost(index_jm1);
      w(i, j - 1, k - 1) = b.w1t_ghost(index_jm1);
      p(i, j - 1, k) = b.pt_ghost(index_jm1);
    }
    if (c2(i, j, k + 1) == 2) {
      u(i, j, k + 1) = b.u2t_ghost(index_kp1);
      u(i - 1, j, k + 1) = b.u1t_ghost(index_kp1);
      v(i, j, k + 1) = b.v2t_ghost(index_kp1);
      v(i, j - 1, k + 1) = b.v1t_ghost(index_kp1);
      w(i, j, k + 1) = b.w2t_ghost(index_kp1);
      p(i, j, k + 1) = b.pt_ghost(index_kp1);
    }
    if (c2(i, j, k - 1) == 2) {
      u(i, j, k - 1) = b.u2t_ghost(index_km1);
      u(i - 1, j, k - 1) = b.u1t_ghost(index_km1);
      v(i, j, k - 1) = b.v2t_ghost(index_km1);
      v(i, j - 1, k - 1) = b.v1t_ghost(index_km1);
      w(i, j, k - 2) = b.w1t_ghost(index_km1);
      p(i, j, k - 1) = b.pt_ghost(index_km1);
    }
  }
}

// velocityBC, src/BoundaryConditions.f90:11-74 (three loops in order)
void velocity_bc(Block& b, real deltat, real uc) {
  const int64_t nx = b.nx, ny = b.ny, nz = b.nz;
  for (int64_t k = 2; k <= nz + 1; ++k)
    for (int64_t j = 2; j <= ny + 1; ++j) {
      b.ut(1, j, k) = uc;
      b.vt(1, j, k) = -b.vt(nx + 1, j, k);
      b.wt(1, j, k) = -b.wt(nx + 1, j, k);
      b.ut(nx + 1, j, k) =
          b.u(nx + 1, j, k) - (deltat / b.deltax(nx + 1)) * uc * (b.u(nx + 1, j, k) - b.u(nx, j, k));
      b.vt(nx + 2, j, k) = -b.vt(nx + 1, j, k) + b.v(nx + 2, j, k) + b.v(nx + 1, j, k) -
                           (2.0 * deltat / b.deltax(nx + 2)) * uc *
                               (b.v(nx + 2, j, k) - b.v(nx + 1, j, k));
      b.wt(nx + 2, j, k) = -b.wt(nx + 1, j, k) + b.w(nx + 2, j, k) + b.w(nx + 1, j, k) -
                           (2.0 * deltat / b.deltax(nx + 2)) * uc *
                               (b.w(nx + 2, j, k) - b.w(nx + 1, j, k));
    }
  for (int64_t k = 2; k <= nz + 1; ++k)
    for (int64_t i = 2; i <= nx + 1; ++i) {
      b.ut(i, 1, k) = b.ut(i, 2, k);
      b.wt(i, 1, k) = b.wt(i, 2, k);
      b.vt(i, 2, k) = 0.0;
      b.ut(i, ny + 2, k) = b.ut(i, ny + 1, k);
      b.wt(i, ny + 2, k) = b.wt(i, ny + 1, k);
      b.vt(i, ny + 1, k) = 0.0;
    }
  for (int64_t j = 2; j <= ny + 1; ++j)
    for (int64_t i = 2; i <= nx + 1; ++i) {
      b.ut(i, j, 1) = b.ut(i, j, 2);
      b.vt(i, j, 1) = b.vt(i, j, 2);
      b.wt(i, j, 1) = 0.0;
      b.ut(i, j, nz + 2) = b.ut(i, j, nz + 1);
      b.vt(i, j, nz + 2) = b.vt(i, j, nz + 1);
      b.wt(i, j, nz + 1) = 0.0;
    }
}

// solidCellBC, src/BoundaryConditions.f90:76-92
void solid_cell_bc(Block& b) {
  for (int64_t n = 1; n <= b.solidCellCount; ++n) {
    const int64_t i = b.solidIndexPtr(n, 1), j = b.solidIndexPtr(n, 2), k = b.solidIndexPtr(n, 3);
    b.ut(i, j, k) = 0.0;
    b.vt(i, j, k) = 0.0;
    b.wt(i, j, k) = 0.0;
    b.p(i, j, k) = 0.0;
  }
}

// solidCellBC_move, src/BoundaryConditions.f90:94-115
void solid_cell_bc_move(Block& b) {
  if (b.move_check != 1) return;
  for (int64_t n = 1; n <= b.solidCellCount; ++n) {
    const int64_t i = b.solidIndexPtr(n, 1), j = b.solidIndexPtr(n, 2), k = b.solidIndexPtr(n, 3);
    b.ut(i, j, k) = 0.0;
    b.vt(i, j, k) = 0.0;
    b.wt(i, j, k) = 0.0;
    b.p(i, j, k) = 0.0;
    b.u(i, j, k) = 0.0;
    b.v(i, j, k) = 0.0;
    b.w(i, j, k) = 0.0;
  }
}

}  // namespace orc
