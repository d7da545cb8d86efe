// Drag / lift integration over the IB elements (stress_calculation,
// src/StressCalc.f90:14-208), FP64.  Each element's viscous and pressure force
// contributions are computed independently, then summed by one CTA in a fixed
// tree order, so the result is deterministic run to run (the reference's
// OpenACC reduction order is unspecified; its serial build sums in element
// order).
#include <cstdio>

#include "bcfd_host.h"
#include "bcfd_dual.cuh"

namespace bcfd {

namespace {

// first i in [s, f] with a(i) <= v < a(i+1); on the non-decreasing grid
// coordinates the bracket is unique, so a binary search finds the scan's i
__device__ int fidx(const DevBlock& B, double v, const double* a, int len, int s, int f) {
  const int lo = max(s, 1), hi = min(f, len - 1);
  if (lo <= hi && v >= a[lo - 1]) {
    int L = lo, H = hi;
    while (L < H) {
      const int m = (L + H + 1) >> 1;
      if (a[m - 1] <= v) L = m;
      else H = m - 1;
    }
    if (v < a[L]) return L;
  }
  set_err(B.err, BCFD_E_NOTFOUND);
  return max(1, min(s, len - 1));
}

__device__ __forceinline__ double bil(double x, double y, double x1, double x2, double y1, double y2,
                                      double f0, double f1, double f2, double f3) {
  const double numer = f0 * (x2 - x) * (y2 - y) + f2 * (x2 - x) * (y - y1) +
                       f1 * (x - x1) * (y2 - y) + f3 * (x - x1) * (y - y1);
  return numer / ((x2 - x1) * (y2 - y1));
}

__device__ __forceinline__ double der(double x, double x2, double x1, double p_x, double p_x2,
                                      double p_x1) {
  const double h2 = fabs(x2 - x), h1 = fabs(x1 - x);
  return (h1 * h1 * p_x2 - h2 * h2 * p_x1 + (h2 * h2 - h1 * h1) * p_x) / (h1 * h2 * (h1 + h2) + 1e-16);
}

// compute_value_and_derivatives with the find_index ranges 2..n+1 of
// StressCalc, split into the bracket search (the 8 stencil points) and the
// evaluation on the 8 values
__device__ void vad_find(const DevBlock& B, double x, double y, double z, const double* xg, int nxg,
                         const double* yg, int nyg, const double* zg, int nzg, int off, int ijk[3],
                         int64_t pos[8]) {
  const Dims& d = B.d;
  const int i = fidx(B, x, xg, nxg, 2, d.nx + 1), j = fidx(B, y, yg, nyg, 2, d.ny + 1),
            k = fidx(B, z, zg, nzg, 2, d.nz + 1);
  const int ii = i - (off == 1), jj = j - (off == 2), kk = k - (off == 3);
#pragma unroll
  for (int q = 0; q < 8; ++q) pos[q] = d.idx(ii + (q & 1), jj + ((q >> 1) & 1), kk + (q >> 2));
  ijk[0] = i;
  ijk[1] = j;
  ijk[2] = k;
}

__device__ void vad_eval(double x, double y, double z, const double* xg, const double* yg, const double* zg,
                         const int ijk[3], const double f[8], double& val, double d3[3]) {
  const int i = ijk[0], j = ijk[1], k = ijk[2];
  const double yj = yg[j - 1], yj1 = yg[j], zk = zg[k - 1], zk1 = zg[k], xi = xg[i - 1], xi1 = xg[i];
  const double t11 = bil(y, z, yj, yj1, zk, zk1, f[0], f[2], f[4], f[6]);
  const double t12 = bil(y, z, yj, yj1, zk, zk1, f[1], f[3], f[5], f[7]);
  const double t21 = bil(x, z, xi, xi1, zk, zk1, f[0], f[1], f[4], f[5]);
  const double t22 = bil(x, z, xi, xi1, zk, zk1, f[2], f[3], f[6], f[7]);
  const double t31 = bil(x, y, xi, xi1, yj, yj1, f[0], f[1], f[2], f[3]);
  const double t32 = bil(x, y, xi, xi1, yj, yj1, f[4], f[5], f[6], f[7]);
  val = t11 + (x - xi) * (t12 - t11) / (xi1 - xi);
  d3[0] = der(x, xi1, xi, val, t12, t11);
  d3[1] = der(y, yj1, yj, val, t22, t21);
  d3[2] = der(z, zk1, zk, val, t32, t31);
}

// probe point and stencils of one element (fields u, v, w, p)
struct ElemStencil {
  double px, py, pz, diag;
  int ijk[4][3];
  int64_t pos[4][8];
};

__device__ ElemStencil elem_stencil(const DevBlock& B, int e) {
  const Dims& d = B.d;
  ElemStencil S;
  const int ic = fidx(B, B.xcent[e], B.x1, d.NX + 1, 2, d.nx + 1);
  const int jc = fidx(B, B.ycent[e], B.y1, d.NY + 1, 2, d.ny + 1);
  const int kc = fidx(B, B.zcent[e], B.z1, d.NZ + 1, 2, d.nz + 1);
  const double dX = B.x1[ic] - B.x1[ic - 1], dY = B.y1[jc] - B.y1[jc - 1], dZ = B.z1[kc] - B.z1[kc - 1];
  S.diag = sqrt(dX * dX + dY * dY + dZ * dZ);
  const double nd = S.diag;
  S.px = B.xcent[e] + nd * B.cosA[e];
  S.py = B.ycent[e] + nd * B.cosB[e];
  S.pz = B.zcent[e] + nd * B.cosG[e];
  vad_find(B, S.px, S.py, S.pz, B.xu, d.NX + 1, B.yu, d.NY, B.zu, d.NZ, 1, S.ijk[0], S.pos[0]);
  vad_find(B, S.px, S.py, S.pz, B.xv, d.NX, B.yv, d.NY + 1, B.zv, d.NZ, 2, S.ijk[1], S.pos[1]);
  vad_find(B, S.px, S.py, S.pz, B.xw, d.NX, B.yw, d.NY, B.zw, d.NZ + 1, 3, S.ijk[2], S.pos[2]);
  vad_find(B, S.px, S.py, S.pz, B.xp, d.NX, B.yp, d.NY, B.zp, d.NZ, 0, S.ijk[3], S.pos[3]);
  return S;
}

// per element: [viscous drag, pressure drag, viscous lift, pressure lift, area, a_xz, a_yz]
// from the element's 4 x 8 stencil values f (u, v, w, p)
__device__ void elem_terms(const DevBlock& B, int e, double mu_f, double rho_f, const ElemStencil& S,
                           const double f[4][8], double o[7]) {
  const double nrm[3] = {B.cosA[e], B.cosB[e], B.cosG[e]};
  const double nd = S.diag, diag = S.diag;
  const double px = S.px, py = S.py, pz = S.pz;
  const int sid = B.surf_id[e];
  const double td = sid == 51 ? B.kin->thetaDot1 : (sid == 52 ? B.kin->thetaDot2 : 0.0);
  const double tdd = sid == 51 ? B.kin->thetaDDot1 : (sid == 52 ? B.kin->thetaDDot2 : 0.0);
  const double us = B.kin->xdot;
  const double vs = -td * (B.zcent[e] - B.kin->piv_z) + B.kin->ydot;
  const double ws = td * (B.ycent[e] - B.kin->piv_y);
  const double ac_z = -(td * td) * (B.zcent[e] - B.kin->piv_z);
  const double ac_y = -(td * td) * (B.ycent[e] - B.kin->piv_y);
  const double at_z = tdd * (B.ycent[e] - B.kin->piv_y);
  const double at_y = -tdd * (B.zcent[e] - B.kin->piv_z);
  const double dpdn = -((ac_z + at_z) * B.cosG[e] + (ac_y + at_y) * B.cosB[e]) - B.kin->yddot * B.cosB[e];
  double val, g[3], ddn[3];
  vad_eval(px, py, pz, B.xu, B.yu, B.zu, S.ijk[0], f[0], val, g);
  ddn[0] = (2.0 / nd) * (val - us) - (g[0] * nrm[0] + g[1] * nrm[1] + g[2] * nrm[2]);
  vad_eval(px, py, pz, B.xv, B.yv, B.zv, S.ijk[1], f[1], val, g);
  ddn[1] = (2.0 / nd) * (val - vs) - (g[0] * nrm[0] + g[1] * nrm[1] + g[2] * nrm[2]);
  vad_eval(px, py, pz, B.xw, B.yw, B.zw, S.ijk[2], f[2], val, g);
  ddn[2] = (2.0 / nd) * (val - ws) - (g[0] * nrm[0] + g[1] * nrm[1] + g[2] * nrm[2]);
  const double alen = B.elen[e];
  const double area = alen / 2.0;
  const double a_yz = 0.5 * fabs(alen * nrm[0]);
  const double a_xz = 0.5 * fabs(alen * nrm[1]);
  const double dd = ddn[0] * nrm[0] + ddn[1] * nrm[1] + ddn[2] * nrm[2];
  const double sh0 = (ddn[0] - dd * nrm[0]) * mu_f * area;
  const double sh1 = (ddn[1] - dd * nrm[1]) * mu_f * area;
  vad_eval(px, py, pz, B.xp, B.yp, B.zp, S.ijk[3], f[3], val, g);
  const double dpdn_e = g[0] * nrm[0] + g[1] * nrm[1] + g[2] * nrm[2];
  const double cval = val - (dpdn_e + dpdn) * diag * 0.5;
  o[0] = sh0;
  o[1] = -cval * area * nrm[0] * rho_f;
  o[2] = sh1;
  o[3] = -cval * area * nrm[1] * rho_f;
  o[4] = area;
  o[5] = a_xz;
  o[6] = a_yz;
}

__global__ void k_stress_elem(DevBlock B, double mu_f, double rho_f, double* part) {
  const double* arr[4] = {B.u, B.v, B.w, B.p};
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < B.ne; e += gridDim.x * blockDim.x) {
    const ElemStencil S = elem_stencil(B, e);
    double f[4][8];
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int q = 0; q < 8; ++q) f[c][q] = arr[c][S.pos[c][q]];
    elem_terms(B, e, mu_f, rho_f, S, f, part + 7 * (int64_t)e);
  }
}

// Weights of a fixed linear combination of the 4 coefficients as a function
// of (u, v, w, p): the element terms are affine in the 32 stencil values, so
// the partial of term q in value c is term(e_c) - term(0).  coef[e][32] and
// pos[e][32] per element; the accumulation is done in element order.
__global__ void k_stress_coef(DevBlock B, double mu_f, double rho_f, const double* scale, double* coef,
                              int64_t* pos) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < B.ne; e += gridDim.x * blockDim.x) {
    const ElemStencil S = elem_stencil(B, e);
    double f[4][8];
    for (int c = 0; c < 4; ++c)
      for (int q = 0; q < 8; ++q) f[c][q] = 0.0;
    double o0[7], o1[7];
    elem_terms(B, e, mu_f, rho_f, S, f, o0);
    for (int c = 0; c < 4; ++c)
      for (int q = 0; q < 8; ++q) {
        f[c][q] = 1.0;
        elem_terms(B, e, mu_f, rho_f, S, f, o1);
        f[c][q] = 0.0;
        double w = 0.0;
        for (int t = 0; t < 4; ++t) w += scale[t] * (o1[t] - o0[t]);
        coef[32 * (int64_t)e + 8 * c + q] = w;
        pos[32 * (int64_t)e + 8 * c + q] = S.pos[c][q];
      }
  }
}

// part[11e + p] = d/d(kinematic scalar p) of sum_t scale[t] * term_t(e) at the
// current fields (the terms are affine in the fields and at most quadratic in
// each scalar, so the central difference with unit steps is exact)
__global__ void k_stress_kin_elem(DevBlock B, double mu_f, double rho_f, const double* scale, double* part) {
  const double* arr[4] = {B.u, B.v, B.w, B.p};
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < B.ne; e += gridDim.x * blockDim.x) {
    const ElemStencil S = elem_stencil(B, e);
    double f[4][8];
    for (int c = 0; c < 4; ++c)
      for (int q = 0; q < 8; ++q) f[c][q] = arr[c][S.pos[c][q]];
    for (int p = 0; p < kKinScalars; ++p) {
      Kin kp = *B.kin, km = *B.kin;
      kin_scalar(kp, p) += 1.0;
      kin_scalar(km, p) -= 1.0;
      DevBlock Bp = B, Bm = B;
      Bp.kin = &kp;
      Bm.kin = &km;
      double op[7], om[7];
      elem_terms(Bp, e, mu_f, rho_f, S, f, op);
      elem_terms(Bm, e, mu_f, rho_f, S, f, om);
      double acc = 0.0;
      for (int t = 0; t < 4; ++t) acc += scale[t] * 0.5 * (op[t] - om[t]);
      part[kKinScalars * (int64_t)e + p] = acc;
    }
  }
}

// gk[p] += sum_e part[11e + p]: fixed-order reduction by one CTA of 256 threads
__global__ void k_stress_kin_sum(const double* part, int ne, double* gk) {
  __shared__ double s[256];
  for (int p = 0; p < kKinScalars; ++p) {
    double acc = 0.0;
    for (int e = threadIdx.x; e < ne; e += blockDim.x) acc += part[kKinScalars * (int64_t)e + p];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
      if ((int)threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
      __syncthreads();
    }
    if (threadIdx.x == 0) gk[p] += s[0];
    __syncthreads();
  }
}

// scale[t] = seed[t] * 2 / aS (aS from the element areas, as k_stress_sum)
__global__ void k_stress_scale(DevBlock B, const double* seed, double* scale) {
  if (blockIdx.x || threadIdx.x) return;
  double sx = 0.0, sy = 0.0;
  for (int e = 0; e < B.ne; ++e) {
    const double alen = B.elen[e];
    sx += 0.5 * fabs(alen * B.cosB[e]);
    sy += 0.5 * fabs(alen * B.cosA[e]);
  }
  const double aSx = 0.5 * sx, aSy = 0.5 * sy;
  scale[0] = seed[0] * 2.0 / aSx;
  scale[1] = seed[1] * 2.0 / aSy;
  scale[2] = seed[2] * 2.0 / aSx;
  scale[3] = seed[3] * 2.0 / aSy;
}

// w[c][pos] += coef over all elements, in element order (one thread)
__global__ void k_stress_accum(int ne, const double* coef, const int64_t* pos, double* w, int64_t np) {
  if (blockIdx.x || threadIdx.x) return;
  for (int e = 0; e < ne; ++e)
    for (int c = 0; c < 4; ++c)
      for (int q = 0; q < 8; ++q) {
        const int64_t r = 32 * (int64_t)e + 8 * c + q;
        w[c * np + pos[r]] += coef[r];
      }
}

// fixed-order pairwise reduction by one CTA
__global__ void k_stress_sum(const double* part, int ne, double* out) {
  __shared__ double s[7][256];
  for (int q = 0; q < 7; ++q) {
    double acc = 0.0;
    for (int e = threadIdx.x; e < ne; e += blockDim.x) acc += part[7 * (int64_t)e + q];
    s[q][threadIdx.x] = acc;
  }
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int q = 0; q < 7; ++q) s[q][threadIdx.x] += s[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double aSx = 0.5 * s[5][0], aSy = 0.5 * s[6][0];
    out[0] = 2.0 * (s[0][0] / aSx);
    out[1] = 2.0 * (s[1][0] / aSy);
    out[2] = 2.0 * (s[2][0] / aSx);
    out[3] = 2.0 * (s[3][0] / aSy);
  }
}

// ---------------------------------------------------------------------------
// Geometric partials of the drag/lift objective (adjoint through moving
// bodies): the derivatives of sum_t seed[t] C_t with respect to each
// element's centroid (lanes 0-2), unit normal (3-5) and element length (6),
// at the current fields, with every bracket and branch of the forward
// evaluation held fixed.  C_t = 2 S_t / aS_t with S_t the sum of the element
// terms and aS the projected-area sums, so an element moves both S_t and aS.
// ---------------------------------------------------------------------------
using G7 = DualN<7>;

__device__ __forceinline__ G7 bil_g(const G7& x, const G7& y, double x1, double x2, double y1, double y2, double f0,
                                    double f1, double f2, double f3) {
  const G7 numer = f0 * (x2 - x) * (y2 - y) + f2 * (x2 - x) * (y - y1) + f1 * (x - x1) * (y2 - y) +
                   f3 * (x - x1) * (y - y1);
  return numer / ((x2 - x1) * (y2 - y1));
}
__device__ __forceinline__ G7 der_g(const G7& x, double x2, double x1, const G7& p_x, const G7& p_x2,
                                    const G7& p_x1) {
  const G7 h2 = fabs(x2 - x), h1 = fabs(x1 - x);
  return (h1 * h1 * p_x2 - h2 * h2 * p_x1 + (h2 * h2 - h1 * h1) * p_x) / (h1 * h2 * (h1 + h2) + 1e-16);
}
__device__ void vad_eval_g(const G7& x, const G7& y, const G7& z, const double* xg, const double* yg,
                           const double* zg, const int ijk[3], const double f[8], G7& val, G7 d3[3]) {
  const int i = ijk[0], j = ijk[1], k = ijk[2];
  const double yj = yg[j - 1], yj1 = yg[j], zk = zg[k - 1], zk1 = zg[k], xi = xg[i - 1], xi1 = xg[i];
  const G7 t11 = bil_g(y, z, yj, yj1, zk, zk1, f[0], f[2], f[4], f[6]);
  const G7 t12 = bil_g(y, z, yj, yj1, zk, zk1, f[1], f[3], f[5], f[7]);
  const G7 t21 = bil_g(x, z, xi, xi1, zk, zk1, f[0], f[1], f[4], f[5]);
  const G7 t22 = bil_g(x, z, xi, xi1, zk, zk1, f[2], f[3], f[6], f[7]);
  const G7 t31 = bil_g(x, y, xi, xi1, yj, yj1, f[0], f[1], f[2], f[3]);
  const G7 t32 = bil_g(x, y, xi, xi1, yj, yj1, f[4], f[5], f[6], f[7]);
  val = t11 + (x - xi) * (t12 - t11) / (xi1 - xi);
  d3[0] = der_g(x, xi1, xi, val, t12, t11);
  d3[1] = der_g(y, yj1, yj, val, t22, t21);
  d3[2] = der_g(z, zk1, zk, val, t32, t31);
}

// elem_terms with the element's geometry seeded: o[0..3] the four terms,
// o[4] a_xz, o[5] a_yz
__device__ void elem_terms_geo(const DevBlock& B, int e, double mu_f, double rho_f, const ElemStencil& S,
                               const double f[4][8], G7 o[6]) {
  const G7 cx = G7::seed(B.xcent[e], 0), cy = G7::seed(B.ycent[e], 1), cz = G7::seed(B.zcent[e], 2);
  const G7 nrm[3] = {G7::seed(B.cosA[e], 3), G7::seed(B.cosB[e], 4), G7::seed(B.cosG[e], 5)};
  const G7 alen = G7::seed(B.elen[e], 6);
  const double nd = S.diag, diag = S.diag;
  const G7 px = cx + nd * nrm[0], py = cy + nd * nrm[1], pz = cz + nd * nrm[2];
  const int sid = B.surf_id[e];
  const Kin& K = *B.kin;
  const double td = sid == 51 ? K.thetaDot1 : (sid == 52 ? K.thetaDot2 : 0.0);
  const double tdd = sid == 51 ? K.thetaDDot1 : (sid == 52 ? K.thetaDDot2 : 0.0);
  const G7 us(K.xdot);
  const G7 vs = -td * (cz - K.piv_z) + K.ydot;
  const G7 ws = td * (cy - K.piv_y);
  const G7 ac_z = -(td * td) * (cz - K.piv_z);
  const G7 ac_y = -(td * td) * (cy - K.piv_y);
  const G7 at_z = tdd * (cy - K.piv_y);
  const G7 at_y = -tdd * (cz - K.piv_z);
  const G7 dpdn = -((ac_z + at_z) * nrm[2] + (ac_y + at_y) * nrm[1]) - K.yddot * nrm[1];
  G7 val, g[3], ddn[3];
  vad_eval_g(px, py, pz, B.xu, B.yu, B.zu, S.ijk[0], f[0], val, g);
  ddn[0] = (2.0 / nd) * (val - us) - (g[0] * nrm[0] + g[1] * nrm[1] + g[2] * nrm[2]);
  vad_eval_g(px, py, pz, B.xv, B.yv, B.zv, S.ijk[1], f[1], val, g);
  ddn[1] = (2.0 / nd) * (val - vs) - (g[0] * nrm[0] + g[1] * nrm[1] + g[2] * nrm[2]);
  vad_eval_g(px, py, pz, B.xw, B.yw, B.zw, S.ijk[2], f[2], val, g);
  ddn[2] = (2.0 / nd) * (val - ws) - (g[0] * nrm[0] + g[1] * nrm[1] + g[2] * nrm[2]);
  const G7 area = alen / 2.0;
  o[5] = 0.5 * fabs(alen * nrm[0]);
  o[4] = 0.5 * fabs(alen * nrm[1]);
  const G7 dd = ddn[0] * nrm[0] + ddn[1] * nrm[1] + ddn[2] * nrm[2];
  o[0] = (ddn[0] - dd * nrm[0]) * mu_f * area;
  o[2] = (ddn[1] - dd * nrm[1]) * mu_f * area;
  vad_eval_g(px, py, pz, B.xp, B.yp, B.zp, S.ijk[3], f[3], val, g);
  const G7 dpdn_e = g[0] * nrm[0] + g[1] * nrm[1] + g[2] * nrm[2];
  const G7 cval = val - (dpdn_e + dpdn) * diag * 0.5;
  o[1] = -cval * area * nrm[0] * rho_f;
  o[3] = -cval * area * nrm[1] * rho_f;
}

// sums[0..3] = S_t, sums[4] = aSx, sums[5] = aSy of the current evaluation
// (k_stress_sum's reduction order)
__global__ void k_stress_sums(const double* part, int ne, double* sums) {
  __shared__ double s[7][256];
  for (int q = 0; q < 7; ++q) {
    double acc = 0.0;
    for (int e = threadIdx.x; e < ne; e += blockDim.x) acc += part[7 * (int64_t)e + q];
    s[q][threadIdx.x] = acc;
  }
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int q = 0; q < 7; ++q) s[q][threadIdx.x] += s[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int q = 0; q < 4; ++q) sums[q] = s[q][0];
    sums[4] = 0.5 * s[5][0];
    sums[5] = 0.5 * s[6][0];
  }
}

// ge[7e + l] += w * d(sum_t seed[t] C_t)/d(geometry lane l of element e)
__global__ void k_stress_geo(DevBlock B, double mu_f, double rho_f, const double* seed, const double* sums,
                             double w, double* ge) {
  const double* arr[4] = {B.u, B.v, B.w, B.p};
  const double aS[4] = {sums[4], sums[5], sums[4], sums[5]};
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < B.ne; e += gridDim.x * blockDim.x) {
    const ElemStencil S = elem_stencil(B, e);
    double f[4][8];
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int q = 0; q < 8; ++q) f[c][q] = arr[c][S.pos[c][q]];
    G7 o[6];
    elem_terms_geo(B, e, mu_f, rho_f, S, f, o);
    for (int l = 0; l < 7; ++l) {
      double g = 0.0;
      for (int t = 0; t < 4; ++t) {
        // d aS_t = 0.5 d(a_xz or a_yz) of this element
        const double daS = 0.5 * ((t & 1) ? o[5].d[l] : o[4].d[l]);
        g += seed[t] * 2.0 * (o[t].d[l] / aS[t] - sums[t] / (aS[t] * aS[t]) * daS);
      }
      ge[7 * (int64_t)e + l] += w * g;
    }
  }
}

}  // namespace

// ge (7 per element) += w * the geometric derivative of sum_t seed[t] * C_t at
// the block's current fields and geometry; scratch: 7 ne + 8 doubles
int launch_stress_geo(HostBlock* hb, double mu_f, double rho_f, const double* seed_dev, double w, double* ge,
                      double* scratch) {
  const int ne = hb->d.ne;
  if (ne <= 0) return BCFD_E_STATE;
  double* part = scratch;
  double* sums = scratch + 7 * (size_t)ne;
  k_stress_elem<<<grid_for(ne, 128), 128, 0, stream()>>>(hb->d, mu_f, rho_f, part);
  TRY_R(note_launch());
  k_stress_sums<<<1, 256, 0, stream()>>>(part, ne, sums);
  TRY_R(note_launch());
  k_stress_geo<<<grid_for(ne, 64), 64, 0, stream()>>>(hb->d, mu_f, rho_f, seed_dev, sums, w, ge);
  TRY_R(note_launch());
  return 0;
}

// w (4 fields, natural layout) += the gradient of sum_t seed[t] * coefficient t
// with respect to (u, v, w, p) at the block's geometry (the coefficients are
// affine in the fields); scratch: 2 * 32 * ne + 8 doubles
int launch_stress_weights(HostBlock* hb, double mu_f, double rho_f, const double* seed_dev, double* w,
                          double* scratch) {
  const int ne = hb->d.ne;
  if (ne <= 0) return BCFD_E_STATE;
  double* scale = scratch;
  double* coef = scratch + 8;
  int64_t* pos = reinterpret_cast<int64_t*>(coef + 32 * (size_t)ne);
  k_stress_scale<<<1, 32, 0, stream()>>>(hb->d, seed_dev, scale);
  TRY_R(note_launch());
  k_stress_coef<<<grid_for(ne, 64), 64, 0, stream()>>>(hb->d, mu_f, rho_f, scale, coef, pos);
  TRY_R(note_launch());
  k_stress_accum<<<1, 32, 0, stream()>>>(ne, coef, pos, w, hb->d.d.npts());
  TRY_R(note_launch());
  return 0;
}

// gk[kKinScalars] += the kinematic derivative of sum_t seed[t] * coefficient
// t at the block's current fields; scratch: 8 + kKinScalars ne doubles
int launch_stress_kin(HostBlock* hb, double mu_f, double rho_f, const double* seed_dev, double* gk,
                      double* scratch) {
  if (hb->d.ne <= 0) return BCFD_E_STATE;
  k_stress_scale<<<1, 32, 0, stream()>>>(hb->d, seed_dev, scratch);
  TRY_R(note_launch());
  // per-element partials after the 8 scale slots (the scratch holds 8 + 64 ne doubles)
  k_stress_kin_elem<<<grid_for(hb->d.ne, 128), 128, 0, stream()>>>(hb->d, mu_f, rho_f, scratch, scratch + 8);
  TRY_R(note_launch());
  k_stress_kin_sum<<<1, 256, 0, stream()>>>(scratch + 8, hb->d.ne, gk);
  TRY_R(note_launch());
  return 0;
}

int launch_stress(HostBlock* hb, double mu_f, double rho_f, double* out_host) {
  const int ne = hb->d.ne;
  if (ne <= 0) return BCFD_E_STATE;
  double* part = nullptr;
  double* out = nullptr;
  // one allocation holds the partials and the 4 coefficients, so no error
  // path can leave half of the scratch allocated
  BCFD_CUDA(cudaMalloc(&part, ((size_t)ne * 7 + 4) * sizeof(double)));
  out = part + (size_t)ne * 7;
  k_stress_elem<<<grid_for(ne, 128), 128, 0, stream()>>>(hb->d, mu_f, rho_f, part);
  int r = note_launch();
  if (!r) {
    k_stress_sum<<<1, 256, 0, stream()>>>(part, ne, out);
    r = note_launch();
  }
  if (!r) {
    cudaError_t e = cudaMemcpyAsync(out_host, out, 4 * sizeof(double), cudaMemcpyDeviceToHost, stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream());
    if (e != cudaSuccess) {
      report_cuda(e, "stress coefficients to host", __FILE__, __LINE__);
      r = BCFD_E_CUDA;
    }
  }
  cudaFree(part);
  return r;
}

// ---- allocation-free variant ------------------------------------------------
// The same two kernels, with the per-element partials and the 4 coefficients
// in a fixed device array of this translation unit instead of cudaMalloc'd
// memory.  Nothing in it has to start at zero: k_stress_elem writes all
// 7 * ne partials that k_stress_sum reads, and k_stress_sum writes out[0..3].
// There is one array per device, so two calls that overlap on one device would
// race on it; launch_stress_noalloc runs under the library lock on the library
// stream and synchronises before returning, so calls through it never overlap.
namespace {
constexpr int kStressNoallocMaxElems = BCFD_STRESS_NOALLOC_MAX_ELEMS;
constexpr size_t kStressScratchDoubles = 7 * (size_t)kStressNoallocMaxElems + 4;
static __device__ __align__(256) double g_stress_scratch[kStressScratchDoubles];
constexpr int kMaxDevices = 64;
double* g_stress_scratch_ptr[kMaxDevices] = {};
}  // namespace

// Set-up, once per device with that device current: the address of the
// device array.  The first call on a device does this, so it should come
// before any stream capture begins on that device.  The cached address is
// valid while the device's primary context lives (the library never resets
// the device).
static int stress_scratch(double** out) {
  int dev = -1;
  BCFD_CUDA(cudaGetDevice(&dev));
  // the library stream belongs to the device bcfd_init selected
  if (dev != lib().device) return BCFD_E_STATE;
  if (dev < 0 || dev >= kMaxDevices) return BCFD_E_ARG;
  if (!g_stress_scratch_ptr[dev]) {
    void* p = nullptr;
    BCFD_CUDA(cudaGetSymbolAddress(&p, g_stress_scratch));
    if (!p) return BCFD_E_CUDA;
    g_stress_scratch_ptr[dev] = (double*)p;
  }
  *out = g_stress_scratch_ptr[dev];
  return 0;
}

int launch_stress_noalloc(HostBlock* hb, double mu_f, double rho_f, double* out_host) {
  const int ne = hb->d.ne;
  if (ne <= 0) return BCFD_E_STATE;
  if (ne > kStressNoallocMaxElems) {
    std::fprintf(stderr,
                 "bcfd_stress_calculation_noalloc: block has %d surface elements, more than the "
                 "%d its fixed device scratch holds (use bcfd_stress_calculation)\n",
                 ne, kStressNoallocMaxElems);
    return BCFD_E_CAPACITY;
  }
  double* scratch = nullptr;
  TRY_R(stress_scratch(&scratch));
  double* part = scratch;
  double* out = scratch + 7 * (size_t)kStressNoallocMaxElems;
  k_stress_elem<<<grid_for(ne, 128), 128, 0, stream()>>>(hb->d, mu_f, rho_f, part);
  TRY_R(note_launch());
  k_stress_sum<<<1, 256, 0, stream()>>>(part, ne, out);
  TRY_R(note_launch());
  BCFD_CUDA(cudaMemcpyAsync(out_host, out, 4 * sizeof(double), cudaMemcpyDeviceToHost, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  return 0;
}

}  // namespace bcfd
