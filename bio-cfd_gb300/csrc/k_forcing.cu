// Immersed-boundary forcing of src/Forcing.f90 on the GPU.
//
// velocityForcing1 and pressureForcing1/Field write the very array their
// probes interpolate from, inside one serial loop over the IB list: a probe
// stencil can read a value that an earlier iteration just wrote.  The GPU
// path reproduces that serial semantics exactly:
//   * a task is one reconstruction (IB cell n, component c) at serial
//     position pos = 6n + c (velocity: U2,U1,V2,V1,W2,W1) or n (pressure);
//   * for every stencil point the task finds the latest task before it that
//     writes that point (a u point u(a,b,c) is written by the U2 task of cell
//     (a,b,c) and the U1 task of cell (a+1,b,c), the later one winning);
//   * tasks are evaluated in rounds: in each round every task whose
//     dependencies finished in earlier rounds runs, reading each stencil
//     value either from the unmodified array or from the dependency's output
//     slot (rounds = dependency depth + 1, one grid barrier each);
//   * last writers scatter their outputs into the array at the end.
// Everything runs in one cooperative launch with bounded grid barriers.  The
// Field / Ghost velocity variants read ut and write u (or ghost arrays) and
// therefore run as plain data-parallel kernels.
#include "bcfd_host.h"
#include "bcfd_dual.cuh"

namespace bcfd {

namespace {

enum Comp { CU2 = 0, CU1, CV2, CV1, CW2, CW1 };

struct Grid3 {
  const double *x, *y, *z;
  int nx, ny, nz;  // array lengths
};

__device__ __forceinline__ Grid3 comp_grid(const DevBlock& B, int axis) {
  const Dims& d = B.d;
  switch (axis) {
    case 1: return {B.xu, B.yu, B.zu, d.NX + 1, d.NY, d.NZ};
    case 2: return {B.xv, B.yv, B.zv, d.NX, d.NY + 1, d.NZ};
    case 3: return {B.xw, B.yw, B.zw, d.NX, d.NY, d.NZ + 1};
    default: return {B.xp, B.yp, B.zp, d.NX, d.NY, d.NZ};
  }
}

// find_index_in_array (src/Forcing.f90:1165-1183): first i in [s, f] with
// a(i) <= v < a(i+1).  Indices outside the array are skipped; when no
// bracket exists the error word is set and a clamped start index returned.
// The grid coordinates are non-decreasing, so a bracket is unique and a
// binary search for the last i with a(i) <= v finds the scan's answer.
__device__ int find_index(const DevBlock& B, double v, const double* a, int len, int s, int f) {
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
  int r = s < 1 ? 1 : s;
  if (r + 1 > len) r = len - 1;
  return r;
}

__device__ __forceinline__ double bilinear(double x, double y, double x1, double x2, double y1,
                                           double y2, double f0, double f1, double f2, double f3) {
  const double numer = f0 * (x2 - x) * (y2 - y) + f2 * (x2 - x) * (y - y1) +
                       f1 * (x - x1) * (y2 - y) + f3 * (x - x1) * (y - y1);
  const double denom = (x2 - x1) * (y2 - y1);
  return numer / denom;
}

__device__ __forceinline__ double linear(double x, double x0, double x1, double y0, double y1) {
  return y0 + (x - x0) * (y1 - y0) / (x1 - x0);
}

__device__ __forceinline__ double derivative(double x, double x2, double x1, double p_x,
                                             double p_x2, double p_x1) {
  const double h2 = fabs(x2 - x);
  const double h1 = fabs(x1 - x);
  return (h1 * h1 * p_x2 - h2 * h2 * p_x1 + (h2 * h2 - h1 * h1) * p_x) /
         (h1 * h2 * (h1 + h2) + 1e-16);
}

// The probe of one reconstruction: position and bracketing indices.
struct Probe {
  double px, py, pz;   // probe point
  int ix, iy, iz;      // find_index results
  int ii, jj, kk;      // stencil base of the variable (offset axis applied)
  double s2n, pt1;
  int e;               // element (0-based)
  int ti, tj, tk;      // written sample (target) index
  int axis;            // 0 p, 1 u, 2 v, 3 w
};

// mode 0: ...Forcing1, 1: ...Field, 2: ...Ghost.  comp < 0 for pressure.
// n is the IB index (0-based) for modes 0/1 and the TS index for mode 2.
__device__ Probe make_probe(const DevBlock& B, int mode, int comp, int n) {
  Probe P;
  const Dims& d = B.d;
  const int ib = mode == 2 ? B.ts_idx[n] - 1 : n;
  const int i = B.ib_i[ib], j = B.ib_j[ib], k = B.ib_k[ib];
  int slot;
  if (comp < 0) {
    slot = N_P;
    P.axis = 0;
  } else {
    // nel / NormDis slots: U1=1, U2=2, V1=3, V2=4, W1=5, W2=6
    slot = comp + ((comp & 1) ? 0 : 2);
    P.axis = 1 + comp / 2;
  }
  P.e = B.nel[slot][ib] - 1;
  const double sg = mode == 2 ? -1.0 : 1.0;
  P.s2n = mode == 2 ? -B.nd[slot][ib] : B.nd[slot][ib];
  const double s2n = P.s2n;
  P.pt1 = 1.5 * sqrt(B.dxa[i - 1] * B.dxa[i - 1] + B.dya[j - 1] * B.dya[j - 1] +
                     B.dza[k - 1] * B.dza[k - 1]) +
          (fabs(s2n) - s2n) * 0.5;
  const Grid3 G = comp_grid(B, P.axis);
  double qx = G.x[i - 1], qy = G.y[j - 1], qz = G.z[k - 1];
  if (comp == CU2) qx = G.x[i];
  if (comp == CV2) qy = G.y[j];
  if (comp == CW2) qz = G.z[k];
  if (sg > 0) {
    P.px = qx + P.pt1 * B.cosA[P.e];
    P.py = qy + P.pt1 * B.cosB[P.e];
    P.pz = qz + P.pt1 * B.cosG[P.e];
  } else {
    P.px = qx - P.pt1 * B.cosA[P.e];
    P.py = qy - P.pt1 * B.cosB[P.e];
    P.pz = qz - P.pt1 * B.cosG[P.e];
  }
  if (mode == 0) {
    P.ix = find_index(B, P.px, G.x, G.nx, 1, d.nx + (comp == CU2 ? 2 : 1));
    P.iy = find_index(B, P.py, G.y, G.ny, 1, d.ny + (comp == CV2 ? 2 : 1));
    P.iz = find_index(B, P.pz, G.z, G.nz, 1, d.nz + (comp == CW2 ? 2 : 1));
    if (comp == CU2 && P.ix == d.nx + 2) P.ix = d.nx + 1;
    if (comp == CU1 && P.ix == 1) P.ix = 2;
    if (comp == CV2 && P.iy == d.ny + 2) P.iy = d.ny + 1;
    if (comp == CV1 && P.iy == 1) P.iy = 2;
    if (comp == CW2 && P.iz == d.nz + 2) P.iz = d.nz + 1;
    if (comp == CW1 && P.iz == 1) P.iz = 2;
  } else {
    P.ix = find_index(B, P.px, G.x, G.nx, i - 7, i + 7);
    P.iy = find_index(B, P.py, G.y, G.ny, j - 7, j + 7);
    P.iz = find_index(B, P.pz, G.z, G.nz, k - 7, k + 7);
  }
  P.ii = P.ix - (P.axis == 1);
  P.jj = P.iy - (P.axis == 2);
  P.kk = P.iz - (P.axis == 3);
  // keep every stencil point inside the array (the reference would read out
  // of bounds here; flag it instead)
  if (P.ii < 1 || P.ii + 1 > d.NX || P.jj < 1 || P.jj + 1 > d.NY || P.kk < 1 || P.kk + 1 > d.NZ) {
    set_err(B.err, BCFD_E_NOTFOUND);
    P.ii = max(1, min(P.ii, d.NX - 1));
    P.jj = max(1, min(P.jj, d.NY - 1));
    P.kk = max(1, min(P.kk, d.NZ - 1));
  }
  P.ti = i - (comp == CU1);
  P.tj = j - (comp == CV1);
  P.tk = k - (comp == CW1);
  return P;
}

// compute_value_and_derivatives (src/Forcing.f90:1091-1161) on the 8 values
// f[a + 2b + 4c] = var(ii+a, jj+b, kk+c)
__device__ void value_and_derivatives(const DevBlock& B, const Probe& P, const double f[8],
                                      double& val, double der[3]) {
  const Grid3 G = comp_grid(B, P.axis);
  const int i = P.ix, j = P.iy, k = P.iz;
  const double x = P.px, y = P.py, z = P.pz;
  const double yj = G.y[j - 1], yj1 = G.y[j], zk = G.z[k - 1], zk1 = G.z[k], xi = G.x[i - 1],
               xi1 = G.x[i];
  const double t11 = bilinear(y, z, yj, yj1, zk, zk1, f[0], f[2], f[4], f[6]);
  const double t12 = bilinear(y, z, yj, yj1, zk, zk1, f[1], f[3], f[5], f[7]);
  const double t21 = bilinear(x, z, xi, xi1, zk, zk1, f[0], f[1], f[4], f[5]);
  const double t22 = bilinear(x, z, xi, xi1, zk, zk1, f[2], f[3], f[6], f[7]);
  const double t31 = bilinear(x, y, xi, xi1, yj, yj1, f[0], f[1], f[2], f[3]);
  const double t32 = bilinear(x, y, xi, xi1, yj, yj1, f[4], f[5], f[6], f[7]);
  val = linear(x, xi, xi1, t11, t12);
  der[0] = derivative(x, xi1, xi, val, t12, t11);
  der[1] = derivative(y, yj1, yj, val, t22, t21);
  der[2] = derivative(z, zk1, zk, val, t32, t31);
}

__device__ __forceinline__ double dotn(const DevBlock& B, int e, const double d[3]) {
  return d[0] * B.cosA[e] + d[1] * B.cosB[e] + d[2] * B.cosG[e];
}

// surface velocity of a sample (src/Forcing.f90: see the oracle for lines);
// the `0 + ydot` forms of Forcing.f90:237 and :551 are kept (they map -0 to +0)
__device__ double surf_velocity(const DevBlock& B, int e, int comp, int mode) {
  const int sid = B.surf_id[e];
  if (comp == CU2 || comp == CU1) return B.kin->xdot;
  if (comp == CV2 || comp == CV1) {
    if (sid == 50) {
      const bool plus0 = (comp == CV1 && mode == 0) || (comp == CV2 && mode == 2);
      return plus0 ? 0.0 + B.kin->ydot : B.kin->ydot;
    }
    const double td = sid == 51 ? B.kin->thetaDot1 : B.kin->thetaDot2;
    if (mode == 0) return -td * (B.zcent[e] - B.kin->piv_z) + B.kin->ydot;
    return -td * (B.zcent[e] - B.kin->piv_z) + (-B.kin->alphaDot) * (B.xcent[e] - B.kin->piv_x) + B.kin->ydot;
  }
  if (sid == 50) return 0.0;
  const double td = sid == 51 ? B.kin->thetaDot1 : B.kin->thetaDot2;
  return td * (B.ycent[e] - B.kin->piv_y);
}

__device__ __forceinline__ double vel_quad(double pos_val, double surf, double dn, double n1,
                                           double s2n) {
  const double cval = surf;
  const double bval = 2.0 / n1 * (pos_val - surf) - dn;
  const double aval = dn / n1 - (pos_val - surf) / (n1 * n1);
  return aval * (s2n * s2n) + bval * s2n + cval;
}

// dpdn of the rigid-body acceleration (src/Forcing.f90:29-52, :381-412)
__device__ double dpdn_body(const DevBlock& B, int e, int mode) {
  const int sid = B.surf_id[e];
  double ac_y = 0, ac_z = 0, at_y = 0, at_z = 0;
  if (sid == 51 || sid == 52) {
    const double td = sid == 51 ? B.kin->thetaDot1 : B.kin->thetaDot2;
    const double tdd = sid == 51 ? B.kin->thetaDDot1 : B.kin->thetaDDot2;
    ac_z = -(td * td) * (B.zcent[e] - B.kin->piv_z);
    ac_y = -(td * td) * (B.ycent[e] - B.kin->piv_y);
    at_z = tdd * (B.ycent[e] - B.kin->piv_y);
    at_y = -tdd * (B.zcent[e] - B.kin->piv_z);
  }
  if (mode == 2)
    return ((ac_z + at_z) * B.cosG[e] + (ac_y + at_y) * B.cosB[e]) + (B.kin->yddot * (B.cosB[e]));
  return -((ac_z + at_z) * B.cosG[e] + (ac_y + at_y) * B.cosB[e]) - B.kin->yddot * B.cosB[e];
}

// value of one reconstruction from its 8 stencil values
__device__ double reconstruct(const DevBlock& B, int mode, int comp, const Probe& P,
                              const double f[8]) {
  double val, der[3];
  value_and_derivatives(B, P, f, val, der);
  const double dn = mode == 2 ? -1.0 * dotn(B, P.e, der) : dotn(B, P.e, der);
  const double n1 = P.pt1 + P.s2n;
  const double s2n = P.s2n;
  if (comp < 0) {
    const double dpdn = dpdn_body(B, P.e, mode);
    const double bval = dpdn;
    const double aval = (dn - dpdn) / (2.0 * n1);
    const double cval = val - (dn + dpdn) * n1 * 0.5;
    return aval * (s2n * s2n) + bval * s2n + cval;
  }
  return vel_quad(val, surf_velocity(B, P.e, comp, mode), dn, n1, s2n);
}

// ---------------------------------------------------------------------------
// Geometric partials of one reconstruction (adjoint through moving bodies):
// the output's derivatives with respect to the centroid (lanes 0-2) and the
// unit normal (lanes 3-5) of the task's element, at the stencil values f the
// forward read.  The bracketing indices, the element and every branch are
// those of the forward evaluation (the discrete choices are held fixed); the
// normal distance s2n = (sample - centroid) . normal of computeNormDistance
// (src/Search.F90:743-861) carries its own derivatives.
// ---------------------------------------------------------------------------
using G6 = DualN<6>;

__device__ __forceinline__ G6 bilinear_g(const G6& x, const G6& y, double x1, double x2, double y1, double y2,
                                         double f0, double f1, double f2, double f3) {
  const G6 numer = f0 * (x2 - x) * (y2 - y) + f2 * (x2 - x) * (y - y1) + f1 * (x - x1) * (y2 - y) +
                   f3 * (x - x1) * (y - y1);
  return numer / ((x2 - x1) * (y2 - y1));
}
__device__ __forceinline__ G6 derivative_g(const G6& x, double x2, double x1, const G6& p_x, const G6& p_x2,
                                           const G6& p_x1) {
  const G6 h2 = fabs(x2 - x), h1 = fabs(x1 - x);
  return (h1 * h1 * p_x2 - h2 * h2 * p_x1 + (h2 * h2 - h1 * h1) * p_x) / (h1 * h2 * (h1 + h2) + 1e-16);
}

// the sample point of NormDis slot `slot` of IB cell (i,j,k) (k_norm_distance)
__device__ __forceinline__ void nd_sample(const DevBlock& B, int slot, int i, int j, int k, double q[3]) {
  q[0] = slot == 1 ? B.x1[i - 1] : slot == 2 ? B.x1[i] : B.xp[i - 1];
  q[1] = slot == 3 ? B.y1[j - 1] : slot == 4 ? B.y1[j] : B.yp[j - 1];
  q[2] = slot == 5 ? B.z1[k - 1] : slot == 6 ? B.z1[k] : B.zp[k - 1];
}

__device__ G6 reconstruct_geo(const DevBlock& B, int mode, int comp, int n, const Probe& P, const double f[8]) {
  const int ib = mode == 2 ? B.ts_idx[n] - 1 : n;
  const int i = B.ib_i[ib], j = B.ib_j[ib], k = B.ib_k[ib];
  const int e = P.e;
  const G6 cx = G6::seed(B.xcent[e], 0), cy = G6::seed(B.ycent[e], 1), cz = G6::seed(B.zcent[e], 2);
  const G6 nx = G6::seed(B.cosA[e], 3), ny = G6::seed(B.cosB[e], 4), nz = G6::seed(B.cosG[e], 5);
  const int slot = comp < 0 ? N_P : comp + ((comp & 1) ? 0 : 2);
  double xs[3];
  nd_sample(B, slot, i, j, k, xs);
  const double sg = mode == 2 ? -1.0 : 1.0;
  G6 s2n = sg * ((xs[0] - cx) * nx + (xs[1] - cy) * ny + (xs[2] - cz) * nz);
  s2n.v = P.s2n;  // the forward's value (its branches)
  const G6 pt1 = 1.5 * ::sqrt(B.dxa[i - 1] * B.dxa[i - 1] + B.dya[j - 1] * B.dya[j - 1] +
                              B.dza[k - 1] * B.dza[k - 1]) +
                 (fabs(s2n) - s2n) * 0.5;
  const Grid3 G = comp_grid(B, P.axis);
  double qx = G.x[i - 1], qy = G.y[j - 1], qz = G.z[k - 1];
  if (comp == CU2) qx = G.x[i];
  if (comp == CV2) qy = G.y[j];
  if (comp == CW2) qz = G.z[k];
  const G6 x = qx + sg * (pt1 * nx), y = qy + sg * (pt1 * ny), z = qz + sg * (pt1 * nz);
  // compute_value_and_derivatives on the forward's brackets
  const int ii = P.ix, jj = P.iy, kk = P.iz;
  const double yj = G.y[jj - 1], yj1 = G.y[jj], zk = G.z[kk - 1], zk1 = G.z[kk], xi = G.x[ii - 1], xi1 = G.x[ii];
  const G6 t11 = bilinear_g(y, z, yj, yj1, zk, zk1, f[0], f[2], f[4], f[6]);
  const G6 t12 = bilinear_g(y, z, yj, yj1, zk, zk1, f[1], f[3], f[5], f[7]);
  const G6 t21 = bilinear_g(x, z, xi, xi1, zk, zk1, f[0], f[1], f[4], f[5]);
  const G6 t22 = bilinear_g(x, z, xi, xi1, zk, zk1, f[2], f[3], f[6], f[7]);
  const G6 t31 = bilinear_g(x, y, xi, xi1, yj, yj1, f[0], f[1], f[2], f[3]);
  const G6 t32 = bilinear_g(x, y, xi, xi1, yj, yj1, f[4], f[5], f[6], f[7]);
  const G6 val = t11 + (x - xi) * (t12 - t11) / (xi1 - xi);
  const G6 d0 = derivative_g(x, xi1, xi, val, t12, t11);
  const G6 d1 = derivative_g(y, yj1, yj, val, t22, t21);
  const G6 d2 = derivative_g(z, zk1, zk, val, t32, t31);
  const G6 dn = sg * (d0 * nx + d1 * ny + d2 * nz);
  const G6 n1 = pt1 + s2n;
  const Kin& K = *B.kin;
  const int sid = B.surf_id[e];
  if (comp < 0) {
    G6 ac_y(0.0), ac_z(0.0), at_y(0.0), at_z(0.0);
    if (sid == 51 || sid == 52) {
      const double td = sid == 51 ? K.thetaDot1 : K.thetaDot2;
      const double tdd = sid == 51 ? K.thetaDDot1 : K.thetaDDot2;
      ac_z = -(td * td) * (cz - K.piv_z);
      ac_y = -(td * td) * (cy - K.piv_y);
      at_z = tdd * (cy - K.piv_y);
      at_y = -tdd * (cz - K.piv_z);
    }
    const G6 dpdn = mode == 2 ? ((ac_z + at_z) * nz + (ac_y + at_y) * ny) + K.yddot * ny
                              : -((ac_z + at_z) * nz + (ac_y + at_y) * ny) - K.yddot * ny;
    const G6 aval = (dn - dpdn) / (2.0 * n1);
    const G6 cval = val - (dn + dpdn) * n1 * 0.5;
    return aval * (s2n * s2n) + dpdn * s2n + cval;
  }
  G6 surf(0.0);
  if (comp == CU2 || comp == CU1) {
    surf = G6(K.xdot);
  } else if (comp == CV2 || comp == CV1) {
    if (sid == 50) {
      surf = G6(K.ydot);
    } else {
      const double td = sid == 51 ? K.thetaDot1 : K.thetaDot2;
      surf = mode == 0 ? -td * (cz - K.piv_z) + K.ydot
                       : -td * (cz - K.piv_z) + (-K.alphaDot) * (cx - K.piv_x) + K.ydot;
    }
  } else if (sid != 50) {
    const double td = sid == 51 ? K.thetaDot1 : K.thetaDot2;
    surf = td * (cy - K.piv_y);
  }
  const G6 bval = 2.0 / n1 * (val - surf) - dn;
  const G6 aval = dn / n1 - (val - surf) / (n1 * n1);
  return aval * (s2n * s2n) + bval * s2n + surf;
}

__device__ __forceinline__ double* comp_array(const DevBlock& B, int axis, bool tfield) {
  switch (axis) {
    case 1: return tfield ? B.ut : B.u;
    case 2: return tfield ? B.vt : B.v;
    case 3: return tfield ? B.wt : B.w;
    default: return B.p;
  }
}

// ---------------------------------------------------------------------------
// the serial-order DAG path (velocityForcing1, pressureForcing1/Field)
// ---------------------------------------------------------------------------
struct DagScratch {
  double* out;    // per task output
  int* dep;       // per task 8 dependency task ids (-1: read the array)
  int* level;     // per task: the round it finished in (0: not yet)
  int* flag;      // [0..2] "work left" flags of the rounds
};

// four read-only point arrays indexed by axis (0 p, 1 u, 2 v, 3 w)
struct Fields4c {
  const double* a[4];
};

struct DagArgs {
  int mode;       // 0 or 1
  int vel;        // 1: velocity (6 tasks per IB cell), 0: pressure
};

// latest task before `pos` writing stencil point (a,b,c) of component axis
__device__ __forceinline__ int last_writer(const DevBlock& B, const DagArgs& g, int axis, int a,
                                           int b, int c, int pos) {
  const Dims& d = B.d;
  if (!g.vel) {
    const int A = B.ibmap[d.idx(a, b, c)];
    return (A >= 0 && A < pos) ? A : -1;
  }
  const int cA = 2 * (axis - 1), cB = cA + 1;  // the "2" and "1" faces of the axis
  const int A = B.ibmap[d.idx(a, b, c)];
  int Bn = -1;
  const int a1 = a + (axis == 1), b1 = b + (axis == 2), c1 = c + (axis == 3);
  if (a1 <= d.NX && b1 <= d.NY && c1 <= d.NZ) Bn = B.ibmap[d.idx(a1, b1, c1)];
  if (Bn >= 0 && 6 * Bn + cB < pos) return 6 * Bn + cB;
  if (A >= 0 && 6 * A + cA < pos) return 6 * A + cA;
  return -1;
}

// is task t the final writer of its target point?
__device__ __forceinline__ bool is_last_writer(const DevBlock& B, const DagArgs& g, int t,
                                               const Probe& P) {
  if (!g.vel) return true;
  const int comp = t % 6;
  if (comp & 1) return true;  // a "1" face task is always the later writer
  const Dims& d = B.d;
  const int a1 = P.ti + (P.axis == 1), b1 = P.tj + (P.axis == 2), c1 = P.tk + (P.axis == 3);
  if (a1 > d.NX || b1 > d.NY || c1 > d.NZ) return true;
  return B.ibmap[d.idx(a1, b1, c1)] < 0;
}

__global__ void __launch_bounds__(256) k_forcing_dag(DevBlock B, DagArgs g, DagScratch s, GridBar gb) {
  const int nib = (int)min(B.cnt[C_IB], (int64_t)B.cap_ib);
  const int nt = g.vel ? 6 * nib : nib;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nthr = gridDim.x * blockDim.x;
  // phase 1: dependencies
  for (int t = tid; t < nt; t += nthr) {
    const int n = g.vel ? t / 6 : t, comp = g.vel ? t % 6 : -1;
    const Probe P = make_probe(B, g.mode, comp, n);
#pragma unroll
    for (int q = 0; q < 8; ++q)
      s.dep[8 * t + q] = last_writer(B, g, P.axis, P.ii + (q & 1), P.jj + ((q >> 1) & 1), P.kk + (q >> 2), t);
    s.level[t] = 0;
  }
  if (!grid_sync(gb)) return;
  // phase 2: evaluate in rounds: in round r every task whose dependencies all
  // finished in earlier rounds computes its output (done = r + 1).  A task
  // finishes in round (its level), so the rounds are the dependency depth
  // plus one, one grid barrier each; the "work left" flag is triple-buffered
  // (set in round r, read after its barrier, cleared for round r + 2).
  int* done = s.level;
  for (int round = 0;; ++round) {
    __shared__ int s_left;
    if (threadIdx.x == 0) s_left = 0;
    __syncthreads();
    int left = 0;
    for (int t = tid; t < nt; t += nthr) {
      if (__ldcg(done + t) != 0) continue;
      bool can = true;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int w = s.dep[8 * t + q];
        if (w >= 0) {
          const int dw = __ldcg(done + w);
          if (dw == 0 || dw > round) can = false;
        }
      }
      if (!can) {
        left = 1;
        continue;
      }
      const int n = g.vel ? t / 6 : t, comp = g.vel ? t % 6 : -1;
      const Probe P = make_probe(B, g.mode, comp, n);
      const double* arr = comp_array(B, P.axis, g.vel != 0);
      double f[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int w = s.dep[8 * t + q];
        f[q] = w >= 0 ? __ldcg(s.out + w)
                      : arr[B.d.idx(P.ii + (q & 1), P.jj + ((q >> 1) & 1), P.kk + (q >> 2))];
      }
      __stcg(s.out + t, reconstruct(B, g.mode, comp, P, f));
      __stcg(done + t, round + 1);
    }
    if (left) atomicOr(&s_left, 1);
    __syncthreads();
    if (threadIdx.x == 0 && s_left) atomicOr(&s.flag[round % 3], 1);
    if (!grid_sync(gb)) return;
    const int any = *((volatile int*)&s.flag[round % 3]);
    if (blockIdx.x == 0 && threadIdx.x == 0) s.flag[(round + 2) % 3] = 0;
    if (!any) break;
    if (round > nt + 2) {  // cannot happen for a DAG; guard the loop anyway
      if (threadIdx.x == 0) set_err(B.err, BCFD_E_TIMEOUT);
      return;
    }
  }
  // phase 4: scatter the final values
  for (int t = tid; t < nt; t += nthr) {
    const int n = g.vel ? t / 6 : t, comp = g.vel ? t % 6 : -1;
    const Probe P = make_probe(B, g.mode, comp, n);
    if (!is_last_writer(B, g, t, P)) continue;
    double* arr = comp_array(B, P.axis, g.vel != 0);
    arr[B.d.idx(P.ti, P.tj, P.tk)] = __ldcg(s.out + t);
  }
}

// velocityForcingField (mode 1): reads ut/vt/wt, writes u/v/w.  No task reads
// another's output, but two tasks write the same face (the "2" face of cell
// (i,j,k) is the "1" face of cell (i+1,j,k)): only the serially later writer
// stores.
__global__ void k_vel_field(DevBlock B) {
  const int nib = (int)min(B.cnt[C_IB], (int64_t)B.cap_ib);
  const int nt = 6 * nib;
  const DagArgs g{1, 1};
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
    const int n = t / 6, comp = t % 6;
    const Probe P = make_probe(B, 1, comp, n);
    if (!is_last_writer(B, g, t, P)) continue;
    const double* src = comp_array(B, P.axis, true);
    double f[8];
#pragma unroll
    for (int q = 0; q < 8; ++q)
      f[q] = src[B.d.idx(P.ii + (q & 1), P.jj + ((q >> 1) & 1), P.kk + (q >> 2))];
    comp_array(B, P.axis, false)[B.d.idx(P.ti, P.tj, P.tk)] = reconstruct(B, 1, comp, P, f);
  }
}

// velocityForcingGhost (mode 2): ghost values and the t-ghost saves
__global__ void k_vel_ghost(DevBlock B) {
  const int nts = (int)B.cnt[C_TS];
  const int nt = 6 * nts;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
    const int n = t / 6, comp = t % 6;
    // ghost slot of the component: U2 2, U1 8, V2 4, V1 10, W2 6, W1 12
    const int gs = ((comp & 1) ? G_U1 : G_U2) + 2 * (comp >> 1);
    const Probe P = make_probe(B, 2, comp, n);
    const double* src = comp_array(B, P.axis, true);
    double f[8];
#pragma unroll
    for (int q = 0; q < 8; ++q)
      f[q] = src[B.d.idx(P.ii + (q & 1), P.jj + ((q >> 1) & 1), P.kk + (q >> 2))];
    B.ghost[gs][n] = reconstruct(B, 2, comp, P, f);
    B.ghost[gs + 1][n] = comp_array(B, P.axis, false)[B.d.idx(P.ti, P.tj, P.tk)];
  }
}

// pressureForcingGhost (mode 2)
__global__ void k_p_ghost(DevBlock B) {
  const int nts = (int)B.cnt[C_TS];
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nts; n += gridDim.x * blockDim.x) {
    const Probe P = make_probe(B, 2, -1, n);
    double f[8];
#pragma unroll
    for (int q = 0; q < 8; ++q)
      f[q] = B.p[B.d.idx(P.ii + (q & 1), P.jj + ((q >> 1) & 1), P.kk + (q >> 2))];
    B.ghost[G_P][n] = reconstruct(B, 2, -1, P, f);
    B.ghost[G_PT][n] = B.p[B.d.idx(P.ti, P.tj, P.tk)];
  }
}

// ---------------------------------------------------------------------------
// Adjoint of the forcing loops.  With the geometry fixed every task is affine
// in its 8 stencil values (interpolation, derivative and the quadratic fit are
// linear in them; the surface velocity and dp/dn are constants), so its
// coefficients are reconstruct(e_q) - reconstruct(0).  The reference's loops
// run the tasks in list order, in place; their transpose runs them in reverse
// order on the adjoint arrays: take the target's adjoint, zero it (the target
// was overwritten), add coefficient x adjoint to each stencil point.  A read
// of a value an earlier task wrote becomes an add that the earlier task picks
// up when its turn comes, which is exactly the chain rule through the serial
// order.  One thread runs the reverse sweep, so the sums have a fixed order.
// ---------------------------------------------------------------------------
__global__ void k_force_coef(DevBlock B, int mode, int vel, ForceCoef fc) {
  const int nib = (int)min(B.cnt[mode == 2 ? C_TS : C_IB], (int64_t)B.cap_ib);
  const int nt = vel ? 6 * nib : nib;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
    const int n = vel ? t / 6 : t, comp = vel ? t % 6 : -1;
    const Probe P = make_probe(B, mode, comp, n);
    double f[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) f[q] = 0.0;
    const double r0 = reconstruct(B, mode, comp, P, f);
    for (int q = 0; q < 8; ++q) {
      f[q] = 1.0;
      fc.coef[8 * (int64_t)t + q] = reconstruct(B, mode, comp, P, f) - r0;
      f[q] = 0.0;
      fc.pos[8 * (int64_t)t + q] = B.d.idx(P.ii + (q & 1), P.jj + ((q >> 1) & 1), P.kk + (q >> 2));
    }
    fc.tgt[t] = B.d.idx(P.ti, P.tj, P.tk);
    fc.axis[t] = P.axis;
    if (fc.elem) fc.elem[t] = P.e;
    // kinematic sensitivities at f = 0: the output is at most quadratic in
    // each scalar (centripetal terms), so the central difference with unit
    // steps is its derivative
    for (int p = 0; p < kKinScalars; ++p) {
      Kin kp = *B.kin, km = *B.kin;
      kin_scalar(kp, p) += 1.0;
      kin_scalar(km, p) -= 1.0;
      DevBlock Bp = B, Bm = B;
      Bp.kin = &kp;
      Bm.kin = &km;
      fc.kc[kKinScalars * (int64_t)t + p] =
          0.5 * (reconstruct(Bp, mode, comp, P, f) - reconstruct(Bm, mode, comp, P, f));
    }
  }
}

__global__ void k_force_rev(DevBlock B, int vel, ForceCoef fc, AdjPtrs a) {
  if (blockIdx.x || threadIdx.x) return;
  const int nib = (int)min(B.cnt[C_IB], (int64_t)B.cap_ib);
  const int nt = vel ? 6 * nib : nib;
  for (int t = nt - 1; t >= 0; --t) {
    const int ax = fc.axis[t];
    double* T = a.tgt[ax];
    double* S = a.src[ax];
    const double o = T[fc.tgt[t]];
    T[fc.tgt[t]] = 0.0;
    for (int q = 0; q < 8; ++q) S[fc.pos[8 * (int64_t)t + q]] += fc.coef[8 * (int64_t)t + q] * o;
    for (int p = 0; p < kKinScalars; ++p) fc.gk[p] += fc.kc[kKinScalars * (int64_t)t + p] * o;
    if (fc.geo) {
      const int e = fc.elem[t];
      for (int l = 0; l < 6; ++l) fc.ge[7 * (int64_t)e + l] += fc.geo[6 * (int64_t)t + l] * o;
    }
  }
}

// velocityForcingGhost / pressureForcingGhost transposed (tasks of TS entry
// n, component comp; the ghost value is affine in the probe's 8 values of
// ut/vt/wt or p, the t-ghost value a copy of u/v/w or p at the TS position):
// the ghost arrays' adjoint gb (14 arrays of cap entries, ghost[] order)
// goes to a.src (the read arrays) and a.tgt (the copied ones), then is zeroed
__global__ void k_ghost_rev(DevBlock B, int vel, ForceCoef fc, AdjPtrs a, double* gb, int64_t cap) {
  if (blockIdx.x || threadIdx.x) return;
  const int nts = (int)min(B.cnt[C_TS], (int64_t)B.cap_ib);
  const int nt = vel ? 6 * nts : nts;
  for (int t = nt - 1; t >= 0; --t) {
    const int n = vel ? t / 6 : t, comp = vel ? t % 6 : -1;
    const int gs = vel ? ((comp & 1) ? G_U1 : G_U2) + 2 * (comp >> 1) : G_P;
    const int ax = fc.axis[t];
    const double o = gb[gs * cap + n];
    gb[gs * cap + n] = 0.0;
    double* S = a.src[ax];
    for (int q = 0; q < 8; ++q) S[fc.pos[8 * (int64_t)t + q]] += fc.coef[8 * (int64_t)t + q] * o;
    for (int p = 0; p < kKinScalars; ++p) fc.gk[p] += fc.kc[kKinScalars * (int64_t)t + p] * o;
    if (fc.geo) {
      const int e = fc.elem[t];
      for (int l = 0; l < 6; ++l) fc.ge[7 * (int64_t)e + l] += fc.geo[6 * (int64_t)t + l] * o;
    }
    const double o2 = gb[(gs + 1) * cap + n];
    gb[(gs + 1) * cap + n] = 0.0;
    a.tgt[ax][fc.tgt[t]] += o2;
  }
}

}  // namespace

// Geometric partials of every task of one forcing call, at the stencil values
// it read: the DAG variants read the output of the latest earlier writer, else
// the array as it was before the call (`pre`); the others read their source
// array, which the call does not change.
__global__ void k_force_geo(DevBlock B, int mode, int vel, Fields4c pre, DagScratch s, int dag, double* geo) {
  const int nib = (int)min(B.cnt[C_IB], (int64_t)B.cap_ib);
  const int nts = (int)min(B.cnt[C_TS], (int64_t)B.cap_ib);
  const int cnt = mode == 2 ? nts : nib;
  const int nt = vel ? 6 * cnt : cnt;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
    const int n = vel ? t / 6 : t, comp = vel ? t % 6 : -1;
    const Probe P = make_probe(B, mode, comp, n);
    const double* src = pre.a[P.axis];
    double f[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int w = dag ? s.dep[8 * t + q] : -1;
      f[q] = w >= 0 ? s.out[w] : src[B.d.idx(P.ii + (q & 1), P.jj + ((q >> 1) & 1), P.kk + (q >> 2))];
    }
    const G6 r = reconstruct_geo(B, mode, comp, n, P, f);
#pragma unroll
    for (int l = 0; l < 6; ++l) geo[6 * (int64_t)t + l] = r.d[l];
  }
}

// transpose of launch_forcing_velocity / launch_forcing_pressure (modes 0 and
// 1) on adjoint arrays indexed by axis (0 p, 1 u, 2 v, 3 w): a.tgt holds the
// adjoint of the written arrays, a.src that of the read ones (the same arrays
// for the in-place loops; ut/vt/wt's for velocityForcingField, which reads ut
// and writes u)
int launch_forcing_adjoint(HostBlock* hb, int mode, int vel, const AdjPtrs& a, const ForceCoef& fc) {
  if (hb->d.ne <= 0) return 0;
  const int64_t cap = (vel ? 6 : 1) * (int64_t)hb->d.cap_ib;
  k_force_coef<<<grid_for(cap, 128, 2048), 128, 0, stream()>>>(hb->d, mode, vel, fc);
  BCFD_LAUNCHED();
  k_force_rev<<<1, 32, 0, stream()>>>(hb->d, vel, fc, a);
  BCFD_LAUNCHED();
  return 0;
}

// transpose of the ghost calls (mode 2): a.src the adjoint of the probed
// arrays by axis (0 p, 1 ut, 2 vt, 3 wt for velocity), a.tgt that of the
// t-ghost sources (p, u, v, w), gb the ghost arrays' adjoint
int launch_ghost_adjoint(HostBlock* hb, int vel, const AdjPtrs& a, const ForceCoef& fc, double* gb, int64_t cap) {
  if (hb->d.ne <= 0) return 0;
  const int64_t n = (vel ? 6 : 1) * (int64_t)hb->d.cap_ib;
  k_force_coef<<<grid_for(n, 128, 2048), 128, 0, stream()>>>(hb->d, 2, vel, fc);
  BCFD_LAUNCHED();
  k_ghost_rev<<<1, 32, 0, stream()>>>(hb->d, vel, fc, a, gb, cap);
  BCFD_LAUNCHED();
  return 0;
}

static DagScratch& dag_scratch(HostBlock* hb, int* status) {
  *status = 0;
  if (!hb->dag_scratch) {
    // sized for the allocated list capacity, so a cap lowered and raised
    // again (bcfd_block_set_list_capacity) never outgrows it
    const int64_t need = 6 * (int64_t)hb->cap_ib_alloc;
    DagScratch* s = new DagScratch{};
    if (cudaMalloc(&s->out, need * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&s->dep, need * 8 * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&s->level, need * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&s->flag, 8 * sizeof(int)) != cudaSuccess)
      *status = BCFD_E_NOMEM;
    hb->dag_scratch = s;
    lib().gen++;
  }
  return *static_cast<DagScratch*>(hb->dag_scratch);
}

void free_dag_scratch(HostBlock* hb) {
  if (!hb->dag_scratch) return;
  DagScratch* s = static_cast<DagScratch*>(hb->dag_scratch);
  for (void* p : {(void*)s->out, (void*)s->dep, (void*)s->level, (void*)s->flag})
    if (p) cudaFree(p);
  delete s;
  hb->dag_scratch = nullptr;
}

static int launch_dag(HostBlock* hb, int mode, int vel) {
  int st = 0;
  DagScratch& s = dag_scratch(hb, &st);
  if (st) return st;
  BCFD_CUDA(cudaMemsetAsync(s.flag, 0, 8 * sizeof(int), stream()));
  BCFD_CUDA(cudaMemsetAsync(hb->bar, 0, 2 * sizeof(unsigned), stream()));
  const int threads = 256;
  const unsigned want = (unsigned)((6 * (int64_t)hb->d.cap_ib + threads - 1) / threads);
  const unsigned grid = coop_grid((const void*)k_forcing_dag, threads, 0, std::min(want, 2u * (unsigned)num_sms()));
  GridBar gb = make_bar(hb->d.err, grid);
  gb.ctr = reinterpret_cast<unsigned long long*>(hb->bar);
  DagArgs g{mode, vel};
  DevBlock B = hb->d;
  void* args[] = {(void*)&B, (void*)&g, (void*)&s, (void*)&gb};
  BCFD_CUDA(launch_coop((const void*)k_forcing_dag, grid, threads, args));
  BCFD_LAUNCHED();
  return 0;
}

// With a recorder (an adjoint run recomputing steps through moving bodies):
// the pre-call copy of the arrays a DAG variant overwrites in place
static int record_pre(HostBlock* hb, int vel, Fields4c* pre) {
  ForceRecorder* R = lib().recorder;
  double* sc = R->scratch(hb);
  if (!sc) return BCFD_E_NOMEM;
  const size_t np = (size_t)hb->d.d.npts(), b = np * sizeof(double);
  const double* src[3] = {vel ? hb->d.ut : hb->d.p, hb->d.vt, hb->d.wt};
  for (int q = 0; q < (vel ? 3 : 1); ++q)
    BCFD_CUDA(cudaMemcpyAsync(sc + q * np, src[q], b, cudaMemcpyDeviceToDevice, stream()));
  if (vel) *pre = Fields4c{{hb->d.p, sc, sc + np, sc + 2 * np}};
  else *pre = Fields4c{{sc, hb->d.ut, hb->d.vt, hb->d.wt}};
  return 0;
}

// ... and the tasks' geometric partials once the call has run
static int record_geo(HostBlock* hb, int mode, int vel, const Fields4c& pre, bool dag) {
  int64_t cnt[N_COUNT];
  BCFD_CUDA(d2h(cnt, hb->d.cnt, sizeof(cnt)));
  const int64_t c = std::min<int64_t>(mode == 2 ? cnt[C_TS] : cnt[C_IB], hb->d.cap_ib);
  const int64_t nt = vel ? 6 * c : c;
  double* geo = lib().recorder->slot(hb, mode, vel, nt);
  if (!geo || nt == 0) return 0;
  int st = 0;
  DagScratch& s = dag_scratch(hb, &st);
  if (st) return st;
  k_force_geo<<<grid_for(nt, 128, 2048), 128, 0, stream()>>>(hb->d, mode, vel, pre, s, dag ? 1 : 0, geo);
  BCFD_LAUNCHED();
  return 0;
}

int launch_forcing_velocity(HostBlock* hb, int mode) {
  if (hb->d.ne <= 0) return 0;
  const bool rec = lib().recorder != nullptr;
  const Fields4c cur{{hb->d.p, hb->d.ut, hb->d.vt, hb->d.wt}};
  if (mode == 0) {
    Fields4c pre = cur;
    if (rec) TRY_R(record_pre(hb, 1, &pre));
    TRY_R(launch_dag(hb, 0, 1));
    return rec ? record_geo(hb, 0, 1, pre, true) : 0;
  }
  if (mode == 1) {
    k_vel_field<<<grid_for(6 * (int64_t)hb->d.cap_ib, 128, 2048), 128, 0, stream()>>>(hb->d);
    BCFD_LAUNCHED();
    return rec ? record_geo(hb, 1, 1, cur, false) : 0;
  }
  k_vel_ghost<<<grid_for(6 * (int64_t)hb->d.cap_ib, 128, 2048), 128, 0, stream()>>>(hb->d);
  BCFD_LAUNCHED();
  return rec ? record_geo(hb, 2, 1, cur, false) : 0;
}

int launch_forcing_pressure(HostBlock* hb, int mode) {
  if (hb->d.ne <= 0) return 0;
  const bool rec = lib().recorder != nullptr;
  const Fields4c cur{{hb->d.p, hb->d.ut, hb->d.vt, hb->d.wt}};
  if (mode == 0 || mode == 1) {
    Fields4c pre = cur;
    if (rec) TRY_R(record_pre(hb, 0, &pre));
    TRY_R(launch_dag(hb, mode, 0));
    return rec ? record_geo(hb, mode, 0, pre, true) : 0;
  }
  k_p_ghost<<<grid_for(hb->d.cap_ib, 128, 2048), 128, 0, stream()>>>(hb->d);
  BCFD_LAUNCHED();
  return rec ? record_geo(hb, 2, 0, cur, false) : 0;
}

}  // namespace bcfd
