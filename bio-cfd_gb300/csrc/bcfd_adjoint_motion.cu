// Adjoint through a moving body's geometry: the transposes from element
// geometry back to the parameters of its motion.
//
//   motion parameters (heave amplitude and frequency, pitch amplitude, phase
//   and frequency)
//     -> per step: the placement of the surface (rotation angle about the x
//        axis and translation, computeSurfaceVariables, src/Search.F90:126-208)
//        and the kinematic scalars the forcing and drag/lift read
//     -> node positions (rotation through the pivot line, then translation)
//     -> element centroid, unit normal and length (computeSurfaceNorm,
//        src/Search.F90:210-258)
//     -> the IB forcing and the drag/lift objective.
//
// The element-geometry adjoints are accumulated by the forcing transposes
// (from partials recorded at the forward's stencil values) and by the
// objective; here they go back to nodes (per-element Jacobians in dual
// numbers, then a per-node gather over the node's elements in a fixed order)
// and from nodes to the placement (a fixed-order reduction).  The chain from
// placements and kinematic scalars to the parameters runs on the host in dual
// numbers through the formulas of the motion (motion_tangent).
#include <cmath>

#include "bcfd_dual.cuh"
#include "bcfd_host.h"

namespace bcfd {
namespace {

using G9 = DualN<9>;

// per element: contributions of its 7 geometry adjoints (centroid, unit
// normal, length) to the 9 coordinates of its 3 nodes, at the current nodes
__global__ void k_elem_node_adj(DevBlock B, double fin, const double* ge, double* contrib) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < B.ne; n += gridDim.x * blockDim.x) {
    const int a = B.elp1[n] - 1, b = B.elp2[n] - 1, c = B.elp3[n] - 1;
    const G9 p1x = G9::seed(B.xnode1[a], 0), p1y = G9::seed(B.ynode1[a], 1), p1z = G9::seed(B.znode1[a], 2);
    const G9 p2x = G9::seed(B.xnode1[b], 3), p2y = G9::seed(B.ynode1[b], 4), p2z = G9::seed(B.znode1[b], 5);
    const G9 p3x = G9::seed(B.xnode1[c], 6), p3y = G9::seed(B.ynode1[c], 7), p3z = G9::seed(B.znode1[c], 8);
    // the expressions of k_surface_norm
    const G9 xc = (p2x + p1x + p3x) / 3.0, yc = (p2y + p1y + p3y) / 3.0, zc = (p2z + p1z + p3z) / 3.0;
    const G9 ca = (p2y - p1y) * (p3z - p1z) - (p3y - p1y) * (p2z - p1z);
    const G9 cb = (p2z - p1z) * (p3x - p1x) - (p3z - p1z) * (p2x - p1x);
    const G9 cg = (p2x - p1x) * (p3y - p1y) - (p3x - p1x) * (p2y - p1y);
    const G9 len = sqrt(ca * ca + cb * cb + cg * cg);
    const G9 out[7] = {xc, yc, zc, fin * ca / len, fin * cb / len, fin * cg / len, len};
    const double* g = ge + 7 * (int64_t)n;
#pragma unroll
    for (int l = 0; l < 9; ++l) {
      double acc = 0.0;
#pragma unroll
      for (int o = 0; o < 7; ++o) acc += g[o] * out[o].d[l];
      contrib[9 * (int64_t)n + l] = acc;
    }
  }
}

// node adjoint = sum over the node's (element, corner) entries in the CSR
// order (fixed), then its contribution to the placement: d/d(angle, tx, ty,
// tz) of the node position, the angle being +theta for surface-51 nodes and
// -theta for surface-52 nodes (place_node)
__global__ void k_node_place_adj(DevBlock B, const int* off, const int* ent, const double* contrib, Place P,
                                 double* part) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < B.nn; j += gridDim.x * blockDim.x) {
    double gx = 0.0, gy = 0.0, gz = 0.0;
    for (int q = off[j]; q < off[j + 1]; ++q) {
      const int e = ent[q] / 3, corner = ent[q] % 3;
      const double* c = contrib + 9 * (int64_t)e + 3 * corner;
      gx += c[0];
      gy += c[1];
      gz += c[2];
    }
    const int id = B.node_id[j];
    double dth = 0.0;
    if (id == 51 || id == 52) {
      const double cs = id == 51 ? P.c1 : P.c2, sn = id == 51 ? P.s1 : P.s2;
      const double y = B.ynode0[j], z = B.znode0[j], pp = P.piv_pt;
      // z' = z c + y s + pp - pp c and y' = -z s + y c + pp s for angle a: d/da
      const double dz = -z * sn + y * cs + pp * sn;
      const double dy = -z * cs - y * sn + pp * cs;
      dth = (gy * dy + gz * dz) * (id == 51 ? 1.0 : -1.0);
    }
    part[4 * (int64_t)j + 0] = dth;
    part[4 * (int64_t)j + 1] = gx;
    part[4 * (int64_t)j + 2] = gy;
    part[4 * (int64_t)j + 3] = gz;
  }
}

// out[4] = sum over nodes of part (one CTA, fixed order)
__global__ void k_sum4(const double* part, int n, double* out) {
  __shared__ double s[4][256];
  for (int q = 0; q < 4; ++q) {
    double acc = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) acc += part[4 * (int64_t)j + q];
    s[q][threadIdx.x] = acc;
  }
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int q = 0; q < 4; ++q) s[q][threadIdx.x] += s[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 4; ++q) out[q] = s[q][0];
}

}  // namespace

// node -> (element, corner) entries of a block's surface, in element order
int build_node_csr(HostBlock* hb, std::vector<int>& off, std::vector<int>& ent) {
  const int ne = hb->d.ne, nn = hb->d.nn;
  if ((int)hb->elem_host.size() < 4 * ne) return BCFD_E_STATE;
  off.assign((size_t)nn + 1, 0);
  for (int e = 0; e < ne; ++e)
    for (int c = 0; c < 3; ++c) {
      const int node = hb->elem_host[(size_t)c * ne + e] - 1;
      if (node < 0 || node >= nn) return BCFD_E_STATE;
      off[(size_t)node + 1]++;
    }
  for (int j = 0; j < nn; ++j) off[(size_t)j + 1] += off[(size_t)j];
  ent.assign((size_t)off[(size_t)nn], 0);
  std::vector<int> fill(off.begin(), off.end() - 1);
  for (int e = 0; e < ne; ++e)
    for (int c = 0; c < 3; ++c) {
      const int node = hb->elem_host[(size_t)c * ne + e] - 1;
      ent[(size_t)fill[(size_t)node]++] = 3 * e + c;
    }
  return 0;
}

// place_bar[4] (host) = the adjoint of the placement P (angle, tx, ty, tz)
// from the element-geometry adjoints ge (7 per element) at the block's current
// nodes (which P placed).  scratch: 9 ne + 4 nn + 4 doubles.
int launch_geometry_place_adj(HostBlock* hb, const double* ge, const int* off_dev, const int* ent_dev,
                              const Place& P, double* scratch, double* place_bar) {
  const int ne = hb->d.ne, nn = hb->d.nn;
  if (ne <= 0 || nn <= 0 || !hb->d.xnode0 || !hb->d.node_id) return BCFD_E_STATE;
  double* contrib = scratch;
  double* part = scratch + 9 * (size_t)ne;
  double* out = part + 4 * (size_t)nn;
  k_elem_node_adj<<<grid_for(ne, 128), 128, 0, stream()>>>(hb->d, (double)hb->inor, ge, contrib);
  BCFD_LAUNCHED();
  k_node_place_adj<<<grid_for(nn, 128), 128, 0, stream()>>>(hb->d, off_dev, ent_dev, contrib, P, part);
  BCFD_LAUNCHED();
  k_sum4<<<1, 256, 0, stream()>>>(part, nn, out);
  BCFD_LAUNCHED();
  BCFD_CUDA(d2h(place_bar, out, 4 * sizeof(double)));
  return 0;
}

// ---------------------------------------------------------------------------
// The motion replayed in dual numbers over the parameters (heave amplitude
// yamp, pitch amplitude a0 in degrees, the shared pitch phase angle in
// radians, pitch frequency freq, heave frequency bfreq): the formulas of the
// initial placement and of the per-step kinematics (shift_surface_nodes_initial
// and stage_surface_variables; src/Search.F90:49-208), from the placement
// through every step up to driver step `last`.  Only the parameter dependence
// is carried: the tow (xpth, piv_x) and the fixed offsets have none.  Entry s
// of `out` belongs to driver step init_ita + s (entry 0: the placement).
// ---------------------------------------------------------------------------
int motion_tangent(const HostBlock* hb, double phase_angle, double freq, double deltat, double tot_at_ita0,
                   int64_t ita0, int64_t last, std::vector<StepTangent>& out) {
  using P5 = DualN<kMotionParams>;
  const BodyMotion& m = hb->motion;
  if (!m.on || !m.placed) return BCFD_E_STATE;
  const double pi = 4.0 * std::atan(1.0);
  const P5 yamp = P5::seed(m.yamp, 0), a0d = P5::seed(m.a0_deg, 1), ph = P5::seed(phase_angle, 2),
           fr = P5::seed(freq, 3), bf = P5::seed(m.bfreq, 4);
  const int64_t first = m.init_ita;
  if (last < first) return BCFD_E_ARG;
  out.assign((size_t)(last - first + 1), StepTangent{});
  auto put = [&](int64_t s, const P5& angle, const P5& ty, const P5 kin[kKinScalars]) {
    StepTangent& T = out[(size_t)(s - first)];
    for (int q = 0; q < kMotionParams; ++q) {
      T.angle[q] = angle.d[q];
      T.ty[q] = ty.d[q];
      for (int p = 0; p < kKinScalars; ++p) T.kin[p][q] = kin[p].d[q];
    }
  };
  // the initial placement
  const double lag = m.lag;
  P5 aoa_b(m.init_aoa), y0(0.0);
  if (lag != 0.0) {
    aoa_b = m.init_aoa + a0d * (sin(ph - lag) - sin(ph));
    y0 = yamp * std::sin(-lag);
  }
  const P5 ysh = m.yshift + y0;
  P5 kin[kKinScalars];
  for (int p = 0; p < kKinScalars; ++p) kin[p] = P5(0.0);
  {
    const P5 angt = 2.0 * pi * bf;
    const double bdfr = 15, bdy = 15 * m.init_dxmin;
    kin[1] = angt * bdy * std::cos(2 * pi * bdfr * m.init_totime);
    kin[2] = -(angt * angt * bdy * std::sin(2 * pi * bdfr * m.init_totime));
    kin[9] = ysh;
  }
  put(first, aoa_b * (pi / 180.0), ysh, kin);
  const P5 a0r = a0d * (pi / 180.0);
  P5 piv_y = ysh;
  for (int64_t s = first + 1; s <= last; ++s) {
    const double totime = tot_at_ita0 + (double)(s - ita0) * deltat;
    P5 parg = 2.0 * pi * fr * (totime + deltat) + ph;
    if (lag != 0.0) parg = parg - lag;
    const P5 angle = a0r * sin(parg);
    const P5 ang_theta = 2.0 * pi * fr;
    const P5 td1 = ang_theta * a0r * cos(parg);
    const P5 tdd1 = -(ang_theta * ang_theta * a0r * sin(parg));
    const P5 angt = 2.0 * pi * bf;
    P5 h0 = angt * totime, h1 = angt * (totime - deltat);
    if (lag != 0.0) {
      h0 = h0 - lag;
      h1 = h1 - lag;
    }
    const P5 yt = yamp * sin(h0);
    piv_y = piv_y + (yt - yamp * sin(h1));
    for (int p = 0; p < kKinScalars; ++p) kin[p] = P5(0.0);
    kin[1] = angt * yamp * cos(h0);
    kin[2] = -(angt * angt * yamp * sin(h0));
    kin[3] = td1;
    kin[4] = tdd1;
    kin[5] = -td1;
    kin[6] = -tdd1;
    kin[9] = piv_y;
    put(s, angle, m.yshift + yt, kin);
  }
  return 0;
}

}  // namespace bcfd
