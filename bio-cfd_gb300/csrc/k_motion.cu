// Rigid-body motion of a block's surface: the initial placement
// shiftSurfaceNodesInitial (src/Search.F90:49-124) and the per-step
// kinematics and node positions computeSurfaceVariables
// (src/Search.F90:126-208).  The kinematic scalars and the rotation's
// cos/sin are evaluated on the host with the reference's expressions (one
// value per step, so the host and the oracle give identical bits) and staged
// in device memory with one copy; one kernel then makes them current and
// moves the nodes: rotation of surface-51 (+angle) and -52 (-angle) nodes
// about the x axis through z = piv_pt, then the translation.  Staging runs
// before a captured step is launched, the kernel inside it, so a step with a
// moving body replays from a CUDA graph.
#include <cmath>

#include "bcfd_host.h"

namespace bcfd {
namespace {

constexpr double kXfact = 0.05;  // src/Search.F90:12

// the staged step: the kinematics take effect, the search origin of the
// moved surface is set, the nodes move
__global__ void k_place_nodes(DevBlock B, const MotionStage* S, Kin* kin, float* org) {
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (t0 == 0) {
    *kin = S->kin;
    if (org)
      for (int q = 0; q < 4; ++q) org[q] = S->org[q];
  }
  const Place P = S->place;
  double* xn = const_cast<double*>(B.xnode1);
  double* yn = const_cast<double*>(B.ynode1);
  double* zn = const_cast<double*>(B.znode1);
  for (int i = t0; i < B.nn; i += gridDim.x * blockDim.x)
    place_node(P, B.node_id[i], B.xnode0[i], B.ynode0[i], B.znode0[i], xn + i, yn + i, zn + i);
}

// the nearest-element search's bound on node distances from the block centre
// after a move: translation + body-frame radius + the rotation about the pivot
// line (a rotation about an axis at distance |piv_pt| from the origin moves a
// point by at most 2|piv_pt| more than its radius)
void update_node_rmax(HostBlock* hb, double piv_pt, double tx, double ty, double tz) {
  const Dims& d = hb->d.d;
  const double cx = 0.5 * (hb->x1[0] + hb->x1[d.nx + 2]), cy = 0.5 * (hb->y1[0] + hb->y1[d.ny + 2]),
               cz = 0.5 * (hb->z1[0] + hb->z1[d.nz + 2]);
  const double ax = tx - cx, ay = ty - cy, az = tz - cz;
  hb->node_rmax = std::sqrt(ax * ax + ay * ay + az * az) + hb->motion_r0 + 2.0 * std::fabs(piv_pt) + 1e-9;
}

// stage a placement: the node bound, the search origin, one upload of the
// kinematics/placement/origin (a pageable source is staged by the copy call,
// so the host struct may change right after)
int stage_place(HostBlock* hb, double aoa1, double piv_pt, double tx, double ty1, double ty2, double tz1,
                double tz2, int two) {
  if (hb->d.nn <= 0) return 0;
  update_node_rmax(hb, piv_pt, tx, ty1 + ty2, tz1 + tz2);
  const double aoa2 = -aoa1;
  MotionStage& S = hb->stage;
  S.kin = hb->kin;
  S.place = Place{std::cos(aoa1), std::sin(aoa1), std::cos(aoa2), std::sin(aoa2), piv_pt, tx, ty1, ty2, tz1, tz2, two};
  float* dev = nullptr;
  TRY_R(search_origin_stage(hb, S.org, &dev));
  BCFD_CUDA(cudaMemcpyAsync(hb->stage_dev, &S, sizeof(S), cudaMemcpyHostToDevice, stream()));
  hb->staged = true;
  return 0;
}

}  // namespace

int apply_surface_variables(HostBlock* hb) {
  if (hb->d.nn <= 0) return upload_kin(hb);
  if (!hb->staged) return BCFD_E_STATE;
  hb->staged = false;
  float* dev = nullptr;
  TRY_R(search_origin_stage(hb, nullptr, &dev));
  k_place_nodes<<<grid_for(hb->d.nn, 128), 128, 0, stream()>>>(hb->d, hb->stage_dev, hb->kin_dev, dev);
  BCFD_LAUNCHED();
  return 0;
}

void staged_node(const HostBlock* hb, int64_t node, double* x, double* y, double* z) {
  const size_t q = (size_t)(node - 1);
  place_node(hb->stage.place, hb->node_id_host[q], hb->node0[0][q], hb->node0[1][q], hb->node0[2][q], x, y, z);
}

int upload_kin(HostBlock* hb) {
  BCFD_CUDA(cudaMemcpyAsync(hb->kin_dev, &hb->kin, sizeof(Kin), cudaMemcpyHostToDevice, stream()));
  return 0;
}

namespace {
}  // namespace

int shift_surface_nodes_initial(HostBlock* hb, double aoa, double piv_pt, int64_t ita, double deltat,
                                double dxmin, double totime) {
  BodyMotion& m = hb->motion;
  const double pi = 4.0 * std::atan(1.0);
  m.placed = true;
  m.init_aoa = aoa;
  m.init_piv_pt = piv_pt;
  m.init_dxmin = dxmin;
  m.init_totime = totime;
  m.init_ita = ita;
  m.a0_deg = m.a0;
  // a lagging body starts where its lagged kinematics put it at t = 0 relative
  // to the shared ones: its angle differs by the pitch's change over the lag,
  // its heave position is yamp sin(-lag) (both 0 without a lag)
  double aoa_b = aoa, y0 = 0.0;
  if (m.lag != 0.0) {
    aoa_b = aoa + m.a0 * (std::sin(m.lag_phase - m.lag) - std::sin(m.lag_phase));
    y0 = m.yamp * std::sin(-m.lag);
  }
  const double aoa1 = aoa_b * pi / 180.0;
  const double bdfr = 15, bdy = 15 * dxmin;
  m.xmove = m.ymove = m.zmove = 0.0;
  m.a0 = m.a0 * pi / 180.0;
  const double angt = 2.0 * pi * m.bfreq;
  m.xpth1 = m.xshift - ((double)ita * dxmin * kXfact);
  m.xpth2 = m.xshift - ((double)ita * dxmin * kXfact);
  m.ypth2 = (m.yamp) * std::sin(angt * m.xshift);
  Kin& D = hb->kin;
  const double ysh = m.lag != 0.0 ? m.yshift + y0 : m.yshift;
  D.piv_x = m.xshift;
  D.piv_y = ysh;
  D.piv_z = m.zshift;
  D.thetaDot1 = D.thetaDot2 = D.alphaDot = 0.0;
  D.thetaDDot1 = D.thetaDDot2 = 0.0;
  m.yt = bdy * std::sin(2 * pi * bdfr * totime);
  D.ydot = angt * bdy * std::cos(2 * pi * bdfr * totime);
  D.yddot = -(angt * angt * bdy * std::sin(2 * pi * bdfr * totime));
  m.xt = m.xshift - ((double)ita * dxmin * kXfact);
  D.xdot = -(dxmin * kXfact) / deltat;
  m.inity_cent = m.nxty_cent = ysh;
  m.initx_cent = m.nxtx_cent = m.xshift;
  m.initz_cent = m.nxtz_cent = m.zshift;
  TRY_R(stage_place(hb, aoa1, piv_pt, m.xshift, ysh, 0.0, m.zshift, 0.0, 0));
  return apply_surface_variables(hb);
}

namespace {

// change_block_coords_interfaces (src/Search.F90:1269-1370), device part:
// cell_n = 1 where the moved block keeps old data (centres strictly inside
// the overlap of the old and new boxes, one cell in from its faces)
__global__ void k_mark_cell_n(DevBlock B, double xs, double xe, double ys, double ye, double zs, double ze,
                              double dx, double dy, double dz) {
  const Dims& d = B.d;
  const int64_t n = d.npts();
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % d.NX);
    const int64_t r = t / d.NX;
    const int j = 1 + (int)(r % d.NY), k = 1 + (int)(r / d.NY);
    const double x = B.xp[i - 1], y = B.yp[j - 1], z = B.zp[k - 1];
    B.cell_n[t] = (x > xs + dx && x < xe - dx && z > zs + dz && z < ze - dz && y > ys + dy && y < ye - dy) ? 1 : 0;
  }
}

// the moved fields: u,v,w,p at the new indices [cpy_mv] from the old indices
// [cpy] (zero elsewhere), one thread per target point
__global__ void k_move_fields(DevBlock B, const double* dum, int64_t x0, int64_t y0, int64_t z0, int64_t nx,
                              int64_t ny, int64_t nz, int64_t ox, int64_t oy, int64_t oz) {
  const Dims& d = B.d;
  const int64_t np = d.npts(), n = nx * ny * nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = t % nx, r = t / nx;
    const int64_t b = r % ny, c = r / ny;
    const int64_t dst = d.idx((int)(x0 + a), (int)(y0 + b), (int)(z0 + c));
    const int64_t src = d.idx((int)(ox + a), (int)(oy + b), (int)(oz + c));
    B.u[dst] = dum[src];
    B.v[dst] = dum[np + src];
    B.w[dst] = dum[2 * np + src];
    B.p[dst] = dum[3 * np + src];
  }
}

}  // namespace

int launch_mark_cell_n(HostBlock* hb, const double box_new[6]) {
  k_mark_cell_n<<<grid_for(hb->d.d.npts(), 256), 256, 0, stream()>>>(hb->d, box_new[0], box_new[1], box_new[2],
                                                                        box_new[3], box_new[4], box_new[5], hb->dx,
                                                                        hb->dy, hb->dz);
  BCFD_LAUNCHED();
  return 0;
}

// u,v,w,p = 0, then the kept data at its new indices; the index ranges must
// lie inside the block (the reference would read outside otherwise)
int launch_move_fields(HostBlock* hb, const double* dum) {
  const Dims& d = hb->d.d;
  const size_t b = (size_t)d.npts() * sizeof(double);
  for (double* f : {hb->d.u, hb->d.v, hb->d.w, hb->d.p}) BCFD_CUDA(cudaMemsetAsync(f, 0, b, stream()));
  const int64_t* c = hb->cpy;
  const int64_t* m = hb->cpy_mv;
  const int64_t nx = m[1] - m[0] + 1, ny = m[3] - m[2] + 1, nz = m[5] - m[4] + 1;
  if (nx <= 0 || ny <= 0 || nz <= 0) return 0;
  const int64_t hi[3] = {d.NX, d.NY, d.NZ};
  for (int a = 0; a < 3; ++a) {
    const int64_t n = a == 0 ? nx : a == 1 ? ny : nz;
    if (m[2 * a] < 1 || m[2 * a] + n - 1 > hi[a] || c[2 * a] < 1 || c[2 * a] + n - 1 > hi[a]) return BCFD_E_STATE;
  }
  k_move_fields<<<grid_for(nx * ny * nz, 256), 256, 0, stream()>>>(hb->d, dum, m[0], m[2], m[4], nx, ny, nz, c[0],
                                                                    c[2], c[4]);
  BCFD_LAUNCHED();
  return 0;
}

int compute_surface_variables(HostBlock* hb, double phase_angle, double piv_pt, int64_t ita, double deltat,
                              double dxmin, double freq, double totime) {
  TRY_R(stage_surface_variables(hb, phase_angle, piv_pt, ita, deltat, dxmin, freq, totime));
  return apply_surface_variables(hb);
}

int stage_surface_variables(HostBlock* hb, double phase_angle, double piv_pt, int64_t ita, double deltat,
                            double dxmin, double freq, double totime) {
  BodyMotion& m = hb->motion;
  Kin& D = hb->kin;
  const double pi = 4.0 * std::atan(1.0);
  // pitch and heave phases; a lagging body subtracts its lag from both
  double parg = 2.0 * pi * freq * (totime + deltat) + phase_angle;
  if (m.lag != 0.0) parg = parg - m.lag;
  const double aoa1 = (m.a0) * std::sin(parg);
  const double ang_theta = 2.0 * pi * freq;
  const double bdfr = m.bfreq, bdy = m.yamp;
  const double angt = 2.0 * pi * bdfr;
  m.xpth2 = m.xshift - ((double)ita * dxmin * kXfact);
  m.ypth2 = (m.yamp) * std::sin(angt * m.xpth2);
  m.xchg = m.xpth2 - m.xpth1;
  m.xpth1 = m.xpth2;
  D.thetaDot1 = ang_theta * m.a0 * std::cos(parg);
  D.thetaDDot1 = -(ang_theta * ang_theta * m.a0 * std::sin(parg));
  D.thetaDot2 = -D.thetaDot1;
  D.thetaDDot2 = -D.thetaDDot1;
  double h0 = angt * (totime), h1 = angt * (totime - deltat);
  if (m.lag != 0.0) {
    h0 = h0 - m.lag;
    h1 = h1 - m.lag;
  }
  m.yt = bdy * std::sin(h0);
  D.ydot = angt * bdy * std::cos(h0);
  D.yddot = -(angt * angt * bdy * std::sin(h0));
  m.xt = m.xpth2;
  D.xdot = -(dxmin * kXfact) / deltat;
  m.ychg = m.yt - bdy * std::sin(h1);
  m.ymove = m.yt;
  m.xmove = m.xchg;
  m.zmove = 0.0;
  D.piv_y = D.piv_y + m.ychg;
  D.piv_x = D.piv_x + m.xmove;
  D.piv_z = D.piv_z + m.zmove;
  m.nxty_cent = m.nxty_cent + m.ychg;
  m.nxtx_cent = m.nxtx_cent + m.xmove;
  return stage_place(hb, aoa1, piv_pt, m.xpth2, m.yshift, m.ymove, m.zshift, m.zmove, 1);
}

}  // namespace bcfd
