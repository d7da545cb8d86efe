// Rigid-body motion of a block's surface, restated from the reference (test
// infrastructure only): node surface ids (src/ReadInput.f90:403-420), the
// initial placement shiftSurfaceNodesInitial (src/Search.F90:49-124) and the
// per-step kinematics and node positions computeSurfaceVariables
// (src/Search.F90:126-208).  Expressions keep the reference's evaluation
// order; pi is modGlobal's 4*atan(1).
#include <cmath>

#include "orc_core.h"

namespace orc {
namespace {
const real kPi = 4.0 * atan(1.0);
const real kXfact = 0.05;  // src/Search.F90:12

// rotation of a surface-51/52 node about the x axis through z = piv_pt
void place(Block& b, int64_t i, real aoa1, real aoa2, real piv_pt, real& xr1, real& yr1,
           real& zr1) {
  const int64_t id = b.ibNodeId(i);
  if (id == 51 || id == 52) {
    const real a = id == 51 ? aoa1 : aoa2;
    xr1 = b.xnode(i);
    zr1 = b.znode(i) * cos(a) + b.ynode(i) * sin(a) + piv_pt - piv_pt * cos(a);
    yr1 = -(b.znode(i) * sin(a)) + b.ynode(i) * cos(a) + piv_pt * sin(a);
  } else {
    xr1 = b.xnode(i);
    zr1 = b.znode(i);
    yr1 = b.ynode(i);
  }
}
}  // namespace

// findDistnode (src/Search.F90:21-47): over the nodes of surface 51, mk is
// the last node whose |z| exceeds the running value, mkx1 / mkx2 those of
// |x| below / above theirs.  The running values take the signed
// coordinate while the tests compare its magnitude, as the reference does.
void find_dist_node(Block& b) {
  real dist = 0.0, dist1 = 999999.0, dist2 = 0.0;
  for (int64_t i = 1; i <= b.ibNodes; ++i) {
    if (b.ibNodeId(i) != 51) continue;
    if (fabs(b.znode(i)) > dist) {
      dist = b.znode(i);
      b.mk = i;
    }
    if (fabs(b.xnode(i)) < dist1) {
      dist1 = b.xnode(i);
      b.mkx1 = i;
    }
    if (fabs(b.xnode(i)) > dist2) {
      dist2 = b.xnode(i);
      b.mkx2 = i;
    }
  }
}

void node_ids_from_elements(Block& b) {
  b.ibNodeId.alloc(b.ibNodes);
  for (int64_t i = 1; i <= b.ibNodes; ++i) b.ibNodeId(i) = 50;
  for (int64_t n = 1; n <= b.ibElems; ++n) {
    const int64_t s = b.ibSurfId(n);
    if (s == 51 || s == 52) {
      b.ibNodeId(b.ibElP1(n)) = s;
      b.ibNodeId(b.ibElP2(n)) = s;
      b.ibNodeId(b.ibElP3(n)) = s;
    }
  }
  for (int64_t n = 1; n <= b.ibElems; ++n)
    if (b.ibSurfId(n) == 50) {
      b.ibNodeId(b.ibElP1(n)) = 50;
      b.ibNodeId(b.ibElP2(n)) = 50;
      b.ibNodeId(b.ibElP3(n)) = 50;
    }
}

void shift_surface_nodes_initial(Block& b, real aoa, real piv_pt, int64_t ita, real deltat,
                                 real dxmin, real totime) {
  // extension: a lagging body starts at its lagged state at t = 0 (angle and
  // heave position); without a lag this is the reference's placement
  real aoa_b = aoa, y0 = 0.0;
  if (b.lag != 0.0) {
    aoa_b = aoa + b.a0 * (sin(b.lag_phase - b.lag) - sin(b.lag_phase));
    y0 = b.yamp * sin(-b.lag);
  }
  const real ysh = b.lag != 0.0 ? b.yshift + y0 : b.yshift;
  const real aoa1 = aoa_b * kPi / 180.0, aoa2 = -aoa1;
  const real bdfr = 15, bdy = 15 * dxmin;
  b.xmove = 0.0;
  b.ymove = 0.0;
  b.zmove = 0.0;
  b.a0 = b.a0 * kPi / 180.0;
  const real angt = 2.0 * kPi * b.bfreq;
  b.xpth1 = b.xshift - ((real)ita * dxmin * kXfact);
  b.xpth2 = b.xshift - ((real)ita * dxmin * kXfact);
  b.ypth2 = (b.yamp) * sin(angt * b.xshift);
  b.piv_x = b.xshift;
  b.piv_y = ysh;
  b.piv_z = b.zshift;
  b.thetaDot = b.thetaDDot = b.thetaDot1 = b.thetaDot2 = b.alphaDot = 0.0;
  b.thetaDDot1 = b.thetaDDot2 = 0.0;
  b.yt = bdy * sin(2 * kPi * bdfr * totime);
  b.ydot = angt * bdy * cos(2 * kPi * bdfr * totime);
  b.yddot = -(angt * angt * bdy * sin(2 * kPi * bdfr * totime));
  b.xt = b.xshift - ((real)ita * dxmin * kXfact);
  b.xdot = -(dxmin * kXfact) / deltat;
  b.inity_cent = ysh;
  b.nxty_cent = ysh;
  b.initx_cent = b.xshift;
  b.nxtx_cent = b.xshift;
  b.initz_cent = b.zshift;
  b.nxtz_cent = b.zshift;
  for (int64_t i = 1; i <= b.ibNodes; ++i) {
    real xr1, yr1, zr1;
    place(b, i, aoa1, aoa2, piv_pt, xr1, yr1, zr1);
    b.xnode1(i) = xr1 + b.xshift;
    b.ynode1(i) = yr1 + ysh;
    b.znode1(i) = zr1 + b.zshift;
  }
}

void compute_surface_variables(Block& b, real phase_angle, real piv_pt, int64_t ita,
                               real deltat, real dxmin, real freq, real totime) {
  real parg = 2.0 * kPi * freq * (totime + deltat) + phase_angle;
  if (b.lag != 0.0) parg = parg - b.lag;  // extension: per-body lag
  const real aoa1 = (b.a0) * sin(parg);
  const real aoa2 = -aoa1;
  const real ang_theta = 2.0 * kPi * freq;
  const real bdfr = b.bfreq, bdy = b.yamp;
  const real angt = 2.0 * kPi * bdfr;
  b.xpth2 = b.xshift - ((real)ita * dxmin * kXfact);
  b.ypth2 = (b.yamp) * sin(angt * b.xpth2);
  b.xchg = b.xpth2 - b.xpth1;
  b.xpth1 = b.xpth2;
  b.thetaDot1 = ang_theta * b.a0 * cos(parg);
  b.thetaDDot1 = -(ang_theta * ang_theta * b.a0 * sin(parg));
  b.thetaDot2 = -b.thetaDot1;
  b.thetaDDot2 = -b.thetaDDot1;
  real h0 = angt * (totime), h1 = angt * (totime - deltat);
  if (b.lag != 0.0) {
    h0 = h0 - b.lag;
    h1 = h1 - b.lag;
  }
  b.yt = bdy * sin(h0);
  b.ydot = angt * bdy * cos(h0);
  b.yddot = -(angt * angt * bdy * sin(h0));
  b.xt = b.xpth2;
  b.xdot = -(dxmin * kXfact) / deltat;
  b.ychg = b.yt - bdy * sin(h1);
  b.ymove = b.yt;
  b.xmove = b.xchg;
  b.zmove = 0.0;
  b.piv_y = b.piv_y + b.ychg;
  b.piv_x = b.piv_x + b.xmove;
  b.piv_z = b.piv_z + b.zmove;
  b.nxty_cent = b.nxty_cent + b.ychg;
  b.nxtx_cent = b.nxtx_cent + b.xmove;
  for (int64_t i = 1; i <= b.ibNodes; ++i) {
    real xr1, yr1, zr1;
    place(b, i, aoa1, aoa2, piv_pt, xr1, yr1, zr1);
    b.xnode1(i) = xr1 + b.xpth2;
    b.ynode1(i) = yr1 + b.yshift + b.ymove;
    b.znode1(i) = zr1 + b.zshift + b.zmove;
  }
}

}  // namespace orc
