// SPDX: test infrastructure, not shipped.
//
// Bio-CFD hot-path ORACLE -- TEST INFRASTRUCTURE ONLY.
//
// Parity status: pinned against the reference's own known-answer tests for
// the interpolation primitives, cellCount_solid_coarse and
// updateVelocity_newv; parity unpinned for the momentum, SOR, forcing,
// Search and coupling routines (the reference ships no golden values for
// them and cannot be compiled here: it is Fortran and no Fortran compiler
// exists on either machine).
//
// A serial FP64 C++ restatement of the reference's per-time-step hot path,
// used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg as
// the checker.  The shipped library (bio-cfd_gb300/) never links, loads or
// calls anything in this directory.
//
// Conventions mirror the reference's Fortran data model (src/Blocks.f90:13-81):
//   * every array is 1-based and column-major (x fastest);
//   * 3-D fields u,v,w,p,ut,vt,wt,b,pc,pco,cell,cell_n are (nx+2,ny+2,nz+2),
//     cell2/nodeIdTag/cell_pr are (nx+3,ny+3,nz+3)  (src/AllocateArrays.f90:25-47);
//   * 1-D grids follow src/ReadInput.f90:206-351.
// Build with -ffp-contract=off: the reference's serial CPU build evaluates
// every expression left to right without fused multiply-adds, and parity
// with the GPU path is checked bit for bit.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <string>

#include "orc_real.h"

#ifndef ORC_NOCHECK
#define ORC_CHECK(cond, what)                                                    \
  do {                                                                           \
    if (!(cond)) {                                                               \
      std::fprintf(stderr, "oracle bounds: %s (%s:%d)\n", what, __FILE__, __LINE__); \
      std::abort();                                                              \
    }                                                                            \
  } while (0)
#else
#define ORC_CHECK(cond, what) ((void)0)
#endif

namespace orc {

template <class T>
struct A1 {
  std::vector<T> d;
  void alloc(int64_t n) { d.assign((size_t)(n > 0 ? n : 0), T(0)); }
  int64_t size() const { return (int64_t)d.size(); }
  T& operator()(int64_t i) {
    ORC_CHECK(i >= 1 && i <= (int64_t)d.size(), "A1 index");
    return d[(size_t)(i - 1)];
  }
  const T& operator()(int64_t i) const {
    ORC_CHECK(i >= 1 && i <= (int64_t)d.size(), "A1 index");
    return d[(size_t)(i - 1)];
  }
};

// column-major (n1, n2) array, 1-based
template <class T>
struct A2 {
  std::vector<T> d;
  int64_t n1 = 0, n2 = 0;
  void alloc(int64_t a, int64_t b) {
    n1 = a > 0 ? a : 0;
    n2 = b > 0 ? b : 0;
    d.assign((size_t)(n1 * n2), T(0));
  }
  T& operator()(int64_t i, int64_t j) {
    ORC_CHECK(i >= 1 && i <= n1 && j >= 1 && j <= n2, "A2 index");
    return d[(size_t)((i - 1) + n1 * (j - 1))];
  }
  const T& operator()(int64_t i, int64_t j) const {
    ORC_CHECK(i >= 1 && i <= n1 && j >= 1 && j <= n2, "A2 index");
    return d[(size_t)((i - 1) + n1 * (j - 1))];
  }
};

// column-major (n1, n2, n3) array, 1-based
template <class T>
struct A3 {
  std::vector<T> d;
  int64_t n1 = 0, n2 = 0, n3 = 0;
  void alloc(int64_t a, int64_t b, int64_t c) {
    n1 = a;
    n2 = b;
    n3 = c;
    d.assign((size_t)(a * b * c), T(0));
  }
  void fill(T v) { std::fill(d.begin(), d.end(), v); }
  T& operator()(int64_t i, int64_t j, int64_t k) {
    ORC_CHECK(i >= 1 && i <= n1 && j >= 1 && j <= n2 && k >= 1 && k <= n3, "A3 index");
    return d[(size_t)((i - 1) + n1 * ((j - 1) + n2 * (k - 1)))];
  }
  const T& operator()(int64_t i, int64_t j, int64_t k) const {
    ORC_CHECK(i >= 1 && i <= n1 && j >= 1 && j <= n2 && k >= 1 && k <= n3, "A3 index");
    return d[(size_t)((i - 1) + n1 * ((j - 1) + n2 * (k - 1)))];
  }
};

using F1 = A1<real>;
using F3 = A3<real>;
using I1 = A1<int64_t>;
using I2 = A2<int64_t>;
using I3 = A3<int64_t>;

// Mirror of Block_t (src/Blocks.f90:13-81), hot-path members only.
struct Block {
  int64_t nx = 0, ny = 0, nz = 0;
  real dx = 0, dy = 0, dz = 0;
  real omega = 1.0;
  real derr1 = 0, derr2 = 0, derrStdSt = 0;
  int64_t nIterPcor = 0, cintp = 3;
  int64_t i_startSearch = 0, i_endSearch = -1, j_startSearch = 0, j_endSearch = -1,
          k_startSearch = 0, k_endSearch = -1;
  int64_t ibCellCount = 0, solidCellCount = 0, fluidCellCount = 0, redCellCount = 0,
          blackCellCount = 0, TSCellCount = 0;
  int64_t ibElems = 0, ibNodes = 0;
  int64_t move_check = 0, blk_mv_tag = 0;
  int64_t mk = 0, mkx1 = 0, mkx2 = 0;  // findDistnode's extreme surface nodes
  // block move (src/Search.F90:997-1370)
  int64_t move_amtx = 0, move_amty = 0, move_amtz = 0;
  int64_t cpy_x_start = 0, cpy_x_end = 0, cpy_y_start = 0, cpy_y_end = 0, cpy_z_start = 0, cpy_z_end = 0;
  int64_t cpy_x_start_mv = 0, cpy_x_end_mv = 0, cpy_y_start_mv = 0, cpy_y_end_mv = 0, cpy_z_start_mv = 0,
          cpy_z_end_mv = 0;
  // kinematics read by the forcing routines
  real xdot = 0, ydot = 0, yddot = 0;
  real thetaDot = 0, thetaDDot = 0, thetaDot1 = 0, thetaDDot1 = 0, thetaDot2 = 0,
         thetaDDot2 = 0, alphaDot = 0;
  real piv_x = 0, piv_y = 0, piv_z = 0;

  F1 deltax, deltay, deltaz, x1, y1, z1, xu, yu, zu, xv, yv, zv, xw, yw, zw, xp, yp, zp;
  A2<real> ca_uu, ck_uu, ca_vv, ck_vv, ca_ww, ck_ww, ca_uv, ck_uv, ca_uw, ck_uw, ca_vu,
      ck_vu, ca_vw, ck_vw, ca_wu, ck_wu, ca_wv, ck_wv;
  A2<real> Acx, Acy, Acz;
  F3 b, u, ut, v, vt, w, wt, p, pc, pco;
  F3 u_dum, v_dum, w_dum, p_dum;
  I3 cell, cell2, cell_n, cell_pr, nodeIdTag;
  I2 fluidIndexPtr, redCellIndexPtr, blackCellIndexPtr, TSIndexPtr, interceptedIndexPtr,
      solidIndexPtr;
  I1 nelp, nelu1, nelu2, nelv1, nelv2, nelw1, nelw2, index_ts;
  F1 xcent, ycent, zcent, cosAlpha, cosBeta, cosGamma, element_length, pNormDis, u1NormDis,
      u2NormDis, v1NormDis, v2NormDis, w1NormDis, w2NormDis, p_ghost, pt_ghost, u2_ghost,
      u2t_ghost, v2_ghost, v2t_ghost, w2_ghost, w2t_ghost, u1_ghost, u1t_ghost, v1_ghost,
      v1t_ghost, w1_ghost, w1t_ghost;
  I1 ibSurfId, ibElP1, ibElP2, ibElP3;
  F1 xnode1, ynode1, znode1;
  // body-frame nodes and their surface ids (src/ReadInput.f90:376-420), and the
  // rigid-body motion state of src/Search.F90:49-208
  F1 xnode, ynode, znode;
  I1 ibNodeId;
  real a0 = 0, bfreq = 0, yamp = 0, xshift = 0, yshift = 0, zshift = 0;
  // per-body phase lag of heave and pitch and the shared pitch phase (an
  // extension of the reference's kinematics; 0 = the reference)
  real lag = 0, lag_phase = 0;
  real xpth1 = 0, xpth2 = 0, ypth2 = 0, xchg = 0, ychg = 0, xmove = 0, ymove = 0, zmove = 0;
  real xt = 0, yt = 0, inity_cent = 0, nxty_cent = 0, initx_cent = 0, nxtx_cent = 0,
         initz_cent = 0, nxtz_cent = 0;
  // drag/lift from the stress integration (src/StressCalc.f90)
  real viscous_drag = 0, pressure_drag = 0, viscous_lift = 0, pressure_lift = 0;
  // first error raised by a routine on this block (0 = none); the reference
  // has undefined behaviour where the oracle records an error instead
  int err = 0;
};

// Mirror of Interface_t (src/Interfaces.f90:8-25).
struct Interface {
  I2 px, ux, vx, wx, py, uy, vy, wy, pz, uz, vz, wz;  // (3, n) tables
  real xintf_start = 0, xintf_end = 0, yintf_start = 0, yintf_end = 0, zintf_start = 0,
         zintf_end = 0;
  real xintf_st_new = 0, xintf_en_new = 0, yintf_st_new = 0, yintf_en_new = 0, zintf_st_new = 0,
         zintf_en_new = 0;
  int64_t a_blk = 1, b_blk = 2;
  int64_t a_msh = 1, b_msh = 2;
  int64_t cxu = 0, cyu = 0, cxp = 0, cyp = 0, cxv = 0, cyv = 0, cxw = 0, cyw = 0, czu = 0,
          czp = 0, czv = 0, czw = 0;
};

// Registry that mirrors the module globals block(:) and intfr(:) (src/modGlobal.f90:9-10).
extern std::vector<Block*> g_blocks;         // g_blocks[g-1] = block(g)
extern std::vector<Interface*> g_interfaces; // g_interfaces[g-1] = intfr(g)
inline Block& blk_of(int64_t g) { return *g_blocks[(size_t)(g - 1)]; }

enum OrcErr { ORC_OK = 0, ORC_E_NOTFOUND = -4 };

// ---- routines (each cites the reference lines it restates) ----
void allocate_arrays(Block& b);
void derive_grids(Block& b);
void non_uni_coeff(Block& b);
void coefficient_matrix(Block& b, bool is_coarse);
void ns_momentum_2order(Block& b, real deltat, real re);
void velocity_bc(Block& b, real deltat, real uc);
void solid_cell_bc(Block& b);
void solid_cell_bc_move(Block& b);
void velocity_forcing1(Block& b);
void pressure_forcing1(Block& b);
void velocity_forcing_field(Block& b);
void pressure_forcing_field(Block& b);
void velocity_forcing_ghost(Block& b);
void pressure_forcing_ghost(Block& b);
void compute_surface_norm(Block& b, int64_t inor);
void tagging_th_core(Block& b);
void selective_retagging_th(Block& b);
void cellcount_solid(Block& b);
void compute_norm_distance(Block& b);
void find_ts_cells(Block& b);
void update_velocity_newv(Block& b);
void compute_div(Block& b);
void correct_pressure(Block& b);
void correct_velocity(Block& b, real deltat);
void redblack_sor_linear(Block& b, int64_t pcItaMax, real deltat, real epsi);
void poisson_solver(int64_t pcItaMax, real epsi, real deltat, real uc, int64_t start,
                    int64_t finish, int64_t step);
void set_interface_detail(const F1& var, real s, real e, int64_t factor, I2& det,
                           int64_t& counter, int64_t starter_in);
void interface_detail(Interface& it);
void fine_block_cell();
void cellcount_solid_coarse(Block& b);
void fine_update_pc_bd();
void fine_update_newv_bd();
void fine_update_bd_mv(int64_t g);
void coarse_update();
void coarse_update_newv();
void coarse_update_pc();
void fine_update_mv(int64_t g);
void stress_calculation(Block& b, real mu_f, real rho_f);
// rigid-body motion (src/Search.F90:49-208, src/ReadInput.f90:403-420)
void node_ids_from_elements(Block& b);
void find_dist_node(Block& b);
void block_move_check(int64_t& coarse_flcnt_check);
void change_block_coords(Block& b);
void change_block_coords_interfaces(Interface& it, Block& b);
void change_block_interface(Interface& it, Block& a, Block& b);
void cellcount_solid_coarse_mv(int64_t& coarse_flcnt_check);
void tagging_th_move(Block& b, int64_t id);
void shift_surface_nodes_initial(Block& b, real aoa, real piv_pt, int64_t ita, real deltat,
                                 real dxmin, real totime);
void compute_surface_variables(Block& b, real phase_angle, real piv_pt, int64_t ita,
                               real deltat, real dxmin, real freq, real totime);

// interpolation primitives (src/Interpolation.f90:16-42)
real linear_interpolation(real x, real x0, real x1, real y0, real y1);
real bilinear_interpolation(real x, real y, real x1, real x2, real y1, real y2,
                              const real f[4]);

}  // namespace orc
