// ORACLE -- TEST INFRASTRUCTURE ONLY (see orc_core.h).
// Flat C entry points so that the Python tests can drive the oracle with
// ctypes.  Arrays are exposed in place (column-major, the Fortran layout).
#include <cstring>
#include <string>
#include <omp.h>

#include "orc_core.h"

using namespace orc;

namespace {

F1* f1_of(Block& b, const std::string& n) {
#define M(x) if (n == #x) return &b.x;
  M(deltax) M(deltay) M(deltaz) M(x1) M(y1) M(z1) M(xu) M(yu) M(zu) M(xv) M(yv) M(zv) M(xw)
  M(yw) M(zw) M(xp) M(yp) M(zp) M(xcent) M(ycent) M(zcent) M(cosAlpha) M(cosBeta) M(cosGamma)
  M(element_length) M(pNormDis) M(u1NormDis) M(u2NormDis) M(v1NormDis) M(v2NormDis)
  M(w1NormDis) M(w2NormDis) M(p_ghost) M(pt_ghost) M(u2_ghost) M(u2t_ghost) M(v2_ghost)
  M(v2t_ghost) M(w2_ghost) M(w2t_ghost) M(u1_ghost) M(u1t_ghost) M(v1_ghost) M(v1t_ghost)
  M(w1_ghost) M(w1t_ghost) M(xnode1) M(ynode1) M(znode1) M(xnode) M(ynode) M(znode)
#undef M
  return nullptr;
}
F3* f3_of(Block& b, const std::string& n) {
#define M(x) if (n == #x) return &b.x;
  M(b) M(u) M(ut) M(v) M(vt) M(w) M(wt) M(p) M(pc) M(pco)
#undef M
  return nullptr;
}
I3* i3_of(Block& b, const std::string& n) {
#define M(x) if (n == #x) return &b.x;
  M(cell) M(cell2) M(cell_n) M(cell_pr) M(nodeIdTag)
#undef M
  return nullptr;
}
I2* i2_of(Block& b, const std::string& n) {
#define M(x) if (n == #x) return &b.x;
  M(fluidIndexPtr) M(redCellIndexPtr) M(blackCellIndexPtr) M(TSIndexPtr)
  M(interceptedIndexPtr) M(solidIndexPtr)
#undef M
  return nullptr;
}
A2<real>* f2_of(Block& b, const std::string& n) {
#define M(x) if (n == #x) return &b.x;
  M(ca_uu) M(ck_uu) M(ca_vv) M(ck_vv) M(ca_ww) M(ck_ww) M(ca_uv) M(ck_uv) M(ca_uw) M(ck_uw)
  M(ca_vu) M(ck_vu) M(ca_vw) M(ck_vw) M(ca_wu) M(ck_wu) M(ca_wv) M(ck_wv) M(Acx) M(Acy) M(Acz)
#undef M
  return nullptr;
}
I1* i1_of(Block& b, const std::string& n) {
#define M(x) if (n == #x) return &b.x;
  M(nelp) M(nelu1) M(nelu2) M(nelv1) M(nelv2) M(nelw1) M(nelw2) M(index_ts) M(ibSurfId)
  M(ibElP1) M(ibElP2) M(ibElP3) M(ibNodeId)
#undef M
  return nullptr;
}
real* fs_of(Block& b, const std::string& n) {
#define M(x) if (n == #x) return &b.x;
  M(dx) M(dy) M(dz) M(omega) M(derr1) M(derr2) M(derrStdSt) M(xdot) M(ydot) M(yddot)
  M(thetaDot) M(thetaDDot) M(thetaDot1) M(thetaDDot1) M(thetaDot2) M(thetaDDot2) M(alphaDot)
  M(piv_x) M(piv_y) M(piv_z) M(viscous_drag) M(pressure_drag) M(viscous_lift) M(pressure_lift)
  M(lag) M(lag_phase) M(a0) M(bfreq) M(yamp) M(xshift) M(yshift) M(zshift) M(xpth1) M(xpth2) M(ypth2) M(xchg) M(ychg)
  M(xmove) M(ymove) M(zmove) M(xt) M(yt) M(inity_cent) M(nxty_cent) M(initx_cent) M(nxtx_cent)
#undef M
  return nullptr;
}
int64_t* is_of(Block& b, const std::string& n) {
#define M(x) if (n == #x) return &b.x;
  M(nx) M(ny) M(nz) M(nIterPcor) M(cintp) M(i_startSearch) M(i_endSearch) M(j_startSearch)
  M(j_endSearch) M(k_startSearch) M(k_endSearch) M(ibCellCount) M(solidCellCount)
  M(fluidCellCount) M(redCellCount) M(blackCellCount) M(TSCellCount) M(ibElems) M(ibNodes)
  M(move_check) M(blk_mv_tag) M(mk) M(mkx1) M(mkx2) M(move_amtx) M(move_amty) M(move_amtz)
#undef M
  return nullptr;
}

// tangents of the call arguments a run differentiates with respect to
// (lane l of the dual build): "uc", "phase_angle", "freq", "aoa", "piv_pt"
struct ArgTangent {
  std::string name;
  int lane;
  double d;
};
std::vector<ArgTangent> g_arg_tangents;

real arg(const char* name, double v) {
  real r = v;
#ifdef ORC_DUAL
  for (const ArgTangent& t : g_arg_tangents)
    if (t.name == name) r.d[t.lane] = t.d;
#else
  (void)name;
#endif
  return r;
}

// element kind of a floating-point array: 0 = double, 2 = dual number
// (value followed by kLanes tangents)
constexpr int kRealKind = kLanes ? 2 : 0;

}  // namespace

extern "C" {

// number of tangent lanes (0: the plain double build)
int orc_lanes() { return kLanes; }

// tangent lane `lane` of a named block scalar (dual build only)
int orc_set_fd(int64_t g, const char* name, int lane, double d) {
  real* p = fs_of(blk_of(g), name);
  if (!p || lane < 0 || lane >= kLanes) return -1;
#ifdef ORC_DUAL
  p->d[lane] = d;
#else
  (void)d;
#endif
  return 0;
}
double orc_get_fd(int64_t g, const char* name, int lane) {
  real* p = fs_of(blk_of(g), name);
  if (!p || lane < 0 || lane >= kLanes) return 0.0;
#ifdef ORC_DUAL
  return p->d[lane];
#else
  return 0.0;
#endif
}
// seeds the tangent of a call argument for every later call that takes it
int orc_arg_tangent(const char* name, int lane, double d) {
  if (lane < 0 || lane >= kLanes) return -1;
  g_arg_tangents.push_back({name, lane, d});
  return 0;
}
void orc_clear_arg_tangents() { g_arg_tangents.clear(); }

void orc_reset() {
  for (Block* b : g_blocks) delete b;
  for (Interface* i : g_interfaces) delete i;
  g_blocks.clear();
  g_interfaces.clear();
}

int64_t orc_block_new(int64_t nx, int64_t ny, int64_t nz) {
  Block* b = new Block();
  b->nx = nx;
  b->ny = ny;
  b->nz = nz;
  allocate_arrays(*b);
  g_blocks.push_back(b);
  return (int64_t)g_blocks.size();
}

void orc_alloc_surface(int64_t g, int64_t n_elems, int64_t n_nodes) {
  Block& b = blk_of(g);
  b.ibElems = n_elems;
  b.ibNodes = n_nodes;
  for (F1* a : {&b.xcent, &b.ycent, &b.zcent, &b.cosAlpha, &b.cosBeta, &b.cosGamma,
                &b.element_length})
    a->alloc(n_elems);
  for (I1* a : {&b.ibSurfId, &b.ibElP1, &b.ibElP2, &b.ibElP3}) a->alloc(n_elems);
  for (F1* a : {&b.xnode1, &b.ynode1, &b.znode1, &b.xnode, &b.ynode, &b.znode}) a->alloc(n_nodes);
  b.ibNodeId.alloc(n_nodes);
}

// Pointer to the storage of a named array; *n = element count, dims = extents
// (column-major), *kind = 0 for double, 1 for int64 and 2 for dual numbers
// (value followed by orc_lanes() tangents per element).  nullptr if unknown.
void* orc_array(int64_t g, const char* name, int64_t* n, int64_t dims[3], int* kind) {
  Block& b = blk_of(g);
  const std::string s(name);
  dims[0] = dims[1] = dims[2] = 1;
  if (F1* a = f1_of(b, s)) { *n = a->size(); dims[0] = *n; *kind = kRealKind; return a->d.data(); }
  if (F3* a = f3_of(b, s)) { *n = (int64_t)a->d.size(); dims[0] = a->n1; dims[1] = a->n2; dims[2] = a->n3; *kind = kRealKind; return a->d.data(); }
  if (I3* a = i3_of(b, s)) { *n = (int64_t)a->d.size(); dims[0] = a->n1; dims[1] = a->n2; dims[2] = a->n3; *kind = 1; return a->d.data(); }
  if (I2* a = i2_of(b, s)) { *n = (int64_t)a->d.size(); dims[0] = a->n1; dims[1] = a->n2; *kind = 1; return a->d.data(); }
  if (auto* a = f2_of(b, s)) { *n = (int64_t)a->d.size(); dims[0] = a->n1; dims[1] = a->n2; *kind = kRealKind; return a->d.data(); }
  if (I1* a = i1_of(b, s)) { *n = a->size(); dims[0] = *n; *kind = 1; return a->d.data(); }
  *n = 0;
  *kind = -1;
  return nullptr;
}

int orc_set_f(int64_t g, const char* name, double v) {
  real* p = fs_of(blk_of(g), name);
  if (!p) return -1;
  *p = v;
  return 0;
}
double orc_get_f(int64_t g, const char* name) {
  real* p = fs_of(blk_of(g), name);
  return p ? val(*p) : 0.0;
}
int orc_set_i(int64_t g, const char* name, int64_t v) {
  int64_t* p = is_of(blk_of(g), name);
  if (!p) return -1;
  *p = v;
  return 0;
}
int64_t orc_get_i(int64_t g, const char* name) {
  int64_t* p = is_of(blk_of(g), name);
  return p ? *p : 0;
}
double orc_linear_interpolation(double x, double x0, double x1, double y0, double y1) {
  return val(linear_interpolation(x, x0, x1, y0, y1));
}
double orc_bilinear_interpolation(double x, double y, double x1, double x2, double y1, double y2,
                                  const double* f) {
  const real fr[4] = {f[0], f[1], f[2], f[3]};
  return val(bilinear_interpolation(x, y, x1, x2, y1, y2, fr));
}

int orc_err(int64_t g) { return blk_of(g).err; }
// threads of the OpenMP loops (1 = the serial loops)
void orc_set_threads(int n) { omp_set_num_threads(n < 1 ? 1 : n); }
int orc_get_threads(void) { return omp_get_max_threads(); }
void orc_clear_err(int64_t g) { blk_of(g).err = 0; }

void orc_derive_grids(int64_t g) { derive_grids(blk_of(g)); }
void orc_non_uni_coeff(int64_t g) { non_uni_coeff(blk_of(g)); }
void orc_coefficient_matrix(int64_t g, int is_coarse) { coefficient_matrix(blk_of(g), is_coarse != 0); }
void orc_ns_momentum(int64_t g, double dt, double re) { ns_momentum_2order(blk_of(g), dt, re); }
void orc_velocity_bc(int64_t g, double dt, double uc) { velocity_bc(blk_of(g), dt, arg("uc", uc)); }
void orc_solid_cell_bc(int64_t g) { solid_cell_bc(blk_of(g)); }
void orc_solid_cell_bc_move(int64_t g) { solid_cell_bc_move(blk_of(g)); }
void orc_velocity_forcing1(int64_t g) { velocity_forcing1(blk_of(g)); }
void orc_pressure_forcing1(int64_t g) { pressure_forcing1(blk_of(g)); }
void orc_velocity_forcing_field(int64_t g) { velocity_forcing_field(blk_of(g)); }
void orc_pressure_forcing_field(int64_t g) { pressure_forcing_field(blk_of(g)); }
void orc_velocity_forcing_ghost(int64_t g) { velocity_forcing_ghost(blk_of(g)); }
void orc_pressure_forcing_ghost(int64_t g) { pressure_forcing_ghost(blk_of(g)); }
void orc_compute_surface_norm(int64_t g, int64_t inor) { compute_surface_norm(blk_of(g), inor); }
void orc_node_ids_from_elements(int64_t g) { node_ids_from_elements(blk_of(g)); }
void orc_find_dist_node(int64_t g) { find_dist_node(blk_of(g)); }
// the block-move stage of app/main.F90:178-230 after computeSurfaceVariables:
// block_move_check, change_block_coords, change_block_coords_interfaces,
// change_block_interface, fine_block_cell + cellCount_solid_coarse_mv (the
// caller runs computeSurfaceNorm next, then orc_tagging_th_move)
void orc_block_move_stage() {
  int64_t flag = 0;
  block_move_check(flag);
  for (size_t g = 1; g < g_blocks.size(); ++g) change_block_coords(*g_blocks[g]);
  for (Interface* it : g_interfaces) change_block_coords_interfaces(*it, blk_of(it->b_blk));
  for (Interface* it : g_interfaces) change_block_interface(*it, blk_of(it->a_blk), blk_of(it->b_blk));
  fine_block_cell();
  cellcount_solid_coarse_mv(flag);
}
void orc_tagging_th_move(int64_t g) { tagging_th_move(blk_of(g), g); }
void orc_shift_surface_nodes_initial(int64_t g, double aoa, double piv_pt, int64_t ita, double deltat,
                                     double dxmin, double totime) {
  shift_surface_nodes_initial(blk_of(g), arg("aoa", aoa), arg("piv_pt", piv_pt), ita, deltat, dxmin, totime);
}
void orc_compute_surface_variables(int64_t g, double phase_angle, double piv_pt, int64_t ita,
                                   double deltat, double dxmin, double freq, double totime) {
  compute_surface_variables(blk_of(g), arg("phase_angle", phase_angle), arg("piv_pt", piv_pt), ita, deltat,
                            dxmin, arg("freq", freq), totime);
}
void orc_tagging_th_core(int64_t g) { tagging_th_core(blk_of(g)); }
void orc_selective_retagging(int64_t g) { selective_retagging_th(blk_of(g)); }
void orc_cellcount_solid(int64_t g) { cellcount_solid(blk_of(g)); }
void orc_cellcount_solid_coarse(int64_t g) { cellcount_solid_coarse(blk_of(g)); }
void orc_compute_norm_distance(int64_t g) { compute_norm_distance(blk_of(g)); }
void orc_find_ts_cells(int64_t g) { find_ts_cells(blk_of(g)); }
void orc_update_velocity_newv(int64_t g) { update_velocity_newv(blk_of(g)); }
void orc_compute_div(int64_t g) { compute_div(blk_of(g)); }
void orc_correct_pressure(int64_t g) { correct_pressure(blk_of(g)); }
void orc_correct_velocity(int64_t g, double dt) { correct_velocity(blk_of(g), dt); }
void orc_redblack_sor(int64_t g, int64_t itmax, double dt, double epsi) {
  redblack_sor_linear(blk_of(g), itmax, dt, epsi);
}
void orc_poisson_solver(int64_t itmax, double epsi, double dt, double uc) {
  poisson_solver(itmax, epsi, dt, arg("uc", uc), 1, (int64_t)g_blocks.size(), 1);
}
void orc_fine_block_cell() { fine_block_cell(); }
void orc_fine_update_pc_bd() { fine_update_pc_bd(); }
void orc_fine_update_newv_bd() { fine_update_newv_bd(); }
void orc_fine_update_bd_mv(int64_t g) { fine_update_bd_mv(g); }
void orc_coarse_update() { coarse_update(); }
void orc_coarse_update_newv() { coarse_update_newv(); }
void orc_coarse_update_pc() { coarse_update_pc(); }
void orc_fine_update_mv(int64_t g) { fine_update_mv(g); }
void orc_stress_calculation(int64_t g, double mu_f, double rho_f) {
  stress_calculation(blk_of(g), mu_f, rho_f);
}

int64_t orc_interface_new(int64_t a, int64_t b, int64_t a_msh, int64_t b_msh, double xs,
                          double xe, double ys, double ye, double zs, double ze) {
  Interface* it = new Interface();
  it->a_blk = a;
  it->b_blk = b;
  it->a_msh = a_msh;
  it->b_msh = b_msh;
  it->xintf_start = xs; it->xintf_end = xe;
  it->yintf_start = ys; it->yintf_end = ye;
  it->zintf_start = zs; it->zintf_end = ze;
  g_interfaces.push_back(it);
  interface_detail(*it);
  return (int64_t)g_interfaces.size();
}

// interface table access: name in {px,py,pz,ux,...,wz}; returns pointer to
// the (3, n) table and its counter.
int64_t* orc_interface_table(int64_t ih, const char* name, int64_t* ncols, int64_t* counter) {
  Interface& it = *g_interfaces[(size_t)(ih - 1)];
  const std::string s(name);
  struct E { const char* n; I2* t; int64_t c; } es[] = {
      {"px", &it.px, it.cxp}, {"py", &it.py, it.cyp}, {"pz", &it.pz, it.czp},
      {"ux", &it.ux, it.cxu}, {"uy", &it.uy, it.cyu}, {"uz", &it.uz, it.czu},
      {"vx", &it.vx, it.cxv}, {"vy", &it.vy, it.cyv}, {"vz", &it.vz, it.czv},
      {"wx", &it.wx, it.cxw}, {"wy", &it.wy, it.cyw}, {"wz", &it.wz, it.czw}};
  for (auto& e : es)
    if (s == e.n) {
      *ncols = e.t->n2;
      *counter = e.c;
      return e.t->d.data();
    }
  *ncols = 0;
  *counter = 0;
  return nullptr;
}

}  // extern "C"
