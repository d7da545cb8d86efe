// C-ABI entry points, part 2: interfaces, poissonSolver orchestration, the
// whole-step driver and the named read-back of device arrays.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "bcfd_host.h"

namespace bcfd {
namespace {

#define TRY(x) do { int _r = (x); if (_r) return _r; } while (0)

// set_interface_detail, src/InterfaceDetail.f90:168-241.  var is the coarse
// coordinate array (1-based meaning, var[i-1]); the table is (3, n) int64.
void set_interface_detail(const std::vector<double>& var, double s, double e, int64_t factor,
                          std::vector<int64_t>& det, int64_t& counter, int64_t starter) {
  const int64_t n = (int64_t)var.size();
  int64_t xx1 = 0, xx2 = 0;
  for (int64_t i = 1; i <= n; ++i)
    if (var[i - 1] > s) {
      xx1 = i;
      break;
    }
  for (int64_t i = xx1; i <= n; ++i)
    if (var[i - 1] > e) {
      xx2 = i - 1;
      break;
    }
  det.clear();
  auto put = [&](int64_t a, int64_t b, int64_t c) {
    det.push_back(a);
    det.push_back(b);
    det.push_back(c);
  };
  put(xx1 - 1, starter - 1, starter - 1);
  int64_t ender = starter + factor - 1;
  counter = 2;
  for (;;) {
    put(xx1, starter, ender);
    starter = ender + 1;
    ender = ender + factor;
    counter = counter + 1;
    xx1 = xx1 + 1;
    if (xx1 > xx2) break;
  }
  put(xx2 + 1, starter, starter);
}

int upload_iface(HostInterface* it) {
  size_t tot = 0;
  for (int t = 0; t < 12; ++t) {
    it->off[t] = (int64_t)tot;
    tot += it->tab[t].size();
  }
  std::vector<int> h(tot);
  for (int t = 0; t < 12; ++t)
    for (size_t q = 0; q < it->tab[t].size(); ++q) h[it->off[t] + q] = (int)it->tab[t][q];
  if (it->dtab) cudaFree(it->dtab);
  BCFD_CUDA(cudaMalloc(&it->dtab, std::max<size_t>(tot, 1) * sizeof(int)));
  BCFD_CUDA(cudaMemcpyAsync(it->dtab, h.data(), tot * sizeof(int), cudaMemcpyHostToDevice, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  return 0;
}

int sync_err(HostBlock* hb) { return take_block_error(hb); }

// Every index the coupling kernels touch must lie inside both blocks' arrays;
// the reference trusts its input files here, the GPU path refuses instead.
bool iface_in_bounds(const HostInterface* it, const HostBlock* A, const HostBlock* B) {
  const int na[3] = {A->d.d.NX, A->d.d.NY, A->d.d.NZ};
  const int nb[3] = {B->d.d.NX, B->d.d.NY, B->d.d.NZ};
  for (int comp = 0; comp < 4; ++comp)
    for (int ax = 0; ax < 3; ++ax) {
      const int t = 3 * comp + ax;
      const bool stag = comp == ax + 1;  // u along x, v along y, w along z
      const int64_t cnt = it->counter[t];
      const auto& T = it->tab[t];
      if ((int64_t)T.size() != 3 * cnt || cnt < 3) return false;
      auto e = [&](int r, int64_t q) { return T[(size_t)(3 * (q - 1) + r - 1)]; };
      const int64_t ga = na[ax] + (stag ? 1 : 0), gb = nb[ax] + (stag ? 1 : 0);  // grid lengths
      for (int64_t q = 1; q <= cnt; ++q) {
        const int64_t loc = e(1, q), s = e(2, q), f = e(3, q);
        // coarse -> fine faces: donors loc-1..loc+1 (loc-2..loc on the staggered axis)
        if (loc - 1 < 1 || loc + 1 > ga) return false;
        if ((stag ? loc - 2 : loc - 1) < 1 || (stag ? loc : loc + 1) > na[ax]) return false;
        if (s < 1 || f > gb || s > f) return false;
        if ((stag ? s - 1 : s) < 1 || (stag ? f - 1 : f) > nb[ax]) return false;
        if (q >= 2 && q <= cnt - 1 && f > nb[ax]) return false;  // cell_n(s) of fineUpdate_mv
        // fine -> coarse restriction entries cintp..cnt-cintp
        if (q >= 3 && q <= cnt - 3) {
          const int64_t l = stag ? f : (s + f - 1) / 2;
          const int64_t lo = stag ? l - 2 : l, hi = stag ? l - 1 : l + 1;
          if (lo < 1 || hi > nb[ax] || (stag ? l - 1 : l) < 1 || (stag ? l : l + 1) > gb) return false;
          if ((stag ? loc - 1 : loc) < 1 || loc > ga || (stag ? loc - 1 : loc) > na[ax]) return false;
        }
      }
    }
  return true;
}

// all registered blocks in registration order
std::vector<std::pair<bcfd_handle, HostBlock*>> blocks() {
  std::vector<std::pair<bcfd_handle, HostBlock*>> v;
  for (size_t q = 0; q < lib().blocks.size(); ++q)
    if (lib().blocks[q]) v.push_back({(bcfd_handle)(q + 1), lib().blocks[q]});
  return v;
}

constexpr int kUVW[3] = {1, 2, 3};
constexpr int kPUVW[4] = {0, 1, 2, 3};

int fine_update_newv_bd() {
  for (HostInterface* it : lib().ifs)
    if (it) TRY(launch_face_fill_set(it, kUVW, 3, 0));
  return 0;
}
constexpr int kP[1] = {0};

int fine_update_pc_bd() {
  for (HostInterface* it : lib().ifs)
    if (it) TRY(launch_face_fill_set(it, kP, 1, 1));
  return 0;
}
int fine_update_bd_mv(HostInterface* it) { return launch_face_fill_set(it, kPUVW, 4, 2); }
int coarse_update() {
  for (HostInterface* it : lib().ifs)
    if (it) TRY(launch_restrict_set(it, kPUVW, 4, 2));
  return 0;
}
int coarse_update_newv() {
  for (HostInterface* it : lib().ifs)
    if (it) TRY(launch_restrict_set(it, kUVW, 3, 0));
  return 0;
}
int coarse_update_pc() {
  for (HostInterface* it : lib().ifs)
    if (it) TRY(launch_restrict_set(it, kP, 1, 1));
  return 0;
}

struct SolveCfg {
  int64_t itmax;
  double epsi, dt, uc;
  int precision;
  double div_tol;
};

// precision 0: FP64, the reference's stop test (drop-in arithmetic);
// 1: FP32 SOR + FP64 defect correction to div_tol; 2: FP64 SOR (reference
// sweeps) to div_tol; 3: division-free FP64 SOR to div_tol.  One batched
// launch over several blocks when batching.
int sor_set(const std::vector<HostBlock*>& v, const SolveCfg& c) {
  if (c.precision == 1) return launch_sor_mixed_set(v, c.itmax, c.dt, c.div_tol);
  if (c.precision >= 2) return launch_sor_set(v, c.itmax, c.dt, c.epsi, c.div_tol, c.precision == 3);
  return launch_sor_set(v, c.itmax, c.dt, c.epsi, 0.0);
}

// poissonSolver, src/PcorVcor.F90:22-220, over the blocks with 1-based
// registration index in [start, finish] by step; no host round trip.  The
// blocks are independent between the interface updates, so each per-block
// phase runs over all of them at once (the reference's per-block loops of
// :86-129 and :160-214 in one launch per phase).
int poisson(const SolveCfg& c, int start, int finish, int step) {
  auto all = blocks();
  auto in = [&](bcfd_handle g) { return g >= start && g <= finish && (g - start) % step == 0; };
  std::vector<HostBlock*> set, fine, first;
  for (auto& [g, hb] : all)
    if (in(g)) {
      set.push_back(hb);
      (g == 1 ? first : fine).push_back(hb);
    }
  phase_mark(PH_CORRECTION);
  // the reference starts every solve from pc = 0; a residual-target solve may
  // start from the last correction instead (same stop, same boundary data)
  const bool warm = lib().warm_start && c.precision >= 1;
  for (HostBlock* hb : set) TRY(launch_zero_poisson(hb, warm));
  phase_mark(PH_COUPLING);
  TRY(fine_update_newv_bd());
  TRY(coarse_update_newv());
  phase_mark(PH_CORRECTION);
  TRY(launch_compute_div(set, c.precision >= 1));
  phase_mark(PH_SOLVE);
  TRY(sor_set(fine, c));
  phase_mark(PH_COUPLING);
  TRY(coarse_update_pc());
  phase_mark(PH_SOLVE);
  TRY(sor_set(first, c));
  phase_mark(PH_COUPLING);
  TRY(fine_update_pc_bd());
  phase_mark(PH_SOLVE);
  TRY(sor_set(fine, c));
  phase_mark(PH_COUPLING);
  TRY(coarse_update_pc());
  phase_mark(PH_CORRECTION);
  TRY(launch_correct_pressure(set));
  TRY(launch_correct_velocity(set, c.dt));
  // the divergence the solve leaves behind (measurement, not in the reference)
  TRY(launch_max_div(set, true));
  for (HostBlock* hb : first) TRY(launch_velocity_bc(hb, c.dt, c.uc));
  TRY(launch_steady_state(set, c.dt));
  TRY(launch_copy_t_to_n(set));
  phase_mark(PH_COUPLING);
  for (HostInterface* it : lib().ifs)
    if (it && get_block(it->b)) TRY(fine_update_bd_mv(it));
  TRY(coarse_update());
  return 0;
}

// One time step in the phase order of app/main.F90:129-265 for blocks whose
// roles are set by bcfd_block_set_role.  A block with domain BCs gets
// velocityBC before and after its IB forcing (main.F90:139-145); body blocks
// get pressureForcing1 and the per-step re-Search of main.F90:232-263.  The
// body is stationary: the kinematics / block-move stage of main.F90:169-230
// leaves the geometry unchanged and is not run.
// ---------------------------------------------------------------------------
// Fine-block moves (app/main.F90:178-230 with src/Search.F90:916-1461): a
// fine block whose moving surface comes within fixed margins of its
// interface box shifts by whole cells, a multiple of the refinement factor.
// The scalar decisions run on the host as the reference's do; the fields,
// tags and lists move on the device.
// ---------------------------------------------------------------------------
int64_t round_move(int64_t m, int64_t factor) {
  if (std::llabs(m) < factor) return m < 0 ? -factor : factor;
  if (m < 0) return m + std::llabs(m) % factor;
  return m - std::llabs(m) % factor;
}

// first 1-based index i in [from, n] with v(i) > s; `keep` when there is none
int64_t first_above(const std::vector<double>& v, int64_t from, int64_t n, double s, int64_t keep) {
  for (int64_t i = std::max<int64_t>(from, 1); i <= n; ++i)
    if (v[(size_t)i - 1] > s) return i;
  return keep;
}

// block_move_check's trigger (src/Search.F90:1020-1030): the moving surface
// within the margins of its fine block's interface box.  The surface nodes
// mk and mkx1 are evaluated on the host from the staged placement (the node
// kernel's own arithmetic), so the decision needs no device read.
bool move_triggered(const HostBlock* c, const HostInterface* it, const HostBlock* fb, double* xmk1_out,
                    bool* ytrig_out) {
  const BodyMotion& m = fb->motion;
  const double mg1 = 3.0 * c->dx;  // cintp * block(1)%dx
  const double marginx = 4.5 * mg1, marginy = 5 * mg1, marginz = 1.52 * mg1;
  double xq, yq, zq, ymk, xmk1;
  staged_node(fb, fb->mk, &xq, &ymk, &zq);
  staged_node(fb, fb->mkx1, &xmk1, &yq, &zq);
  const double yval_up = std::fmax(ymk, m.nxty_cent + 0.02), yval_dw = std::fmin(ymk, m.nxty_cent - 0.02);
  const double piv_z = fb->kin.piv_z;
  const double* box = it->box;  // xs, xe, ys, ye, zs, ze
  const bool ytrig = std::fabs(yval_dw - box[2]) <= marginy || std::fabs(yval_up - box[3]) <= marginy;
  if (xmk1_out) *xmk1_out = xmk1;
  if (ytrig_out) *ytrig_out = ytrig;
  return std::fabs(xmk1 - box[0]) <= marginx || std::fabs(piv_z - box[4]) <= marginz ||
         std::fabs(piv_z - box[5]) <= marginz || ytrig;
}

bool movable(const HostBlock* fb) {
  return fb && fb->motion.on && fb->mk >= 1 && fb->mkx1 >= 1 && !fb->node_id_host.empty();
}

// a staged step that will move a fine block (such a step runs eagerly)
bool any_move_pending() {
  HostBlock* c = get_block(1);
  if (!c) return false;
  for (HostInterface* it : lib().ifs) {
    if (!it) continue;
    HostBlock* fb = get_block(it->b);
    if (movable(fb) && move_triggered(c, it, fb, nullptr, nullptr)) return true;
  }
  return false;
}

// block_move_check, change_block_coords, change_block_coords_interfaces,
// change_block_interface, fine_block_cell and cellCount_solid_coarse_mv
int block_move_stage() {
  HostBlock* c = get_block(1);
  if (!c) return 0;
  int64_t flag = 0;
  struct Moved {
    HostInterface* it;
    HostBlock* fb;
    double box_new[6];
  };
  std::vector<Moved> moved;
  for (HostInterface* it : lib().ifs) {
    if (!it) continue;
    HostBlock* fb = get_block(it->b);
    if (!movable(fb)) continue;
    BodyMotion& m = fb->motion;
    const double mg1 = 3.0 * c->dx;  // cintp * block(1)%dx
    const double marginx = 4.5 * mg1;
    const int64_t factor = it->b_msh / it->a_msh;
    const double piv_z = fb->kin.piv_z;
    double* box = it->box;  // xs, xe, ys, ye, zs, ze
    int64_t* amt = fb->move_amt;
    amt[0] = amt[1] = amt[2] = 0;
    double xmk1 = 0.0;
    bool ytrig = false;
    if (!move_triggered(c, it, fb, &xmk1, &ytrig)) continue;
    fb->move_check = 1;
    fb->blk_mv_tag = 1;
    flag = 1;
    if (ytrig) {
      amt[1] = round_move((int64_t)std::floor((m.nxty_cent - m.inity_cent) / fb->dy), factor);
      m.inity_cent = m.nxty_cent;
    }
    if (std::fabs(xmk1 - box[0]) < marginx) {
      amt[0] = round_move((int64_t)std::floor((m.nxtx_cent - m.initx_cent) / fb->dx) - factor, factor);
      m.initx_cent = m.nxtx_cent;
    }
    if (std::fabs(piv_z - box[4]) < (0.500 - 0.410 - mg1) || std::fabs(piv_z - box[5]) < (0.600 - 0.500 - mg1)) {
      amt[2] = round_move((int64_t)std::floor((m.nxtz_cent - m.initz_cent) / fb->dz), factor);
      m.initz_cent = m.nxtz_cent;
    }
    const double ch[3] = {amt[0] * fb->dx, amt[1] * fb->dy, amt[2] * fb->dz};
    Moved mv{it, fb, {0, 0, 0, 0, 0, 0}};
    for (int a = 0; a < 3; ++a) {
      mv.box_new[2 * a] = std::fmax(box[2 * a], box[2 * a] + ch[a]);
      mv.box_new[2 * a + 1] = std::fmin(box[2 * a + 1], box[2 * a + 1] + ch[a]);
      box[2 * a] = box[2 * a] + ch[a];
      box[2 * a + 1] = box[2 * a + 1] + ch[a];
    }
    // the old indices whose centres lie in the overlap of the old and new boxes
    const std::vector<double>* cen[3] = {&fb->xp, &fb->yp, &fb->zp};
    const int64_t npa[3] = {fb->d.d.NX, fb->d.d.NY, fb->d.d.NZ};
    for (int a = 0; a < 3; ++a) {
      fb->cpy[2 * a] = first_above(*cen[a], 1, npa[a], mv.box_new[2 * a], fb->cpy[2 * a]);
      fb->cpy[2 * a + 1] =
          first_above(*cen[a], fb->cpy[2 * a], npa[a], mv.box_new[2 * a + 1], fb->cpy[2 * a + 1] + 1) - 1;
    }
    const size_t np = (size_t)fb->d.d.npts();
    if (!fb->mv_dum) {
      void* p = nullptr;
      if (cudaMalloc(&p, 4 * np * sizeof(double)) != cudaSuccess) return BCFD_E_NOMEM;
      fb->allocs.push_back(p);
      fb->mv_dum = static_cast<double*>(p);
      lib().gen++;
    }
    const double* src[4] = {fb->d.u, fb->d.v, fb->d.w, fb->d.p};
    for (int q = 0; q < 4; ++q)
      BCFD_CUDA(cudaMemcpyAsync(fb->mv_dum + q * np, src[q], np * sizeof(double), cudaMemcpyDeviceToDevice,
                                stream()));
    moved.push_back(mv);
  }
  if (!flag) return 0;
  // change_block_coords
  for (Moved& mv : moved)
    TRY(shift_block_grid(mv.fb, mv.fb->move_amt[0] * mv.fb->dx, mv.fb->move_amt[1] * mv.fb->dy,
                         mv.fb->move_amt[2] * mv.fb->dz));
  // change_block_coords_interfaces: cell_n, the new index ranges, the fields
  for (Moved& mv : moved) {
    HostBlock* fb = mv.fb;
    TRY(launch_mark_cell_n(fb, mv.box_new));
    const std::vector<double>* cen[3] = {&fb->xp, &fb->yp, &fb->zp};
    const int64_t npa[3] = {fb->d.d.NX, fb->d.d.NY, fb->d.d.NZ};
    for (int a = 0; a < 3; ++a) {
      fb->cpy_mv[2 * a] = first_above(*cen[a], 1, npa[a], mv.box_new[2 * a], fb->cpy_mv[2 * a]);
      fb->cpy_mv[2 * a + 1] =
          first_above(*cen[a], fb->cpy_mv[2 * a], npa[a], mv.box_new[2 * a + 1], fb->cpy_mv[2 * a + 1] + 1) - 1;
    }
    TRY(launch_move_fields(fb, fb->mv_dum));
  }
  // change_block_interface: the coarse indices of the tables shift by the
  // move in coarse cells
  for (Moved& mv : moved) {
    HostInterface* it = mv.it;
    const int64_t factor = it->b_msh / it->a_msh;
    for (int t = 0; t < 12; ++t) {
      const int64_t inc = mv.fb->move_amt[t % 3] / factor;
      for (int64_t q = 0; q < it->counter[t]; ++q) it->tab[t][(size_t)(3 * q)] += inc;
    }
    HostBlock* A = get_block(it->a);
    if (!A || !iface_in_bounds(it, A, mv.fb)) return BCFD_E_STATE;  // moved out of the coarse block
    TRY(upload_iface(it));
  }
  // fine_block_cell and cellCount_solid_coarse_mv (the coarse tags are the
  // same as before when nothing moved, so both run only after a move)
  TRY(launch_fine_block_cell(c, nullptr, true));
  for (HostInterface* it : lib().ifs)
    if (it && it->a == 1) TRY(launch_fine_block_cell(c, it, false));
  TRY(launch_cellcount(c, true));
  return 0;
}

// The host part of a step, run before its launches (and outside a captured
// step): app/main.F90:130-131, then the kinematics of every moving body,
// staged in device memory for the step's node kernel.  The kinematics depend
// only on the loop counters, never on the flow, so evaluating them before the
// step's first half gives the values the reference computes after it.
int step_begin(const bcfd_step_config& cfg) {
  Lib& L = lib();
  L.ita = L.ita + 1;
  L.totime = L.totime + cfg.deltat;
  for (auto& [g, hb] : blocks())
    if (hb->motion.on)
      TRY(stage_surface_variables(hb, L.phase_angle, L.piv_pt, L.ita, cfg.deltat, L.dxmin, L.freq, L.totime));
  return 0;
}

// The device part of a step (everything a captured step holds); a step whose
// staged motion moves a fine block runs it eagerly.
int step_body(const bcfd_step_config& cfg) {
  SolveCfg c{cfg.pc_ita_max, cfg.epsi, cfg.deltat, cfg.uc, cfg.precision, cfg.div_tol};
  auto all = blocks();
  Lib& L = lib();
  std::vector<HostBlock*> every;
  for (auto& [g, hb] : all) every.push_back(hb);
  // nsMomentum2order of every block in one launch (blocks are independent)
  phase_mark(PH_MOMENTUM);
  TRY(launch_momentum(every, cfg.deltat, cfg.re, cfg.precision == 1));
  for (auto& [g, hb] : all) {
    if (hb->is_coarse) {
      phase_mark(PH_MOMENTUM);
      TRY(launch_velocity_bc(hb, cfg.deltat, cfg.uc));
    }
    if (hb->has_body) {
      phase_mark(PH_FORCING);
      TRY(launch_solid_bc(hb, false));
      TRY(launch_forcing_velocity(hb, 0));
    }
    if (hb->is_coarse) {
      phase_mark(PH_MOMENTUM);
      TRY(launch_velocity_bc(hb, cfg.deltat, cfg.uc));
    }
  }
  TRY(poisson(c, 1, (int)lib().blocks.size(), 1));
  phase_mark(PH_FORCING);
  for (auto& [g, hb] : all)
    if (hb->has_body) TRY(launch_forcing_pressure(hb, 0));
  phase_mark(PH_SEARCH);
  // moving bodies (app/main.F90:169-176, 213-215): the staged kinematics
  // take effect and the nodes move
  bool moving = false;
  for (auto& [g, hb] : all)
    if (hb->motion.on) {
      hb->blk_mv_tag = 0;
      TRY(apply_surface_variables(hb));
      moving = true;
    }
  // the fine-block moves (main.F90:178-211), then the normals, then the
  // re-tagging of the moved blocks (tagging_th_move, :226-230)
  bool ifaces = false;
  for (HostInterface* it : L.ifs) ifaces |= it != nullptr;
  if (moving && ifaces) TRY(block_move_stage());
  for (auto& [g, hb] : all)
    if (hb->motion.on) TRY(launch_surface_norm(hb, L.inor));
  if (moving && ifaces)
    for (auto& [g, hb] : all) {
      if (g == 1 || hb->move_check != 1) continue;
      TRY(launch_tagging(hb));
      for (HostInterface* it : L.ifs)
        if (it && it->b == g) {
          TRY(launch_fine_update_mv(it));
          TRY(fine_update_bd_mv(it));
        }
    }
  for (auto& [g, hb] : all) {
    if (!hb->has_body) continue;
    // app/main.F90:238-239: a block that moved this step was re-tagged whole
    // (blk_mv_tag = 1 skips the selective pass), then the tag is cleared
    if (hb->blk_mv_tag == 0) TRY(launch_retagging(hb));
    hb->blk_mv_tag = 0;
    TRY(launch_cellcount(hb, false));
    if (hb->move_check == 1) {
      TRY(launch_solid_bc(hb, true));
      TRY(launch_copy_n_to_t(hb));
    }
    hb->move_check = 0;
    TRY(launch_norm_distance(hb));
    TRY(launch_find_ts(hb));
    phase_mark(PH_FORCING_FIELD);
    TRY(launch_forcing_velocity(hb, 1));
    TRY(launch_forcing_pressure(hb, 1));
    TRY(launch_forcing_velocity(hb, 2));
    TRY(launch_forcing_pressure(hb, 2));
    phase_mark(PH_SEARCH);
  }
  return 0;
}

int step_once(const bcfd_step_config& cfg) {
  TRY(step_begin(cfg));
  return step_body(cfg);
}

// Everything a captured step's launches depend on: the step configuration,
// every block's device view (all device pointers and scalars the kernels
// receive) and host-side switches, the interfaces' device tables, and the
// generation of the scratch buffers.  A different key means a new capture.
std::vector<unsigned char> step_key(const bcfd_step_config& c) {
  std::vector<unsigned char> k;
  auto put = [&](const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    k.insert(k.end(), b, b + n);
  };
  put(&c.deltat, sizeof c.deltat);
  put(&c.re, sizeof c.re);
  put(&c.uc, sizeof c.uc);
  put(&c.epsi, sizeof c.epsi);
  put(&c.pc_ita_max, sizeof c.pc_ita_max);
  put(&c.precision, sizeof c.precision);
  put(&c.div_tol, sizeof c.div_tol);
  const Lib& L = lib();
  put(&L.gen, sizeof L.gen);
  put(&L.batch, sizeof L.batch);
  put(&L.wait_limit_ns, sizeof L.wait_limit_ns);
  put(&L.warm_start, sizeof L.warm_start);
  for (const HostBlock* hb : L.blocks) {
    const unsigned char none = 0;
    if (!hb) { put(&none, 1); continue; }
    put(&hb->d, sizeof hb->d);
    const int sw[11] = {hb->is_coarse, hb->has_body, (int)hb->move_check, (int)hb->blk_mv_tag, hb->dc_inner,
                        hb->dc_variant, hb->solve_threads, hb->solve_ctas_per_sm, hb->solve_sync,
                        hb->dc_threads, hb->dc_ctas_per_sm};
    put(sw, sizeof sw);
    put(&hb->dc_omega, sizeof hb->dc_omega);
    put(&hb->omega, sizeof hb->omega);
    put(&hb->bar, sizeof hb->bar);
    put(&hb->prog, sizeof hb->prog);
  }
  for (const HostInterface* it : L.ifs) {
    const unsigned char none = 0;
    if (!it) { put(&none, 1); continue; }
    put(&it->a, sizeof it->a);
    put(&it->b, sizeof it->b);
    put(&it->dtab, sizeof it->dtab);
    put(it->counter, sizeof it->counter);
    put(it->off, sizeof it->off);
    put(it->box, sizeof it->box);
  }
  return k;
}

// n time steps as replays of one captured step.  When the key changed, the
// first step runs eagerly (one-time allocations and host-side state changes
// happen there, outside any capture), then one step is captured, not run.
int run_steps_graph(const bcfd_step_config& cfg, int64_t n) {
  Lib& L = lib();
  for (int64_t done = 0; done < n; ++done) {
    TRY(step_begin(cfg));
    // a fine-block move changes grids, tables and launch shapes: eager
    if (any_move_pending()) {
      TRY(step_body(cfg));
      continue;
    }
    const std::vector<unsigned char> key = step_key(cfg);
    if (!L.step_graph || key != L.step_key) {
      if (L.step_graph) cudaGraphExecDestroy(L.step_graph);
      L.step_graph = nullptr;
      L.step_key.clear();
      if (key != L.eager_key) {
        // the first step under a new key runs eagerly (one-time allocations);
        // the key it leaves is the one captured next
        TRY(step_body(cfg));
        L.eager_key = step_key(cfg);
        continue;
      }
      cudaGraph_t g = nullptr;
      const int64_t k0 = L.launches;
      BCFD_CUDA(cudaStreamBeginCapture(stream(), cudaStreamCaptureModeRelaxed));
      const int r = step_body(cfg);
      const cudaError_t e = cudaStreamEndCapture(stream(), &g);
      if (r) {
        if (g) cudaGraphDestroy(g);
        return r;
      }
      BCFD_CUDA(e);
      const cudaError_t ei = cudaGraphInstantiate(&L.step_graph, g, 0);
      cudaGraphDestroy(g);
      BCFD_CUDA(ei);
      L.step_kernels = L.launches - k0;
      L.launches = k0;
      L.step_key = key;
    }
    BCFD_CUDA(cudaGraphLaunch(L.step_graph, stream()));
    L.launches += L.step_kernels;
    for (auto& [g, hb] : blocks()) hb->staged = false;  // applied by the replay
  }
  return 0;
}

}  // namespace

int run_one_step(const bcfd_step_config& cfg) { return step_once(cfg); }

}  // namespace bcfd

using namespace bcfd;

#define LOCK() ::bcfd::LibLock _lk

extern "C" {

int bcfd_interface_create(bcfd_handle a, bcfd_handle b, int64_t a_msh, int64_t b_msh,
                          const double* box, bcfd_handle* out) {
  LOCK();
  HostBlock* A = get_block(a);
  HostBlock* B = get_block(b);
  if (!A || !B) return BCFD_E_HANDLE;
  if (!box || !out || a_msh <= 0 || b_msh <= 0 || b_msh % a_msh) return BCFD_E_ARG;
  HostInterface* it = new HostInterface();
  it->a = a;
  it->b = b;
  it->a_msh = a_msh;
  it->b_msh = b_msh;
  std::copy(box, box + 6, it->box);
  const int64_t f = b_msh / a_msh;
  const std::vector<double>* g[12] = {&A->xp, &A->yp, &A->zp, &A->xu, &A->yu, &A->zu,
                                      &A->xv, &A->yv, &A->zv, &A->xw, &A->yw, &A->zw};
  const int starter[12] = {2, 2, 2, 3, 2, 2, 2, 3, 2, 2, 2, 3};
  for (int t = 0; t < 12; ++t) {
    const int ax = t % 3;
    set_interface_detail(*g[t], box[2 * ax], box[2 * ax + 1], f, it->tab[t], it->counter[t], starter[t]);
  }
  if (!iface_in_bounds(it, A, B)) {
    delete it;
    return BCFD_E_ARG;
  }
  int r = upload_iface(it);
  if (r) {
    delete it;
    return r;
  }
  lib().ifs.push_back(it);
  *out = (bcfd_handle)lib().ifs.size();
  return 0;
}

int bcfd_interface_table(bcfd_handle h, const char* name, int64_t* out, int64_t n, int64_t* counter) {
  LOCK();
  HostInterface* it = get_iface(h);
  if (!it) return BCFD_E_HANDLE;
  static const char* names[12] = {"px", "py", "pz", "ux", "uy", "uz", "vx", "vy", "vz", "wx", "wy", "wz"};
  for (int t = 0; t < 12; ++t)
    if (name && std::strcmp(name, names[t]) == 0) {
      if (counter) *counter = it->counter[t];
      const int64_t m = std::min<int64_t>(n, (int64_t)it->tab[t].size());
      if (out) std::copy(it->tab[t].begin(), it->tab[t].begin() + m, out);
      return 0;
    }
  return BCFD_E_ARG;
}

int bcfd_coupling_apply(bcfd_handle h, int comp, int op, const double* in, double* out) {
  LOCK();
  HostInterface* it = get_iface(h);
  if (!it) return BCFD_E_HANDLE;
  if (!in || !out || comp < 0 || comp > 3 || op < 0 || op > 3) return BCFD_E_ARG;
  HostBlock* a = get_block(it->a);
  HostBlock* b = get_block(it->b);
  if (!a || !b) return BCFD_E_HANDLE;
  // 0 P (coarse -> fine), 1 P^T (fine -> coarse), 2 R (fine -> coarse),
  // 3 R^T (coarse -> fine)
  const size_t na = (size_t)a->d.d.npts(), nb = (size_t)b->d.d.npts();
  const size_t nin = (op == 0 || op == 3) ? na : nb, nout = (op == 0 || op == 3) ? nb : na;
  double *din = nullptr, *dout = nullptr;
  BCFD_CUDA(cudaMalloc(&din, nin * sizeof(double)));
  if (cudaMalloc(&dout, nout * sizeof(double)) != cudaSuccess) {
    cudaFree(din);
    return BCFD_E_NOMEM;
  }
  int r = 0;
  if (h2d(din, in, nin * sizeof(double)) != cudaSuccess ||
      h2d(dout, out, nout * sizeof(double)) != cudaSuccess)
    r = BCFD_E_CUDA;
  if (!r) r = coupling_apply(it, comp, op, din, dout);
  if (!r && cudaStreamSynchronize(stream()) != cudaSuccess) r = BCFD_E_CUDA;
  if (!r && d2h(out, dout, nout * sizeof(double)) != cudaSuccess) r = BCFD_E_CUDA;
  cudaFree(din);
  cudaFree(dout);
  return r;
}

int bcfd_fine_update_pc_bd(void) { LOCK(); return fine_update_pc_bd(); }
int bcfd_fine_update_newv_bd(void) { LOCK(); return fine_update_newv_bd(); }
int bcfd_fine_update_bd_mv(bcfd_handle h) {
  LOCK();
  HostInterface* it = get_iface(h);
  if (!it) return BCFD_E_HANDLE;
  return fine_update_bd_mv(it);
}
int bcfd_coarse_update(void) { LOCK(); return coarse_update(); }
int bcfd_coarse_update_newv(void) { LOCK(); return coarse_update_newv(); }
int bcfd_coarse_update_pc(void) { LOCK(); return coarse_update_pc(); }
int bcfd_fine_update_mv(bcfd_handle h) {
  LOCK();
  HostInterface* it = get_iface(h);
  if (!it) return BCFD_E_HANDLE;
  return launch_fine_update_mv(it);
}

int bcfd_poisson_solver(int64_t pc_ita_max, double epsi, int64_t ita, double deltat, double totime,
                        double uc, double* total_time, int start, int finish, int step) {
  LOCK();
  (void)ita;
  if (step <= 0 || start < 1) return BCFD_E_ARG;
  SolveCfg c{pc_ita_max, epsi, deltat, uc, 0, 0.0};
  TRY(poisson(c, start, finish, step));
  int err = 0;
  for (auto& [g, hb] : blocks())
    if (g >= start && g <= finish && (g - start) % step == 0) {
      const int e = sync_err(hb);
      if (e && !err) err = e;
      if (total_time) *total_time = totime + *total_time;
    }
  return err;
}

int bcfd_block_move_stage(int64_t* moved) {
  LOCK();
  std::vector<int64_t> before;
  for (HostBlock* hb : lib().blocks) before.push_back(hb ? hb->move_check : 0);
  TRY(block_move_stage());
  int64_t any = 0;
  for (size_t q = 0; q < lib().blocks.size(); ++q)
    if (lib().blocks[q] && lib().blocks[q]->move_check == 1 && before[q] != 1) any = 1;
  if (moved) *moved = any;
  return 0;
}

int bcfd_tagging_th_move(bcfd_handle h) {
  LOCK();
  HostBlock* hb = get_block(h);
  if (!hb) return BCFD_E_HANDLE;
  if (hb->move_check != 1) return 0;
  TRY(launch_tagging(hb));
  for (HostInterface* it : lib().ifs)
    if (it && it->b == h) {
      TRY(launch_fine_update_mv(it));
      TRY(fine_update_bd_mv(it));
    }
  return 0;
}

int bcfd_run_steps(const bcfd_step_config* cfg, int64_t n_steps) {
  LOCK();
  if (!cfg || n_steps < 0 || cfg->precision < 0 || cfg->precision > 3) return BCFD_E_ARG;
  if (cfg->precision >= 1 && !(cfg->div_tol > 0.0)) return BCFD_E_ARG;
  if (cfg->use_graph && !lib().prof_on) {
    TRY(run_steps_graph(*cfg, n_steps));
  } else {
    for (int64_t s = 0; s < n_steps; ++s) TRY(step_once(*cfg));
  }
  int err = 0;
  for (auto& [g, hb] : blocks()) {
    const int e = sync_err(hb);
    if (e && !err) err = e;
  }
  return err;
}

int bcfd_block_write(bcfd_handle h, const char* name, const double* data, int64_t n) {
  LOCK();
  HostBlock* hb = get_block(h);
  if (!hb) return BCFD_E_HANDLE;
  if (!name || !data || n < 0) return BCFD_E_ARG;
  const std::string s(name);
  DevBlock& D = hb->d;
  int64_t cnt[6];
  BCFD_CUDA(cudaMemcpyAsync(cnt, D.cnt, sizeof(cnt), cudaMemcpyDeviceToHost, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  const int64_t nts = std::min<int64_t>(cnt[C_TS], D.cap_ib);
  const char* gn[14] = {"p_ghost", "pt_ghost", "u2_ghost", "u2t_ghost", "v2_ghost", "v2t_ghost", "w2_ghost",
                        "w2t_ghost", "u1_ghost", "u1t_ghost", "v1_ghost", "v1t_ghost", "w1_ghost", "w1t_ghost"};
  for (int q = 0; q < 14; ++q)
    if (s == gn[q]) {
      if (n != nts) return BCFD_E_ARG;
      if (n) BCFD_CUDA(cudaMemcpyAsync(D.ghost[q], data, n * sizeof(double), cudaMemcpyHostToDevice, stream()));
      BCFD_CUDA(cudaStreamSynchronize(stream()));
      return 0;
    }
  return BCFD_E_NOTFOUND;
}

int bcfd_block_read(bcfd_handle h, const char* name, void* out, int64_t n, int64_t* written) {
  LOCK();
  HostBlock* hb = get_block(h);
  if (!hb) return BCFD_E_HANDLE;
  if (!name || !out) return BCFD_E_ARG;
  const std::string s(name);
  const Dims& d = hb->d.d;
  DevBlock& D = hb->d;
  int64_t cnt[6];
  BCFD_CUDA(cudaMemcpyAsync(cnt, D.cnt, sizeof(cnt), cudaMemcpyDeviceToHost, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  const int64_t nib = std::min<int64_t>(cnt[C_IB], D.cap_ib), nts = cnt[C_TS];
  auto dcopy = [&](const double* src, int64_t m) -> int {
    m = std::min(m, n);
    BCFD_CUDA(cudaMemcpyAsync(out, src, m * sizeof(double), cudaMemcpyDeviceToHost, stream()));
    BCFD_CUDA(cudaStreamSynchronize(stream()));
    if (written) *written = m;
    return 0;
  };
  auto icopy = [&](const int* src, int64_t m) -> int {
    m = std::min(m, n);
    std::vector<int> t((size_t)m);
    BCFD_CUDA(cudaMemcpyAsync(t.data(), src, m * sizeof(int), cudaMemcpyDeviceToHost, stream()));
    BCFD_CUDA(cudaStreamSynchronize(stream()));
    for (int64_t q = 0; q < m; ++q) ((int64_t*)out)[q] = t[q];
    if (written) *written = m;
    return 0;
  };
  auto hcopy = [&](const std::vector<double>& v) -> int {
    const int64_t m = std::min<int64_t>(n, (int64_t)v.size());
    std::copy(v.begin(), v.begin() + m, (double*)out);
    if (written) *written = m;
    return 0;
  };
  if (s == "pc" || s == "b") {
    double* tmp;
    BCFD_CUDA(cudaMalloc(&tmp, d.npts() * sizeof(double)));
    double* const* src = s == "pc" ? D.pc : D.bpk;
    int r = launch_unpack(hb, src, tmp);
    if (!r) r = dcopy(tmp, d.npts());
    cudaFree(tmp);
    return r;
  }
  if (s == "mk" || s == "mkx1" || s == "mkx2") {
    if (n < 1) return BCFD_E_ARG;
    *(int64_t*)out = s == "mk" ? hb->mk : s == "mkx1" ? hb->mkx1 : hb->mkx2;
    if (written) *written = 1;
    return 0;
  }
  {
    // the block-move switches and amounts of Block_t
    const char* fn[5] = {"move_check", "blk_mv_tag", "move_amtx", "move_amty", "move_amtz"};
    const int64_t fv[5] = {hb->move_check, hb->blk_mv_tag, hb->move_amt[0], hb->move_amt[1], hb->move_amt[2]};
    for (int q = 0; q < 5; ++q)
      if (s == fn[q]) {
        if (n < 1) return BCFD_E_ARG;
        static_cast<int64_t*>(out)[0] = fv[q];
        if (written) *written = 1;
        return 0;
      }
  }
  if (s == "xnode1") return dcopy(D.xnode1, D.nn);
  if (s == "ynode1") return dcopy(D.ynode1, D.nn);
  if (s == "znode1") return dcopy(D.znode1, D.nn);
  {
    // kinematic scalars the forcing routines read
    const char* kn[10] = {"xdot", "ydot", "yddot", "thetaDot1", "thetaDDot1", "thetaDot2", "thetaDDot2",
                          "piv_x", "piv_y", "piv_z"};
    const Kin& K = hb->kin;
    const double kv[10] = {K.xdot, K.ydot, K.yddot, K.thetaDot1, K.thetaDDot1, K.thetaDot2, K.thetaDDot2,
                           K.piv_x, K.piv_y, K.piv_z};
    for (int q = 0; q < 10; ++q)
      if (s == kn[q]) {
        if (n < 1) return BCFD_E_ARG;
        static_cast<double*>(out)[0] = kv[q];
        if (written) *written = 1;
        return 0;
      }
  }
  const char* fnames[7] = {"xcent", "ycent", "zcent", "cosAlpha", "cosBeta", "cosGamma", "element_length"};
  double* fptr[7] = {D.xcent, D.ycent, D.zcent, D.cosA, D.cosB, D.cosG, D.elen};
  for (int q = 0; q < 7; ++q)
    if (s == fnames[q]) return dcopy(fptr[q], D.ne);
  const char* ndn[7] = {"pNormDis", "u1NormDis", "u2NormDis", "v1NormDis", "v2NormDis", "w1NormDis", "w2NormDis"};
  const char* neln[7] = {"nelp", "nelu1", "nelu2", "nelv1", "nelv2", "nelw1", "nelw2"};
  for (int q = 0; q < 7; ++q) {
    if (s == ndn[q]) return dcopy(D.nd[q], nib);
    if (s == neln[q]) return icopy(D.nel[q], nib);
  }
  const char* gn[14] = {"p_ghost", "pt_ghost", "u2_ghost", "u2t_ghost", "v2_ghost", "v2t_ghost", "w2_ghost",
                        "w2t_ghost", "u1_ghost", "u1t_ghost", "v1_ghost", "v1t_ghost", "w1_ghost", "w1t_ghost"};
  for (int q = 0; q < 14; ++q)
    if (s == gn[q]) return dcopy(D.ghost[q], nts);
  if (s == "index_ts") return icopy(D.ts_idx, nts);
  if (s == "Acx") return hcopy(hb->Acx);
  if (s == "Acy") return hcopy(hb->Acy);
  if (s == "Acz") return hcopy(hb->Acz);
  const char* tn[N_TAB] = {"uu", "vv", "ww", "uv", "uw", "vu", "vw", "wu", "wv"};
  for (int t = 0; t < N_TAB; ++t) {
    if (s == std::string("ca_") + tn[t]) return hcopy(hb->ca[t]);
    if (s == std::string("ck_") + tn[t]) return hcopy(hb->ck[t]);
  }
  const char* grn[18] = {"x1", "y1", "z1", "deltax", "deltay", "deltaz", "xu", "yu", "zu",
                         "xv", "yv", "zv", "xw", "yw", "zw", "xp", "yp", "zp"};
  const std::vector<double>* grv[18] = {&hb->x1, &hb->y1, &hb->z1, &hb->dxa, &hb->dya, &hb->dza,
                                        &hb->xu, &hb->yu, &hb->zu, &hb->xv, &hb->yv, &hb->zv,
                                        &hb->xw, &hb->yw, &hb->zw, &hb->xp, &hb->yp, &hb->zp};
  for (int q = 0; q < 18; ++q)
    if (s == grn[q]) return hcopy(*grv[q]);
  // index lists as (count, 3) column-major int64
  auto list_out = [&](const std::vector<int>& ijk, int64_t m, int64_t cap) -> int {
    if (3 * m > n) return BCFD_E_ARG;
    int64_t* o = (int64_t*)out;
    for (int64_t q = 0; q < m; ++q) {
      o[q] = ijk[q];
      o[m + q] = ijk[cap + q];
      o[2 * m + q] = ijk[2 * cap + q];
    }
    if (written) *written = 3 * m;
    return 0;
  };
  if (s == "interceptedIndexPtr") {
    std::vector<int> t(3 * (size_t)nib);
    BCFD_CUDA(cudaMemcpyAsync(t.data(), D.ib_i, nib * sizeof(int), cudaMemcpyDeviceToHost, stream()));
    BCFD_CUDA(cudaMemcpyAsync(t.data() + nib, D.ib_j, nib * sizeof(int), cudaMemcpyDeviceToHost, stream()));
    BCFD_CUDA(cudaMemcpyAsync(t.data() + 2 * nib, D.ib_k, nib * sizeof(int), cudaMemcpyDeviceToHost, stream()));
    BCFD_CUDA(cudaStreamSynchronize(stream()));
    return list_out(t, nib, nib);
  }
  if (s == "TSIndexPtr") {
    std::vector<int> ts((size_t)nts), ii((size_t)nib), jj((size_t)nib), kk((size_t)nib);
    BCFD_CUDA(cudaMemcpyAsync(ts.data(), D.ts_idx, nts * sizeof(int), cudaMemcpyDeviceToHost, stream()));
    BCFD_CUDA(cudaMemcpyAsync(ii.data(), D.ib_i, nib * sizeof(int), cudaMemcpyDeviceToHost, stream()));
    BCFD_CUDA(cudaMemcpyAsync(jj.data(), D.ib_j, nib * sizeof(int), cudaMemcpyDeviceToHost, stream()));
    BCFD_CUDA(cudaMemcpyAsync(kk.data(), D.ib_k, nib * sizeof(int), cudaMemcpyDeviceToHost, stream()));
    BCFD_CUDA(cudaStreamSynchronize(stream()));
    std::vector<int> t(3 * (size_t)nts);
    for (int64_t q = 0; q < nts; ++q) {
      t[q] = ii[ts[q] - 1];
      t[nts + q] = jj[ts[q] - 1];
      t[2 * nts + q] = kk[ts[q] - 1];
    }
    return list_out(t, nts, nts);
  }
  int which = -1;
  if (s == "fluidIndexPtr" || s == "redCellIndexPtr" || s == "blackCellIndexPtr") which = 0;
  if (s == "solidIndexPtr") which = 1;
  if (which >= 0) {
    const int64_t cap = (int64_t)d.nx * d.ny * d.nz;
    int* buf;
    BCFD_CUDA(cudaMalloc(&buf, 3 * cap * sizeof(int)));
    int64_t m = 0;
    int r = launch_build_list(hb, which, buf, cap, &m);
    std::vector<int> t(3 * (size_t)cap);
    if (!r) {
      const cudaError_t e = d2h(t.data(), buf, 3 * cap * sizeof(int));
      if (e != cudaSuccess) {
        report_cuda(e, "index lists to host", __FILE__, __LINE__);
        r = BCFD_E_CUDA;
      }
    }
    cudaFree(buf);
    if (r) return r;
    if (s == "redCellIndexPtr" || s == "blackCellIndexPtr") {
      const int want = s == "redCellIndexPtr" ? 1 : 0;
      std::vector<int> u;
      std::vector<int> a, b2, c2;
      for (int64_t q = 0; q < m; ++q)
        if (((t[q] + t[cap + q] + t[2 * cap + q]) & 1) == want) {
          a.push_back(t[q]);
          b2.push_back(t[cap + q]);
          c2.push_back(t[2 * cap + q]);
        }
      const int64_t mm = (int64_t)a.size();
      u.insert(u.end(), a.begin(), a.end());
      u.insert(u.end(), b2.begin(), b2.end());
      u.insert(u.end(), c2.begin(), c2.end());
      return list_out(u, mm, mm);
    }
    return list_out(t, m, cap);
  }
  return BCFD_E_ARG;
}

}  // extern "C"
