// Host-side objects of the library: registered blocks and interfaces, the
// library stream and the launch helpers.  Shared by the .cu translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "bcfd_internal.cuh"
#include "bcfd_batch.cuh"

namespace bcfd {

// rigid-body motion state of a block's surface (Block_t members used by
// src/Search.F90:49-208)
struct BodyMotion {
  bool on = false;
  double a0 = 0, bfreq = 0, yamp = 0, xshift = 0, yshift = 0, zshift = 0;
  double xpth1 = 0, xpth2 = 0, ypth2 = 0, xchg = 0, ychg = 0, xmove = 0, ymove = 0, zmove = 0;
  double xt = 0, yt = 0, inity_cent = 0, nxty_cent = 0, initx_cent = 0, nxtx_cent = 0,
         initz_cent = 0, nxtz_cent = 0;
  // phase lag of this body's heave and pitch behind the kinematics all bodies
  // share (radians; 0 = the reference's single-phase kinematics) and the
  // shared pitch phase angle its initial placement is taken against
  double lag = 0, lag_phase = 0;
  // the initial placement's inputs (shiftSurfaceNodesInitial) and the pitch
  // amplitude as given in degrees, for the replay of the motion in the adjoint
  bool placed = false;
  double init_aoa = 0, init_piv_pt = 0, init_dxmin = 0, init_totime = 0, a0_deg = 0;
  int64_t init_ita = 0;
};

// Node placement of one step (computeSurfaceVariables): the rotation's
// cos/sin for surface-51 (+angle) and -52 (-angle) nodes about the x axis
// through z = piv_pt, then the translation
struct Place {
  double c1, s1, c2, s2, piv_pt;
  double tx, ty1, ty2, tz1, tz2;
  int two;  // 1: y = (yr1 + ty1) + ty2, z = (zr1 + tz1) + tz2; 0: one term
};

// one node moved by a Place, in the reference's evaluation order (the same
// expression on the host and the device)
__host__ __device__ inline void place_node(const Place& P, int id, double x, double y, double z, double* xo,
                                           double* yo, double* zo) {
  double xr1 = x, yr1 = y, zr1 = z;
  if (id == 51 || id == 52) {
    const double c = id == 51 ? P.c1 : P.c2, s = id == 51 ? P.s1 : P.s2;
    zr1 = z * c + y * s + P.piv_pt - P.piv_pt * c;
    yr1 = -(z * s) + y * c + P.piv_pt * s;
  }
  *xo = xr1 + P.tx;
  *yo = P.two ? (yr1 + P.ty1) + P.ty2 : yr1 + P.ty1;
  *zo = P.two ? (zr1 + P.tz1) + P.tz2 : zr1 + P.tz1;
}

// What a moving block's step needs from the host, uploaded in one copy: the
// kinematics that take effect when the nodes move, the placement, and the
// search origin/radius of the moved surface
struct MotionStage {
  Kin kin;
  Place place;
  float org[4];
};

struct HostBlock {
  int index = -1;                  // registration order (device table slot)
  BodyMotion motion;
  double motion_r0 = 0.0;          // largest body-frame node radius
  Kin kin{};                       // host copy of the device kinematics (d.kin)
  Kin* kin_dev = nullptr;          // the device kinematics the kernels read
  MotionStage* stage_dev = nullptr;
  MotionStage stage{};             // last staged placement
  bool staged = false;             // a step's motion is staged but not applied
  // body-frame nodes and surface ids on the host (moving blocks)
  std::vector<double> node0[3];
  std::vector<int8_t> node_id_host;
  std::vector<int> elem_host;      // elp1 | elp2 | elp3 | surf_id, as uploaded
  std::vector<int> elem_perm;      // search order -> element index (Morton order of the centroids)
  int elem_perm_gen = 0;           // bumped when elem_perm changes
  DevBlock d{};
  std::vector<void*> allocs;  // device allocations owned by the block
  // host copies of the 1-D grids (1-based meaning, v[i-1])
  std::vector<double> x1, y1, z1, dxa, dya, dza, xu, yu, zu, xv, yv, zv, xw, yw, zw, xp, yp, zp;
  std::vector<double> Acx, Acy, Acz;  // column-major (n,3)
  std::vector<double> ca[N_TAB], ck[N_TAB];
  double dx = 0, dy = 0, dz = 0, omega = 1.0;
  int64_t move_check = 0, blk_mv_tag = 0;
  bool is_coarse = false, has_body = false;
  bool coeffs_ready = false;
  int64_t inor = 1;
  BlockStats* stats = nullptr;     // device
  double* grid_buf = nullptr;      // device buffer holding all 1-D arrays
  double* coef_buf = nullptr;      // device Acx/Acy/Acz + ca/ck tables
  float* grid_f32 = nullptr;       // device dxa/dya/dza rounded to FP32
  double* lcoef = nullptr;         // device per-line factors of correctVelocity (see DevBlock::lcoef)
  double lcoef_dt = 0.0;           // the deltat they were computed for (0: not computed)
  float* coef_f32 = nullptr;       // device Acx/Acy/Acz rounded to FP32
  float* pcf2 = nullptr;           // second FP32 correction buffer (both colours) of the temporal-blocked sweeps
  int64_t mk = 0, mkx1 = 0, mkx2 = 0;  // findDistnode's extreme surface nodes (1-based)
  // fine-block moves (src/Search.F90:997-1370): the last move and the index
  // ranges of the old (cpy) and new (cpy_mv) positions of the moved data,
  // which keep their values when a search finds no index, as the reference's
  double* mv_dum = nullptr;  // u, v, w, p before the move
  int64_t move_amt[3] = {0, 0, 0};
  int64_t cpy[6] = {0, 0, 0, 0, 0, 0}, cpy_mv[6] = {0, 0, 0, 0, 0, 0};
  int surf_cap_e = 0, surf_cap_n = 0;
  int cap_ib_alloc = 0;            // IB/TS list entries allocated (d.cap_ib may be set lower)
  // per-block barrier words for persistent kernels: [count, gen]
  unsigned* bar = nullptr;
  unsigned* prog = nullptr;        // per-tile phase counters of the tiled solves
  // mixed-precision solve: FP32 sweeps per correction and their relaxation
  // (0 = defaults chosen from the block size)
  int dc_inner = 0;
  double dc_omega = 0.0;
  // mixed solve kernel: 0 = library default, 1 = grid-wide phase barriers,
  // 3 = neighbour sync, 4 = temporal-blocked
  int dc_variant = 0;
  int solve_threads = 0;           // threads per CTA of the tiled solves (0: 256)
  int solve_ctas_per_sm = 0;       // co-resident CTAs per SM cap (0: occupancy limit)
  int solve_sync = 0;              // FP64 solve: 0 point-to-point, 1 grid-wide phase barriers
  int sor_rev = 0;                 // FP64 solve: black half-sweep first (adjoint solves)
  int dc_threads = 0;              // FP32 correction: threads per CTA (0: 256)
  int dc_ctas_per_sm = 0;          // FP32 correction: CTAs per SM cap (0: occupancy limit)
  // largest distance of a surface node from the block centre (for the FP32
  // prefilter bound of the nearest-element search)
  double node_rmax = 0.0;
  // scratch owned by the search and forcing translation units
  void* search_scratch = nullptr;
  void* dag_scratch = nullptr;
};

void free_search_scratch(HostBlock* hb);
void free_dag_scratch(HostBlock* hb);

struct HostInterface {
  bcfd_handle a = 0, b = 0;  // block handles (a coarse, b fine)
  int64_t a_msh = 1, b_msh = 2;
  double box[6] = {0, 0, 0, 0, 0, 0};
  // 12 tables (3, cap) int64 in the reference layout, order px py pz ux uy uz vx vy vz wx wy wz
  std::vector<int64_t> tab[12];
  int64_t counter[12] = {0};
  int64_t cap[12] = {0};
  int* dtab = nullptr;  // device copy, int32, same layout, each table at offset off[t]
  int64_t off[12] = {0};
};

enum TabId { TPX = 0, TPY, TPZ, TUX, TUY, TUZ, TVX, TVY, TVZ, TWX, TWY, TWZ };

// Records, during the forward recomputation of an adjoint run through moving
// bodies, what the transposes need from each forcing call: the geometric
// partials of every task at the stencil values it read (k_force_geo).
struct ForceRecorder {
  virtual ~ForceRecorder() = default;
  // device buffer of 6 * nt doubles for call (mode, vel) of block hb in the
  // step being recomputed (nullptr: nothing to record)
  virtual double* slot(HostBlock* hb, int mode, int vel, int64_t nt) = 0;
  // device scratch of 3 point arrays of the block (the pre-call copies)
  virtual double* scratch(HostBlock* hb) = 0;
};

struct Lib {
  std::recursive_mutex mu;
  bool ready = false;
  int device = 0;
  int nsm = 0;
  cudaStream_t s = nullptr;
  std::vector<HostBlock*> blocks;      // handle h -> blocks[h-1] (nullptr when destroyed)
  std::vector<HostInterface*> ifs;     // interface handle -> ifs[h-1]
  int64_t launches = 0;
  // measurement window
  bool prof_on = false;
  int64_t* prof_dev = nullptr;            // device solve log
  std::vector<cudaEvent_t> prof_events;   // begin/end pairs, in order
  size_t prof_used = 0;
  int64_t prof_launch0 = 0;
  // per-phase split of the window: an event at every phase boundary of an
  // eagerly issued step, and the summed device time per phase of the last window
  std::vector<cudaEvent_t> phase_events;
  std::vector<int> phase_ids;
  size_t phase_used = 0;
  double phase_ms[8] = {0};
  // bumped whenever a scratch buffer that captured kernels point at is
  // (re)allocated, so a captured step graph is rebuilt
  uint64_t gen = 0;
  // device table of all blocks' views for batched launches
  bool batch = true;                 // phases over several blocks in one launch
  DevBlock* dtab = nullptr;
  size_t dtab_cap = 0;
  std::vector<DevBlock> htab;        // what the device table holds
  // time and motion inputs of the native driver (app/main.F90 variables)
  int64_t ita = 0;
  double totime = 0.0;
  double phase_angle = 0.0, piv_pt = 0.0, freq = 0.0, dxmin = 0.0;
  int64_t inor = 1;
  // captured time step (bcfd_run_steps with use_graph)
  cudaGraphExec_t step_graph = nullptr;
  std::vector<unsigned char> step_key;  // what the capture depends on
  std::vector<unsigned char> eager_key; // the key left by the last eager step
  int adj_precision = 1;  // zero-BC and adjoint solves: 0 FP64 SOR, 1 FP32 sweeps + FP64 correction
  uint64_t wait_limit_ns = kBarrierLimitNs;  // longest single device-side wait
  bool warm_start = false;  // residual-target solves start from the last correction
  ForceRecorder* recorder = nullptr;  // set by an adjoint run while it recomputes steps
  int64_t step_kernels = 0;              // kernels in the captured step
};

Lib& lib();

// Held by every entry point: serialises calls and, once bcfd_init has run,
// makes the library's device current on the calling thread, so a host thread
// other than the one that called bcfd_init (which starts on device 0) can
// call in.  The calling thread's current device is left at the library's.
struct LibLock {
  std::lock_guard<std::recursive_mutex> g;
  LibLock() : g(lib().mu) {
    if (lib().ready) {
      int cur = -1;
      if (cudaGetDevice(&cur) != cudaSuccess || cur != lib().device) cudaSetDevice(lib().device);
    }
  }
};

HostBlock* get_block(bcfd_handle h);
HostInterface* get_iface(bcfd_handle h);

// record one kernel launch (for the launch counter) and check the launch
int note_launch(cudaError_t e = cudaGetLastError());
#define BCFD_LAUNCHED() do { int _r = ::bcfd::note_launch(); if (_r) return _r; } while (0)
#define TRY_R(x) do { int _r = (x); if (_r) return _r; } while (0)
#define BCFD_CUDA(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) { ::bcfd::report_cuda(_e, #x, __FILE__, __LINE__); return BCFD_E_CUDA; } } while (0)
void report_cuda(cudaError_t e, const char* what, const char* file, int line);

// host <-> device copies ordered on the library stream (a non-blocking
// stream: plain cudaMemcpy / cudaMemset on the legacy stream would race with
// its kernels); d2h returns once the data is on the host
inline cudaError_t h2d(void* dst, const void* src, size_t bytes) {
  return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream());
}
inline cudaError_t d2h(void* dst, const void* src, size_t bytes) {
  const cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream());
  return e != cudaSuccess ? e : cudaStreamSynchronize(stream());
}

// read and clear a block's device error word (synchronises)
int take_block_error(HostBlock* hb);

// ---- launchers implemented by the kernel translation units (return status) ----
// k_poisson.cu
int launch_compute_div(HostBlock* hb);
int launch_correct_pressure(HostBlock* hb);
int launch_correct_velocity(HostBlock* hb, double dt);
// the same phases over several blocks (one launch per phase when batching)
// fast: reciprocal spacings (residual-target solves) instead of the
// reference's divisions
int launch_compute_div(const std::vector<HostBlock*>& hbs, bool fast);
int launch_correct_pressure(const std::vector<HostBlock*>& hbs);
int launch_correct_velocity(const std::vector<HostBlock*>& hbs, double dt);
int launch_steady_state(const std::vector<HostBlock*>& hbs, double dt);
int launch_max_div(const std::vector<HostBlock*>& hbs, bool tfield);
int launch_copy_t_to_n(const std::vector<HostBlock*>& hbs);
int launch_momentum(const std::vector<HostBlock*>& hbs, double dt, double re, bool fp32);
// fast = 1 (residual-target solves only): the division-free FP64 update
int launch_sor_set(const std::vector<HostBlock*>& hbs, int64_t itmax, double dt, double epsi, double res_tol,
                   int fast = 0);
bool tb_solve_fits(HostBlock* hb);
bool zm_solve_fits(HostBlock* hb);
double mixed_omega_of(const HostBlock* hb);
int launch_sor_mixed_set(const std::vector<HostBlock*>& hbs, int64_t itmax, double dt, double div_tol);
// res_tol > 0: stop on the FP64 residual dt*max|b/dt - A pc| <= res_tol
int launch_sor(HostBlock* hb, int64_t itmax, double dt, double epsi, double res_tol = 0.0, int fast = 0);
// warm = true: the solve starts from the previous correction at its updated
// cells (residual-target solves only) instead of from 0
int launch_zero_poisson(HostBlock* hb, bool warm = false);
int launch_steady_state(HostBlock* hb, double dt);
int launch_copy_t_to_n(HostBlock* hb);
int launch_copy_n_to_t(HostBlock* hb);
int launch_update_masks(HostBlock* hb);
int launch_pack(HostBlock* hb, const double* natural_dev, double* packed[2]);
int launch_unpack(HostBlock* hb, double* const packed[2], double* natural_dev);
int launch_max_div(HostBlock* hb, bool tfield);
// measurement window: device log of solves (nullptr when inactive) and CUDA
// events around each persistent solve launch
int64_t* prof_log();
void prof_mark(bool begin);
// phases of a time step for the measurement window's split (bcfd_profile_phases)
enum StepPhase {
  PH_MOMENTUM = 0,   // nsMomentum2order and the domain BCs
  PH_FORCING,        // solid-cell BCs, velocityForcing1, pressureForcing1
  PH_SOLVE,          // the Poisson solves (incl. their right-hand sides)
  PH_COUPLING,       // coarse/fine face fills and restrictions
  PH_CORRECTION,     // zeroing, divergence, corrections, reductions, copies
  PH_SEARCH,         // body motion, normals, block moves, re-Search and lists
  PH_FORCING_FIELD,  // forcing on the re-searched geometry (Field, Ghost)
  PH_COUNT
};
// marks the start of phase `ph` on the library stream (no-op outside a
// measurement window or while a stream capture is running)
void phase_mark(int ph);
int launch_sor_mixed(HostBlock* hb, int64_t itmax, double dt, double div_tol);
// k_momentum.cu
int launch_momentum(HostBlock* hb, double dt, double re, bool fp32);
int launch_momentum_tangent(HostBlock* hb, double dt, double re, const double* const du[4], double* const val[3],
                            double* const tan[3]);
int solve_zero_bc_dev(HostBlock* hb, const double* r, double* x, double tol, int64_t itmax, bool transpose);
int run_one_step(const bcfd_step_config& cfg);
// scratch of the thin-surface overlay's adjoint: last (7 ints per point),
// contrib (14 doubles per point), gb (the ghost arrays' adjoint, 14 x cap)
struct MomTsAdj {
  int* last = nullptr;
  double* contrib = nullptr;
  double* gb = nullptr;
  int64_t cap = 0;
};
int launch_momentum_adjoint(HostBlock* hb, double dt, double re, const double* const sb[3], double* const ab[4],
                            uint32_t* foot, const MomTsAdj* ts = nullptr);
int launch_velocity_bc(HostBlock* hb, double dt, double uc);
int launch_solid_bc(HostBlock* hb, bool move);
// k_search.cu
int launch_surface_norm(HostBlock* hb, int64_t inor);
int launch_tagging(HostBlock* hb);
int launch_retagging(HostBlock* hb);
int launch_cellcount(HostBlock* hb, bool coarse);
int launch_norm_distance(HostBlock* hb);
int launch_find_ts(HostBlock* hb);
int launch_fine_block_cell(HostBlock* a, HostInterface* it, bool first);
// fine-block moves: grid shift (host grids, derived grids, upload), the
// cell_n marks of the data the block keeps, the moved fields
int shift_block_grid(HostBlock* hb, double cx, double cy, double cz);
int launch_mark_cell_n(HostBlock* hb, const double box_new[6]);
int launch_move_fields(HostBlock* hb, const double* dum);
int launch_build_list(HostBlock* hb, int which, int* out_ijk, int64_t cap, int64_t* count_host);
// k_forcing.cu
int launch_forcing_velocity(HostBlock* hb, int mode);  // 0 forcing1, 1 field, 2 ghost
int launch_forcing_pressure(HostBlock* hb, int mode);
// k_interp.cu
// the face fill / restriction of components comps[0..nc) of an interface
// (which: 0 t-fields, 1 pc, 2 n-fields)
int launch_face_fill_set(HostInterface* it, const int* comps, int nc, int which);
int launch_restrict_set(HostInterface* it, const int* comps, int nc, int which);
int launch_fine_update_mv(HostInterface* it);
// op 0: face fill P, 1: P^T (accumulates), 2: restriction R, 3: R^T (accumulates)
int coupling_apply(HostInterface* it, int comp, int op, const double* in, double* out);
// k_stress.cu
int launch_stress(HostBlock* hb, double mu_f, double rho_f, double* out_host);
// k_motion.cu
int shift_surface_nodes_initial(HostBlock* hb, double aoa, double piv_pt, int64_t ita, double deltat,
                                double dxmin, double totime);
int compute_surface_variables(HostBlock* hb, double phase_angle, double piv_pt, int64_t ita, double deltat,
                              double dxmin, double freq, double totime);
// computeSurfaceVariables in two halves: the host's kinematics and the
// staged upload (outside a captured step), then the node kernel that applies
// them (inside it)
int stage_surface_variables(HostBlock* hb, double phase_angle, double piv_pt, int64_t ita, double deltat,
                            double dxmin, double freq, double totime);
int apply_surface_variables(HostBlock* hb);
// a node's position under the staged placement (host, the kernel's arithmetic)
void staged_node(const HostBlock* hb, int64_t node, double* x, double* y, double* z);
// the device kinematics from the host copy (set_kinematics, set-up)
int upload_kin(HostBlock* hb);
// bcfd_api.cu: the FP32 sweep tables (axr | ayr | azr) of three line tables
void append_sweep_tables(const Dims& d, const std::vector<double>& Ax, const std::vector<double>& Ay,
                         const std::vector<double>& Az, std::vector<float>& f, size_t* axr_off, size_t* ayr_off,
                         size_t* azr_off);
// k_search.cu: the search origin/radius for the block's current grid and
// node bound, recorded as the device's value (the caller puts it there)
int search_origin_stage(HostBlock* hb, float h[4], float** dev);
int launch_stress_noalloc(HostBlock* hb, double mu_f, double rho_f, double* out_host);
// adjoint of the forcing loops (k_forcing.cu): per-task coefficient scratch
// (capacity 6 * cap_ib tasks) and the adjoint arrays by axis (0 p, 1 u, 2 v, 3 w)
// kinematic scalars the forcing and drag/lift depend on: the 8 of
// bcfd_block_set_kinematics and the pivot (piv_x, piv_y, piv_z)
constexpr int kKinScalars = 11;
struct ForceCoef {
  int64_t* tgt;
  int* axis;
  int64_t* pos;
  double* coef;
  double* kc;  // per task, d(output)/d(kinematic scalar p), p < kKinScalars (bcfd_block_set_kinematics order)
  double* gk;  // kKinScalars accumulators: dJ/d(kinematic scalar p)
  int* elem;         // per task: its element (0-based)
  const double* geo; // per task: 6 geometric partials recorded forward (nullptr: geometry fixed)
  double* ge;        // per element: 7 accumulators dJ/d(centroid, unit normal, length) (with geo)
};
// the 8 rigid-body kinematic scalars of a block, in bcfd_block_set_kinematics order
__host__ __device__ inline double& kin_scalar(Kin& K, int p) {
  switch (p) {
    case 0: return K.xdot;
    case 1: return K.ydot;
    case 2: return K.yddot;
    case 3: return K.thetaDot1;
    case 4: return K.thetaDDot1;
    case 5: return K.thetaDot2;
    case 6: return K.thetaDDot2;
    case 7: return K.alphaDot;
    case 8: return K.piv_x;
    case 9: return K.piv_y;
    default: return K.piv_z;
  }
}
struct AdjPtrs {
  double* tgt[4];
  double* src[4];
};
int launch_stress_kin(HostBlock* hb, double mu_f, double rho_f, const double* seed_dev, double* gk,
                      double* scratch);
int launch_forcing_adjoint(HostBlock* hb, int mode, int vel, const AdjPtrs& a, const ForceCoef& fc);
int launch_ghost_adjoint(HostBlock* hb, int vel, const AdjPtrs& a, const ForceCoef& fc, double* gb, int64_t cap);
int launch_stress_geo(HostBlock* hb, double mu_f, double rho_f, const double* seed_dev, double w, double* ge,
                      double* scratch);

// ---- adjoint through moving geometry (bcfd_adjoint_motion.cu) ----
constexpr int kMotionParams = 5;  // yamp, a0 (deg), phase angle (rad), freq, bfreq
// derivatives of one step's placement (rotation angle, y translation) and
// kinematic scalars with respect to the motion parameters
struct StepTangent {
  double angle[kMotionParams];
  double ty[kMotionParams];
  double kin[kKinScalars][kMotionParams];
};
int motion_tangent(const HostBlock* hb, double phase_angle, double freq, double deltat, double tot_at_ita0,
                   int64_t ita0, int64_t last, std::vector<StepTangent>& out);
int build_node_csr(HostBlock* hb, std::vector<int>& off, std::vector<int>& ent);
int launch_geometry_place_adj(HostBlock* hb, const double* ge, const int* off_dev, const int* ent_dev,
                              const Place& P, double* scratch, double* place_bar);
int launch_stress_weights(HostBlock* hb, double mu_f, double rho_f, const double* seed_dev, double* w,
                          double* scratch);

// Refresh the device table of block views (no copy when unchanged, so a
// captured step contains none).
int sync_block_table();

enum class Extent { Interior, Points };

inline int64_t op_cells(const HostBlock* hb, Extent e) {
  const Dims& d = hb->d.d;
  return e == Extent::Interior ? (int64_t)d.nx * d.ny * d.nz : d.npts();
}

// One phase operation over the given blocks: one launch per block, or, with
// batching on and several blocks, one launch per group of up to kMaxBatch
// blocks.  `cap` bounds the CTAs of one block.
template <class Op, int NT>
int launch_op(const std::vector<HostBlock*>& hbs, const Op& op, Extent ext, unsigned cap) {
  if (hbs.empty()) return 0;
  if (hbs.size() == 1 || !lib().batch) {
    for (HostBlock* hb : hbs) {
      k_one<Op, NT><<<grid_for(op_cells(hb, ext), NT, cap), NT, 0, stream()>>>(hb->d, op);
      if (int r = note_launch()) return r;
    }
    return 0;
  }
  if (int r = sync_block_table()) return r;
  for (size_t g0 = 0; g0 < hbs.size(); g0 += kMaxBatch) {
    BlockSet S{};
    S.tab = lib().dtab;
    S.nb = (int)std::min<size_t>(kMaxBatch, hbs.size() - g0);
    int grid = 0;
    for (int m = 0; m < S.nb; ++m) {
      const HostBlock* hb = hbs[g0 + m];
      S.ids[m] = hb->index;
      S.cta_off[m] = grid;
      grid += (int)grid_for(op_cells(hb, ext), NT, cap);
    }
    S.cta_off[S.nb] = grid;
    k_set<Op, NT><<<grid, NT, 0, stream()>>>(S, op);
    if (int r = note_launch()) return r;
  }
  return 0;
}

}  // namespace bcfd
