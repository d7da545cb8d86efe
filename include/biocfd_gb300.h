/*
 * biocfd_gb300.h -- C ABI of the GB300-native Bio-CFD hot path.
 *
 * Each entry point replaces one Fortran module subroutine of the reference
 * (BioFSILab/Bio-CFD) on its per-time-step path; the reference routine is
 * cited beside the declaration as file:line.  A thin ISO_C_BINDING shim keeps
 * the reference's module and subroutine names, so app/main.F90 relinks
 * unchanged (the shim is bio-cfd_gb300/fortran/biocfd_gb300_shim.f90).
 *
 * Conventions
 *   - Block data live on the GPU.  A block is registered once and addressed
 *     by an opaque handle; the Fortran Block_t arrays are host mirrors that
 *     are copied in with the upload calls and out with the download calls.
 *   - Arrays passed in or out have the reference's layout: column-major,
 *     1-based extents of src/AllocateArrays.f90 / src/ReadInput.f90, FP64
 *     reals and int64 integers, so a Fortran caller passes c_loc(arr).
 *   - Every function returns 0 (BCFD_OK) or a negative bcfd_status.  Calls
 *     enqueue work on the library stream; calls that return data to the host
 *     synchronise.  Calls on different handles may come from different host
 *     threads (they are serialised inside the library).
 */
#ifndef BIOCFD_GB300_H
#define BIOCFD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int64_t bcfd_handle;

enum bcfd_status {
  BCFD_OK = 0,
  BCFD_E_HANDLE = -1,      /* unknown block or interface handle               */
  BCFD_E_NOMEM = -2,       /* device allocation failed                        */
  BCFD_E_NONFINITE = -3,   /* NaN/Inf in a residual or reduction              */
  BCFD_E_NOTFOUND = -4,    /* probe bracket not found (find_index_in_array)   */
  BCFD_E_TIMEOUT = -5,     /* a bounded device-side wait gave up              */
  BCFD_E_ARG = -6,         /* invalid argument                                */
  BCFD_E_CUDA = -7,        /* CUDA runtime error                              */
  BCFD_E_STATE = -8,       /* call out of order (e.g. lists before tagging)   */
  BCFD_E_CAPACITY = -9     /* a list outgrew its device capacity              */
};

/* ---- library ---------------------------------------------------------- */
int bcfd_init(int device);
int bcfd_finalize(void);
int bcfd_synchronize(void);
/* the cudaStream_t all work is enqueued on (for event timing by a caller) */
int bcfd_get_stream(void** stream);
const char* bcfd_status_string(int status);
/* number of kernels this library has launched since bcfd_init */
int64_t bcfd_kernel_launches(void);
/* 1 (default): the per-block phases of a time step (momentum, divergence,
 * corrections, reductions, copies, and the Poisson solves of the blocks that
 * are solved together) run over all blocks in one launch per phase, driven by
 * a device table of block views; 0: one launch per block.  Same results. */
int bcfd_set_batching(int on);
/* 1: the Poisson solves of the residual-target precisions (1-3 of
 * bcfd_step_config) start from the previous step's correction pc at the cells
 * they update instead of from pc = 0 (no counterpart in the reference, which
 * zeroes pc before every poissonSolver, src/PcorVcor.F90:74-80).  The stop
 * test, the operator and the boundary data (0 at solid cells and faces, the
 * coupling ghosts) are unchanged, so each solve still ends at the requested
 * residual; only its starting point differs.  0 (default): zero start.  The
 * drop-in precision 0 always starts from 0. */
int bcfd_set_warm_start(int on);
/* Longest time (ns) any single device-side wait of a persistent kernel (the
 * grid barriers and the neighbour-tile waits of the Poisson solves, the
 * forcing's level barriers) may spin before the kernel gives up: it records
 * BCFD_E_TIMEOUT, every CTA leaves its loops and the call that launched it
 * returns BCFD_E_TIMEOUT; the context stays usable.  0 restores the default
 * (2 s); at most 600 s.  No counterpart in the reference (its OpenACC loops
 * do not wait on each other). */
int bcfd_set_wait_limit_ns(int64_t ns);
/* Self-check of the bounded waits (no counterpart in the reference): launches
 * one grid barrier that nothing can complete and returns in *status what the
 * device recorded (BCFD_E_TIMEOUT once the wait limit passed) and in
 * *waited_ms (may be NULL) the kernel's duration.  The context stays usable. */
int bcfd_check_wait_limit(int* status, double* waited_ms);
/* Caps the entries of a block's IB / thin-surface lists (no counterpart in
 * the reference, whose lists are allocated to fit): 0 restores the allocated
 * capacity, min(interior cells, 4M); a lower cap makes a list that outgrows
 * it report BCFD_E_CAPACITY (entries beyond it are dropped, never written). */
int bcfd_block_set_list_capacity(bcfd_handle h, int64_t cap);

/* ---- block registration and host mirrors (src/Blocks.f90:13-81) --------- */
/* Allocates the per-block device arrays of src/AllocateArrays.f90:15-57 and
 * sets the grid from x1(1:nx+3), y1, z1 and deltax(1:nx+2), deltay, deltaz
 * (src/ReadInput.f90:250-351); xu..zp are derived as the reference does. */
int bcfd_block_create(int64_t nx, int64_t ny, int64_t nz, const double* x1, const double* y1,
                      const double* z1, const double* deltax, const double* deltay,
                      const double* deltaz, bcfd_handle* out);
int bcfd_block_destroy(bcfd_handle h);
/* after a block move (src/Search.F90:1208-1264): new x1/y1/z1, deltas kept */
int bcfd_block_set_grid(bcfd_handle h, const double* x1, const double* y1, const double* z1);
/* Block_t scalars: dx, dy, dz (src/ReadInput.f90:233-239) and omega (:353-360) */
int bcfd_block_set_scalars(bcfd_handle h, double dx, double dy, double dz, double omega);
/* body_search.dat box of tagging_th_core (src/ReadInput.f90:103-111) */
int bcfd_block_set_search_box(bcfd_handle h, int64_t i0, int64_t i1, int64_t j0, int64_t j1,
                              int64_t k0, int64_t k1);
/* surface mesh (src/ReadInput.f90:365-426): element node ids (1-based),
 * physical tags, and the shifted node coordinates xnode1/ynode1/znode1 */
int bcfd_block_set_surface(bcfd_handle h, int64_t n_elems, int64_t n_nodes, const int64_t* elp1,
                           const int64_t* elp2, const int64_t* elp3, const int64_t* surf_id,
                           const double* xnode1, const double* ynode1, const double* znode1);
/* new node positions after the body kinematics (src/Search.F90:126-208) */
int bcfd_block_set_nodes(bcfd_handle h, const double* xnode1, const double* ynode1,
                         const double* znode1);
/* rigid-body kinematics read by the forcing routines: kin[11] =
 * {xdot, ydot, yddot, thetaDot1, thetaDDot1, thetaDot2, thetaDDot2, alphaDot,
 *  piv_x, piv_y, piv_z} */
int bcfd_block_set_kinematics(bcfd_handle h, const double* kin);
/* Block_t move_check / blk_mv_tag (a negative value leaves that flag as it is) */
int bcfd_block_set_flags(bcfd_handle h, int64_t move_check, int64_t blk_mv_tag);
/* fields (nx+2,ny+2,nz+2); any pointer may be NULL */
int bcfd_block_upload_fields(bcfd_handle h, const double* u, const double* v, const double* w,
                             const double* p, const double* ut, const double* vt, const double* wt);
int bcfd_block_download_fields(bcfd_handle h, double* u, double* v, double* w, double* p,
                               double* ut, double* vt, double* wt);
/* tags: cell, cell_n (nx+2)^3 and cell2, nodeIdTag, cell_pr (nx+3)^3, int64 */
int bcfd_block_upload_tags(bcfd_handle h, const int64_t* cell, const int64_t* cell2,
                           const int64_t* node_id_tag, const int64_t* cell_n,
                           const int64_t* cell_pr);
int bcfd_block_download_tags(bcfd_handle h, int64_t* cell, int64_t* cell2, int64_t* node_id_tag,
                             int64_t* cell_n, int64_t* cell_pr);
/* counts[6] = ibCellCount, solidCellCount, fluidCellCount, redCellCount,
 * blackCellCount, TSCellCount */
int bcfd_block_get_counts(bcfd_handle h, int64_t* counts);
/* the per-block Poisson statistics nIterPcor, derr2, derrStdSt */
int bcfd_block_get_sor_stats(bcfd_handle h, int64_t* n_iter, double* derr2, double* derr_std_st);
int bcfd_block_set_sor_iter(bcfd_handle h, int64_t n_iter);
/* named host read-back of any other device array, in the reference layout:
 * "pc", "b", "xcent", ..., "pNormDis", "nelp", "p_ghost", "fluidIndexPtr",
 * "interceptedIndexPtr", "solidIndexPtr", "redCellIndexPtr", "TSIndexPtr",
 * "index_ts", "Acx", "ca_uu", "x1", "xnode1", "xdot", ..., "mk", "move_check",
 * "blk_mv_tag", "move_amtx", ...  (reals as double, integers as int64);
 * n = capacity in elements, *written = elements written */
int bcfd_block_read(bcfd_handle h, const char* name, void* out, int64_t n, int64_t* written);
/* named host write of the device arrays a caller may need to set besides
 * the fields: the 14 TS ghost arrays ("p_ghost", "pt_ghost", ..., "w1t_ghost",
 * Block_t's ghost components; n must equal the TS cell count), e.g. to resume
 * a plate's state mid-run.  BCFD_E_NOTFOUND for other names. */
int bcfd_block_write(bcfd_handle h, const char* name, const double* data, int64_t n);

/* ---- setup routines ------------------------------------------------------ */
int bcfd_non_uni_coeff(bcfd_handle h);                    /* src/NavierStokes.f90:13-250 */
int bcfd_coefficient_matrix(bcfd_handle h, int is_coarse); /* src/CoefficientMatrix.f90:10-71 */

/* ---- momentum predictor and boundary conditions --------------------------- */
int bcfd_ns_momentum_2order(bcfd_handle h, double deltat, double re); /* src/NavierStokes.f90:252-912 */
int bcfd_velocity_bc(bcfd_handle h, double deltat, double uc);        /* src/BoundaryConditions.f90:11-74 */
int bcfd_solid_cell_bc(bcfd_handle h);                                /* src/BoundaryConditions.f90:76-92 */
int bcfd_solid_cell_bc_move(bcfd_handle h);                           /* src/BoundaryConditions.f90:94-115 */

/* ---- immersed-boundary forcing ------------------------------------------ */
int bcfd_velocity_forcing1(bcfd_handle h);       /* src/Forcing.f90:92-360   */
int bcfd_pressure_forcing1(bcfd_handle h);       /* src/Forcing.f90:14-90    */
int bcfd_velocity_forcing_field(bcfd_handle h);  /* src/Forcing.f90:813-1075 */
int bcfd_pressure_forcing_field(bcfd_handle h);  /* src/Forcing.f90:737-811  */
int bcfd_velocity_forcing_ghost(bcfd_handle h);  /* src/Forcing.f90:450-734  */
int bcfd_pressure_forcing_ghost(bcfd_handle h);  /* src/Forcing.f90:362-448  */

/* ---- Search / tagging ---------------------------------------------------- */
int bcfd_compute_surface_norm(bcfd_handle h, int64_t inor); /* src/Search.F90:210-258  */

/* ---- rigid-body motion of a block's surface (src/Search.F90:49-208) ---- */
/* p[6] = a0 (pitch amplitude in degrees, as read), bfreq (heave frequency),
 * yamp (heave amplitude), xshift, yshift, zshift (body placement).  The nodes
 * set with the surface become the body frame (xnode of Block_t); node surface
 * ids follow src/ReadInput.f90:403-420. */
int bcfd_block_set_body_motion(bcfd_handle h, const double* p);
/* A phase lag of this body's heave and pitch behind the kinematics that every
 * body shares (no counterpart in the reference, whose kinematics take one
 * phase angle for all bodies: src/Search.F90:142, app/main.F90:62,173).  With
 * lag L (radians) the body pitches a0 sin(2 pi freq (t + dt) + phase - L) and
 * heaves yamp sin(2 pi bfreq t - L); its initial placement
 * (bcfd_shift_surface_nodes_initial) starts it where the lagged kinematics
 * put it at t = 0: angle aoa + a0 (sin(phase_angle - L) - sin(phase_angle))
 * and heave position yamp sin(-L), where phase_angle is the pitch phase the
 * bodies share (radians).  L = 0 (the default, and what
 * bcfd_block_set_body_motion resets to) is the reference's arithmetic bit for
 * bit.  Call after bcfd_block_set_body_motion, before the initial placement;
 * BCFD_E_STATE without body motion. */
int bcfd_block_set_body_lag(bcfd_handle h, double lag, double phase_angle);
int bcfd_shift_surface_nodes_initial(bcfd_handle h, double aoa, double piv_pt, int64_t ita,
                                     double deltat, double dxmin, double totime); /* src/Search.F90:49-124 */
int bcfd_compute_surface_variables(bcfd_handle h, double phase_angle, double piv_pt, int64_t ita,
                                   double deltat, double dxmin, double freq,
                                   double totime);                             /* src/Search.F90:126-208 */
/* inputs of app/main.F90 the native driver needs for moving bodies (phase
 * angle in radians) and its time counters ita / totime, which bcfd_run_steps
 * advances like main.F90:130-131 */
int bcfd_set_motion_inputs(double phase_angle, double piv_pt, double freq, double dxmin, int64_t inor,
                           int64_t ita, double totime);
int bcfd_get_time(int64_t* ita, double* totime);
int bcfd_tagging_th(bcfd_handle h);                         /* src/Search.F90:260-413  */
int bcfd_selective_retagging_th(bcfd_handle h);             /* src/Search.F90:520-651  */
int bcfd_cellcount_solid(bcfd_handle h);                    /* src/Search.F90:653-741  */
int bcfd_compute_norm_distance(bcfd_handle h);              /* src/Search.F90:743-861  */
int bcfd_find_ts_cells(bcfd_handle h);                      /* src/Search.F90:434-518  */
int bcfd_cellcount_solid_coarse(bcfd_handle h);             /* src/Search.F90:1463-1532 */
int bcfd_fine_block_cell(void);                             /* src/Search.F90:863-914  */

/* ---- pressure correction ------------------------------------------------- */
int bcfd_compute_div(bcfd_handle h);                        /* src/PcorVcor.F90:222-243 */
int bcfd_correct_pressure(bcfd_handle h);                   /* src/PcorVcor.F90:245-259 */
int bcfd_correct_velocity(bcfd_handle h, double deltat);    /* src/PcorVcor.F90:261-286 */
int bcfd_redblack_sor_linear(bcfd_handle h, int64_t pc_ita_max, double deltat,
                             double epsi);                  /* src/PcorVcor.F90:288-377 */
int bcfd_update_velocity_newv(bcfd_handle h);               /* src/PcorVcor.F90:379-397 */
/* poissonSolver over the registered blocks start..finish by step (1-based
 * registration order; block 1 is the coarse block): src/PcorVcor.F90:22-220.
 * totalTime accumulates totime per block as in the reference. */
int bcfd_poisson_solver(int64_t pc_ita_max, double epsi, int64_t ita, double deltat,
                        double totime, double uc, double* total_time, int start, int finish,
                        int step);

/* ---- inter-block coupling ------------------------------------------------ */
/* interface between coarse block a and fine block b at mesh ratio b_msh/a_msh
 * over box[6] = {xs, xe, ys, ye, zs, ze}; builds the tables of
 * src/InterfaceDetail.f90:10-165 (set_interface_detail :168-241) */
int bcfd_interface_create(bcfd_handle a, bcfd_handle b, int64_t a_msh, int64_t b_msh,
                          const double* box, bcfd_handle* out);
/* table read-back: name in {px,py,pz,ux,...,wz}; out (3, n) int64 */
int bcfd_interface_table(bcfd_handle it, const char* name, int64_t* out, int64_t n,
                         int64_t* counter);
int bcfd_fine_update_pc_bd(void);              /* src/FineInterp_bound.f90:17-107   */
int bcfd_fine_update_newv_bd(void);            /* src/FineInterp_bound.f90:109-309  */
int bcfd_fine_update_bd_mv(bcfd_handle it);    /* src/FineInterp_bound.f90:311-544  */
int bcfd_coarse_update(void);                  /* src/CoarseInterp.f90:16-204       */
int bcfd_coarse_update_newv(void);             /* src/CoarseInterp.f90:206-346      */
int bcfd_coarse_update_pc(void);               /* src/CoarseInterp.f90:347-437      */
int bcfd_fine_update_mv(bcfd_handle it);       /* src/FineInterp.f90:10-281         */

/* ---- adjoint of the pressure Poisson solve (no counterpart in the reference) --
 * Both solve on the fluid cells of a block with zero boundary data, FP64
 * red-black SOR to max|r - A x| <= tol (at most itmax sweep pairs); r and x
 * are natural-layout (nx+2)(ny+2)(nz+2) arrays, x is 0 off the fluid cells.
 * The adjoint runs the same solve kernel with the transposed line tables of
 * A and the colour sweeps in reverse order.  They use the block's Poisson
 * arrays as scratch (call between time steps). */
/* the solver of bcfd_poisson_solve_zero_bc / _adjoint and of the adjoint
 * solves in bcfd_adjoint_run (no counterpart in the reference): 0 FP64 SOR,
 * 1 (default) FP32 red-black sweeps with FP64 defect correction; both stop at
 * the same FP64 residual target */
int bcfd_adjoint_set_solver(int precision);
int bcfd_poisson_solve_zero_bc(bcfd_handle h, const double* r, double* x, double tol, int64_t itmax);
int bcfd_poisson_solve_adjoint(bcfd_handle h, const double* r, double* x, double tol, int64_t itmax);
/* tangent-linear model of nsMomentum2order (no counterpart in the reference):
 * at the block's current u,v,w,p, (ut,vt,wt) = the predictor's values (bitwise
 * those of bcfd_ns_momentum_2order; the block's own ut,vt,wt are untouched)
 * and (dut,dvt,dwt) = its exact derivative along (du,dv,dw,dp); natural-layout
 * host arrays, outputs 0 off the fluid cells.  Not for cells within reach of
 * thin-surface cells (BCFD_E_STATE). */
int bcfd_momentum_tangent(bcfd_handle h, double deltat, double re, const double* du, const double* dv,
                          const double* dw, const double* dp, double* ut, double* vt, double* wt, double* dut,
                          double* dvt, double* dwt);
/* adjoint of nsMomentum2order (no counterpart in the reference): at the
 * block's current u,v,w,p, (ub,vb,wb,pb) = J^T (utb,vtb,wtb) with J the
 * Jacobian of the predictor's fluid-cell outputs (the transpose of
 * bcfd_momentum_tangent), accumulated per input point in a fixed order
 * (deterministic).  Natural-layout host arrays; same thin-surface limit. */
int bcfd_momentum_adjoint(bcfd_handle h, double deltat, double re, const double* utb, const double* vtb,
                          const double* wtb, double* ub, double* vb, double* wb, double* pb);
/* The same with the thin-surface (TS) overlay of a plate (surfaces 51/52,
 * src/NavierStokes.f90:310-490, 860-907) transposed (no counterpart in the
 * reference).  ub,vb,wb,pb on entry: the adjoint of u,v,w,p after the call
 * (the loop leaves t-ghost values at the TS positions it restores); on
 * return: the adjoint of u,v,w,p before it.  gb (14 x n_ts, the ghost[]
 * order p, pt, u2, u2t, v2, v2t, w2, w2t, u1, u1t, v1, v1t, w1, w1t of
 * bcfd_block_read) receives the adjoint of the ghost arrays the predictor
 * read.  The block's ghost arrays must hold the values of the forward call. */
int bcfd_momentum_adjoint_ts(bcfd_handle h, double deltat, double re, const double* utb, const double* vtb,
                             const double* wtb, double* ub, double* vb, double* wb, double* pb, double* gb);
/* Transpose of velocityForcingGhost and pressureForcingGhost
 * (src/Forcing.f90:450-734, 362-448) at the block's current geometry and
 * kinematics (no counterpart in the reference): each ghost value is affine in
 * the 8 probe values of ut/vt/wt (p for the pressure ghost), each t-ghost
 * value a copy of u/v/w (p) at the TS position.  Adds G^T gb to
 * (ub, vb, wb, pb, utb, vtb, wtb); gb as in bcfd_momentum_adjoint_ts. */
int bcfd_forcing_ghost_adjoint(bcfd_handle h, const double* gb, double* ub, double* vb, double* wb, double* pb,
                               double* utb, double* vtb, double* wtb);

/* ---- coupling maps and their transposes (no counterpart in the reference) --
 * Interface h, component comp (0 p, 1 u, 2 v, 3 w), natural-layout host
 * arrays of the coarse (a) and fine (b) blocks:
 *   op 0: out(fine)   = P in(coarse)   the face fill of src/FineInterp_bound.f90
 *   op 1: out(coarse) += P^T in(fine)  deterministic gather per coarse donor
 *   op 2: out(coarse) = R in(fine)     the restriction of src/CoarseInterp.f90
 *   op 3: out(fine)   += R^T in(coarse) scatter (donor boxes are disjoint)
 * ops 0 and 2 overwrite only the points they fill. */
int bcfd_coupling_apply(bcfd_handle h, int comp, int op, const double* in, double* out);

/* ---- drag / lift (src/StressCalc.f90:14-208, FP64, deterministic order) --- */
/* out[4] = viscous drag, pressure drag, viscous lift, pressure lift coefficients */
int bcfd_stress_calculation(bcfd_handle h, double mu_f, double rho_f, double* out);
/* The same computation and result without any device allocation; this entry
 * point has no counterpart in the reference.  bcfd_stress_calculation
 * cudaMallocs and cudaFrees its scratch on every call, and cudaFree waits for
 * the whole device, so a caller that samples drag/lift every step while other
 * streams run, or one whose memory is held by a caching allocator, uses this
 * instead.  Scratch is a fixed 7 * BCFD_STRESS_NOALLOC_MAX_ELEMS + 4 doubles
 * (1.8 MB) per device inside the library; nothing in it has to start at zero.
 * A block with more than BCFD_STRESS_NOALLOC_MAX_ELEMS surface elements
 * returns BCFD_E_CAPACITY.  The first call on a device does set-up (looks up
 * the scratch address), so make it before any stream capture begins.  Calls
 * through the library are serialised and synchronise before returning; two
 * calls overlapping on one device by any other route would race on the
 * scratch. */
#define BCFD_STRESS_NOALLOC_MAX_ELEMS 32768
int bcfd_stress_calculation_noalloc(bcfd_handle h, double mu_f, double rho_f, double* out);

/* ---- whole time step (the phase order of app/main.F90:129-265) ----------- */
typedef struct bcfd_step_config {
  double deltat;       /* time step                                            */
  double re;           /* the reference's `re` argument, 1/nu                  */
  double uc;           /* inflow velocity                                      */
  double epsi;         /* SOR stop threshold on max |pc - pco|                 */
  int64_t pc_ita_max;  /* SOR iteration cap                                    */
  int precision;       /* 0: FP64 reference arithmetic and stop test (drop-in);
                          1: FP32 SOR + FP64 defect correction to div_tol;
                          2: FP64 SOR (reference sweeps) to div_tol;
                          3: FP64 SOR without divisions (fused residual, the
                             inverse diagonal by Newton-Raphson) to div_tol   */
  double div_tol;      /* precision 1-3: target FP64 Poisson residual in
                          divergence units, deltat * max|b/deltat - A pc|;
                          must be > 0 (BCFD_E_ARG otherwise).  The residual
                          is checked at an adaptive cadence (after each FP32
                          correction, whose length follows the measured
                          reduction rate; every 5 to 64 FP64 sweep pairs)    */
  int use_graph;       /* capture the step in a CUDA graph and replay it       */
} bcfd_step_config;

/* Runs n_steps time steps over every registered block and interface with the
 * per-block roles set by bcfd_block_set_role (domain BCs / immersed body). */
int bcfd_block_set_role(bcfd_handle h, int is_coarse, int has_body);
int bcfd_run_steps(const bcfd_step_config* cfg, int64_t n_steps);
/* the fine-block moves of app/main.F90:178-211 after computeSurfaceVariables:
 * block_move_check, change_block_coords, change_block_coords_interfaces,
 * change_block_interface (src/Search.F90:997-1461), then fine_block_cell and
 * cellCount_solid_coarse_mv (:863-995) when a block moved; *moved = 1 then.
 * Only blocks with body motion are checked.  BCFD_E_STATE when a move would
 * take a fine block's coupling stencils outside the coarse block. */
int bcfd_block_move_stage(int64_t* moved);
/* tagging_th_move (src/Search.F90:415-432): a block that moved is re-tagged
 * and refilled from the coarse block (fineUpdate_mv, fineUpdate_bd_mv) */
int bcfd_tagging_th_move(bcfd_handle h);
/* Discrete adjoint of n_steps whole time steps (no counterpart in the
 * reference).  Scope: block 1 with the domain BCs plus fine blocks coupled to
 * it by interfaces, FP64 drop-in steps (cfg->precision 0), stationary immersed
 * bodies without thin-surface cells (BCFD_E_STATE for body motion).  The
 * objective and the returned gradients refer to block h.  Runs the steps
 * forward from the blocks' state with ut,vt,wt = u,v,w, checkpointing
 * (u,v,w,p,ut,vt,wt of every block) every `every` steps in HBM, and returns
 *   J = (1/N) sum_{n=1..N} ( <W, x^n> + sum_t stress_seed[t] * C_t(x^n) )
 * for natural-layout weights W = (wu,wv,ww,wp) over (u,v,w,p) and, when
 * stress_seed (4 values) is non-null, the drag/lift coefficients C_t of
 * bcfd_stress_calculation with (mu_f, rho_f) (a body is required).  When any
 * gradient output is non-null it then runs the reverse pass, recomputing each
 * segment from its checkpoint, and returns dJ/duc, dJ/d(u,v,w,p)^0 and
 * dj_dkin[8], the derivative with respect to the body's rigid-body kinematic
 * scalars in bcfd_block_set_kinematics order (xdot, ydot, yddot, thetaDot1,
 * thetaDDot1, thetaDot2, thetaDDot2, alphaDot) held constant over the run
 * with the geometry fixed (the body's surface velocity and acceleration in
 * the forcing and in the coefficients); the
 * adjoint Poisson solves run to max|r - A^T y| <= adj_tol (at most adj_itmax
 * iterations).  The tags must not change during the run (BCFD_E_STATE
 * otherwise).  The blocks are left at the forward run's final state. */
int bcfd_adjoint_run(bcfd_handle h, const bcfd_step_config* cfg, int64_t n_steps, int64_t every, const double* wu,
                     const double* wv, const double* ww, const double* wp, const double* stress_seed, double mu_f,
                     double rho_f, double adj_tol, int64_t adj_itmax, double* J, double* dj_duc,
                     double* dj_dkin, double* gu, double* gv, double* gw, double* gp);
/* Discrete adjoint of n_steps whole time steps through moving bodies (no
 * counterpart in the reference): the objective J of bcfd_adjoint_run on block
 * h, whose body moves, and dj_dmotion[5] = dJ/d of its motion parameters
 * (heave amplitude yamp, pitch amplitude a0 in degrees, the pitch phase angle
 * in radians, the pitch frequency freq, the heave frequency bfreq of
 * bcfd_block_set_body_motion and bcfd_set_motion_inputs), plus dJ/duc and
 * dJ/d(u,v,w,p)^0 as there.  Other moving bodies of the run (a plate in
 * tandem, with its own phase lag) move with the run and contribute to the
 * parameters they share with block h's body -- the phase angle and the
 * pitch frequency -- through their geometry and kinematics too.  The
 * parameters reach J through every step's node placement (rotation about x
 * through the pivot, translation), the element centroids, normals and lengths
 * (src/Search.F90:126-258), the normal distances and probe points of the IB
 * forcing (src/Forcing.f90) and the drag/lift of the moving surface, and
 * through the rigid-body kinematic scalars the forcing and drag/lift read; the
 * discrete choices (tags, lists, nearest elements, probe brackets, upwind
 * branches) are those of the forward run at each step.  Each segment of
 * `every` steps is recomputed from its checkpoint (fields, tags, nodes and
 * motion state).  Thin-surface cells (surfaces 51/52 of a plate) are
 * differentiated through the predictor's ghost substitution and restore and
 * through the ghost calls.  Refused (BCFD_E_STATE): a fine-block move during
 * the run, precision /= 0.  The blocks are left at the forward run's final
 * state. */
int bcfd_adjoint_run_motion(bcfd_handle h, const bcfd_step_config* cfg, int64_t n_steps, int64_t every,
                            const double* wu, const double* wv, const double* ww, const double* wp,
                            const double* stress_seed, double mu_f, double rho_f, double adj_tol, int64_t adj_itmax,
                            double* J, double* dj_duc, double* dj_dmotion, double* gu, double* gv, double* gw,
                            double* gp);
/* max over fluid cells of |div u| of the current u,v,w (FP64, the backward
 * differences times the reciprocal spacings: within an ulp of the divided
 * form of computeDiv) */
int bcfd_max_divergence(bcfd_handle h, double* out);
/* out[0] = max over fluid cells of |div ut| right after the last velocity
 * correction; out[1] = deltat * max over fluid cells of |b/deltat - A pc|, the
 * FP64 Poisson residual of the last solve in divergence units (the divergence
 * the correction leaves wherever the operators are consistent) */
int bcfd_block_get_divergence(bcfd_handle h, double* out);
/* mixed-precision solve parameters of a block: FP32 sweep pairs of the first
 * correction and the most of any later one (0: 64), their relaxation factor
 * (0 selects the default, bcfd_block_get_mixed_omega) and the kernel variant
 * (0: the library's choice, 1: tiled cooperative with grid-wide phase
 * barriers, 3: tiled cooperative with point-to-point neighbour sync, 4:
 * temporal-blocked sweeps, one grid barrier per sweep pair, when the block's
 * halo'd tiles fit in shared memory, else 1; 5: z-marching sweeps, two
 * sweep pairs per pass over the block with the correction staged in shared
 * memory by TMA, when a packed row fits one TMA box (nx <= 509), else 1;
 * 1, 3, 4 and 5 give bitwise the same corrections; 2 is not accepted) */
int bcfd_block_set_mixed_params(bcfd_handle h, int64_t inner_sweeps, double omega, int variant);
/* the relaxation factor block h's FP32 correction sweeps use (its setting or
 * the default: 2 / (1 + sqrt(1 - rho^2)), rho = (cos(pi/nx) + cos(pi/ny) +
 * cos(pi/nz)) / 3; at most 1.99), before its rounding to FP32 (no counterpart
 * in the reference) */
int bcfd_block_get_mixed_omega(bcfd_handle h, double* omega);
/* launch shape of a block's tiled Poisson solves (the autotuner's knobs; no
 * effect on results): threads per CTA (0 = the default: 512 for the FP64
 * solve, 256 for the mixed one, which takes at most 256; else 128/256/512), cap
 * on co-resident CTAs per SM (0 = occupancy limit), and the FP64 solve's
 * phase sync (0 point-to-point between neighbour tiles, 1 grid-wide) */
int bcfd_block_set_solve_launch(bcfd_handle h, int threads, int ctas_per_sm, int fp64_sync);
/* out[6] = FP64 solve threads, CTAs/SM cap, sync; FP32 correction threads,
 * CTAs/SM cap, variant (0 = library default) */
int bcfd_block_get_solve_launch(bcfd_handle h, int* out);
/* Autotuner (no counterpart in the reference): for every block, times short
 * solves under each candidate launch shape of the FP64 solve and of the FP32
 * correction (threads per CTA, CTAs per SM, which sets the tile shape, the
 * phase synchronisation, the sweep variant) and keeps the fastest; results are
 * cached per block shape.  The blocks whose solves batching would run side
 * by side in one launch (every block after the first, when there are several)
 * keep that launch only if it beats their best launches one after the other
 * (timed, per precision).  None of these changes the arithmetic.  The blocks'
 * solve state is restored afterwards.  *n_tuned = shapes newly timed. */
int bcfd_autotune(int64_t* n_tuned);
/* measurement: exactly n_pairs red-black sweep pairs of the block's Poisson
 * system b = the current computeDiv result (deltat = 1), stop test disabled.
 * precision 0: the FP64 reference sweeps on pc; 1: one FP32 correction of
 * n_pairs sweeps (with its two FP64 residual passes and the FP64 update);
 * 2: the division-free FP64 sweeps of bcfd_step_config precision 3.
 * Changes pc; for timing and roofline measurement only. */
int bcfd_block_sor_sweeps(bcfd_handle h, int64_t n_pairs, int precision);

/* ---- measurement window (no counterpart in the reference) ----------------- */
typedef struct bcfd_profile_report {
  int64_t sor_launches;   /* persistent Poisson-solve launches in the window      */
  double sor_ms;          /* their summed device time (CUDA events, library stream) */
  double sor_bytes;       /* algorithmic bytes they moved (4w+1 B per cell sweep
                             pair, w = 8 FP64 / 4 FP32; 13 B per cell per two
                             pairs for the z-marching sweeps; plus the FP64
                             residual and update passes of the mixed solve)       */
  int64_t sor_sweeps;     /* red+black sweep pairs done by them                    */
  int64_t kernel_launches;/* kernels launched in the window                        */
} bcfd_profile_report;
int bcfd_profile_begin(void);
int bcfd_profile_end(bcfd_profile_report* out);
/* Device time (ms) per phase of the time steps issued eagerly (use_graph 0)
 * inside the last measurement window, summed over the window's steps:
 * ms[0] nsMomentum2order and the domain BCs, [1] solid-cell BCs,
 * velocityForcing1 and pressureForcing1, [2] the Poisson solves, [3] the
 * coarse/fine face fills and restrictions, [4] zeroing, divergence,
 * pressure and velocity corrections, reductions and copies, [5] body motion,
 * normals, fine-block moves, re-Search and index lists, [6] the forcing on
 * the re-searched geometry (Field and Ghost variants).  n <= 7 entries. */
int bcfd_profile_phases(double* ms, int n);
/* Measured arithmetic rates of this GPU (no counterpart in the reference):
 * out[0] FP64 fused multiply-add GFLOP/s (2 per FMA), out[1] FP64 IEEE
 * divisions in G/s, out[2] FP32 fused multiply-add GFLOP/s; chains of
 * independent operations on every SM, best of three CUDA-event timings. */
int bcfd_measure_alu_rates(double* out);

#ifdef __cplusplus
}
#endif
#endif /* BIOCFD_GB300_H */
