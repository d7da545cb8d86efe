// Discrete adjoint of whole time steps of one body-free block with the domain
// boundary conditions (the coarse-block phase order of app/main.F90:129-265
// without bodies or interfaces), with forward checkpoints every K steps and
// recomputation in between.
//
// One step maps the state x = (u,v,w,p) to x' (the work arrays start as
// ut = u, which the ut -> u copy at the end of every step maintains):
//   S1 ut,vt,wt = M(x) on the fluid cells         nsMomentum2order
//   S2,S3 velocityBC twice (reads x and uc)        BoundaryConditions.f90:11-74
//   S4 b = D ut                                    computeDiv
//   S5 pc = A^{-1} (b / deltat), pc = 0 off fluid REDBLACKSOR_linear
//   S6 p' = p + pc on the fluid cells              correctPressure
//   S7 ut -= deltat G pc                           correctVelocity
//   S9 velocityBC (third time, after the solve)    poissonSolver
//   S11 u' = ut                                    updateVelocity
// The objective is J = (1/N) sum_{n=1..N} <W, x^n> for weights W over the four
// fields (a pressure integral over a control surface, a momentum flux through
// a plane, a probe mean).  The reverse pass applies the transposes in the
// opposite order: the BC assignments in reverse, the correction and
// divergence as gathers, the solve with A^T (the same SOR kernel on the
// transposed line tables, colours reversed) and the momentum adjoint at the
// step's own input state, recomputed from the nearest checkpoint.  Each
// adjoint value is a sum in a fixed order: the result is deterministic.
#include <array>

#include "bcfd_host.h"

namespace bcfd {
namespace {

struct Fields4 {
  double *u, *v, *w, *p;
};

__device__ __forceinline__ bool fluid_at(const DevBlock& B, int i, int j, int k) {
  const Dims& d = B.d;
  return i >= 2 && i <= d.nx + 1 && j >= 2 && j <= d.ny + 1 && k >= 2 && k <= d.nz + 1 &&
         B.cell[d.idx(i, j, k)] == 0;
}

// ---- velocityBC, transposed (kernel order z, y, x; assignments reversed) ----
// x faces (BoundaryConditions.f90:20-40); ucl[line] accumulates dJ/duc
__global__ void k_vbc_x_adj(DevBlock B, double deltat, double uc, double* ut_b, double* vt_b, double* wt_b,
                            Fields4 s, double* ucl) {
  const Dims& d = B.d;
  const int n = d.ny * d.nz;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int j = 2 + t % d.ny, k = 2 + t / d.ny;
    const int nx = d.nx;
    const int64_t c1 = d.idx(1, j, k), cn = d.idx(nx, j, k), cn1 = d.idx(nx + 1, j, k), cn2 = d.idx(nx + 2, j, k);
    const double ax = deltat / B.dxa[nx], bx = 2.0 * deltat / B.dxa[nx + 1];
    double g = 0.0, a;
    a = wt_b[cn2];
    wt_b[cn2] = 0.0;
    wt_b[cn1] -= a;
    s.w[cn2] += (1.0 - bx * uc) * a;
    s.w[cn1] += (1.0 + bx * uc) * a;
    g -= bx * (B.w[cn2] - B.w[cn1]) * a;
    a = vt_b[cn2];
    vt_b[cn2] = 0.0;
    vt_b[cn1] -= a;
    s.v[cn2] += (1.0 - bx * uc) * a;
    s.v[cn1] += (1.0 + bx * uc) * a;
    g -= bx * (B.v[cn2] - B.v[cn1]) * a;
    a = ut_b[cn1];
    ut_b[cn1] = 0.0;
    s.u[cn1] += (1.0 - ax * uc) * a;
    s.u[cn] += ax * uc * a;
    g -= ax * (B.u[cn1] - B.u[cn]) * a;
    a = wt_b[c1];
    wt_b[c1] = 0.0;
    wt_b[cn1] -= a;
    a = vt_b[c1];
    vt_b[c1] = 0.0;
    vt_b[cn1] -= a;
    a = ut_b[c1];
    ut_b[c1] = 0.0;
    g += a;
    ucl[t] += g;
  }
}

// y faces (BoundaryConditions.f90:42-58)
__global__ void k_vbc_y_adj(DevBlock B, double* ut_b, double* vt_b, double* wt_b) {
  const Dims& d = B.d;
  const int n = d.nx * d.nz;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int i = 2 + t % d.nx, k = 2 + t / d.nx;
    const int ny = d.ny;
    const int64_t a1 = d.idx(i, 1, k), a2 = d.idx(i, 2, k), an1 = d.idx(i, ny + 1, k), an2 = d.idx(i, ny + 2, k);
    vt_b[an1] = 0.0;
    wt_b[an1] += wt_b[an2];
    wt_b[an2] = 0.0;
    ut_b[an1] += ut_b[an2];
    ut_b[an2] = 0.0;
    vt_b[a2] = 0.0;
    wt_b[a2] += wt_b[a1];
    wt_b[a1] = 0.0;
    ut_b[a2] += ut_b[a1];
    ut_b[a1] = 0.0;
  }
}

// z faces (BoundaryConditions.f90:60-73)
__global__ void k_vbc_z_adj(DevBlock B, double* ut_b, double* vt_b, double* wt_b) {
  const Dims& d = B.d;
  const int n = d.nx * d.ny;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int i = 2 + t % d.nx, j = 2 + t / d.nx;
    const int nz = d.nz;
    const int64_t b1 = d.idx(i, j, 1), b2 = d.idx(i, j, 2), bn1 = d.idx(i, j, nz + 1), bn2 = d.idx(i, j, nz + 2);
    wt_b[bn1] = 0.0;
    vt_b[bn1] += vt_b[bn2];
    vt_b[bn2] = 0.0;
    ut_b[bn1] += ut_b[bn2];
    ut_b[bn2] = 0.0;
    wt_b[b1] = 0.0;  // the z pass zeroes w at k = 1 (the y pass zeroes v at j = 2)
    vt_b[b2] += vt_b[b1];
    vt_b[b1] = 0.0;
    ut_b[b2] += ut_b[b1];
    ut_b[b1] = 0.0;
  }
}

// correctVelocity and correctPressure transposed: pcb = adjoint of pc at every
// position the corrections read (the fluid cells, and the non-fluid neighbours
// whose pc is boundary data of the solve: fine-block ghosts, coarse cells
// under a fine block)
__global__ void k_correct_adj(DevBlock B, double dt, const double* ut_b, const double* vt_b, const double* wt_b,
                              const double* p_b, double* pcb) {
  const Dims& d = B.d;
  const int64_t n = d.npts(), sy = d.NX, sz = (int64_t)d.NX * d.NY;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(x % d.NX);
    const int64_t r = x / d.NX;
    const int j = 1 + (int)(r % d.NY), k = 1 + (int)(r / d.NY);
    double g = 0.0;
    if (fluid_at(B, i, j, k)) {
      g = p_b[x];
      g += dt / (0.5 * (B.dxa[i] + B.dxa[i - 1])) * ut_b[x];
      g += dt / (0.5 * (B.dya[j] + B.dya[j - 1])) * vt_b[x];
      g += dt / (0.5 * (B.dza[k] + B.dza[k - 1])) * wt_b[x];
    }
    if (fluid_at(B, i - 1, j, k)) g -= dt / (0.5 * (B.dxa[i - 1] + B.dxa[i - 2])) * ut_b[x - 1];
    if (fluid_at(B, i, j - 1, k)) g -= dt / (0.5 * (B.dya[j - 1] + B.dya[j - 2])) * vt_b[x - sy];
    if (fluid_at(B, i, j, k - 1)) g -= dt / (0.5 * (B.dza[k - 1] + B.dza[k - 2])) * wt_b[x - sz];
    pcb[x] = g;
  }
}

// The solve with boundary data: on the fluid cells A_ff pc = b/dt - A_fn g,
// g the pc held at non-fluid neighbours.  Given y = A_ff^{-T} pcb_f, the
// adjoint of g is pcb_g - A_fn^T y (pc at a non-fluid position also passes
// through unchanged); the fluid cells' incoming pc (the initial guess) has
// no influence at convergence.  A_fn's entries are the line-table
// coefficients of the fluid row for that neighbour.
__global__ void k_dirichlet_adj(DevBlock B, const double* y, double* pcb) {
  const Dims& d = B.d;
  const int64_t n = d.npts(), sy = d.NX, sz = (int64_t)d.NX * d.NY;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(x % d.NX);
    const int64_t r = x / d.NX;
    const int j = 1 + (int)(r % d.NY), k = 1 + (int)(r / d.NY);
    if (fluid_at(B, i, j, k)) {
      pcb[x] = 0.0;
      continue;
    }
    double s = 0.0;
    // x is the left neighbour of (i+1) and the right neighbour of (i-1), ...
    if (fluid_at(B, i + 1, j, k)) s += B.Acx[(i + 1) - 2] * y[x + 1];
    if (fluid_at(B, i - 1, j, k)) s += B.Acx[(i - 1) - 2 + 2 * nx] * y[x - 1];
    if (fluid_at(B, i, j + 1, k)) s += B.Acy[(j + 1) - 2] * y[x + sy];
    if (fluid_at(B, i, j - 1, k)) s += B.Acy[(j - 1) - 2 + 2 * ny] * y[x - sy];
    if (fluid_at(B, i, j, k + 1)) s += B.Acz[(k + 1) - 2] * y[x + sz];
    if (fluid_at(B, i, j, k - 1)) s += B.Acz[(k - 1) - 2 + 2 * nz] * y[x - sz];
    pcb[x] -= s;
  }
}

// a[x] = 0 where mask[x] != 0 (positions a coupling map overwrote)
__global__ void k_zero_masked(int64_t n, double* a, const double* mask) {
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x)
    if (mask[x] != 0.0) a[x] = 0.0;
}

__global__ void k_fill(int64_t n, double* a, double v) {
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x)
    a[x] = v;
}

// computeDiv transposed with the solve's 1/deltat: ut_b += D^T (y / deltat)
__global__ void k_div_adj(DevBlock B, double dt, const double* y, double* ut_b, double* vt_b, double* wt_b) {
  const Dims& d = B.d;
  const int64_t n = d.npts(), sy = d.NX, sz = (int64_t)d.NX * d.NY;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(x % d.NX);
    const int64_t r = x / d.NX;
    const int j = 1 + (int)(r % d.NY), k = 1 + (int)(r / d.NY);
    double gu = 0.0, gv = 0.0, gw = 0.0;
    if (fluid_at(B, i, j, k)) {
      const double bb = y[x] / dt;
      gu += bb / B.dxa[i - 1];
      gv += bb / B.dya[j - 1];
      gw += bb / B.dza[k - 1];
    }
    if (fluid_at(B, i + 1, j, k)) gu -= (y[x + 1] / dt) / B.dxa[i];
    if (fluid_at(B, i, j + 1, k)) gv -= (y[x + sy] / dt) / B.dya[j];
    if (fluid_at(B, i, j, k + 1)) gw -= (y[x + sz] / dt) / B.dza[k];
    ut_b[x] += gu;
    vt_b[x] += gv;
    wt_b[x] += gw;
  }
}

// u = ut (updateVelocity, all points) transposed: the adjoint of u moves to ut
__global__ void k_copy_adj(int64_t n, double* ub, double* vb, double* wb, double* utb, double* vtb, double* wtb) {
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    utb[x] += ub[x];
    vtb[x] += vb[x];
    wtb[x] += wb[x];
    ub[x] = 0.0;
    vb[x] = 0.0;
    wb[x] = 0.0;
  }
}

// solidCellBC transposed: ut, vt, wt and p are overwritten with 0 at solid cells
__global__ void k_solid_adj(DevBlock B, double* utb, double* vtb, double* wtb, double* pb) {
  const Dims& d = B.d;
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 2 + (int)(t % d.nx);
    const int64_t r = t / d.nx;
    const int j = 2 + (int)(r % d.ny), k = 2 + (int)(r / d.ny);
    const int64_t c = d.idx(i, j, k);
    if (B.cell[c] != 1) continue;
    utb[c] = 0.0;
    vtb[c] = 0.0;
    wtb[c] = 0.0;
    pb[c] = 0.0;
  }
}

// the predictor overwrote ut, vt, wt on the fluid cells
__global__ void k_zero_fluid(DevBlock B, double* utb, double* vtb, double* wtb) {
  const Dims& d = B.d;
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 2 + (int)(t % d.nx);
    const int64_t r = t / d.nx;
    const int j = 2 + (int)(r % d.ny), k = 2 + (int)(r / d.ny);
    const int64_t c = d.idx(i, j, k);
    if (B.cell[c] != 0) continue;
    utb[c] = 0.0;
    vtb[c] = 0.0;
    wtb[c] = 0.0;
  }
}

// y += a * w over n values
__global__ void k_axpy(const double* w, double a, double* y, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    y[t] += a * w[t];
}

// part[cta] += sum over this CTA's fixed share of <w, x> (4 fields): a fixed
// grid and a fixed tree, so the per-CTA sums are reproducible
constexpr int kDotCtas = 256, kDotThreads = 256;
__global__ void __launch_bounds__(kDotThreads) k_dot_acc(const double* w, Fields4 x, int64_t np, double* part) {
  __shared__ double sh[kDotThreads];
  double acc = 0.0;
  for (int q = 0; q < 4; ++q) {
    const double* xs = q == 0 ? x.u : q == 1 ? x.v : q == 2 ? x.w : x.p;
    const double* ws = w + q * np;
    for (int64_t t = blockIdx.x * (int64_t)kDotThreads + threadIdx.x; t < np; t += (int64_t)kDotCtas * kDotThreads)
      acc += ws[t] * xs[t];
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kDotThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] += sh[0];
}

#define ACK(x) \
  do { \
    if ((x) != cudaSuccess) return BCFD_E_CUDA; \
  } while (0)

// the step state: u, v, w, p and the work arrays ut, vt, wt (with a body the
// work arrays differ from u, v, w between steps at the forced faces)
constexpr int kStateFields = 7;

double* const* state_arrays(HostBlock* hb, double* out[kStateFields]) {
  DevBlock& D = hb->d;
  out[0] = D.u;
  out[1] = D.v;
  out[2] = D.w;
  out[3] = D.p;
  out[4] = D.ut;
  out[5] = D.vt;
  out[6] = D.wt;
  return out;
}

int save_state(HostBlock* hb, double* slot) {
  const size_t np = (size_t)hb->d.d.npts(), b = np * sizeof(double);
  double* f[kStateFields];
  state_arrays(hb, f);
  for (int q = 0; q < kStateFields; ++q)
    ACK(cudaMemcpyAsync(slot + q * np, f[q], b, cudaMemcpyDeviceToDevice, stream()));
  return 0;
}

int load_state(HostBlock* hb, const double* slot) {
  const size_t np = (size_t)hb->d.d.npts(), b = np * sizeof(double);
  double* f[kStateFields];
  state_arrays(hb, f);
  for (int q = 0; q < kStateFields; ++q)
    ACK(cudaMemcpyAsync(f[q], slot + q * np, b, cudaMemcpyDeviceToDevice, stream()));
  return 0;
}

// The ghost arrays (velocityForcingGhost / pressureForcingGhost, the last
// calls of a step) are read by the next step's predictor.  At a step's end
// they are a function of the state the step leaves and of the body's TS
// list, so a loaded state regenerates them; at the run's start they are
// whatever an earlier step or the caller left, and are saved.
int save_ghosts(HostBlock* hb, double* slot) {
  const size_t cap = (size_t)hb->d.cap_ib;
  for (int g = 0; g < 14; ++g)
    ACK(cudaMemcpyAsync(slot + g * cap, hb->d.ghost[g], cap * sizeof(double), cudaMemcpyDeviceToDevice, stream()));
  return 0;
}
int load_ghosts(HostBlock* hb, const double* slot) {
  const size_t cap = (size_t)hb->d.cap_ib;
  for (int g = 0; g < 14; ++g)
    ACK(cudaMemcpyAsync(hb->d.ghost[g], slot + g * cap, cap * sizeof(double), cudaMemcpyDeviceToDevice, stream()));
  return 0;
}
int regen_ghosts(HostBlock* hb) {
  TRY_R(launch_forcing_velocity(hb, 2));
  return launch_forcing_pressure(hb, 2);
}

int launch_vbc_adj(HostBlock* hb, double dt, double uc, double* tb[3], const Fields4& s, double* ucl) {
  const Dims& d = hb->d.d;
  k_vbc_z_adj<<<grid_for((int64_t)d.nx * d.ny, 128), 128, 0, stream()>>>(hb->d, tb[0], tb[1], tb[2]);
  BCFD_LAUNCHED();
  k_vbc_y_adj<<<grid_for((int64_t)d.nx * d.nz, 128), 128, 0, stream()>>>(hb->d, tb[0], tb[1], tb[2]);
  BCFD_LAUNCHED();
  k_vbc_x_adj<<<grid_for((int64_t)d.ny * d.nz, 128), 128, 0, stream()>>>(hb->d, dt, uc, tb[0], tb[1], tb[2], s, ucl);
  BCFD_LAUNCHED();
  return 0;
}

// per block: the adjoint arrays and scratch
struct AdjBlock {
  HostBlock* hb = nullptr;
  double* A = nullptr;     // adjoint of the 7 state arrays, in place through a step
  double* pcb = nullptr;   // adjoint of pc
  double* y = nullptr;     // A_ff^{-T} pcb
  double* bb = nullptr;    // accumulated y of the block's solves (adjoint of b, times deltat)
  uint32_t* foot = nullptr;
  ForceCoef fc{};          // forcing coefficients and kinematic accumulators (body blocks)
  MomTsAdj ts{};           // the thin-surface overlay's adjoint (body blocks)
  double* ucl = nullptr;   // dJ/duc per x-face line (coarse block)
  bool body = false;
  int64_t np = 0;
  double* F(int q) const { return A + q * np; }
};

// device allocations freed with the owner
struct DevMem {
  std::vector<void*> ptrs;
  ~DevMem() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  T* get(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return static_cast<T*>(p);
  }
};

// the overlay's adjoint scratch of a body block (zeroed ghost adjoint)
int alloc_ts_adj(AdjBlock& a, DevMem& mem) {
  if (!a.body) return 0;
  const int64_t cap = a.hb->d.cap_ib;
  a.ts.last = mem.get<int>(7 * (size_t)a.np);
  a.ts.contrib = mem.get<double>(14 * (size_t)a.np);
  a.ts.gb = mem.get<double>(14 * (size_t)cap);
  a.ts.cap = cap;
  if (!a.ts.last || !a.ts.contrib || !a.ts.gb) return BCFD_E_NOMEM;
  ACK(cudaMemsetAsync(a.ts.gb, 0, 14 * (size_t)cap * sizeof(double), stream()));
  return 0;
}

// positions a coupling map overwrites, per interface and component: the fine
// block's face-fill targets and the coarse block's restriction targets
struct IfaceMasks {
  HostInterface* it = nullptr;
  AdjBlock* a = nullptr;   // coarse
  AdjBlock* b = nullptr;   // fine
  double* face[4] = {nullptr, nullptr, nullptr, nullptr};
  double* restr[4] = {nullptr, nullptr, nullptr, nullptr};
};

// f = P c (face fill into the fine block) transposed: c_bar += P^T f_bar on
// the written positions, then f_bar = 0 there
int face_fill_adj(IfaceMasks& m, int comp, double* fine_bar, double* coarse_bar) {
  TRY_R(coupling_apply(m.it, comp, 1, fine_bar, coarse_bar));
  k_zero_masked<<<grid_for(m.b->np, 256), 256, 0, stream()>>>(m.b->np, fine_bar, m.face[comp]);
  BCFD_LAUNCHED();
  return 0;
}

// c = R f (restriction into the coarse block) transposed
int restrict_adj(IfaceMasks& m, int comp, double* coarse_bar, double* fine_bar) {
  TRY_R(coupling_apply(m.it, comp, 3, coarse_bar, fine_bar));
  k_zero_masked<<<grid_for(m.a->np, 256), 256, 0, stream()>>>(m.a->np, coarse_bar, m.restr[comp]);
  BCFD_LAUNCHED();
  return 0;
}

// solve transposed: y = A_ff^{-T} pcb, bb += y, pcb -> adjoint of the boundary data
int solve_adj(AdjBlock& a, double tol, int64_t itmax) {
  TRY_R(solve_zero_bc_dev(a.hb, a.pcb, a.y, tol, itmax, true));
  k_axpy<<<grid_for(a.np, 256), 256, 0, stream()>>>(a.y, 1.0, a.bb, a.np);
  BCFD_LAUNCHED();
  k_dirichlet_adj<<<grid_for(a.np, 256), 256, 0, stream()>>>(a.hb->d, a.y, a.pcb);
  BCFD_LAUNCHED();
  return 0;
}

// One whole step transposed, in place on every block's adjoint arrays (each
// block holds the step's input state).  The forward order is that of the
// native step (app/main.F90:129-265 with poissonSolver, PcorVcor.F90:22-220):
//   predictor (all blocks); per block: velocityBC (coarse), solidCellBC and
//   velocityForcing1 (body), velocityBC (coarse);
//   Poisson: fineUpdate_newv_bd (ut faces), coarseUpdate_newv, div, solve
//   fine, coarseUpdate_pc, solve coarse, fineUpdate_pc_bd, solve fine,
//   coarseUpdate_pc, correctPressure, correctVelocity, velocityBC (block 1),
//   ut -> u, fineUpdate_bd_mv (u, v, w, p faces), coarseUpdate (u, v, w, p);
//   pressureForcing1; velocityForcingField, pressureForcingField (body).
// The recorded geometric partials of the forcing calls of the step being
// transposed (moving bodies; nullptr with the geometry fixed).  Call index
// 2 * mode + vel.
struct StepGeo {
  const double* geo[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
};

// the part of a step after the body moved, transposed: pressureForcingGhost,
// velocityForcingGhost (the ghost arrays the next step's predictor read),
// pressureForcingField, velocityForcingField (the geometry and kinematics of
// the step's end)
int adjoint_step_second(std::vector<AdjBlock>& B, const std::vector<StepGeo>* geo) {
  for (size_t q = 0; q < B.size(); ++q) {
    AdjBlock& a = B[q];
    if (!a.body) continue;
    const AdjPtrs pin{{a.F(3), a.F(1), a.F(2), a.F(3)}, {a.F(3), a.F(1), a.F(2), a.F(3)}};
    const AdjPtrs field{{a.F(3), a.F(0), a.F(1), a.F(2)}, {a.F(3), a.F(4), a.F(5), a.F(6)}};
    ForceCoef fc = a.fc;
    if (a.ts.gb) {
      fc.geo = geo ? (*geo)[q].geo[4] : nullptr;
      TRY_R(launch_ghost_adjoint(a.hb, 0, field, fc, a.ts.gb, a.ts.cap));
      fc.geo = geo ? (*geo)[q].geo[5] : nullptr;
      TRY_R(launch_ghost_adjoint(a.hb, 1, field, fc, a.ts.gb, a.ts.cap));
    }
    fc.geo = geo ? (*geo)[q].geo[2] : nullptr;
    TRY_R(launch_forcing_adjoint(a.hb, 1, 0, pin, fc));
    fc.geo = geo ? (*geo)[q].geo[3] : nullptr;
    TRY_R(launch_forcing_adjoint(a.hb, 1, 1, field, fc));
  }
  return 0;
}

// the part of a step before the body moved, transposed (the geometry and
// kinematics the step started with)
int adjoint_step_first(std::vector<AdjBlock>& B, std::vector<IfaceMasks>& M, const bcfd_step_config& c, double tol,
                       int64_t itmax, const std::vector<StepGeo>* geo) {
  std::vector<AdjBlock*> fine, first;
  for (AdjBlock& a : B) (a.hb->is_coarse ? first : fine).push_back(&a);
  auto tb = [](AdjBlock& a) {
    return std::array<double*, 3>{a.F(4), a.F(5), a.F(6)};
  };
  // pressureForcing1
  for (size_t q = 0; q < B.size(); ++q) {
    AdjBlock& a = B[q];
    if (!a.body) continue;
    const AdjPtrs pin{{a.F(3), a.F(1), a.F(2), a.F(3)}, {a.F(3), a.F(1), a.F(2), a.F(3)}};
    ForceCoef fc = a.fc;
    fc.geo = geo ? (*geo)[q].geo[0] : nullptr;
    TRY_R(launch_forcing_adjoint(a.hb, 0, 0, pin, fc));
  }
  // coarseUpdate (u,v,w,p) and fineUpdate_bd_mv (u,v,w,p), reversed
  const int f_of[4] = {3, 0, 1, 2};  // comp 0 p, 1 u, 2 v, 3 w -> state field
  for (auto m = M.rbegin(); m != M.rend(); ++m)
    for (int comp = 3; comp >= 0; --comp) TRY_R(restrict_adj(*m, comp, m->a->F(f_of[comp]), m->b->F(f_of[comp])));
  for (auto m = M.rbegin(); m != M.rend(); ++m)
    for (int comp = 3; comp >= 0; --comp) TRY_R(face_fill_adj(*m, comp, m->b->F(f_of[comp]), m->a->F(f_of[comp])));
  // ut -> u, velocityBC of block 1, the corrections
  for (AdjBlock& a : B) {
    k_copy_adj<<<grid_for(a.np, 256), 256, 0, stream()>>>(a.np, a.F(0), a.F(1), a.F(2), a.F(4), a.F(5), a.F(6));
    BCFD_LAUNCHED();
  }
  for (AdjBlock* a : first) {
    auto t = tb(*a);
    double* tt[3] = {t[0], t[1], t[2]};
    TRY_R(launch_vbc_adj(a->hb, c.deltat, c.uc, tt, Fields4{a->F(0), a->F(1), a->F(2), a->F(3)}, a->ucl));
  }
  for (AdjBlock& a : B) {
    k_correct_adj<<<grid_for(a.np, 256), 256, 0, stream()>>>(a.hb->d, c.deltat, a.F(4), a.F(5), a.F(6), a.F(3), a.pcb);
    BCFD_LAUNCHED();
    ACK(cudaMemsetAsync(a.bb, 0, a.np * sizeof(double), stream()));
  }
  // coarseUpdate_pc, solve fine, fineUpdate_pc_bd, solve coarse, coarseUpdate_pc, solve fine
  for (auto m = M.rbegin(); m != M.rend(); ++m) TRY_R(restrict_adj(*m, 0, m->a->pcb, m->b->pcb));
  for (AdjBlock* a : fine) TRY_R(solve_adj(*a, tol, itmax));
  for (auto m = M.rbegin(); m != M.rend(); ++m) TRY_R(face_fill_adj(*m, 0, m->b->pcb, m->a->pcb));
  for (AdjBlock* a : first) TRY_R(solve_adj(*a, tol, itmax));
  for (auto m = M.rbegin(); m != M.rend(); ++m) TRY_R(restrict_adj(*m, 0, m->a->pcb, m->b->pcb));
  for (AdjBlock* a : fine) TRY_R(solve_adj(*a, tol, itmax));
  // div (with the solves' 1/deltat), coarseUpdate_newv, fineUpdate_newv_bd
  for (AdjBlock& a : B) {
    auto t = tb(a);
    k_div_adj<<<grid_for(a.np, 256), 256, 0, stream()>>>(a.hb->d, c.deltat, a.bb, t[0], t[1], t[2]);
    BCFD_LAUNCHED();
  }
  for (auto m = M.rbegin(); m != M.rend(); ++m)
    for (int comp = 3; comp >= 1; --comp) TRY_R(restrict_adj(*m, comp, m->a->F(3 + comp), m->b->F(3 + comp)));
  for (auto m = M.rbegin(); m != M.rend(); ++m)
    for (int comp = 3; comp >= 1; --comp) TRY_R(face_fill_adj(*m, comp, m->b->F(3 + comp), m->a->F(3 + comp)));
  // per block: velocityBC, [velocityForcing1, solidCellBC], velocityBC, reversed
  for (size_t q = 0; q < B.size(); ++q) {
    AdjBlock& a = B[q];
    auto t = tb(a);
    double* tt[3] = {t[0], t[1], t[2]};
    const Fields4 s{a.F(0), a.F(1), a.F(2), a.F(3)};
    if (a.hb->is_coarse) TRY_R(launch_vbc_adj(a.hb, c.deltat, c.uc, tt, s, a.ucl));
    if (a.body) {
      const AdjPtrs vin{{a.F(3), a.F(4), a.F(5), a.F(6)}, {a.F(3), a.F(4), a.F(5), a.F(6)}};
      ForceCoef fc = a.fc;
      fc.geo = geo ? (*geo)[q].geo[1] : nullptr;
      TRY_R(launch_forcing_adjoint(a.hb, 0, 1, vin, fc));
      const int64_t ni = (int64_t)a.hb->d.d.nx * a.hb->d.d.ny * a.hb->d.d.nz;
      k_solid_adj<<<grid_for(ni, 256), 256, 0, stream()>>>(a.hb->d, a.F(4), a.F(5), a.F(6), a.F(3));
      BCFD_LAUNCHED();
    }
    if (a.hb->is_coarse) TRY_R(launch_vbc_adj(a.hb, c.deltat, c.uc, tt, s, a.ucl));
  }
  // the predictor
  for (AdjBlock& a : B) {
    auto t = tb(a);
    const double* sb[3] = {t[0], t[1], t[2]};
    double* ab[4] = {a.F(0), a.F(1), a.F(2), a.F(3)};
    TRY_R(launch_momentum_adjoint(a.hb, c.deltat, c.re, sb, ab, a.foot, a.ts.gb ? &a.ts : nullptr));
    const int64_t ni = (int64_t)a.hb->d.d.nx * a.hb->d.d.ny * a.hb->d.d.nz;
    k_zero_fluid<<<grid_for(ni, 256), 256, 0, stream()>>>(a.hb->d, t[0], t[1], t[2]);
    BCFD_LAUNCHED();
  }
  return 0;
}

int adjoint_step(std::vector<AdjBlock>& B, std::vector<IfaceMasks>& M, const bcfd_step_config& c, double tol,
                 int64_t itmax) {
  TRY_R(adjoint_step_second(B, nullptr));
  return adjoint_step_first(B, M, c, tol, itmax, nullptr);
}

// the registered blocks in registration order
std::vector<std::pair<bcfd_handle, HostBlock*>> registered_blocks() {
  std::vector<std::pair<bcfd_handle, HostBlock*>> v;
  for (size_t q = 0; q < lib().blocks.size(); ++q)
    if (lib().blocks[q]) v.push_back({(bcfd_handle)(q + 1), lib().blocks[q]});
  return v;
}

// ---- moving bodies -----------------------------------------------------------
constexpr int kCalls = 6;  // forcing calls of a step, index 2 * mode + vel

// what a recomputed step leaves for the transposes, for the moving body: the
// tags and nodes after the step (its end geometry), the host motion state,
// and the geometric partials of its forcing calls
struct BodyRec {
  int8_t* cell = nullptr;
  int8_t* cell2 = nullptr;
  int8_t* ntag = nullptr;
  double* nodes = nullptr;
  Kin kin{};
  MotionStage stage{};
  BodyMotion motion{};
  double node_rmax = 0.0;
  double* geo[kCalls] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  int64_t nt[kCalls] = {0, 0, 0, 0, 0, 0};
};

int save_body(HostBlock* hb, BodyRec& r, DevMem& mem) {
  const DevBlock& D = hb->d;
  const size_t np = (size_t)D.d.npts(), np3 = (size_t)D.d.npts3(), nn = (size_t)D.nn;
  if (!r.cell) {
    r.cell = mem.get<int8_t>(np);
    r.cell2 = mem.get<int8_t>(np3);
    r.ntag = mem.get<int8_t>(np3);
    r.nodes = mem.get<double>(3 * nn);
    if (!r.cell || !r.cell2 || !r.ntag || !r.nodes) return BCFD_E_NOMEM;
  }
  ACK(cudaMemcpyAsync(r.cell, D.cell, np, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(r.cell2, D.cell2, np3, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(r.ntag, D.nodeTag, np3, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(r.nodes, D.xnode1, nn * sizeof(double), cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(r.nodes + nn, D.ynode1, nn * sizeof(double), cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(r.nodes + 2 * nn, D.znode1, nn * sizeof(double), cudaMemcpyDeviceToDevice, stream()));
  r.kin = hb->kin;
  r.stage = hb->stage;
  r.motion = hb->motion;
  r.node_rmax = hb->node_rmax;
  return 0;
}

// the body's state after a recorded step: tags, nodes, kinematics and motion,
// then what follows from them (normals, lists and masks, normal distances,
// thin-surface list)
int restore_body(HostBlock* hb, const BodyRec& r) {
  DevBlock& D = hb->d;
  const size_t np = (size_t)D.d.npts(), np3 = (size_t)D.d.npts3(), nn = (size_t)D.nn;
  ACK(cudaMemcpyAsync(D.cell, r.cell, np, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(D.cell2, r.cell2, np3, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(D.nodeTag, r.ntag, np3, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(const_cast<double*>(D.xnode1), r.nodes, nn * sizeof(double), cudaMemcpyDeviceToDevice,
                      stream()));
  ACK(cudaMemcpyAsync(const_cast<double*>(D.ynode1), r.nodes + nn, nn * sizeof(double), cudaMemcpyDeviceToDevice,
                      stream()));
  ACK(cudaMemcpyAsync(const_cast<double*>(D.znode1), r.nodes + 2 * nn, nn * sizeof(double),
                      cudaMemcpyDeviceToDevice, stream()));
  hb->kin = r.kin;
  hb->stage = r.stage;
  hb->staged = false;
  hb->motion = r.motion;
  hb->node_rmax = r.node_rmax;
  TRY_R(upload_kin(hb));
  TRY_R(launch_surface_norm(hb, hb->inor));
  TRY_R(launch_cellcount(hb, false));
  TRY_R(launch_norm_distance(hb));
  return launch_find_ts(hb);
}

// the recorder of a segment's recomputation: per step, the geometric
// partials of every moving body's forcing calls
struct MoveRecorder : ForceRecorder {
  std::vector<HostBlock*> bodies;
  std::vector<BodyRec*> cur;  // per body: the record of the step being recomputed
  std::vector<double*> sc;    // per body: 3 point arrays of scratch
  DevMem* mem = nullptr;
  bool oom = false;
  int find(HostBlock* hb) const {
    for (size_t i = 0; i < bodies.size(); ++i)
      if (bodies[i] == hb) return (int)i;
    return -1;
  }
  double* slot(HostBlock* hb, int mode, int vel, int64_t nt) override {
    const int i = find(hb);
    if (i < 0 || !cur[(size_t)i] || nt <= 0) return nullptr;
    BodyRec* r = cur[(size_t)i];
    const int c = 2 * mode + vel;
    r->nt[c] = nt;
    r->geo[c] = mem->get<double>(6 * (size_t)nt);
    if (!r->geo[c]) oom = true;
    return r->geo[c];
  }
  double* scratch(HostBlock* hb) override {
    const int i = find(hb);
    return i < 0 ? nullptr : sc[(size_t)i];
  }
};

}  // namespace
}  // namespace bcfd

using namespace bcfd;

extern "C" {

int bcfd_adjoint_run(bcfd_handle h, const bcfd_step_config* cfg, int64_t n_steps, int64_t every, const double* wu,
                     const double* wv, const double* ww, const double* wp, const double* stress_seed, double mu_f,
                     double rho_f, double adj_tol, int64_t adj_itmax, double* J, double* dj_duc,
                     double* dj_dkin, double* gu, double* gv, double* gw, double* gp) {
  LibLock lk;
  HostBlock* hb = get_block(h);
  if (!hb) return BCFD_E_HANDLE;
  if (!cfg || n_steps < 1 || every < 1 || !wu || !wv || !ww || !wp || !J || !(adj_tol > 0.0) || adj_itmax < 1)
    return BCFD_E_ARG;
  if (cfg->precision != 0) return BCFD_E_STATE;
  // the blocks: block 1 with the domain BCs, the others fine blocks coupled
  // to it by interfaces; no moving bodies, no thin-surface cells
  auto all = registered_blocks();
  if (all.empty() || !all.front().second->is_coarse) return BCFD_E_STATE;
  for (auto& [g, b] : all) {
    if (b->motion.on || !b->d.ca[0] || !b->d.Acx) return BCFD_E_STATE;
    if (g != all.front().first && b->is_coarse) return BCFD_E_STATE;
  }
  std::vector<HostInterface*> ifs;
  for (HostInterface* it : lib().ifs)
    if (it) ifs.push_back(it);
  if (all.size() > 1 && ifs.empty()) return BCFD_E_STATE;
  const bool body = hb->has_body && hb->d.ne > 0;
  if (stress_seed && !body) return BCFD_E_STATE;
  const bool use_stress = stress_seed != nullptr;
  const bool grad = dj_duc || dj_dkin || gu || gv || gw || gp;
  const int nb = (int)all.size();
  int hidx = -1;
  for (int q = 0; q < nb; ++q)
    if (all[q].second == hb) hidx = q;
  std::vector<int64_t> npb(nb), off(nb + 1, 0);
  for (int q = 0; q < nb; ++q) {
    npb[q] = all[q].second->d.d.npts();
    off[q + 1] = off[q] + kStateFields * npb[q];
  }
  const size_t S = (size_t)off[nb];  // doubles of one state of all blocks
  const int64_t np = hb->d.d.npts();
  const size_t fb = (size_t)np * sizeof(double);
  const int64_t K = std::min(every, n_steps);
  const int64_t ncp = (n_steps + K - 1) / K;
  DevMem mem;
  double* W = mem.get<double>(4 * np);
  double* cps = mem.get<double>((size_t)ncp * S);
  double* fin = mem.get<double>(S);
  double* part = mem.get<double>(kDotCtas);
  if (!W || !cps || !fin || !part) return BCFD_E_NOMEM;
  const double* wh[4] = {wu, wv, ww, wp};
  for (int q = 0; q < 4; ++q) ACK(h2d(W + q * np, wh[q], fb));
  ACK(cudaMemsetAsync(part, 0, kDotCtas * sizeof(double), stream()));
  auto save_all = [&](double* slot) -> int {
    for (int q = 0; q < nb; ++q) TRY_R(save_state(all[q].second, slot + off[q]));
    return 0;
  };
  auto load_all = [&](const double* slot) -> int {
    for (int q = 0; q < nb; ++q) TRY_R(load_state(all[q].second, slot + off[q]));
    return 0;
  };
  Lib& L = lib();
  const int64_t ita0 = L.ita;
  const double tot0 = L.totime;
  bcfd_step_config c = *cfg;
  c.use_graph = 0;
  const Fields4 bx{hb->d.u, hb->d.v, hb->d.w, hb->d.p};

  // forward: the work arrays start equal to u, v, w; checkpoints; objective
  for (auto& [g, b] : all) {
    const size_t bytes = (size_t)b->d.d.npts() * sizeof(double);
    ACK(cudaMemcpyAsync(b->d.ut, b->d.u, bytes, cudaMemcpyDeviceToDevice, stream()));
    ACK(cudaMemcpyAsync(b->d.vt, b->d.v, bytes, cudaMemcpyDeviceToDevice, stream()));
    ACK(cudaMemcpyAsync(b->d.wt, b->d.w, bytes, cudaMemcpyDeviceToDevice, stream()));
  }
  TRY_R(save_all(cps));
  std::vector<double*> g0(nb, nullptr);
  for (int q = 0; q < nb; ++q) {
    HostBlock* b = all[q].second;
    if (!b->has_body || b->d.ne <= 0) continue;
    g0[q] = mem.get<double>(14 * (size_t)b->d.cap_ib);
    if (!g0[q]) return BCFD_E_NOMEM;
    TRY_R(save_ghosts(b, g0[q]));
  }
  // the ghost arrays of the state after step n (n = 0: the run's start)
  auto ghosts_at = [&](int64_t n) -> int {
    for (int q = 0; q < nb; ++q)
      if (g0[q]) TRY_R(n == 0 ? load_ghosts(all[q].second, g0[q]) : regen_ghosts(all[q].second));
    return 0;
  };
  // the transpose assumes the tags the run starts with hold throughout
  // (stationary bodies: the per-step re-Search reproduces them)
  std::vector<std::vector<int8_t>> tags0(nb);
  for (int q = 0; q < nb; ++q) {
    tags0[q].resize((size_t)npb[q]);
    ACK(d2h(tags0[q].data(), all[q].second->d.cell, (size_t)npb[q]));
  }
  double jstress = 0.0;
  for (int64_t n = 1; n <= n_steps; ++n) {
    TRY_R(run_one_step(c));
    k_dot_acc<<<kDotCtas, kDotThreads, 0, stream()>>>(W, bx, np, part);
    BCFD_LAUNCHED();
    if (use_stress) {
      double co[4];
      // the fixed scratch when the body fits in it (no allocation per
      // step), else the allocating launch: same kernels, same result
      if (hb->d.ne <= BCFD_STRESS_NOALLOC_MAX_ELEMS)
        TRY_R(launch_stress_noalloc(hb, mu_f, rho_f, co));
      else
        TRY_R(launch_stress(hb, mu_f, rho_f, co));
      for (int t = 0; t < 4; ++t) jstress += stress_seed[t] * co[t];
    }
    if (n % K == 0 && n < n_steps) TRY_R(save_all(cps + (size_t)(n / K) * S));
  }
  TRY_R(save_all(fin));
  std::vector<double> ph(kDotCtas);
  ACK(d2h(ph.data(), part, kDotCtas * sizeof(double)));
  double jsum = 0.0;
  for (double v : ph) jsum += v;
  *J = (jsum + jstress) / (double)n_steps;
  int err = 0;
  for (int q = 0; q < nb && !err; ++q) {
    err = take_block_error(all[q].second);
    std::vector<int8_t> t1((size_t)npb[q]);
    ACK(d2h(t1.data(), all[q].second->d.cell, (size_t)npb[q]));
    if (!err && t1 != tags0[q]) err = BCFD_E_STATE;
  }
  if (err || !grad) {
    L.ita = ita0 + n_steps;
    L.totime = tot0 + n_steps * cfg->deltat;
    return err;
  }

  // per-block adjoint buffers
  std::vector<AdjBlock> AB(nb);
  for (int q = 0; q < nb; ++q) {
    AdjBlock& a = AB[q];
    a.hb = all[q].second;
    a.np = npb[q];
    a.body = a.hb->has_body && a.hb->d.ne > 0;
    a.A = mem.get<double>(kStateFields * a.np);
    a.pcb = mem.get<double>(a.np);
    a.y = mem.get<double>(a.np);
    a.bb = mem.get<double>(a.np);
    a.foot = mem.get<uint32_t>(16);
    a.ucl = mem.get<double>((size_t)a.hb->d.d.ny * a.hb->d.d.nz);
    const size_t ntask = a.body ? 6 * (size_t)a.hb->d.cap_ib : 1;
    a.fc.tgt = mem.get<int64_t>(ntask);
    a.fc.axis = mem.get<int>(ntask);
    a.fc.pos = mem.get<int64_t>(8 * ntask);
    a.fc.coef = mem.get<double>(8 * ntask);
    a.fc.kc = mem.get<double>(kKinScalars * ntask);
    a.fc.gk = mem.get<double>(kKinScalars);
    if (!a.A || !a.pcb || !a.y || !a.bb || !a.foot || !a.ucl || !a.fc.tgt || !a.fc.axis || !a.fc.pos ||
        !a.fc.coef || !a.fc.kc || !a.fc.gk)
      return BCFD_E_NOMEM;
    TRY_R(alloc_ts_adj(a, mem));
    ACK(cudaMemsetAsync(a.A, 0, kStateFields * a.np * sizeof(double), stream()));
    ACK(cudaMemsetAsync(a.ucl, 0, (size_t)a.hb->d.d.ny * a.hb->d.d.nz * sizeof(double), stream()));
    ACK(cudaMemsetAsync(a.fc.gk, 0, kKinScalars * sizeof(double), stream()));
  }
  // coupling masks: the positions each map writes (the maps are partitions of
  // unity, so a field of ones maps to ones exactly there)
  std::vector<IfaceMasks> M;
  for (HostInterface* it : ifs) {
    IfaceMasks m;
    m.it = it;
    for (int q = 0; q < nb; ++q) {
      if (all[q].first == it->a) m.a = &AB[q];
      if (all[q].first == it->b) m.b = &AB[q];
    }
    if (!m.a || !m.b) return BCFD_E_STATE;
    double* ones_a = mem.get<double>(m.a->np);
    double* ones_b = mem.get<double>(m.b->np);
    if (!ones_a || !ones_b) return BCFD_E_NOMEM;
    k_fill<<<grid_for(m.a->np, 256), 256, 0, stream()>>>(m.a->np, ones_a, 1.0);
    BCFD_LAUNCHED();
    k_fill<<<grid_for(m.b->np, 256), 256, 0, stream()>>>(m.b->np, ones_b, 1.0);
    BCFD_LAUNCHED();
    for (int comp = 0; comp < 4; ++comp) {
      m.face[comp] = mem.get<double>(m.b->np);
      m.restr[comp] = mem.get<double>(m.a->np);
      if (!m.face[comp] || !m.restr[comp]) return BCFD_E_NOMEM;
      ACK(cudaMemsetAsync(m.face[comp], 0, m.b->np * sizeof(double), stream()));
      ACK(cudaMemsetAsync(m.restr[comp], 0, m.a->np * sizeof(double), stream()));
      TRY_R(coupling_apply(it, comp, 0, ones_a, m.face[comp]));
      TRY_R(coupling_apply(it, comp, 2, ones_b, m.restr[comp]));
    }
    M.push_back(m);
  }
  // objective weights per step on block h: W plus the coefficients' weights
  AdjBlock& ah = AB[hidx];
  if (use_stress) {
    double* sd = mem.get<double>(4);
    double* ss = mem.get<double>(8 + std::max<size_t>(64, kKinScalars) * (size_t)hb->d.ne);
    if (!sd || !ss) return BCFD_E_NOMEM;
    ACK(h2d(sd, stress_seed, 4 * sizeof(double)));
    TRY_R(launch_stress_weights(hb, mu_f, rho_f, sd, W, ss));
    // the coefficients' own dependence on the kinematic scalars (the same at
    // every step: (1/N) * N times)
    TRY_R(launch_stress_kin(hb, mu_f, rho_f, sd, ah.fc.gk, ss));
  }
  double* tape = mem.get<double>((size_t)K * S);
  if (!tape) return BCFD_E_NOMEM;
  const double wn = 1.0 / (double)n_steps;
  k_axpy<<<grid_for(4 * np, 256), 256, 0, stream()>>>(W, wn, ah.A, 4 * np);
  BCFD_LAUNCHED();
  for (int64_t m = ncp - 1; m >= 0; --m) {
    const int64_t n0 = m * K, n1 = std::min(n0 + K, n_steps);
    const double* cp = cps + (size_t)m * S;
    ACK(cudaMemcpyAsync(tape, cp, S * sizeof(double), cudaMemcpyDeviceToDevice, stream()));
    TRY_R(load_all(cp));
    TRY_R(ghosts_at(n0));
    L.ita = ita0 + n0;
    L.totime = tot0 + n0 * cfg->deltat;
    for (int64_t n = n0 + 1; n < n1; ++n) {
      TRY_R(run_one_step(c));
      TRY_R(save_all(tape + (size_t)(n - n0) * S));
    }
    for (int64_t n = n1; n > n0; --n) {
      TRY_R(load_all(tape + (size_t)(n - 1 - n0) * S));
      TRY_R(ghosts_at(n - 1));
      TRY_R(adjoint_step(AB, M, c, adj_tol, adj_itmax));
      if (n - 1 >= 1) {
        k_axpy<<<grid_for(4 * np, 256), 256, 0, stream()>>>(W, wn, ah.A, 4 * np);
        BCFD_LAUNCHED();
      }
    }
  }
  // leave the blocks at the forward run's final state
  TRY_R(load_all(fin));
  TRY_R(ghosts_at(n_steps));
  L.ita = ita0 + n_steps;
  L.totime = tot0 + n_steps * cfg->deltat;
  // the run started from ut = u, vt = v, wt = w: their adjoints add up
  k_axpy<<<grid_for(3 * np, 256), 256, 0, stream()>>>(ah.A + 4 * np, 1.0, ah.A, 3 * np);
  BCFD_LAUNCHED();
  double* gh[4] = {gu, gv, gw, gp};
  for (int q = 0; q < 4; ++q)
    if (gh[q]) ACK(cudaMemcpyAsync(gh[q], ah.A + q * np, fb, cudaMemcpyDeviceToHost, stream()));
  if (dj_dkin) ACK(d2h(dj_dkin, ah.fc.gk, 8 * sizeof(double)));
  double duc = 0.0;
  for (AdjBlock& a : AB) {
    if (!a.hb->is_coarse) continue;
    std::vector<double> ul((size_t)a.hb->d.d.ny * a.hb->d.d.nz);
    ACK(d2h(ul.data(), a.ucl, ul.size() * sizeof(double)));
    for (double v : ul) duc += v;
  }
  if (dj_duc) *dj_duc = duc;
  ACK(cudaStreamSynchronize(stream()));
  for (auto& [g, b] : all) {
    const int e = take_block_error(b);
    if (e) return e;
  }
  return 0;
}

// The moving-body run: the objective's moving body on block h, and any other
// moving bodies.  Forward as above, with every moving body's tags, nodes and
// motion state checkpointed beside the fields.  In
// reverse each segment is recomputed with the forcing recorder on (per step:
// the forcing calls' geometric partials, the tags, nodes and motion state the
// step leaves), then every step is transposed in two halves: the part after
// the body moved with the step's end geometry and kinematics restored, then
// the part before with the start's; after the first half the element-geometry
// and kinematic adjoints of the end geometry are complete and go through the
// nodes and the placement to the motion parameters.
int bcfd_adjoint_run_motion(bcfd_handle h, const bcfd_step_config* cfg, int64_t n_steps, int64_t every,
                            const double* wu, const double* wv, const double* ww, const double* wp,
                            const double* stress_seed, double mu_f, double rho_f, double adj_tol, int64_t adj_itmax,
                            double* J, double* dj_duc, double* dj_dmotion, double* gu, double* gv, double* gw,
                            double* gp) {
  LibLock lk;
  HostBlock* hb = get_block(h);
  if (!hb) return BCFD_E_HANDLE;
  if (!cfg || n_steps < 1 || every < 1 || !wu || !wv || !ww || !wp || !J || !(adj_tol > 0.0) || adj_itmax < 1)
    return BCFD_E_ARG;
  if (cfg->precision != 0) return BCFD_E_STATE;
  auto all = registered_blocks();
  if (all.empty() || !all.front().second->is_coarse) return BCFD_E_STATE;
  for (auto& [g, b] : all) {
    if (!b->d.ca[0] || !b->d.Acx) return BCFD_E_STATE;
    if (g != all.front().first && b->is_coarse) return BCFD_E_STATE;
  }
  if (!hb->motion.on) return BCFD_E_STATE;
  // the moving bodies (the objective's and any others, e.g. a plate in tandem)
  std::vector<int> movers;
  for (int q = 0; q < (int)all.size(); ++q) {
    HostBlock* b = all[q].second;
    if (!b->motion.on) continue;
    if (!b->motion.placed || !b->has_body || b->d.ne <= 0 || b->d.nn <= 0) return BCFD_E_STATE;
    movers.push_back(q);
  }
  const int nmov = (int)movers.size();
  std::vector<HostInterface*> ifs;
  for (HostInterface* it : lib().ifs)
    if (it) ifs.push_back(it);
  if (all.size() > 1 && ifs.empty()) return BCFD_E_STATE;
  const bool use_stress = stress_seed != nullptr;
  const int nb = (int)all.size();
  int hidx = -1;
  for (int q = 0; q < nb; ++q)
    if (all[q].second == hb) hidx = q;
  std::vector<int64_t> npb(nb), off(nb + 1, 0);
  for (int q = 0; q < nb; ++q) {
    npb[q] = all[q].second->d.d.npts();
    off[q + 1] = off[q] + kStateFields * npb[q];
  }
  const size_t S = (size_t)off[nb];
  const int64_t np = hb->d.d.npts();
  const size_t fb = (size_t)np * sizeof(double);
  const int64_t K = std::min(every, n_steps);
  const int64_t ncp = (n_steps + K - 1) / K;
  const int ne = hb->d.ne;
  DevMem mem;
  double* W = mem.get<double>(4 * np);
  double* cps = mem.get<double>((size_t)ncp * S);
  double* fin = mem.get<double>(S);
  double* part = mem.get<double>(kDotCtas);
  if (!W || !cps || !fin || !part) return BCFD_E_NOMEM;
  // per moving body: its state at the checkpoints and at the end
  std::vector<std::vector<BodyRec>> cprec((size_t)nmov, std::vector<BodyRec>((size_t)ncp));
  std::vector<BodyRec> finrec((size_t)nmov);
  auto mover = [&](int mi) { return all[(size_t)movers[(size_t)mi]].second; };
  auto save_bodies = [&](std::vector<BodyRec>* recs, size_t at, DevMem& m) -> int {
    for (int mi = 0; mi < nmov; ++mi) TRY_R(save_body(mover(mi), recs[mi][at], m));
    return 0;
  };
  const double* wh[4] = {wu, wv, ww, wp};
  for (int q = 0; q < 4; ++q) ACK(h2d(W + q * np, wh[q], fb));
  ACK(cudaMemsetAsync(part, 0, kDotCtas * sizeof(double), stream()));
  auto save_all = [&](double* slot) -> int {
    for (int q = 0; q < nb; ++q) TRY_R(save_state(all[q].second, slot + off[q]));
    return 0;
  };
  auto load_all = [&](const double* slot) -> int {
    for (int q = 0; q < nb; ++q) TRY_R(load_state(all[q].second, slot + off[q]));
    return 0;
  };
  Lib& L = lib();
  const int64_t ita0 = L.ita;
  const double tot0 = L.totime;
  bcfd_step_config c = *cfg;
  c.use_graph = 0;
  const Fields4 bx{hb->d.u, hb->d.v, hb->d.w, hb->d.p};
  auto fail = [&](int e) {
    L.ita = ita0 + n_steps;
    L.totime = tot0 + n_steps * cfg->deltat;
    return e;
  };

  // forward, checkpointing fields and the body's state
  for (auto& [g, b] : all) {
    const size_t bytes = (size_t)b->d.d.npts() * sizeof(double);
    ACK(cudaMemcpyAsync(b->d.ut, b->d.u, bytes, cudaMemcpyDeviceToDevice, stream()));
    ACK(cudaMemcpyAsync(b->d.vt, b->d.v, bytes, cudaMemcpyDeviceToDevice, stream()));
    ACK(cudaMemcpyAsync(b->d.wt, b->d.w, bytes, cudaMemcpyDeviceToDevice, stream()));
  }
  TRY_R(save_all(cps));
  TRY_R(save_bodies(cprec.data(), 0, mem));
  std::vector<double*> g0(nb, nullptr);
  for (int q = 0; q < nb; ++q) {
    HostBlock* b = all[q].second;
    if (!b->has_body || b->d.ne <= 0) continue;
    g0[q] = mem.get<double>(14 * (size_t)b->d.cap_ib);
    if (!g0[q]) return BCFD_E_NOMEM;
    TRY_R(save_ghosts(b, g0[q]));
  }
  // the ghost arrays of the state after step n (n = 0: the run's start), with
  // the body's state of that step restored
  auto ghosts_at = [&](int64_t n) -> int {
    for (int q = 0; q < nb; ++q)
      if (g0[q]) TRY_R(n == 0 ? load_ghosts(all[q].second, g0[q]) : regen_ghosts(all[q].second));
    return 0;
  };
  double jstress = 0.0;
  for (int64_t n = 1; n <= n_steps; ++n) {
    TRY_R(run_one_step(c));
    // a fine-block move changes the blocks' structure: not differentiated
    for (int mi = 0; mi < nmov; ++mi) {
      const HostBlock* b = mover(mi);
      if (b->move_amt[0] || b->move_amt[1] || b->move_amt[2]) return fail(BCFD_E_STATE);
    }
    k_dot_acc<<<kDotCtas, kDotThreads, 0, stream()>>>(W, bx, np, part);
    BCFD_LAUNCHED();
    if (use_stress) {
      double co[4];
      if (ne <= BCFD_STRESS_NOALLOC_MAX_ELEMS)
        TRY_R(launch_stress_noalloc(hb, mu_f, rho_f, co));
      else
        TRY_R(launch_stress(hb, mu_f, rho_f, co));
      for (int t = 0; t < 4; ++t) jstress += stress_seed[t] * co[t];
    }
    if (n % K == 0 && n < n_steps) {
      TRY_R(save_all(cps + (size_t)(n / K) * S));
      TRY_R(save_bodies(cprec.data(), (size_t)(n / K), mem));
    }
  }
  TRY_R(save_all(fin));
  for (int mi = 0; mi < nmov; ++mi) TRY_R(save_body(mover(mi), finrec[(size_t)mi], mem));
  std::vector<double> ph(kDotCtas);
  ACK(d2h(ph.data(), part, kDotCtas * sizeof(double)));
  double jsum = 0.0;
  for (double v : ph) jsum += v;
  *J = (jsum + jstress) / (double)n_steps;
  for (int q = 0; q < nb; ++q) {
    const int e = take_block_error(all[q].second);
    if (e) return fail(e);
  }
  const bool grad = dj_duc || dj_dmotion || gu || gv || gw || gp;
  if (!grad) return fail(0);

  // each moving body's parameter tangents for every driver step of the run
  std::vector<std::vector<StepTangent>> tan((size_t)nmov);
  std::vector<int64_t> first((size_t)nmov);
  for (int mi = 0; mi < nmov; ++mi) {
    HostBlock* b = mover(mi);
    TRY_R(motion_tangent(b, L.phase_angle, L.freq, cfg->deltat, tot0, ita0, ita0 + n_steps, tan[(size_t)mi]));
    first[(size_t)mi] = b->motion.init_ita;
    if (ita0 < first[(size_t)mi]) return fail(BCFD_E_STATE);
  }
  // per-block adjoint buffers
  std::vector<AdjBlock> AB(nb);
  for (int q = 0; q < nb; ++q) {
    AdjBlock& a = AB[q];
    a.hb = all[q].second;
    a.np = npb[q];
    a.body = a.hb->has_body && a.hb->d.ne > 0;
    a.A = mem.get<double>(kStateFields * a.np);
    a.pcb = mem.get<double>(a.np);
    a.y = mem.get<double>(a.np);
    a.bb = mem.get<double>(a.np);
    a.foot = mem.get<uint32_t>(16);
    a.ucl = mem.get<double>((size_t)a.hb->d.d.ny * a.hb->d.d.nz);
    const size_t ntask = a.body ? 6 * (size_t)a.hb->cap_ib_alloc : 1;
    a.fc.tgt = mem.get<int64_t>(ntask);
    a.fc.axis = mem.get<int>(ntask);
    a.fc.pos = mem.get<int64_t>(8 * ntask);
    a.fc.coef = mem.get<double>(8 * ntask);
    a.fc.kc = mem.get<double>(kKinScalars * ntask);
    a.fc.gk = mem.get<double>(kKinScalars);
    if (!a.A || !a.pcb || !a.y || !a.bb || !a.foot || !a.ucl || !a.fc.tgt || !a.fc.axis || !a.fc.pos ||
        !a.fc.coef || !a.fc.kc || !a.fc.gk)
      return fail(BCFD_E_NOMEM);
    TRY_R(alloc_ts_adj(a, mem));
    if (a.hb->motion.on) {
      const size_t ne_q = (size_t)a.hb->d.ne;
      a.fc.elem = mem.get<int>(ntask);
      a.fc.ge = mem.get<double>(7 * ne_q);
      if (!a.fc.elem || !a.fc.ge) return fail(BCFD_E_NOMEM);
      ACK(cudaMemsetAsync(a.fc.ge, 0, 7 * ne_q * sizeof(double), stream()));
    }
    ACK(cudaMemsetAsync(a.A, 0, kStateFields * a.np * sizeof(double), stream()));
    ACK(cudaMemsetAsync(a.ucl, 0, (size_t)a.hb->d.d.ny * a.hb->d.d.nz * sizeof(double), stream()));
    ACK(cudaMemsetAsync(a.fc.gk, 0, kKinScalars * sizeof(double), stream()));
  }
  std::vector<IfaceMasks> M;
  for (HostInterface* it : ifs) {
    IfaceMasks m;
    m.it = it;
    for (int q = 0; q < nb; ++q) {
      if (all[q].first == it->a) m.a = &AB[q];
      if (all[q].first == it->b) m.b = &AB[q];
    }
    if (!m.a || !m.b) return fail(BCFD_E_STATE);
    double* ones_a = mem.get<double>(m.a->np);
    double* ones_b = mem.get<double>(m.b->np);
    if (!ones_a || !ones_b) return fail(BCFD_E_NOMEM);
    k_fill<<<grid_for(m.a->np, 256), 256, 0, stream()>>>(m.a->np, ones_a, 1.0);
    BCFD_LAUNCHED();
    k_fill<<<grid_for(m.b->np, 256), 256, 0, stream()>>>(m.b->np, ones_b, 1.0);
    BCFD_LAUNCHED();
    for (int comp = 0; comp < 4; ++comp) {
      m.face[comp] = mem.get<double>(m.b->np);
      m.restr[comp] = mem.get<double>(m.a->np);
      if (!m.face[comp] || !m.restr[comp]) return fail(BCFD_E_NOMEM);
      ACK(cudaMemsetAsync(m.face[comp], 0, m.b->np * sizeof(double), stream()));
      ACK(cudaMemsetAsync(m.restr[comp], 0, m.a->np * sizeof(double), stream()));
      TRY_R(coupling_apply(it, comp, 0, ones_a, m.face[comp]));
      TRY_R(coupling_apply(it, comp, 2, ones_b, m.restr[comp]));
    }
    M.push_back(m);
  }
  AdjBlock& ah = AB[hidx];
  // the objective at the state the blocks hold (geometry and kinematics of
  // the same step): field weights, drag/lift weights, their geometric and
  // kinematic partials, each with the time average's 1/N
  const double wn = 1.0 / (double)n_steps;
  int ne_max = 0, nn_max = 0;
  for (int mi = 0; mi < nmov; ++mi) {
    ne_max = std::max(ne_max, mover(mi)->d.ne);
    nn_max = std::max(nn_max, mover(mi)->d.nn);
  }
  double* sd = mem.get<double>(4);
  double* sdw = mem.get<double>(4);
  double* ss = mem.get<double>(8 + (size_t)std::max(64, kKinScalars) * ne);
  double* gscr = mem.get<double>(9 * (size_t)ne_max + 4 * (size_t)nn_max + 4);
  if (!sd || !sdw || !ss || !gscr) return fail(BCFD_E_NOMEM);
  // per moving body: the recorder's scratch and the node -> element CSR
  std::vector<double*> pre((size_t)nmov);
  std::vector<int*> csr_off((size_t)nmov), csr_ent((size_t)nmov);
  for (int mi = 0; mi < nmov; ++mi) {
    HostBlock* b = mover(mi);
    pre[(size_t)mi] = mem.get<double>(3 * (size_t)b->d.d.npts());
    std::vector<int> hoff, hent;
    TRY_R(build_node_csr(b, hoff, hent));
    csr_off[(size_t)mi] = mem.get<int>(hoff.size());
    csr_ent[(size_t)mi] = mem.get<int>(std::max<size_t>(hent.size(), 1));
    if (!pre[(size_t)mi] || !csr_off[(size_t)mi] || !csr_ent[(size_t)mi]) return fail(BCFD_E_NOMEM);
    ACK(h2d(csr_off[(size_t)mi], hoff.data(), hoff.size() * sizeof(int)));
    if (!hent.empty()) ACK(h2d(csr_ent[(size_t)mi], hent.data(), hent.size() * sizeof(int)));
  }
  if (use_stress) {
    double sw[4];
    for (int t = 0; t < 4; ++t) sw[t] = stress_seed[t] * wn;
    ACK(h2d(sd, stress_seed, 4 * sizeof(double)));
    ACK(h2d(sdw, sw, 4 * sizeof(double)));
  }
  auto objective = [&]() -> int {
    k_axpy<<<grid_for(4 * np, 256), 256, 0, stream()>>>(W, wn, ah.A, 4 * np);
    BCFD_LAUNCHED();
    if (use_stress) {
      TRY_R(launch_stress_weights(hb, mu_f, rho_f, sdw, ah.A, ss));
      TRY_R(launch_stress_geo(hb, mu_f, rho_f, sd, wn, ah.fc.ge, ss));
      TRY_R(launch_stress_kin(hb, mu_f, rho_f, sdw, ah.fc.gk, ss));
    }
    return 0;
  };
  // the geometry and kinematics of driver step `st` (each moving body's
  // current state, placed by its Place) are complete: their adjoints go to
  // the parameters.  The objective's body contributes to all five; another
  // moving body only to those it shares (the pitch phase angle and
  // frequency), its own amplitudes and heave frequency being other parameters.
  double dmot[kMotionParams] = {0, 0, 0, 0, 0};
  auto flush = [&](int64_t st, const std::vector<const Place*>& P) -> int {
    for (int mi = 0; mi < nmov; ++mi) {
      const int q0 = movers[(size_t)mi];
      HostBlock* b = all[(size_t)q0].second;
      AdjBlock& a = AB[(size_t)q0];
      double pb[4], gk[kKinScalars];
      TRY_R(launch_geometry_place_adj(b, a.fc.ge, csr_off[(size_t)mi], csr_ent[(size_t)mi], *P[(size_t)mi], gscr,
                                      pb));
      ACK(d2h(gk, a.fc.gk, kKinScalars * sizeof(double)));
      const StepTangent& T = tan[(size_t)mi][(size_t)(st - first[(size_t)mi])];
      for (int q = 0; q < kMotionParams; ++q) {
        if (q0 != hidx && q != 2 && q != 3) continue;
        double v = pb[0] * T.angle[q] + pb[2] * T.ty[q];
        for (int p = 0; p < kKinScalars; ++p) v += gk[p] * T.kin[p][q];
        dmot[q] += v;
      }
      ACK(cudaMemsetAsync(a.fc.ge, 0, 7 * (size_t)b->d.ne * sizeof(double), stream()));
      ACK(cudaMemsetAsync(a.fc.gk, 0, kKinScalars * sizeof(double), stream()));
    }
    return 0;
  };
  double* tape = mem.get<double>((size_t)K * S);
  if (!tape) return fail(BCFD_E_NOMEM);
  TRY_R(objective());  // at x^N with the end geometry (the blocks' state now)
  MoveRecorder rec;
  for (int mi = 0; mi < nmov; ++mi) rec.bodies.push_back(mover(mi));
  rec.cur.assign((size_t)nmov, nullptr);
  rec.sc = pre;
  std::vector<StepGeo> geo((size_t)nb);
  std::vector<const Place*> places((size_t)nmov);
  for (int64_t m = ncp - 1; m >= 0; --m) {
    const int64_t n0 = m * K, n1 = std::min(n0 + K, n_steps);
    const double* cp = cps + (size_t)m * S;
    ACK(cudaMemcpyAsync(tape, cp, S * sizeof(double), cudaMemcpyDeviceToDevice, stream()));
    TRY_R(load_all(cp));
    for (int mi = 0; mi < nmov; ++mi) TRY_R(restore_body(mover(mi), cprec[(size_t)mi][(size_t)m]));
    TRY_R(ghosts_at(n0));
    L.ita = ita0 + n0;
    L.totime = tot0 + n0 * cfg->deltat;
    DevMem seg;
    std::vector<std::vector<BodyRec>> recs((size_t)nmov, std::vector<BodyRec>((size_t)(n1 - n0 + 1)));
    rec.mem = &seg;
    L.recorder = &rec;
    int r = 0;
    for (int64_t n = n0 + 1; n <= n1 && !r; ++n) {
      for (int mi = 0; mi < nmov; ++mi) rec.cur[(size_t)mi] = &recs[(size_t)mi][(size_t)(n - n0)];
      r = run_one_step(c);
      if (!r) r = save_bodies(recs.data(), (size_t)(n - n0), seg);
      if (!r && n < n1) r = save_all(tape + (size_t)(n - n0) * S);
    }
    L.recorder = nullptr;
    rec.cur.assign((size_t)nmov, nullptr);
    if (r) return fail(r);
    if (rec.oom) return fail(BCFD_E_NOMEM);
    for (int64_t n = n1; n > n0; --n) {
      for (int mi = 0; mi < nmov; ++mi) {
        const BodyRec& re = recs[(size_t)mi][(size_t)(n - n0)];
        for (int k2 = 0; k2 < kCalls; ++k2) geo[(size_t)movers[(size_t)mi]].geo[k2] = re.geo[k2];
        // after the bodies moved: the step's end geometry and kinematics
        TRY_R(restore_body(mover(mi), re));
        places[(size_t)mi] = &re.stage.place;
      }
      TRY_R(adjoint_step_second(AB, &geo));
      TRY_R(flush(ita0 + n, places));
      // before: the geometry, kinematics and state the step started from
      for (int mi = 0; mi < nmov; ++mi) {
        const BodyRec& rs =
            (n - 1 == n0) ? cprec[(size_t)mi][(size_t)m] : recs[(size_t)mi][(size_t)(n - 1 - n0)];
        TRY_R(restore_body(mover(mi), rs));
      }
      TRY_R(load_all(tape + (size_t)(n - 1 - n0) * S));
      TRY_R(ghosts_at(n - 1));
      TRY_R(adjoint_step_first(AB, M, c, adj_tol, adj_itmax, &geo));
      if (n - 1 >= 1) TRY_R(objective());
    }
  }
  // the run's start: its geometry and kinematics
  for (int mi = 0; mi < nmov; ++mi) places[(size_t)mi] = &cprec[(size_t)mi][0].stage.place;
  TRY_R(flush(ita0, places));
  // leave the blocks at the forward run's final state
  TRY_R(load_all(fin));
  for (int mi = 0; mi < nmov; ++mi) TRY_R(restore_body(mover(mi), finrec[(size_t)mi]));
  TRY_R(ghosts_at(n_steps));
  L.ita = ita0 + n_steps;
  L.totime = tot0 + n_steps * cfg->deltat;
  k_axpy<<<grid_for(3 * np, 256), 256, 0, stream()>>>(ah.A + 4 * np, 1.0, ah.A, 3 * np);
  BCFD_LAUNCHED();
  double* ghp[4] = {gu, gv, gw, gp};
  for (int q = 0; q < 4; ++q)
    if (ghp[q]) ACK(cudaMemcpyAsync(ghp[q], ah.A + q * np, fb, cudaMemcpyDeviceToHost, stream()));
  double duc = 0.0;
  for (AdjBlock& a : AB) {
    if (!a.hb->is_coarse) continue;
    std::vector<double> ul((size_t)a.hb->d.d.ny * a.hb->d.d.nz);
    ACK(d2h(ul.data(), a.ucl, ul.size() * sizeof(double)));
    for (double v : ul) duc += v;
  }
  if (dj_duc) *dj_duc = duc;
  if (dj_dmotion)
    for (int q = 0; q < kMotionParams; ++q) dj_dmotion[q] = dmot[q];
  ACK(cudaStreamSynchronize(stream()));
  for (auto& [g, b] : all) {
    const int e = take_block_error(b);
    if (e) return e;
  }
  return 0;
}

}  // extern "C"
