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

// correctVelocity and correctPressure transposed: pcb = adjoint of pc (zero
// off the fluid cells, where pc is held at zero)
__global__ void k_correct_adj(DevBlock B, double dt, const double* ut_b, const double* vt_b, const double* wt_b,
                              const double* p_b, double* pcb) {
  const Dims& d = B.d;
  const int64_t n = d.npts(), sy = d.NX, sz = (int64_t)d.NX * d.NY;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(x % d.NX);
    const int64_t r = x / d.NX;
    const int j = 1 + (int)(r % d.NY), k = 1 + (int)(r / d.NY);
    if (!fluid_at(B, i, j, k)) {
      pcb[x] = 0.0;
      continue;
    }
    double g = p_b[x];
    g += dt / (0.5 * (B.dxa[i] + B.dxa[i - 1])) * ut_b[x];
    g += dt / (0.5 * (B.dya[j] + B.dya[j - 1])) * vt_b[x];
    g += dt / (0.5 * (B.dza[k] + B.dza[k - 1])) * wt_b[x];
    if (fluid_at(B, i - 1, j, k)) g -= dt / (0.5 * (B.dxa[i - 1] + B.dxa[i - 2])) * ut_b[x - 1];
    if (fluid_at(B, i, j - 1, k)) g -= dt / (0.5 * (B.dya[j - 1] + B.dya[j - 2])) * vt_b[x - sy];
    if (fluid_at(B, i, j, k - 1)) g -= dt / (0.5 * (B.dza[k - 1] + B.dza[k - 2])) * wt_b[x - sz];
    pcb[x] = g;
  }
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
    if (B.cell[c] != 0 || B.tsnear[c]) continue;
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

struct AdjBuffers {
  double* A;     // adjoint of the 7 state arrays (kept in place through the step)
  double* pcb;   // adjoint of pc
  double* y;     // A^{-T} pcb
  double* ucl;   // dJ/duc per x-face line
  uint32_t* foot;
  ForceCoef fc;  // forcing coefficients (blocks with a body)
};

// One step transposed, in place on the adjoint arrays (the block holds the
// step's input state; tags, IB lists and probes are those of the run, which a
// stationary body keeps).  The forward order is that of the native step:
// predictor, velocityBC, [solidCellBC, velocityForcing1], velocityBC, the
// Poisson phase (div, solve, correctPressure, correctVelocity, velocityBC,
// ut -> u), [pressureForcing1, velocityForcingField, pressureForcingField].
int adjoint_step(HostBlock* hb, const bcfd_step_config& c, const AdjBuffers& a, double tol, int64_t itmax) {
  const int64_t np = hb->d.d.npts();
  double* A[kStateFields];
  for (int q = 0; q < kStateFields; ++q) A[q] = a.A + q * np;
  double* tb[3] = {A[4], A[5], A[6]};
  const Fields4 s{A[0], A[1], A[2], A[3]};
  const bool body = hb->has_body && hb->d.ne > 0;
  if (body) {
    const AdjPtrs pin{{A[3], A[1], A[2], A[3]}, {A[3], A[1], A[2], A[3]}};
    const AdjPtrs field{{A[3], A[0], A[1], A[2]}, {A[3], A[4], A[5], A[6]}};
    TRY_R(launch_forcing_adjoint(hb, 1, 0, pin, a.fc));    // pressureForcingField
    TRY_R(launch_forcing_adjoint(hb, 1, 1, field, a.fc));  // velocityForcingField: reads ut, writes u
    TRY_R(launch_forcing_adjoint(hb, 0, 0, pin, a.fc));    // pressureForcing1
  }
  k_copy_adj<<<grid_for(np, 256), 256, 0, stream()>>>(np, A[0], A[1], A[2], A[4], A[5], A[6]);
  BCFD_LAUNCHED();
  TRY_R(launch_vbc_adj(hb, c.deltat, c.uc, tb, s, a.ucl));
  k_correct_adj<<<grid_for(np, 256), 256, 0, stream()>>>(hb->d, c.deltat, tb[0], tb[1], tb[2], A[3], a.pcb);
  BCFD_LAUNCHED();
  TRY_R(solve_zero_bc_dev(hb, a.pcb, a.y, tol, itmax, true));
  k_div_adj<<<grid_for(np, 256), 256, 0, stream()>>>(hb->d, c.deltat, a.y, tb[0], tb[1], tb[2]);
  BCFD_LAUNCHED();
  TRY_R(launch_vbc_adj(hb, c.deltat, c.uc, tb, s, a.ucl));
  if (body) {
    const AdjPtrs vin{{A[3], A[4], A[5], A[6]}, {A[3], A[4], A[5], A[6]}};
    TRY_R(launch_forcing_adjoint(hb, 0, 1, vin, a.fc));  // velocityForcing1, in place on ut
    const int64_t ni = (int64_t)hb->d.d.nx * hb->d.d.ny * hb->d.d.nz;
    k_solid_adj<<<grid_for(ni, 256), 256, 0, stream()>>>(hb->d, A[4], A[5], A[6], A[3]);
    BCFD_LAUNCHED();
  }
  TRY_R(launch_vbc_adj(hb, c.deltat, c.uc, tb, s, a.ucl));
  const double* sb[3] = {tb[0], tb[1], tb[2]};
  double* ab[4] = {A[0], A[1], A[2], A[3]};
  TRY_R(launch_momentum_adjoint(hb, c.deltat, c.re, sb, ab, a.foot));
  const int64_t ni = (int64_t)hb->d.d.nx * hb->d.d.ny * hb->d.d.nz;
  k_zero_fluid<<<grid_for(ni, 256), 256, 0, stream()>>>(hb->d, tb[0], tb[1], tb[2]);
  BCFD_LAUNCHED();
  return 0;
}

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

}  // namespace
}  // namespace bcfd

using namespace bcfd;

extern "C" {

int bcfd_adjoint_run(bcfd_handle h, const bcfd_step_config* cfg, int64_t n_steps, int64_t every, const double* wu,
                     const double* wv, const double* ww, const double* wp, const double* stress_seed, double mu_f,
                     double rho_f, double adj_tol, int64_t adj_itmax, double* J, double* dj_duc,
                     double* dj_dkin, double* gu, double* gv, double* gw, double* gp) {
  std::lock_guard<std::recursive_mutex> lk(lib().mu);
  HostBlock* hb = get_block(h);
  if (!hb) return BCFD_E_HANDLE;
  if (!cfg || n_steps < 1 || every < 1 || !wu || !wv || !ww || !wp || !J || !(adj_tol > 0.0) || adj_itmax < 1)
    return BCFD_E_ARG;
  int live = 0;
  for (HostBlock* b : lib().blocks) live += b != nullptr;
  for (HostInterface* it : lib().ifs)
    if (it) return BCFD_E_STATE;
  if (live != 1 || !hb->is_coarse || hb->motion.on || cfg->precision != 0) return BCFD_E_STATE;
  if (!hb->d.ca[0] || !hb->d.Acx) return BCFD_E_STATE;
  const bool body = hb->has_body && hb->d.ne > 0;
  const bool use_stress = stress_seed && body;
  if (stress_seed && !body) return BCFD_E_STATE;
  if (body && hb->d.ne > BCFD_STRESS_NOALLOC_MAX_ELEMS) return BCFD_E_CAPACITY;
  const bool grad = dj_duc || dj_dkin || gu || gv || gw || gp;
  const Dims& d = hb->d.d;
  const int64_t np = d.npts();
  const size_t fb = (size_t)np * sizeof(double);
  const int64_t K = std::min(every, n_steps);
  const int64_t ncp = (n_steps + K - 1) / K;  // checkpoints at 0, K, 2K, ... < N
  const size_t S = (size_t)kStateFields * np;
  DevMem mem;
  double* W = mem.get<double>(4 * np);
  double* cps = mem.get<double>((size_t)ncp * S);
  double* fin = mem.get<double>(S);
  double* part = mem.get<double>(kDotCtas);
  if (!W || !cps || !fin || !part) return BCFD_E_NOMEM;
  const double* wh[4] = {wu, wv, ww, wp};
  for (int q = 0; q < 4; ++q) ACK(h2d(W + q * np, wh[q], fb));
  ACK(cudaMemsetAsync(part, 0, kDotCtas * sizeof(double), stream()));
  Lib& L = lib();
  const int64_t ita0 = L.ita;
  const double tot0 = L.totime;
  bcfd_step_config c = *cfg;
  c.use_graph = 0;
  const Fields4 bx{hb->d.u, hb->d.v, hb->d.w, hb->d.p};

  // forward: the work arrays start equal to u, v, w; checkpoints; objective
  ACK(cudaMemcpyAsync(hb->d.ut, hb->d.u, fb, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(hb->d.vt, hb->d.v, fb, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(hb->d.wt, hb->d.w, fb, cudaMemcpyDeviceToDevice, stream()));
  TRY_R(save_state(hb, cps));
  // the transpose assumes the tags the run starts with hold throughout
  // (a stationary body: the per-step re-Search reproduces them)
  std::vector<int8_t> tags0((size_t)np), tags1((size_t)np);
  ACK(d2h(tags0.data(), hb->d.cell, (size_t)np));
  double jstress = 0.0;
  for (int64_t n = 1; n <= n_steps; ++n) {
    TRY_R(run_one_step(c));
    k_dot_acc<<<kDotCtas, kDotThreads, 0, stream()>>>(W, bx, np, part);
    BCFD_LAUNCHED();
    if (use_stress) {
      double co[4];
      TRY_R(launch_stress_noalloc(hb, mu_f, rho_f, co));
      for (int t = 0; t < 4; ++t) jstress += stress_seed[t] * co[t];
    }
    if (n % K == 0 && n < n_steps) TRY_R(save_state(hb, cps + (size_t)(n / K) * S));
  }
  TRY_R(save_state(hb, fin));
  std::vector<double> ph(kDotCtas);
  ACK(d2h(ph.data(), part, kDotCtas * sizeof(double)));
  double jsum = 0.0;
  for (double v : ph) jsum += v;
  *J = (jsum + jstress) / (double)n_steps;
  int err = take_block_error(hb);
  ACK(d2h(tags1.data(), hb->d.cell, (size_t)np));
  if (!err && tags0 != tags1) err = BCFD_E_STATE;
  if (err || !grad) {
    L.ita = ita0 + n_steps;
    L.totime = tot0 + n_steps * cfg->deltat;
    return err;
  }

  // objective weights per step: W plus the stress coefficients' weights
  bool kin_stress = false;
  double* stress_seed_dev = nullptr;
  double* stress_scratch = nullptr;
  if (use_stress) {
    double* sd = mem.get<double>(4);
    double* ss = mem.get<double>(8 + 64 * (size_t)hb->d.ne);
    if (!sd || !ss) return BCFD_E_NOMEM;
    ACK(h2d(sd, stress_seed, 4 * sizeof(double)));
    TRY_R(launch_stress_weights(hb, mu_f, rho_f, sd, W, ss));
    kin_stress = true;
    stress_seed_dev = sd;
    stress_scratch = ss;
  }
  // reverse: recompute each segment from its checkpoint, then step back
  double* tape = mem.get<double>((size_t)K * S);
  AdjBuffers a;
  a.A = mem.get<double>(S);
  a.pcb = mem.get<double>(np);
  a.y = mem.get<double>(np);
  a.ucl = mem.get<double>((size_t)d.ny * d.nz);
  a.foot = mem.get<uint32_t>(16);
  const size_t ntask = 6 * (size_t)hb->d.cap_ib;
  a.fc.tgt = mem.get<int64_t>(body ? ntask : 1);
  a.fc.axis = mem.get<int>(body ? ntask : 1);
  a.fc.pos = mem.get<int64_t>(body ? 8 * ntask : 1);
  a.fc.coef = mem.get<double>(body ? 8 * ntask : 1);
  a.fc.kc = mem.get<double>(body ? 8 * ntask : 1);
  a.fc.gk = mem.get<double>(8);
  if (!tape || !a.A || !a.pcb || !a.y || !a.ucl || !a.foot || !a.fc.tgt || !a.fc.axis || !a.fc.pos || !a.fc.coef ||
      !a.fc.kc || !a.fc.gk)
    return BCFD_E_NOMEM;
  ACK(cudaMemsetAsync(a.fc.gk, 0, 8 * sizeof(double), stream()));
  // the coefficients' own dependence on the kinematic scalars (the same at
  // every step: (1/N) * N times)
  if (kin_stress) TRY_R(launch_stress_kin(hb, mu_f, rho_f, stress_seed_dev, a.fc.gk, stress_scratch));
  ACK(cudaMemsetAsync(a.ucl, 0, (size_t)d.ny * d.nz * sizeof(double), stream()));
  ACK(cudaMemsetAsync(a.A, 0, S * sizeof(double), stream()));
  const double wn = 1.0 / (double)n_steps;
  k_axpy<<<grid_for(4 * np, 256), 256, 0, stream()>>>(W, wn, a.A, 4 * np);
  BCFD_LAUNCHED();
  for (int64_t m = ncp - 1; m >= 0; --m) {
    const int64_t n0 = m * K, n1 = std::min(n0 + K, n_steps);
    const double* cp = cps + (size_t)m * S;
    ACK(cudaMemcpyAsync(tape, cp, S * sizeof(double), cudaMemcpyDeviceToDevice, stream()));
    TRY_R(load_state(hb, cp));
    L.ita = ita0 + n0;
    L.totime = tot0 + n0 * cfg->deltat;
    for (int64_t n = n0 + 1; n < n1; ++n) {
      TRY_R(run_one_step(c));
      TRY_R(save_state(hb, tape + (size_t)(n - n0) * S));
    }
    for (int64_t n = n1; n > n0; --n) {
      TRY_R(load_state(hb, tape + (size_t)(n - 1 - n0) * S));
      TRY_R(adjoint_step(hb, c, a, adj_tol, adj_itmax));
      if (n - 1 >= 1) {
        k_axpy<<<grid_for(4 * np, 256), 256, 0, stream()>>>(W, wn, a.A, 4 * np);
        BCFD_LAUNCHED();
      }
    }
  }
  // leave the block at the forward run's final state
  TRY_R(load_state(hb, fin));
  L.ita = ita0 + n_steps;
  L.totime = tot0 + n_steps * cfg->deltat;
  // the run started from ut = u, vt = v, wt = w: their adjoints add up
  k_axpy<<<grid_for(3 * np, 256), 256, 0, stream()>>>(a.A + 4 * np, 1.0, a.A, 3 * np);
  BCFD_LAUNCHED();
  double* gh[4] = {gu, gv, gw, gp};
  for (int q = 0; q < 4; ++q)
    if (gh[q]) ACK(cudaMemcpyAsync(gh[q], a.A + q * np, fb, cudaMemcpyDeviceToHost, stream()));
  std::vector<double> ul((size_t)d.ny * d.nz);
  ACK(d2h(ul.data(), a.ucl, ul.size() * sizeof(double)));
  if (dj_dkin) ACK(d2h(dj_dkin, a.fc.gk, 8 * sizeof(double)));
  if (dj_duc) {
    double sum = 0.0;
    for (double v : ul) sum += v;
    *dj_duc = sum;
  }
  return take_block_error(hb);
}

}  // extern "C"
