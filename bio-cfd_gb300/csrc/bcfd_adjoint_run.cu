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

// the work arrays start as ut = u: positions the predictor does not write
// pass their adjoint to the state; p' = p + pc passes p's adjoint through
__global__ void k_pass_adj(DevBlock B, const double* ut_b, const double* vt_b, const double* wt_b,
                           const double* p_b, Fields4 s) {
  const Dims& d = B.d;
  const int64_t n = d.npts();
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(x % d.NX);
    const int64_t r = x / d.NX;
    const int j = 1 + (int)(r % d.NY), k = 1 + (int)(r / d.NY);
    if (!fluid_at(B, i, j, k)) {
      s.u[x] += ut_b[x];
      s.v[x] += vt_b[x];
      s.w[x] += wt_b[x];
    }
    s.p[x] += p_b[x];
  }
}

// y = x + a * w over 4 consecutive fields
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

int save_state(HostBlock* hb, double* slot) {
  const size_t np = (size_t)hb->d.d.npts(), b = np * sizeof(double);
  DevBlock& D = hb->d;
  ACK(cudaMemcpyAsync(slot, D.u, b, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(slot + np, D.v, b, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(slot + 2 * np, D.w, b, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(slot + 3 * np, D.p, b, cudaMemcpyDeviceToDevice, stream()));
  return 0;
}

// the state into the block, with ut = u (the invariant at a step's start)
int load_state(HostBlock* hb, const double* slot) {
  const size_t np = (size_t)hb->d.d.npts(), b = np * sizeof(double);
  DevBlock& D = hb->d;
  ACK(cudaMemcpyAsync(D.u, slot, b, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(D.v, slot + np, b, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(D.w, slot + 2 * np, b, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(D.p, slot + 3 * np, b, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(D.ut, slot, b, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(D.vt, slot + np, b, cudaMemcpyDeviceToDevice, stream()));
  ACK(cudaMemcpyAsync(D.wt, slot + 2 * np, b, cudaMemcpyDeviceToDevice, stream()));
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
  double* lam;   // adjoint of the step's output state (4 fields)
  double* acc;   // adjoint of the step's input state (4 fields)
  double* tb;    // adjoint of ut,vt,wt (3 fields)
  double* pcb;   // adjoint of pc
  double* y;     // A^{-T} pcb
  double* ucl;   // dJ/duc per x-face line
  uint32_t* foot;
};

// one reverse step: lam (adjoint of x^n) -> acc (adjoint of x^{n-1}); the
// block holds x^{n-1}
int adjoint_step(HostBlock* hb, const bcfd_step_config& c, const AdjBuffers& a, double tol, int64_t itmax) {
  const int64_t np = hb->d.d.npts();
  const size_t b = (size_t)np * sizeof(double);
  double* tb[3] = {a.tb, a.tb + np, a.tb + 2 * np};
  const double* pb = a.lam + 3 * np;
  const Fields4 s{a.acc, a.acc + np, a.acc + 2 * np, a.acc + 3 * np};
  ACK(cudaMemcpyAsync(a.tb, a.lam, 3 * b, cudaMemcpyDeviceToDevice, stream()));  // S11
  ACK(cudaMemsetAsync(a.acc, 0, 4 * b, stream()));
  TRY_R(launch_vbc_adj(hb, c.deltat, c.uc, tb, s, a.ucl));  // S9
  k_correct_adj<<<grid_for(np, 256), 256, 0, stream()>>>(hb->d, c.deltat, tb[0], tb[1], tb[2], pb, a.pcb);  // S7, S6
  BCFD_LAUNCHED();
  TRY_R(solve_zero_bc_dev(hb, a.pcb, a.y, tol, itmax, true));  // S5
  k_div_adj<<<grid_for(np, 256), 256, 0, stream()>>>(hb->d, c.deltat, a.y, tb[0], tb[1], tb[2]);  // S4
  BCFD_LAUNCHED();
  TRY_R(launch_vbc_adj(hb, c.deltat, c.uc, tb, s, a.ucl));  // S3
  TRY_R(launch_vbc_adj(hb, c.deltat, c.uc, tb, s, a.ucl));  // S2
  const double* sb[3] = {tb[0], tb[1], tb[2]};
  double* ab[4] = {s.u, s.v, s.w, s.p};
  TRY_R(launch_momentum_adjoint(hb, c.deltat, c.re, sb, ab, a.foot));  // S1
  k_pass_adj<<<grid_for(np, 256), 256, 0, stream()>>>(hb->d, tb[0], tb[1], tb[2], pb, s);
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
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return static_cast<T*>(p);
  }
};

}  // namespace
}  // namespace bcfd

using namespace bcfd;

extern "C" {

int bcfd_adjoint_run(bcfd_handle h, const bcfd_step_config* cfg, int64_t n_steps, int64_t every, const double* wu,
                     const double* wv, const double* ww, const double* wp, double adj_tol, int64_t adj_itmax,
                     double* J, double* dj_duc, double* gu, double* gv, double* gw, double* gp) {
  std::lock_guard<std::recursive_mutex> lk(lib().mu);
  HostBlock* hb = get_block(h);
  if (!hb) return BCFD_E_HANDLE;
  if (!cfg || n_steps < 1 || every < 1 || !wu || !wv || !ww || !wp || !J || !(adj_tol > 0.0) || adj_itmax < 1)
    return BCFD_E_ARG;
  int live = 0;
  for (HostBlock* b : lib().blocks) live += b != nullptr;
  for (HostInterface* it : lib().ifs)
    if (it) return BCFD_E_STATE;
  if (live != 1 || !hb->is_coarse || hb->has_body || hb->motion.on || cfg->precision != 0) return BCFD_E_STATE;
  if (!hb->d.ca[0] || !hb->d.Acx) return BCFD_E_STATE;
  const bool grad = dj_duc || gu || gv || gw || gp;
  const Dims& d = hb->d.d;
  const int64_t np = d.npts();
  const size_t fb = (size_t)np * sizeof(double);
  const int64_t K = std::min(every, n_steps);
  const int64_t ncp = (n_steps + K - 1) / K;  // checkpoints at 0, K, 2K, ... < N
  DevMem mem;
  double* W = mem.get<double>(4 * np);
  double* cps = mem.get<double>((size_t)ncp * 4 * np);
  double* fin = mem.get<double>(4 * np);
  double* part = mem.get<double>(kDotCtas);
  if (!W || !cps || !fin || !part) return BCFD_E_NOMEM;
  const double* wh[4] = {wu, wv, ww, wp};
  for (int q = 0; q < 4; ++q) ACK(cudaMemcpyAsync(W + q * np, wh[q], fb, cudaMemcpyHostToDevice, stream()));
  ACK(cudaMemsetAsync(part, 0, kDotCtas * sizeof(double), stream()));
  Lib& L = lib();
  const int64_t ita0 = L.ita;
  const double tot0 = L.totime;
  bcfd_step_config c = *cfg;
  c.use_graph = 0;
  const Fields4 bx{hb->d.u, hb->d.v, hb->d.w, hb->d.p};

  // forward: checkpoints, objective
  TRY_R(save_state(hb, cps));
  TRY_R(load_state(hb, cps));
  for (int64_t n = 1; n <= n_steps; ++n) {
    TRY_R(run_one_step(c));
    k_dot_acc<<<kDotCtas, kDotThreads, 0, stream()>>>(W, bx, np, part);
    BCFD_LAUNCHED();
    if (n % K == 0 && n < n_steps) TRY_R(save_state(hb, cps + (size_t)(n / K) * 4 * np));
  }
  TRY_R(save_state(hb, fin));
  std::vector<double> ph(kDotCtas);
  ACK(cudaMemcpyAsync(ph.data(), part, kDotCtas * sizeof(double), cudaMemcpyDeviceToHost, stream()));
  ACK(cudaStreamSynchronize(stream()));
  double jsum = 0.0;
  for (double v : ph) jsum += v;
  *J = jsum / (double)n_steps;
  int err = take_block_error(hb);
  if (err || !grad) {
    L.ita = ita0 + n_steps;
    L.totime = tot0 + n_steps * cfg->deltat;
    return err;
  }

  // reverse: recompute each segment from its checkpoint, then step back
  double* tape = mem.get<double>((size_t)K * 4 * np);
  AdjBuffers a;
  a.lam = mem.get<double>(4 * np);
  a.acc = mem.get<double>(4 * np);
  a.tb = mem.get<double>(3 * np);
  a.pcb = mem.get<double>(np);
  a.y = mem.get<double>(np);
  a.ucl = mem.get<double>((size_t)d.ny * d.nz);
  a.foot = mem.get<uint32_t>(16);
  if (!tape || !a.lam || !a.acc || !a.tb || !a.pcb || !a.y || !a.ucl || !a.foot) return BCFD_E_NOMEM;
  ACK(cudaMemsetAsync(a.ucl, 0, (size_t)d.ny * d.nz * sizeof(double), stream()));
  ACK(cudaMemsetAsync(a.lam, 0, 4 * fb, stream()));
  const double wn = 1.0 / (double)n_steps;
  k_axpy<<<grid_for(4 * np, 256), 256, 0, stream()>>>(W, wn, a.lam, 4 * np);
  BCFD_LAUNCHED();
  for (int64_t m = ncp - 1; m >= 0; --m) {
    const int64_t n0 = m * K, n1 = std::min(n0 + K, n_steps);
    const double* cp = cps + (size_t)m * 4 * np;
    ACK(cudaMemcpyAsync(tape, cp, 4 * fb, cudaMemcpyDeviceToDevice, stream()));
    TRY_R(load_state(hb, cp));
    L.ita = ita0 + n0;
    L.totime = tot0 + n0 * cfg->deltat;
    for (int64_t n = n0 + 1; n < n1; ++n) {
      TRY_R(run_one_step(c));
      TRY_R(save_state(hb, tape + (size_t)(n - n0) * 4 * np));
    }
    for (int64_t n = n1; n > n0; --n) {
      TRY_R(load_state(hb, tape + (size_t)(n - 1 - n0) * 4 * np));
      TRY_R(adjoint_step(hb, c, a, adj_tol, adj_itmax));
      std::swap(a.lam, a.acc);
      if (n - 1 >= 1) {
        k_axpy<<<grid_for(4 * np, 256), 256, 0, stream()>>>(W, wn, a.lam, 4 * np);
        BCFD_LAUNCHED();
      }
    }
  }
  // leave the block at x^N, as the forward run left it
  TRY_R(load_state(hb, fin));
  L.ita = ita0 + n_steps;
  L.totime = tot0 + n_steps * cfg->deltat;
  double* gh[4] = {gu, gv, gw, gp};
  for (int q = 0; q < 4; ++q)
    if (gh[q]) ACK(cudaMemcpyAsync(gh[q], a.lam + q * np, fb, cudaMemcpyDeviceToHost, stream()));
  std::vector<double> ul((size_t)d.ny * d.nz);
  ACK(cudaMemcpyAsync(ul.data(), a.ucl, ul.size() * sizeof(double), cudaMemcpyDeviceToHost, stream()));
  ACK(cudaStreamSynchronize(stream()));
  if (dj_duc) {
    double sum = 0.0;
    for (double v : ul) sum += v;
    *dj_duc = sum;
  }
  return take_block_error(hb);
}

}  // extern "C"
