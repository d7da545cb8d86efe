// Pressure-correction kernels: divergence, red-black SOR (one persistent
// cooperative launch per solve), pressure / velocity correction, the
// steady-state reduction and the ut -> u copy of src/PcorVcor.F90.
//
// The Poisson correction pc lives in a colour-packed layout: one array per
// colour with (h, j, k) -> h + NXH*((j-1) + NY*(k-1)), h = (i-1)/2.  A red
// cell's x-neighbours are black cells at h-1/h (i odd) or h/h+1 (i even); its
// y and z neighbours are black cells at the same h.  Because the reference
// copies pc into pco after every sweep pair (src/PcorVcor.F90:363-372), its red
// sweep reads black values of the previous iteration and its black sweep reads
// the new red values -- exactly an in-place red-black sweep on one array, so
// no pco array and no copy exist here.  The stop test max|pc - pco| over the
// fluid cells is the max of |new - old| of both half-sweeps, fused into them.
#include "bcfd_host.h"

namespace bcfd {

namespace {

// interior-row decomposition of one colour: item t -> (h, j, k)
struct RowMap {
  int NXH, ny;
  __device__ void at(int64_t t, int& h, int& j, int& k) const {
    h = (int)(t % NXH);
    const int64_t r = t / NXH;
    j = 2 + (int)(r % ny);
    k = 2 + (int)(r / ny);
  }
};

// computeDiv (src/PcorVcor.F90:222-243) over the fluid cells; b lands in the
// packed layout.  Non-fluid cells keep the zero of the start of the solve.
__global__ void k_div(DevBlock B) {
  const Dims& d = B.d;
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 2 + (int)(t % d.nx);
    const int64_t r = t / d.nx;
    const int j = 2 + (int)(r % d.ny), k = 2 + (int)(r / d.ny);
    const int64_t c = d.idx(i, j, k);
    if (B.cell[c] != 0) continue;
    const double bv = (B.ut[c] - B.ut[c - 1]) / B.dxa[i - 1] +
                      (B.vt[c] - B.vt[c - d.NX]) / B.dya[j - 1] +
                      (B.wt[c] - B.wt[c - (int64_t)d.NX * d.NY]) / B.dza[k - 1];
    B.bpk[colour_of(i, j, k)][d.pidx(i, j, k)] = bv;
  }
}

// rhs = b / deltat, once per solve (the reference divides inside every sweep;
// the quotient is the same IEEE value)
__global__ void k_rhs(DevBlock B, double dt) {
  const int64_t n = B.d.npacked();
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    B.rhs[0][t] = B.bpk[0][t] / dt;
    B.rhs[1][t] = B.bpk[1][t] / dt;
  }
}

// One half-sweep of colour C, FP64, reference arithmetic (no FMA; the
// expression order of src/PcorVcor.F90:319-327).
template <int C>
__device__ __forceinline__ void half_sweep64(const DevBlock& B, const RowMap& rm, int64_t total,
                                             double omega, double& lmax) {
  const Dims& d = B.d;
  const double* __restrict__ o = B.pc[1 - C];
  double* __restrict__ own = B.pc[C];
  const double* __restrict__ rhs = B.rhs[C];
  const uint8_t* __restrict__ upd = B.upd[C];
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int64_t sy = d.NXH, sz = (int64_t)d.NXH * d.NY;
  const int S = gridDim.x * blockDim.x;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  Walk3 w;
  w.init(t, S, d.NXH, d.ny);
  for (; t < (int)total; t += S, w.next()) {
    const int h = w.a, j = 2 + w.b, k = 2 + w.c;
    const int64_t pi = h + sy * (j - 1) + sz * (k - 1);
    if (!upd[pi]) continue;
    int i = 2 * h + 1;
    if (((i + j + k) & 1) != C) ++i;
    const int64_t row = sy * (j - 1) + sz * (k - 1);
    // values written by other CTAs in this launch: read through L2 (ld.cg)
    const double pl = __ldcg(o + row + ((i - 2) >> 1));
    const double pr = __ldcg(o + row + (i >> 1));
    const double ps = __ldcg(o + pi - sy), pn = __ldcg(o + pi + sy);
    const double pb = __ldcg(o + pi - sz), pt = __ldcg(o + pi + sz);
    const double old = __ldcg(own + pi);
    const double ax1 = B.Acx[i - 2], ax2 = B.Acx[i - 2 + nx], ax3 = B.Acx[i - 2 + 2 * nx];
    const double ay1 = B.Acy[j - 2], ay2 = B.Acy[j - 2 + ny], ay3 = B.Acy[j - 2 + 2 * ny];
    const double az1 = B.Acz[k - 2], az2 = B.Acz[k - 2 + nz], az3 = B.Acz[k - 2 + 2 * nz];
    double v = rhs[pi] - ax1 * pl - ax3 * pr - ay1 * ps - ay3 * pn - az1 * pb - az3 * pt;
    v = v / (ax2 + ay2 + az2);
    const double nv = (1.0 - omega) * old + omega * v;
    own[pi] = nv;
    lmax = fmax(lmax, fabs(nv - old));
  }
}

// max over fluid cells of colour C of |b/dt - A pc| (FP64, FMA allowed: this
// is a stop test of the residual-target mode, not reference arithmetic)
template <int C>
__device__ __forceinline__ double resid_max64(const DevBlock& B, const RowMap& rm, int64_t total) {
  const Dims& d = B.d;
  const double* own = B.pc[C];
  const double* o = B.pc[1 - C];
  const int64_t sy = d.NXH, sz = (int64_t)d.NXH * d.NY;
  double m = 0.0;
  const int S = gridDim.x * blockDim.x;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  Walk3 w;
  w.init(t, S, d.NXH, d.ny);
  for (; t < (int)total; t += S, w.next()) {
    const int h = w.a, j = 2 + w.b, k = 2 + w.c;
    const int64_t pi = h + sy * (j - 1) + sz * (k - 1);
    if (!B.upd[C][pi]) continue;
    int i = 2 * h + 1;
    if (((i + j + k) & 1) != C) ++i;
    const int64_t row = pi - h;
    double ax = (B.Acx[i - 2 + d.nx] + B.Acy[j - 2 + d.ny] + B.Acz[k - 2 + d.nz]) * __ldcg(own + pi);
    ax = fma(B.Acx[i - 2], __ldcg(o + row + ((i - 2) >> 1)), ax);
    ax = fma(B.Acx[i - 2 + 2 * d.nx], __ldcg(o + row + (i >> 1)), ax);
    ax = fma(B.Acy[j - 2], __ldcg(o + pi - sy), ax);
    ax = fma(B.Acy[j - 2 + 2 * d.ny], __ldcg(o + pi + sy), ax);
    ax = fma(B.Acz[k - 2], __ldcg(o + pi - sz), ax);
    ax = fma(B.Acz[k - 2 + 2 * d.nz], __ldcg(o + pi + sz), ax);
    m = fmax(m, fabs(B.rhs[C][pi] - ax));
  }
  return m;
}

struct SorArgs {
  int64_t itmax;
  double epsi, omega;
  int64_t* log;   // measurement log (nullptr outside a profiling window)
  double res_tol; // > 0: stop on dt * max|b/dt - A pc| <= res_tol instead of
                  // the reference's increment test (same check cadence)
  double dt;
};

// append {sweep pairs, FP64 residual passes, fluid cells, precision}
__device__ __forceinline__ void log_solve(int64_t* log, int64_t sweeps, int64_t res_passes,
                                          int64_t fluid, int64_t precision) {
  if (!log) return;
  const unsigned long long s = atomicAdd(reinterpret_cast<unsigned long long*>(log), 1ull);
  if (s < kProfLogCap) {
    int64_t* e = log + 1 + 4 * s;
    e[0] = sweeps;
    e[1] = res_passes;
    e[2] = fluid;
    e[3] = precision;
  }
}

// REDBLACKSOR_linear (src/PcorVcor.F90:288-377) as one cooperative launch.
// nIterPcor continues from stats->niter (the fine blocks accumulate it over
// two solves per step, :78, :98, :116) and the stop test runs whenever the
// accumulated count is a multiple of 5, exactly as the reference does.
__global__ void __launch_bounds__(256) k_sor64(DevBlock B, SorArgs a, GridBar gb) {
  __shared__ double sh[32];
  const RowMap rm{B.d.NXH, B.d.ny};
  const int64_t total = (int64_t)B.d.NXH * B.d.ny * B.d.nz;
  BlockStats* st = B.stats;
  int64_t it = st->niter;
  double derr4 = 11111.0;
  int check = 0;
  bool ok = true;
  for (;;) {
    ++it;
    double lmax = 0.0;
    half_sweep64<1>(B, rm, total, a.omega, lmax);
    if (!grid_sync(gb)) { ok = false; break; }
    half_sweep64<0>(B, rm, total, a.omega, lmax);
    const bool chk = (it % 5) == 0;
    if (chk && a.res_tol > 0.0) {
      // residual-target mode: the residual needs the whole sweep pair done
      if (!grid_sync(gb)) { ok = false; break; }
      lmax = fmax(resid_max64<1>(B, rm, total), resid_max64<0>(B, rm, total)) * a.dt;
    }
    if (chk) {
      const double m = block_max(lmax, sh);
      if (threadIdx.x == 0) atomic_max_nonneg(&st->slot[check & 1], m);
    }
    if (!grid_sync(gb)) { ok = false; break; }
    if (chk) {
      derr4 = *((volatile double*)&st->slot[check & 1]);
      if (blockIdx.x == 0 && threadIdx.x == 0) st->slot[(check + 1) & 1] = 0.0;
      ++check;
    }
    if (a.res_tol > 0.0 ? (derr4 <= a.res_tol) : (derr4 < a.epsi)) break;
    if (it > a.itmax) break;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    log_solve(a.log, it - st->niter, 0, B.cnt[C_FLUID], 0);
    st->niter = it;
    st->derr2 = derr4;
    if (ok && !(derr4 == derr4)) set_err(B.err, BCFD_E_NONFINITE);
  }
}

// ---------------------------------------------------------------------------
// FP32 SOR + FP64 defect correction (the mixed-precision Poisson solve).
//   x = pc (FP64, packed).  Outer loop: r = b/dt - A x in FP64 over the fluid
//   cells (stored as FP32 in rhsf), stop when dt * max|r| <= div_tol (the
//   divergence the correction leaves behind), else solve A e = r with M
//   red-black FP32 SOR sweeps from e = 0 (non-fluid cells are zero Dirichlet
//   data for e) and update x += e in FP64.
// ---------------------------------------------------------------------------
struct DcArgs {
  int64_t max_outer;
  int inner;          // FP32 sweeps per correction
  float omega;        // relaxation of the FP32 sweeps
  double dt, div_tol;
  int64_t* log;
};

// grid-stride walk over the interior packed positions of colour C: h, j, k,
// the cell's i and its packed index pi
#define FOR_PACKED(C_, total_)                                  \
  const int _S = gridDim.x * blockDim.x;                        \
  int _t = blockIdx.x * blockDim.x + threadIdx.x;               \
  Walk3 _w;                                                     \
  _w.init(_t, _S, B.d.NXH, B.d.ny);                             \
  for (; _t < (int)(total_); _t += _S, _w.next())
#define PACKED_CELL(C_)                                                                   \
  const int h = _w.a, j = 2 + _w.b, k = 2 + _w.c;                                         \
  const int64_t pi = h + (int64_t)B.d.NXH * (j - 1) + (int64_t)B.d.NXH * B.d.NY * (k - 1); \
  const int i = 2 * h + 1 + ((((2 * h + 1) + j + k) & 1) != (C_))

// FP64 residual of colour C into rhsf[C]; returns the local max |r|
template <int C>
__device__ __forceinline__ double residual64(const DevBlock& B, int64_t total) {
  const Dims& d = B.d;
  const double* __restrict__ own = B.pc[C];
  const double* __restrict__ o = B.pc[1 - C];
  const int64_t sy = d.NXH, sz = (int64_t)d.NXH * d.NY;
  double m = 0.0;
  FOR_PACKED(C, total) {
    PACKED_CELL(C);
    if (!B.upd[C][pi]) continue;
    const int64_t row = pi - (i - 1) / 2;
    const double ax1 = B.Acx[i - 2], ax2 = B.Acx[i - 2 + d.nx], ax3 = B.Acx[i - 2 + 2 * d.nx];
    const double ay1 = B.Acy[j - 2], ay2 = B.Acy[j - 2 + d.ny], ay3 = B.Acy[j - 2 + 2 * d.ny];
    const double az1 = B.Acz[k - 2], az2 = B.Acz[k - 2 + d.nz], az3 = B.Acz[k - 2 + 2 * d.nz];
    double ax = (ax2 + ay2 + az2) * __ldcg(own + pi);
    ax = fma(ax1, __ldcg(o + row + ((i - 2) >> 1)), ax);
    ax = fma(ax3, __ldcg(o + row + (i >> 1)), ax);
    ax = fma(ay1, __ldcg(o + pi - sy), ax);
    ax = fma(ay3, __ldcg(o + pi + sy), ax);
    ax = fma(az1, __ldcg(o + pi - sz), ax);
    ax = fma(az3, __ldcg(o + pi + sz), ax);
    const double r = B.rhs[C][pi] - ax;
    B.rhsf[C][pi] = (float)r;
    m = fmax(m, fabs(r));
  }
  return m;
}

// one FP32 half-sweep on the correction e (stored in pcf)
template <int C>
__device__ __forceinline__ void half_sweep32(const DevBlock& B, int64_t total, float omega) {
  const Dims& d = B.d;
  const float* __restrict__ o = B.pcf[1 - C];
  float* __restrict__ own = B.pcf[C];
  const int64_t sy = d.NXH, sz = (int64_t)d.NXH * d.NY;
  FOR_PACKED(C, total) {
    PACKED_CELL(C);
    if (!B.upd[C][pi]) continue;
    const int64_t row = pi - (i - 1) / 2;
    const float ax1 = B.Acxf[i - 2], ax2 = B.Acxf[i - 2 + d.nx], ax3 = B.Acxf[i - 2 + 2 * d.nx];
    const float ay1 = B.Acyf[j - 2], ay2 = B.Acyf[j - 2 + d.ny], ay3 = B.Acyf[j - 2 + 2 * d.ny];
    const float az1 = B.Aczf[k - 2], az2 = B.Aczf[k - 2 + d.nz], az3 = B.Aczf[k - 2 + 2 * d.nz];
    float s = B.rhsf[C][pi];
    s = __fmaf_rn(-ax1, __ldcg(o + row + ((i - 2) >> 1)), s);
    s = __fmaf_rn(-ax3, __ldcg(o + row + (i >> 1)), s);
    s = __fmaf_rn(-ay1, __ldcg(o + pi - sy), s);
    s = __fmaf_rn(-ay3, __ldcg(o + pi + sy), s);
    s = __fmaf_rn(-az1, __ldcg(o + pi - sz), s);
    s = __fmaf_rn(-az3, __ldcg(o + pi + sz), s);
    const float old = __ldcg(own + pi);
    const float nv = __fmaf_rn(omega, __fdividef(s, ax2 + ay2 + az2) - old, old);
    own[pi] = nv;
  }
}

template <int C>
__device__ __forceinline__ void apply_correction(const DevBlock& B, int64_t np) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < np;
       t += (int64_t)gridDim.x * blockDim.x) {
    if (!B.upd[C][t]) continue;
    B.pc[C][t] = B.pc[C][t] + (double)__ldcg(B.pcf[C] + t);
    B.pcf[C][t] = 0.0f;
  }
}

__global__ void __launch_bounds__(256) k_sor_dc(DevBlock B, DcArgs a, GridBar gb) {
  __shared__ double sh[32];
  const RowMap rm{B.d.NXH, B.d.ny};
  const int64_t total = (int64_t)B.d.NXH * B.d.ny * B.d.nz;
  const int64_t np = B.d.npacked();
  BlockStats* st = B.stats;
  int64_t sweeps = 0;
  double res = 0.0;
  int64_t outer = 0;
  for (;; ++outer) {
    double m = residual64<1>(B, total);
    m = fmax(m, residual64<0>(B, total));
    m = block_max(m, sh);
    if (threadIdx.x == 0) atomic_max_nonneg(&st->slot[outer & 1], m);
    if (!grid_sync(gb)) return;
    res = *((volatile double*)&st->slot[outer & 1]);
    if (blockIdx.x == 0 && threadIdx.x == 0) st->slot[(outer + 1) & 1] = 0.0;
    if (a.dt * res <= a.div_tol || outer >= a.max_outer || !(res == res)) break;
    for (int it = 0; it < a.inner; ++it) {
      half_sweep32<1>(B, total, a.omega);
      if (!grid_sync(gb)) return;
      half_sweep32<0>(B, total, a.omega);
      if (!grid_sync(gb)) return;
    }
    sweeps += a.inner;
    apply_correction<1>(B, np);
    apply_correction<0>(B, np);
    if (!grid_sync(gb)) return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    log_solve(a.log, sweeps, outer + 1, B.cnt[C_FLUID], 1);
    st->niter = st->niter + sweeps;
    st->derr2 = a.dt * res;
    if (!(res == res)) set_err(B.err, BCFD_E_NONFINITE);
  }
}

// dt * max over fluid cells of |b/dt - A pc| (FP64, measurement) -> stats->pad[1]
__global__ void k_resid(DevBlock B, double dt) {
  __shared__ double sh[32];
  const int64_t total = (int64_t)B.d.NXH * B.d.ny * B.d.nz;
  const RowMap rm{B.d.NXH, B.d.ny};
  const double m = block_max(fmax(resid_max64<1>(B, rm, total), resid_max64<0>(B, rm, total)), sh);
  if (threadIdx.x == 0) atomic_max_nonneg(&B.stats->pad[1], m * dt);
}

// correctPressure (src/PcorVcor.F90:245-259)
__global__ void k_correct_p(DevBlock B) {
  const Dims& d = B.d;
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 2 + (int)(t % d.nx);
    const int64_t r = t / d.nx;
    const int j = 2 + (int)(r % d.ny), k = 2 + (int)(r / d.ny);
    const int64_t c = d.idx(i, j, k);
    if (B.cell[c] != 0) continue;
    B.p[c] = B.p[c] + B.pc[colour_of(i, j, k)][d.pidx(i, j, k)];
  }
}

__device__ __forceinline__ double pc_at(const DevBlock& B, int i, int j, int k) {
  return B.pc[colour_of(i, j, k)][B.d.pidx(i, j, k)];
}

// correctVelocity (src/PcorVcor.F90:261-286)
__global__ void k_correct_v(DevBlock B, double dt) {
  const Dims& d = B.d;
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 2 + (int)(t % d.nx);
    const int64_t r = t / d.nx;
    const int j = 2 + (int)(r % d.ny), k = 2 + (int)(r / d.ny);
    const int64_t c = d.idx(i, j, k);
    if (B.cell[c] != 0) continue;
    const double p0 = pc_at(B, i, j, k);
    B.ut[c] = B.ut[c] - dt / (0.5 * (B.dxa[i] + B.dxa[i - 1])) * (pc_at(B, i + 1, j, k) - p0);
    B.vt[c] = B.vt[c] - dt / (0.5 * (B.dya[j] + B.dya[j - 1])) * (pc_at(B, i, j + 1, k) - p0);
    B.wt[c] = B.wt[c] - dt / (0.5 * (B.dza[k] + B.dza[k - 1])) * (pc_at(B, i, j, k + 1) - p0);
  }
}

// steady-state error max |ut - u| / dt over the fluid cells (src/PcorVcor.F90:135-153)
__global__ void k_steady(DevBlock B, double dt) {
  __shared__ double sh[32];
  const Dims& d = B.d;
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  double m = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 2 + (int)(t % d.nx);
    const int64_t r = t / d.nx;
    const int j = 2 + (int)(r % d.ny), k = 2 + (int)(r / d.ny);
    const int64_t c = d.idx(i, j, k);
    if (B.cell[c] != 0) continue;
    const double eu = fabs((B.ut[c] - B.u[c])) / dt;
    const double ev = fabs((B.vt[c] - B.v[c])) / dt;
    const double ew = fabs((B.wt[c] - B.w[c])) / dt;
    m = fmax(fmax(fmax(m, eu), ev), ew);
  }
  m = block_max(m, sh);
  if (threadIdx.x == 0) atomic_max_nonneg(&B.stats->derr_std_st, m);
}

// max |div| over the fluid cells of (u,v,w) (slot maxdiv) or, right after
// the velocity correction, of (ut,vt,wt) (slot derr_pad[0]); FP64
__global__ void k_maxdiv(DevBlock B, int tfield) {
  __shared__ double sh[32];
  const Dims& d = B.d;
  const double* U = tfield ? B.ut : B.u;
  const double* V = tfield ? B.vt : B.v;
  const double* W = tfield ? B.wt : B.w;
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  double m = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 2 + (int)(t % d.nx);
    const int64_t r = t / d.nx;
    const int j = 2 + (int)(r % d.ny), k = 2 + (int)(r / d.ny);
    const int64_t c = d.idx(i, j, k);
    if (B.cell[c] != 0) continue;
    const double dv = (U[c] - U[c - 1]) / B.dxa[i - 1] + (V[c] - V[c - d.NX]) / B.dya[j - 1] +
                      (W[c] - W[c - (int64_t)d.NX * d.NY]) / B.dza[k - 1];
    m = fmax(m, fabs(dv));
  }
  m = block_max(m, sh);
  if (threadIdx.x == 0) atomic_max_nonneg(tfield ? &B.stats->pad[0] : &B.stats->maxdiv, m);
}

__global__ void k_copy3(double* a, double* b, double* c, const double* x, const double* y,
                        const double* z, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    a[t] = x[t];
    b[t] = y[t];
    c[t] = z[t];
  }
}

// SOR update masks from the cell tags (the red/black lists of cellCount_solid)
__global__ void k_masks(DevBlock B) {
  const Dims& d = B.d;
  const int64_t n = d.npts();
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % d.NX);
    const int64_t r = t / d.NX;
    const int j = 1 + (int)(r % d.NY), k = 1 + (int)(r / d.NY);
    const bool interior = i >= 2 && i <= d.nx + 1 && j >= 2 && j <= d.ny + 1 && k >= 2 && k <= d.nz + 1;
    B.upd[colour_of(i, j, k)][d.pidx(i, j, k)] = (interior && B.cell[t] == 0) ? 1 : 0;
  }
  // the dummy slot of an odd NX row stays 0 (set by the initial memset)
}

__global__ void k_pack(DevBlock B, const double* nat, double* p0, double* p1) {
  const Dims& d = B.d;
  const int64_t n = d.npts();
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % d.NX);
    const int64_t r = t / d.NX;
    const int j = 1 + (int)(r % d.NY), k = 1 + (int)(r / d.NY);
    (colour_of(i, j, k) ? p1 : p0)[d.pidx(i, j, k)] = nat[t];
  }
}

__global__ void k_unpack(DevBlock B, const double* p0, const double* p1, double* nat) {
  const Dims& d = B.d;
  const int64_t n = d.npts();
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % d.NX);
    const int64_t r = t / d.NX;
    const int j = 1 + (int)(r % d.NY), k = 1 + (int)(r / d.NY);
    nat[t] = (colour_of(i, j, k) ? p1 : p0)[d.pidx(i, j, k)];
  }
}

}  // namespace

int launch_compute_div(HostBlock* hb) {
  const int64_t n = (int64_t)hb->d.d.nx * hb->d.d.ny * hb->d.d.nz;
  k_div<<<grid_for(n, 256), 256, 0, stream()>>>(hb->d);
  BCFD_LAUNCHED();
  return 0;
}

int launch_correct_pressure(HostBlock* hb) {
  const int64_t n = (int64_t)hb->d.d.nx * hb->d.d.ny * hb->d.d.nz;
  k_correct_p<<<grid_for(n, 256), 256, 0, stream()>>>(hb->d);
  BCFD_LAUNCHED();
  return 0;
}

int launch_correct_velocity(HostBlock* hb, double dt) {
  const int64_t n = (int64_t)hb->d.d.nx * hb->d.d.ny * hb->d.d.nz;
  k_correct_v<<<grid_for(n, 256), 256, 0, stream()>>>(hb->d, dt);
  BCFD_LAUNCHED();
  return 0;
}

int launch_zero_poisson(HostBlock* hb) {
  const size_t bytes = (size_t)hb->d.d.npacked() * sizeof(double);
  for (int c = 0; c < 2; ++c) {
    BCFD_CUDA(cudaMemsetAsync(hb->d.pc[c], 0, bytes, stream()));
    BCFD_CUDA(cudaMemsetAsync(hb->d.bpk[c], 0, bytes, stream()));
  }
  // nIterPcor = 0, derr2 = 0, derrStdSt = 0 (src/PcorVcor.F90:78-80)
  BCFD_CUDA(cudaMemsetAsync(hb->d.stats, 0, sizeof(BlockStats), stream()));
  return 0;
}

static int launch_residual(HostBlock* hb, double dt) {
  BCFD_CUDA(cudaMemsetAsync(&hb->d.stats->pad[1], 0, sizeof(double), stream()));
  const int64_t total = (int64_t)hb->d.d.NXH * hb->d.d.ny * hb->d.d.nz;
  k_resid<<<grid_for(total, 256, 1024), 256, 0, stream()>>>(hb->d, dt);
  BCFD_LAUNCHED();
  return 0;
}

int launch_sor(HostBlock* hb, int64_t itmax, double dt, double epsi, double res_tol) {
  DevBlock& B = hb->d;
  const int64_t np = B.d.npacked();
  k_rhs<<<grid_for(np, 256), 256, 0, stream()>>>(B, dt);
  BCFD_LAUNCHED();
  // fresh stop-test slots and barrier words for this launch
  BCFD_CUDA(cudaMemsetAsync(&B.stats->slot[0], 0, 2 * sizeof(double), stream()));
  BCFD_CUDA(cudaMemsetAsync(hb->bar, 0, 2 * sizeof(unsigned), stream()));
  const int64_t total = (int64_t)B.d.NXH * B.d.ny * B.d.nz;
  const int threads = 256;
  unsigned want = (unsigned)((total + threads - 1) / threads);
  const unsigned grid = coop_grid((const void*)k_sor64, threads, 0, want);
  SorArgs a{itmax, epsi, hb->omega, prof_log(), res_tol, dt};
  GridBar gb = make_bar(B.err, grid);
  gb.count = hb->bar;
  gb.gen = hb->bar + 1;
  void* args[] = {(void*)&B, (void*)&a, (void*)&gb};
  prof_mark(true);
  BCFD_CUDA(launch_coop((const void*)k_sor64, grid, threads, args));
  prof_mark(false);
  BCFD_LAUNCHED();
  return launch_residual(hb, dt);
}

int launch_sor_mixed(HostBlock* hb, int64_t itmax, double dt, double div_tol) {
  DevBlock& B = hb->d;
  const int64_t np = B.d.npacked();
  k_rhs<<<grid_for(np, 256), 256, 0, stream()>>>(B, dt);
  BCFD_LAUNCHED();
  const int nmax0 = std::max(B.d.nx, std::max(B.d.ny, B.d.nz));
  if (hb->dc_variant != 1 && cluster_solve_fits(hb)) {
    // the whole block fits in one cluster's distributed shared memory
    const int inner = hb->dc_inner > 0 ? hb->dc_inner : 64;
    const double om = hb->dc_omega > 0 ? hb->dc_omega : 2.0 / (1.0 + std::sin(3.14159265358979323846 / nmax0));
    TRY_R(launch_sor_cluster(hb, itmax, dt, div_tol, inner, (float)std::min(1.97, std::max(1.0, om))));
    return launch_residual(hb, dt);
  }
  for (int c = 0; c < 2; ++c) BCFD_CUDA(cudaMemsetAsync(B.pcf[c], 0, np * sizeof(float), stream()));
  BCFD_CUDA(cudaMemsetAsync(&B.stats->slot[0], 0, 2 * sizeof(double), stream()));
  BCFD_CUDA(cudaMemsetAsync(hb->bar, 0, 2 * sizeof(unsigned), stream()));
  const int64_t total = (int64_t)B.d.NXH * B.d.ny * B.d.nz;
  const int threads = 256;
  const unsigned grid = coop_grid((const void*)k_sor_dc, threads, 0, (unsigned)((total + threads - 1) / threads));
  const int nmax = std::max(B.d.nx, std::max(B.d.ny, B.d.nz));
  DcArgs a;
  a.inner = hb->dc_inner > 0 ? hb->dc_inner : 64;
  double om = hb->dc_omega > 0 ? hb->dc_omega : 2.0 / (1.0 + std::sin(3.14159265358979323846 / nmax));
  a.omega = (float)std::min(1.97, std::max(1.0, om));
  a.max_outer = itmax / a.inner + 1;
  a.dt = dt;
  a.div_tol = div_tol;
  a.log = prof_log();
  GridBar gb = make_bar(B.err, grid);
  gb.count = hb->bar;
  gb.gen = hb->bar + 1;
  void* args[] = {(void*)&B, (void*)&a, (void*)&gb};
  prof_mark(true);
  BCFD_CUDA(launch_coop((const void*)k_sor_dc, grid, threads, args));
  prof_mark(false);
  BCFD_LAUNCHED();
  return launch_residual(hb, dt);
}

int launch_steady_state(HostBlock* hb, double dt) {
  const int64_t n = (int64_t)hb->d.d.nx * hb->d.d.ny * hb->d.d.nz;
  BCFD_CUDA(cudaMemsetAsync(&hb->d.stats->derr_std_st, 0, sizeof(double), stream()));
  k_steady<<<grid_for(n, 256, 1024), 256, 0, stream()>>>(hb->d, dt);
  BCFD_LAUNCHED();
  return 0;
}

int launch_max_div(HostBlock* hb, bool tfield) {
  const int64_t n = (int64_t)hb->d.d.nx * hb->d.d.ny * hb->d.d.nz;
  double* slot = tfield ? &hb->d.stats->pad[0] : &hb->d.stats->maxdiv;
  BCFD_CUDA(cudaMemsetAsync(slot, 0, sizeof(double), stream()));
  k_maxdiv<<<grid_for(n, 256, 1024), 256, 0, stream()>>>(hb->d, tfield ? 1 : 0);
  BCFD_LAUNCHED();
  return 0;
}

int launch_copy_t_to_n(HostBlock* hb) {
  const int64_t n = hb->d.d.npts();
  k_copy3<<<grid_for(n, 256), 256, 0, stream()>>>(hb->d.u, hb->d.v, hb->d.w, hb->d.ut, hb->d.vt,
                                                   hb->d.wt, n);
  BCFD_LAUNCHED();
  return 0;
}

int launch_copy_n_to_t(HostBlock* hb) {
  const int64_t n = hb->d.d.npts();
  k_copy3<<<grid_for(n, 256), 256, 0, stream()>>>(hb->d.ut, hb->d.vt, hb->d.wt, hb->d.u, hb->d.v,
                                                   hb->d.w, n);
  BCFD_LAUNCHED();
  return 0;
}

int launch_update_masks(HostBlock* hb) {
  const int64_t n = hb->d.d.npts();
  k_masks<<<grid_for(n, 256), 256, 0, stream()>>>(hb->d);
  BCFD_LAUNCHED();
  return 0;
}

int launch_pack(HostBlock* hb, const double* nat, double* packed[2]) {
  const int64_t n = hb->d.d.npts();
  k_pack<<<grid_for(n, 256), 256, 0, stream()>>>(hb->d, nat, packed[0], packed[1]);
  BCFD_LAUNCHED();
  return 0;
}

int launch_unpack(HostBlock* hb, double* const packed[2], double* nat) {
  const int64_t n = hb->d.d.npts();
  k_unpack<<<grid_for(n, 256), 256, 0, stream()>>>(hb->d, packed[0], packed[1], nat);
  BCFD_LAUNCHED();
  return 0;
}

}  // namespace bcfd
