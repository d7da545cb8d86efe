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
#include <cuda.h>
#include <cudaTypedefs.h>

#include "bcfd_host.h"

namespace bcfd {

namespace {

// computeDiv (src/PcorVcor.F90:222-243) over the fluid cells; b lands in the
// packed layout.  Non-fluid cells keep the zero of the start of the solve.
// With `fast` (the residual-target solves, which reproduce no reference bits)
// the differences are multiplied by the reciprocal spacings instead of divided
// by the spacings: b within an ulp, without three FP64 divisions per cell.
struct DivOp {
  int fast;
  __device__ void run(const DevBlock& B, int cta, int ncta) const {
    const Dims& d = B.d;
    const double* rx = B.lcoef + (d.NX + d.NY + d.NZ);
    const double* ry = rx + d.NX;
    const double* rz = ry + d.NY;
    FOR_INTERIOR(B, cta, ncta) {
      INTERIOR_CELL(B);
      if (B.cell[c] != 0) continue;
      const double du = B.ut[c] - B.ut[c - 1], dv = B.vt[c] - B.vt[c - d.NX],
                   dw = B.wt[c] - B.wt[c - (int64_t)d.NX * d.NY];
      const double bv = fast ? du * rx[i - 1] + dv * ry[j - 1] + dw * rz[k - 1]
                             : du / B.dxa[i - 1] + dv / B.dya[j - 1] + dw / B.dza[k - 1];
      B.bpk[colour_of(i, j, k)][d.pidx(i, j, k)] = bv;
    }
  }
};

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

// ---------------------------------------------------------------------------
// Tiled persistent solves.  Each CTA of a cooperative launch owns one 2-D
// tile of interior rows (j in [j0, j0+nj), k in [k0, k0+nk), every h of both
// colours).  A red-black half-sweep reads the other colour only at face
// neighbours, so instead of a grid-wide barrier between half-sweeps each CTA
// waits for the (at most four) CTAs owning the face-adjacent tiles: every
// phase (half-sweep, residual pass, correction) ends with the CTA publishing
// its count of completed phases, and a phase starts once the neighbours have
// completed as many phases as this CTA.  That orders both the reads of the
// neighbours' previous-phase values and the overwrite of values they read in
// that phase, so every cell sees exactly the values a grid-wide barrier
// would give it.  Grid-wide barriers remain only where a global max is taken.
// With `global` set, every phase boundary is a grid-wide barrier instead
// (fewer round trips per phase when a phase is only ~1 cell per thread).
// ---------------------------------------------------------------------------
// largest CTA of the FP64 tiled solve, and the FP32 solve's largest CTA (its
// four-cell runs need ~80 registers: three CTAs of 256 threads per SM)
constexpr int kSolveMaxThreads = 512;
constexpr int kDcThreads = 256;

struct TileMap {
  int tj, tk;      // rows per tile along j and k
  int ntj, ntk;    // tiles along j and k (gridDim.x == ntj * ntk)
  unsigned* prog;  // completed-phase count per tile, zeroed before the launch
  int global;      // 1: phase boundaries are grid-wide barriers
};

struct Tile {
  int j0, nj, k0, nk;  // first interior row and row counts of this CTA's tile
  int a, b;            // tile coordinates
};

__device__ __forceinline__ Tile my_tile(const Dims& d, const TileMap& tm, int cta) {
  Tile t;
  t.a = cta % tm.ntj;
  t.b = cta / tm.ntj;
  t.j0 = 2 + t.a * tm.tj;
  t.k0 = 2 + t.b * tm.tk;
  t.nj = min(tm.tj, d.ny + 2 - t.j0);
  t.nk = min(tm.tk, d.nz + 2 - t.k0);
  return t;
}

// publish `done` completed phases of this CTA, after all its threads' writes
__device__ __forceinline__ void tile_publish(const TileMap& tm, const Tile& t, unsigned done) {
  if (tm.global) return;
  __syncthreads();
  if (threadIdx.x == 0) {
    fence_acq_rel_gpu();
    st_relaxed(tm.prog + kTileStride * (t.a + tm.ntj * t.b), done);
  }
}

// wait until the face-neighbour tiles have completed `need` phases (lanes 0-3
// of warp 0 poll one neighbour each); false once the launch was abandoned
__device__ __forceinline__ bool tile_wait(const TileMap& tm, const GridBar& gb, const Tile& t,
                                          unsigned need) {
  if (tm.global) return need == 0 ? true : grid_sync(gb);
  __shared__ int s_ok;
  if (threadIdx.x < 32) {
    const int q = threadIdx.x;
    int na = t.a, nb = t.b;
    bool have = false;
    if (q == 0 && t.a > 0) { na = t.a - 1; have = true; }
    else if (q == 1 && t.a + 1 < tm.ntj) { na = t.a + 1; have = true; }
    else if (q == 2 && t.b > 0) { nb = t.b - 1; have = true; }
    else if (q == 3 && t.b + 1 < tm.ntk) { nb = t.b + 1; have = true; }
    int ok = 1;
    if (have) {
      const unsigned* f = tm.prog + kTileStride * (na + tm.ntj * nb);
      const unsigned long long t0 = globaltimer_ns();
      unsigned spins = 0;
      while (ld_relaxed(f) < need) {
        if (((++spins) & 63u) == 0) {
          if ((ld_relaxed_u64(gb.ctr) & kBarAbandon) || ld_acquire_i(gb.err) != 0) {
            atomicOr(gb.ctr, kBarAbandon);
            ok = 0;
            break;
          }
          if (globaltimer_ns() - t0 > gb.limit_ns) {
            atomicCAS(gb.err, 0, BCFD_E_TIMEOUT);
            atomicOr(gb.ctr, kBarAbandon);
            ok = 0;
            break;
          }
        }
      }
      fence_acq_rel_gpu();
    }
    ok = __all_sync(0xffffffffu, ok);
    if (q == 0) s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// A tile position of colour C: packed index, row start, cell indices and
// whether the cell is updated.  A position past the tile end maps onto the
// tile's first row (addresses in range, never updated).  `ic` is i clamped to
// the interior for the coefficient tables (cells that are not updated may sit
// at i = 1 or nx + 2); every neighbour address of a tile row is in range.
struct Pos {
  int64_t pi, row;
  int i, ic, j, k;
  bool on;
};

template <int C>
__device__ __forceinline__ Pos tile_pos(const DevBlock& B, const Tile& t, const Walk3& w, bool valid) {
  Pos p;
  const int h = valid ? w.a : 0;
  p.j = valid ? t.j0 + w.b : t.j0;
  p.k = valid ? t.k0 + w.c : t.k0;
  p.row = (int64_t)B.d.NXH * (p.j - 1) + (int64_t)B.d.NXH * B.d.NY * (p.k - 1);
  p.pi = p.row + h;
  p.i = 2 * h + 1 + ((((2 * h + 1) + p.j + p.k) & 1) != C);
  p.ic = min(max(p.i, 2), B.d.nx + 1);
  p.on = valid && B.upd[C][p.pi] != 0;
  return p;
}

// reference SOR update of one FP64 cell (no FMA; the expression order of
// src/PcorVcor.F90:319-327); `old` returns the previous value
template <int C>
__device__ __forceinline__ double sor64_cell(const DevBlock& B, const Pos& p, double omega, double& old) {
  const Dims& d = B.d;
  const double* __restrict__ o = B.pc[1 - C];
  const int64_t sy = d.NXH, sz = (int64_t)d.NXH * d.NY;
  const int i = p.ic, j = p.j, k = p.k, nx = d.nx, ny = d.ny, nz = d.nz;
  // values written by other CTAs in this launch: read through L2 (ld.cg)
  const double pl = __ldcg(o + p.row + ((p.i - 2) >> 1));
  const double pr = __ldcg(o + p.row + (p.i >> 1));
  const double ps = __ldcg(o + p.pi - sy), pn = __ldcg(o + p.pi + sy);
  const double pb = __ldcg(o + p.pi - sz), pt = __ldcg(o + p.pi + sz);
  old = __ldcg(B.pc[C] + p.pi);
  const double ax1 = B.Acx[i - 2], ax2 = B.Acx[i - 2 + nx], ax3 = B.Acx[i - 2 + 2 * nx];
  const double ay1 = B.Acy[j - 2], ay2 = B.Acy[j - 2 + ny], ay3 = B.Acy[j - 2 + 2 * ny];
  const double az1 = B.Acz[k - 2], az2 = B.Acz[k - 2 + nz], az3 = B.Acz[k - 2 + 2 * nz];
  double v = B.rhs[C][p.pi] - ax1 * pl - ax3 * pr - ay1 * ps - ay3 * pn - az1 * pb - az3 * pt;
  v = v / (ax2 + ay2 + az2);
  return (1.0 - omega) * old + omega * v;
}

// One half-sweep of colour C over the tile, FP64, reference arithmetic; one
// cell per pass (the FP64 sweep is bound by the FP64 divide, and the lower
// register count keeps two CTAs of 512 threads per SM)
// SOR update of one FP64 cell without a division, for solves that stop on
// the FP64 residual (precision 3): r = b/dt - A_offdiag pc by fused
// multiply-adds, then x + omega r / d.  1/d is an FP32 reciprocal refined by
// one Newton-Raphson step in FP64 (y1 = y0 + y0 (1 - d y0)), accurate to a
// few FP64 ulps; the iteration's fixed point A x = b does not depend on it.
template <int C>
__device__ __forceinline__ double sor64f_cell(const DevBlock& B, const Pos& p, double omega, double& old) {
  const Dims& d = B.d;
  const double* __restrict__ o = B.pc[1 - C];
  const int64_t sy = d.NXH, sz = (int64_t)d.NXH * d.NY;
  const int i = p.ic, j = p.j, k = p.k, nx = d.nx, ny = d.ny, nz = d.nz;
  const double pl = __ldcg(o + p.row + ((p.i - 2) >> 1));
  const double pr = __ldcg(o + p.row + (p.i >> 1));
  const double ps = __ldcg(o + p.pi - sy), pn = __ldcg(o + p.pi + sy);
  const double pb = __ldcg(o + p.pi - sz), pt = __ldcg(o + p.pi + sz);
  old = __ldcg(B.pc[C] + p.pi);
  const double ax1 = B.Acx[i - 2], ax2 = B.Acx[i - 2 + nx], ax3 = B.Acx[i - 2 + 2 * nx];
  const double ay1 = B.Acy[j - 2], ay2 = B.Acy[j - 2 + ny], ay3 = B.Acy[j - 2 + 2 * ny];
  const double az1 = B.Acz[k - 2], az2 = B.Acz[k - 2 + nz], az3 = B.Acz[k - 2 + 2 * nz];
  const double dg = ax2 + ay2 + az2;
  double r = fma(-dg, old, B.rhs[C][p.pi]);
  r = fma(-ax1, pl, r);
  r = fma(-ax3, pr, r);
  r = fma(-ay1, ps, r);
  r = fma(-ay3, pn, r);
  r = fma(-az1, pb, r);
  r = fma(-az3, pt, r);
  const double y0 = (double)__frcp_rn((float)dg);
  const double y1 = fma(y0, fma(-dg, y0, 1.0), y0);
  return fma(omega * y1, r, old);
}

template <int C>
__device__ __forceinline__ void tile_half64(const DevBlock& B, const Tile& t, double omega, double& lmax,
                                            int fast) {
  double* __restrict__ own = B.pc[C];
  const int n = B.d.NXH * t.nj * t.nk;
  Walk3 w;
  w.init(threadIdx.x, blockDim.x, B.d.NXH, t.nj);
  for (int q = threadIdx.x; q < n; q += blockDim.x, w.next()) {
    const Pos p = tile_pos<C>(B, t, w, true);
    if (!p.on) continue;
    double old;
    const double nv = fast ? sor64f_cell<C>(B, p, omega, old) : sor64_cell<C>(B, p, omega, old);
    own[p.pi] = nv;
    lmax = nmax(lmax, fabs(nv - old));
  }
}

// FP64 residual b/dt - A pc of one cell of colour C (FMA allowed: a stop test
// and correction source, not reference arithmetic)
template <int C>
__device__ __forceinline__ double resid64_cell(const DevBlock& B, const Pos& p) {
  const Dims& d = B.d;
  const double* __restrict__ own = B.pc[C];
  const double* __restrict__ o = B.pc[1 - C];
  const int64_t sy = d.NXH, sz = (int64_t)d.NXH * d.NY;
  const int i = p.ic, j = p.j, k = p.k;
  const double ax1 = B.Acx[i - 2], ax2 = B.Acx[i - 2 + d.nx], ax3 = B.Acx[i - 2 + 2 * d.nx];
  const double ay1 = B.Acy[j - 2], ay2 = B.Acy[j - 2 + d.ny], ay3 = B.Acy[j - 2 + 2 * d.ny];
  const double az1 = B.Acz[k - 2], az2 = B.Acz[k - 2 + d.nz], az3 = B.Acz[k - 2 + 2 * d.nz];
  double ax = (ax2 + ay2 + az2) * __ldcg(own + p.pi);
  ax = fma(ax1, __ldcg(o + p.row + ((p.i - 2) >> 1)), ax);
  ax = fma(ax3, __ldcg(o + p.row + (p.i >> 1)), ax);
  ax = fma(ay1, __ldcg(o + p.pi - sy), ax);
  ax = fma(ay3, __ldcg(o + p.pi + sy), ax);
  ax = fma(az1, __ldcg(o + p.pi - sz), ax);
  ax = fma(az3, __ldcg(o + p.pi + sz), ax);
  return B.rhs[C][p.pi] - ax;
}

// max |residual| of colour C over the tile, one cell per pass (the stop test
// of the FP64 residual-target solve)
template <int C>
__device__ __forceinline__ double tile_resid_max64(const DevBlock& B, const Tile& t) {
  double m = 0.0;
  const int n = B.d.NXH * t.nj * t.nk;
  Walk3 w;
  w.init(threadIdx.x, blockDim.x, B.d.NXH, t.nj);
  for (int q = threadIdx.x; q < n; q += blockDim.x, w.next()) {
    const Pos p = tile_pos<C>(B, t, w, true);
    if (p.on) m = nmax(m, fabs(resid64_cell<C>(B, p)));
  }
  return m;
}

// max over fluid cells of colour C of |b/dt - A pc| (grid-stride; measurement)
template <int C>
__device__ __forceinline__ double resid_max64(const DevBlock& B, int64_t total) {
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
    m = nmax(m, fabs(B.rhs[C][pi] - ax));
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
  int rev;        // 1: black half-sweep first (the adjoint solve's order)
  int fast;       // 1: division-free update (not the reference's arithmetic)
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

// The three stop-test slots rotate: slot c % 3 collects check c; after the
// grid barrier of check c every CTA has read check c-1, so slot (c+2) % 3 is
// cleared for check c+2 by CTA 0.
__device__ __forceinline__ double take_slot(BlockStats* st, int c, int cta) {
  const double v = *((volatile double*)&st->slot[c % 3]);
  if (cta == 0 && threadIdx.x == 0) st->slot[(c + 2) % 3] = 0.0;
  return v;
}

// REDBLACKSOR_linear (src/PcorVcor.F90:288-377) as one cooperative launch.
// nIterPcor continues from stats->niter (the fine blocks accumulate it over
// two solves per step, :78, :98, :116) and the stop test runs whenever the
// accumulated count is a multiple of 5, exactly as the reference does.  In
// residual-target mode (not a reference routine) the FP64 residual is checked
// first after 5 pairs, then after as many pairs as the reduction per pair
// measured between the last two checks needs to reach the target (15% and one
// pair of margin, 5 to 64): each check is a full FP64 residual pass.
// `cta` is this CTA's index among the block's CTAs (a batched launch runs
// several blocks' solves side by side, each with its own barrier and tiles)
__device__ __forceinline__ void sor64_body(const DevBlock& B, const SorArgs& a, const GridBar& gb,
                                           const TileMap& tm, int cta) {
  __shared__ double sh[32];
  const Tile t = my_tile(B.d, tm, cta);
  BlockStats* st = B.stats;
  const int64_t it0 = st->niter;
  // every CTA has read niter before CTA 0 may rewrite it at the end
  if (!grid_sync(gb)) return;
  int64_t it = it0;
  int r5 = (int)(it0 % 5);  // it mod 5, kept incrementally
  double derr4 = 11111.0;
  int check = 0;
  unsigned ph = 0;
  bool ok = true;
  const bool target_mode = a.res_tol > 0.0;
  int64_t next_check = it0 + 5, it_prev = it0;  // residual-target mode
  double res_prev = -1.0;
  for (;;) {
    ++it;
    if (++r5 == 5) r5 = 0;
    double lmax = 0.0;
    if (!tile_wait(tm, gb, t, ph)) { ok = false; break; }
    if (a.rev) tile_half64<0>(B, t, a.omega, lmax, a.fast);
    else tile_half64<1>(B, t, a.omega, lmax, a.fast);
    tile_publish(tm, t, ++ph);
    if (!tile_wait(tm, gb, t, ph)) { ok = false; break; }
    if (a.rev) tile_half64<1>(B, t, a.omega, lmax, a.fast);
    else tile_half64<0>(B, t, a.omega, lmax, a.fast);
    tile_publish(tm, t, ++ph);
    if (target_mode ? it >= next_check : r5 == 0) {
      if (target_mode) {
        // residual-target mode: the residual needs the neighbours' sweep pair
        if (!tile_wait(tm, gb, t, ph)) { ok = false; break; }
        lmax = nmax(tile_resid_max64<1>(B, t), tile_resid_max64<0>(B, t)) * a.dt;
        tile_publish(tm, t, ++ph);
      }
      const double m = block_max(lmax, sh);
      if (threadIdx.x == 0) atomic_max_nonneg(&st->slot[check % 3], m);
      if (!grid_sync(gb)) { ok = false; break; }
      derr4 = take_slot(st, check, cta);
      ++check;
      if (target_mode) {
        int64_t gap = 5;
        if (res_prev > 0.0 && derr4 < res_prev && derr4 > a.res_tol) {
          const double per_pair = log(derr4 / res_prev) / (double)(it - it_prev);  // < 0
          const double need = log(a.res_tol / derr4) / per_pair;                   // > 0
          gap = (int64_t)fmin(64.0, fmax(5.0, ceil(need * 1.15) + 1.0));
        }
        res_prev = derr4;
        it_prev = it;
        next_check = it + gap;
      }
    }
    if (a.res_tol > 0.0 ? (derr4 <= a.res_tol) : (derr4 < a.epsi)) break;
    if (it > a.itmax || non_finite(derr4)) break;
  }
  if (cta == 0 && threadIdx.x == 0) {
    log_solve(a.log, it - it0, 0, B.cnt[C_FLUID], 0);
    st->niter = it;
    st->derr2 = derr4;
    if (ok && non_finite(derr4)) set_err(B.err, BCFD_E_NONFINITE);
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
// largest relaxation factor of the FP32 correction sweeps
constexpr double kMixedOmegaMax = 1.99;

// the default relaxation factor of the FP32 correction sweeps: the classical
// optimum 2 / (1 + sqrt(1 - rho^2)) of red-black SOR for the 7-point Laplacian
// on an nx x ny x nz box with Dirichlet boundaries, rho = (cos(pi/nx) +
// cos(pi/ny) + cos(pi/nz)) / 3 the Jacobi spectral radius (1 - rho formed
// from sin^2 terms, free of cancellation)
double mixed_omega_default(const Dims& d) {
  const double pi = 3.14159265358979323846;
  auto s2 = [&](int n) {
    const double x = std::sin(pi / (2.0 * n));
    return 2.0 * x * x;  // 1 - cos(pi / n)
  };
  const double e = (s2(d.nx) + s2(d.ny) + s2(d.nz)) / 3.0;  // 1 - rho
  return 2.0 / (1.0 + std::sqrt(e * (2.0 - e)));
}

struct DcArgs {
  int64_t max_outer;
  int inner;          // FP32 sweep pairs of the first correction (and the most of any)
  float omega;        // relaxation of the FP32 sweeps
  double dt, inv_dt, div_tol;
  int64_t* log;
};

// Sweep pairs of the next correction.  The first takes a.inner; each later
// one takes what the residual reduction per pair measured over the previous
// correction needs to reach the target (15% and two pairs of margin), at
// least kMinInner and at most a.inner, so the last correction of a solve does
// not run a full a.inner pairs past the target.  Every CTA computes it from
// the same two residuals, so all agree.
constexpr int kMinInner = 16;
__device__ __forceinline__ int next_inner(const DcArgs& a, int outer, double res, double res_prev, int prev) {
  const double target = a.div_tol * a.inv_dt;
  if (outer == 0 || !(res < res_prev) || !(res > target) || !(target > 0.0)) return a.inner;
  const double per_pair = log(res / res_prev) / (double)prev;  // < 0
  const double need = log(target / res) / per_pair;             // > 0
  if (!(need < (double)a.inner)) return a.inner;
  return min(a.inner, max(kMinInner, (int)ceil(need * 1.15) + 2));
}

// one FP32 half-sweep of colour C over the tile.  Each thread updates a run
// of four consecutive packed cells h0..h0+3 of one row (h0 a multiple of 4;
// rows are 16-byte aligned): the run shares one x-parity `par` (its cells sit
// at i = 2h+1+par), so its x-neighbours are the other colour's h-1+par and
// h+par, i.e. the centre float4 plus one scalar; y/z neighbours, own values
// and right-hand side are float4 loads, the masks one 4-byte load, and the
// run is written back with one float4 store (cells that are not updated keep
// their value; no other CTA writes them in this phase).
template <int C>
__device__ __forceinline__ void tile_half32(const DevBlock& B, const Tile& t, float omega) {
  const Dims& d = B.d;
  const float* __restrict__ o = B.pcf[1 - C];
  float* __restrict__ own = B.pcf[C];
  const float* __restrict__ rhs = B.rhsf[C];
  const uint8_t* __restrict__ upd = B.upd[C];
  const int nq = d.NXH >> 2;
  const int64_t sy = d.NXH, sz = (int64_t)d.NXH * d.NY;
  const int n = nq * t.nj * t.nk;
  Walk3 w;
  w.init(threadIdx.x, blockDim.x, nq, t.nj);
  for (int q = threadIdx.x; q < n; q += blockDim.x, w.next()) {
    const int h0 = 4 * w.a, j = t.j0 + w.b, k = t.k0 + w.c;
    const int64_t row = (int64_t)d.NXH * (j - 1) + sz * (k - 1);
    const int64_t pi = row + h0;
    // every load of the run is issued before any result is needed (no early
    // exit on the mask: all addresses of a tile row are in range)
    const uchar4 m = *reinterpret_cast<const uchar4*>(upd + pi);
    const int par = ((1 + j + k) & 1) != C;
    const float4 oc = *reinterpret_cast<const float4*>(o + pi);
    const float4 os = *reinterpret_cast<const float4*>(o + pi - sy);
    const float4 on = *reinterpret_cast<const float4*>(o + pi + sy);
    const float4 ob = *reinterpret_cast<const float4*>(o + pi - sz);
    const float4 ot = *reinterpret_cast<const float4*>(o + pi + sz);
    const float4 r4 = *reinterpret_cast<const float4*>(rhs + pi);
    const float4 e4 = *reinterpret_cast<const float4*>(own + pi);
    // the one x-neighbour outside the centre float4 (in range: row +- 1)
    const float ox = par ? o[pi + 4] : o[pi - 1];
    const float4 cy = B.ayr[j - 2], cz = B.azr[k - 2];
    const float ay1 = cy.x, ay2 = cy.y, ay3 = cy.z;
    const float az1 = cz.x, az2 = cz.y, az3 = cz.z;
    // the run's x coefficients: three float4 loads of a small table (the
    // same FP32 values as Acxf at the run's cells)
    const float4* __restrict__ ar = B.axr + (int64_t)(3 * par) * nq + w.a;
    const float4 c1 = ar[0], c2 = ar[nq], c3 = ar[2 * nq];
    const float axv1[4] = {c1.x, c1.y, c1.z, c1.w}, axv2[4] = {c2.x, c2.y, c2.z, c2.w},
                axv3[4] = {c3.x, c3.y, c3.z, c3.w};
    const float oxs[6] = {par ? oc.x : ox, oc.x, oc.y, oc.z, oc.w, par ? ox : oc.w};
    const float sv[4] = {os.x, os.y, os.z, os.w}, nv4[4] = {on.x, on.y, on.z, on.w};
    const float bv[4] = {ob.x, ob.y, ob.z, ob.w}, tv[4] = {ot.x, ot.y, ot.z, ot.w};
    const float rv[4] = {r4.x, r4.y, r4.z, r4.w};
    float ev[4] = {e4.x, e4.y, e4.z, e4.w};
    const unsigned char mv[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      // cell i = 2(h0+u)+1+par; left neighbour h0+u-1+par, right h0+u+par
      // constant indices after unrolling (a runtime index would put oxs in
      // local memory)
      const float left = par ? oxs[u + 1] : oxs[u];
      const float right = par ? oxs[u + 2] : oxs[u + 1];
      const float ax1 = axv1[u], ax2 = axv2[u], ax3 = axv3[u];
      float s = rv[u];
      s = __fmaf_rn(-ax1, left, s);
      s = __fmaf_rn(-ax3, right, s);
      s = __fmaf_rn(-ay1, sv[u], s);
      s = __fmaf_rn(-ay3, nv4[u], s);
      s = __fmaf_rn(-az1, bv[u], s);
      s = __fmaf_rn(-az3, tv[u], s);
      const float nvv = __fmaf_rn(omega, __fdividef(s, ax2 + ay2 + az2) - ev[u], ev[u]);
      ev[u] = mv[u] ? nvv : ev[u];
    }
    *reinterpret_cast<float4*>(own + pi) = make_float4(ev[0], ev[1], ev[2], ev[3]);
  }
}

// FP64 residual r = b * (1/dt) - A pc of colour C over the tile, two
// consecutive packed cells per thread (double2 loads; rows are 16-byte
// aligned), written to rhsf as the FP32 right-hand side of the correction (0
// at cells that are not updated).  The pair shares one x-parity `par`: its
// x-neighbours are the other colour's centre double2 plus one scalar.
// Returns the local max |r|.  (b * (1/dt) differs from b / dt by at most half
// an ulp, far below any residual target.)
template <int C>
__device__ __forceinline__ double tile_residual64v(const DevBlock& B, const Tile& t, double inv_dt) {
  const Dims& d = B.d;
  const double* __restrict__ x = B.pc[C];
  const double* __restrict__ o = B.pc[1 - C];
  const double* __restrict__ bb = B.bpk[C];
  const uint8_t* __restrict__ upd = B.upd[C];
  float* __restrict__ rf = B.rhsf[C];
  const int nh = d.NXH >> 1;
  const int64_t sy = d.NXH, sz = (int64_t)d.NXH * d.NY;
  const int n = nh * t.nj * t.nk;
  double m = 0.0;
  Walk3 w;
  w.init(threadIdx.x, blockDim.x, nh, t.nj);
  for (int q = threadIdx.x; q < n; q += blockDim.x, w.next()) {
    const int h0 = 2 * w.a, j = t.j0 + w.b, k = t.k0 + w.c;
    const int64_t pi = (int64_t)d.NXH * (j - 1) + sz * (k - 1) + h0;
    const uchar2 mk = *reinterpret_cast<const uchar2*>(upd + pi);
    const int par = ((1 + j + k) & 1) != C;
    const double2 oc = *reinterpret_cast<const double2*>(o + pi);
    const double2 os = *reinterpret_cast<const double2*>(o + pi - sy);
    const double2 on = *reinterpret_cast<const double2*>(o + pi + sy);
    const double2 ob = *reinterpret_cast<const double2*>(o + pi - sz);
    const double2 ot = *reinterpret_cast<const double2*>(o + pi + sz);
    const double2 x2 = *reinterpret_cast<const double2*>(x + pi);
    const double2 b2 = *reinterpret_cast<const double2*>(bb + pi);
    const double ox = par ? o[pi + 2] : o[pi - 1];
    const double ay1 = B.Acy[j - 2], ay2 = B.Acy[j - 2 + d.ny], ay3 = B.Acy[j - 2 + 2 * d.ny];
    const double az1 = B.Acz[k - 2], az2 = B.Acz[k - 2 + d.nz], az3 = B.Acz[k - 2 + 2 * d.nz];
    double r[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const double left = u == 0 ? (par ? oc.x : ox) : (par ? oc.y : oc.x);
      const double right = u == 0 ? (par ? oc.y : oc.x) : (par ? ox : oc.y);
      const int ic = min(max(2 * (h0 + u) + 1 + par, 2), d.nx + 1);
      const double ax1 = B.Acx[ic - 2], ax2 = B.Acx[ic - 2 + d.nx], ax3 = B.Acx[ic - 2 + 2 * d.nx];
      double ax = (ax2 + ay2 + az2) * (u == 0 ? x2.x : x2.y);
      ax = fma(ax1, left, ax);
      ax = fma(ax3, right, ax);
      ax = fma(ay1, u == 0 ? os.x : os.y, ax);
      ax = fma(ay3, u == 0 ? on.x : on.y, ax);
      ax = fma(az1, u == 0 ? ob.x : ob.y, ax);
      ax = fma(az3, u == 0 ? ot.x : ot.y, ax);
      r[u] = (u == 0 ? b2.x : b2.y) * inv_dt - ax;
    }
    if (mk.x) m = nmax(m, fabs(r[0]));
    if (mk.y) m = nmax(m, fabs(r[1]));
    *reinterpret_cast<float2*>(rf + pi) = make_float2(mk.x ? (float)r[0] : 0.0f, mk.y ? (float)r[1] : 0.0f);
  }
  return m;
}

// x += e in FP64 over the tile's updated cells of colour C, e back to 0; runs
// of four packed cells (float4 / 2 x double2)
template <int C>
__device__ __forceinline__ void tile_apply4(const DevBlock& B, const Tile& t) {
  const Dims& d = B.d;
  double* __restrict__ x = B.pc[C];
  float* __restrict__ e = B.pcf[C];
  const uint8_t* __restrict__ upd = B.upd[C];
  const int nq = d.NXH >> 2;
  const int64_t sz = (int64_t)d.NXH * d.NY;
  const int n = nq * t.nj * t.nk;
  Walk3 w;
  w.init(threadIdx.x, blockDim.x, nq, t.nj);
  for (int q = threadIdx.x; q < n; q += blockDim.x, w.next()) {
    const int64_t pi = (int64_t)d.NXH * (t.j0 + w.b - 1) + sz * (t.k0 + w.c - 1) + 4 * w.a;
    const uchar4 mk = *reinterpret_cast<const uchar4*>(upd + pi);
    const float4 e4 = *reinterpret_cast<const float4*>(e + pi);
    double2 a = *reinterpret_cast<const double2*>(x + pi);
    double2 b = *reinterpret_cast<const double2*>(x + pi + 2);
    if (mk.x) a.x = a.x + (double)e4.x;
    if (mk.y) a.y = a.y + (double)e4.y;
    if (mk.z) b.x = b.x + (double)e4.z;
    if (mk.w) b.y = b.y + (double)e4.w;
    *reinterpret_cast<double2*>(x + pi) = a;
    *reinterpret_cast<double2*>(x + pi + 2) = b;
    *reinterpret_cast<float4*>(e + pi) = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

__device__ __forceinline__ void sor_dc_body(const DevBlock& B, const DcArgs& a, const GridBar& gb,
                                            const TileMap& tm, int cta) {
  __shared__ double sh[32];
  const Tile t = my_tile(B.d, tm, cta);
  BlockStats* st = B.stats;
  int64_t sweeps = 0;
  double res = 0.0, res_prev = 0.0;
  int inner = a.inner;
  unsigned ph = 0;
  int outer = 0;
  for (;; ++outer) {
    if (!tile_wait(tm, gb, t, ph)) return;
    double m = nmax(tile_residual64v<1>(B, t, a.inv_dt), tile_residual64v<0>(B, t, a.inv_dt));
    tile_publish(tm, t, ++ph);
    m = block_max(m, sh);
    if (threadIdx.x == 0) atomic_max_nonneg(&st->slot[outer % 3], m);
    if (!grid_sync(gb)) return;
    res = take_slot(st, outer, cta);
    if (a.dt * res <= a.div_tol || outer >= a.max_outer || non_finite(res)) break;
    inner = next_inner(a, outer, res, res_prev, inner);
    res_prev = res;
    for (int it = 0; it < inner; ++it) {
      if (!tile_wait(tm, gb, t, ph)) return;
      tile_half32<1>(B, t, a.omega);
      tile_publish(tm, t, ++ph);
      if (!tile_wait(tm, gb, t, ph)) return;
      tile_half32<0>(B, t, a.omega);
      tile_publish(tm, t, ++ph);
    }
    sweeps += inner;
    if (!tile_wait(tm, gb, t, ph)) return;
    tile_apply4<1>(B, t);
    tile_apply4<0>(B, t);
    tile_publish(tm, t, ++ph);
  }
  if (cta == 0 && threadIdx.x == 0) {
    log_solve(a.log, sweeps, outer + 1, B.cnt[C_FLUID], 1);
    st->niter = st->niter + sweeps;
    st->derr2 = a.dt * res;
    st->pad[1] = a.dt * res;  // the residual this solve leaves behind
    if (non_finite(res)) set_err(B.err, BCFD_E_NONFINITE);
  }
}

__global__ void __launch_bounds__(kSolveMaxThreads, 2) k_sor64(DevBlock B, SorArgs a, GridBar gb, TileMap tm) {
  sor64_body(B, a, gb, tm, (int)blockIdx.x);
}

// MINB CTAs of 256 threads per SM: 3 (80 registers, no spill) or 4 (64
// registers, a few spilled: more warps, so more loads in flight on large blocks)
template <int MINB>
__global__ void __launch_bounds__(kDcThreads, MINB) k_sor_dc(DevBlock B, DcArgs a, GridBar gb, TileMap tm) {
  sor_dc_body(B, a, gb, tm, (int)blockIdx.x);
}

// ---------------------------------------------------------------------------
// Temporal-blocked FP32 sweeps (variant 4): one grid barrier per sweep pair
// instead of two.  Each CTA copies the rows of its tile plus two halo rows on
// each side in j and k (both colours of the correction e, the right-hand side
// and the masks) into shared memory, runs the red half-sweep over the tile
// grown by one row and the black half-sweep over the tile, and writes the
// tile's rows to the other of two e buffers.  The halo's red values are
// recomputed from the inputs the owning CTA uses, with the same operations,
// so every cell gets exactly the values of the two-barrier sweep (bitwise);
// the second buffer keeps a round's reads of the neighbours' rows from racing
// with their writes.  Small blocks only: the halo'd tile has to fit in
// shared memory (18 bytes per packed cell position).
// ---------------------------------------------------------------------------
constexpr int kTbThreads = 512;
constexpr int kTbPad = 4;  // floats before and after each shared row (zero)

struct TbSmem {
  int rj, rk, pitch;  // rows along j and k incl. halo, row pitch in floats
  float* e;           // [2 colours][rk][rj][pitch]
  float* r;
  uint8_t* m;
  __device__ __forceinline__ int rows() const { return rj * rk; }
  __device__ __forceinline__ int off(int c, int jj, int kk) const {
    return (c * rows() + kk * rj + jj) * pitch + kTbPad;
  }
};

__device__ __forceinline__ TbSmem tb_smem(float* base, const TileMap& tm, const Dims& d) {
  TbSmem s;
  s.rj = tm.tj + 4;
  s.rk = tm.tk + 4;
  s.pitch = d.NXH + 2 * kTbPad;
  const int n = 2 * s.rj * s.rk * s.pitch;
  s.e = base;
  s.r = base + n;
  s.m = reinterpret_cast<uint8_t*>(base + 2 * n);
  return s;
}

// asynchronous global -> shared copies (cp.async): a thread issues all its
// copies before waiting once, so the few CTAs of this variant keep many
// loads in flight
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// copy the halo'd rows of e (both colours; and of r and the masks when
// `inputs`) from global memory; rows outside the arrays read as zero.  The
// caller synchronises the CTA afterwards.
__device__ __forceinline__ void tb_load(const DevBlock& B, const Tile& t, const TbSmem& s, const float* const E[2],
                                        bool inputs) {
  const Dims& d = B.d;
  const int nq = d.NXH >> 2;
  const int64_t sz = (int64_t)d.NXH * d.NY;
  const int n = s.rows() * nq;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int a = q % nq, rr = q / nq;
    const int jj = rr % s.rj, kk = rr / s.rj;
    const int j = t.j0 - 2 + jj, k = t.k0 - 2 + kk;
    const bool in = j >= 1 && j <= d.NY && k >= 1 && k <= d.NZ;
    const int64_t pi = (int64_t)d.NXH * (j - 1) + sz * (k - 1) + 4 * a;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const int o = s.off(c, jj, kk) + 4 * a;
      if (in) {
        cp_async16(s.e + o, E[c] + pi);
        if (inputs) {
          cp_async16(s.r + o, B.rhsf[c] + pi);
          cp_async4(s.m + o, B.upd[c] + pi);
        }
      } else {
        *reinterpret_cast<float4*>(s.e + o) = make_float4(0.f, 0.f, 0.f, 0.f);
        if (inputs) {
          *reinterpret_cast<float4*>(s.r + o) = make_float4(0.f, 0.f, 0.f, 0.f);
          *reinterpret_cast<uchar4*>(s.m + o) = make_uchar4(0, 0, 0, 0);
        }
      }
    }
  }
  cp_async_wait_all();
}

// zero the row pads once (the x-neighbour of a row's first/last run reads a
// pad; those cells are never updated)
__device__ __forceinline__ void tb_zero_pads(const TbSmem& s) {
  const int n = 2 * s.rows();
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int c = q / s.rows(), rr = q % s.rows();
    const int o = s.off(c, rr % s.rj, rr / s.rj);
    for (int u = 1; u <= kTbPad; ++u) {
      s.e[o - u] = 0.f;
      s.e[o + (s.pitch - 2 * kTbPad) + u - 1] = 0.f;
    }
  }
}

// one half-sweep of colour C over the rows lo .. rj-1-lo (j) and lo .. rk-1-lo
// (k) of the shared tile: the arithmetic of tile_half32
template <int C>
__device__ __forceinline__ void tb_half(const DevBlock& B, const Tile& t, const TbSmem& s, int lo, float omega) {
  const Dims& d = B.d;
  const int nq = d.NXH >> 2;
  const int wj = s.rj - 2 * lo, wk = s.rk - 2 * lo;
  const int n = wj * wk * nq;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int a = q % nq, rr = q / nq;
    const int jj = lo + rr % wj, kk = lo + rr / wj;
    const int j = t.j0 - 2 + jj, k = t.k0 - 2 + kk;
    if (j < 2 || j > d.ny + 1 || k < 2 || k > d.nz + 1) continue;  // ghost rows hold no updated cell
    const int oo = s.off(1 - C, jj, kk) + 4 * a, ow = s.off(C, jj, kk) + 4 * a;
    const int sy = s.pitch, sz = s.rj * s.pitch;
    const uchar4 m = *reinterpret_cast<const uchar4*>(s.m + ow);
    const int par = ((1 + j + k) & 1) != C;
    const float4 oc = *reinterpret_cast<const float4*>(s.e + oo);
    const float4 os = *reinterpret_cast<const float4*>(s.e + oo - sy);
    const float4 on = *reinterpret_cast<const float4*>(s.e + oo + sy);
    const float4 ob = *reinterpret_cast<const float4*>(s.e + oo - sz);
    const float4 ot = *reinterpret_cast<const float4*>(s.e + oo + sz);
    const float4 r4 = *reinterpret_cast<const float4*>(s.r + ow);
    const float4 e4 = *reinterpret_cast<const float4*>(s.e + ow);
    const float ox = par ? s.e[oo + 4] : s.e[oo - 1];
    const float4 cy = B.ayr[j - 2], cz = B.azr[k - 2];
    const float ay1 = cy.x, ay2 = cy.y, ay3 = cy.z;
    const float az1 = cz.x, az2 = cz.y, az3 = cz.z;
    const float4* __restrict__ ar = B.axr + (int64_t)(3 * par) * nq + a;
    const float4 c1 = ar[0], c2 = ar[nq], c3 = ar[2 * nq];
    const float axv1[4] = {c1.x, c1.y, c1.z, c1.w}, axv2[4] = {c2.x, c2.y, c2.z, c2.w},
                axv3[4] = {c3.x, c3.y, c3.z, c3.w};
    const float oxs[6] = {par ? oc.x : ox, oc.x, oc.y, oc.z, oc.w, par ? ox : oc.w};
    const float sv[4] = {os.x, os.y, os.z, os.w}, nv4[4] = {on.x, on.y, on.z, on.w};
    const float bv[4] = {ob.x, ob.y, ob.z, ob.w}, tv[4] = {ot.x, ot.y, ot.z, ot.w};
    const float rv[4] = {r4.x, r4.y, r4.z, r4.w};
    float ev[4] = {e4.x, e4.y, e4.z, e4.w};
    const unsigned char mv[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float left = par ? oxs[u + 1] : oxs[u];
      const float right = par ? oxs[u + 2] : oxs[u + 1];
      const float ax1 = axv1[u], ax2 = axv2[u], ax3 = axv3[u];
      float sm = rv[u];
      sm = __fmaf_rn(-ax1, left, sm);
      sm = __fmaf_rn(-ax3, right, sm);
      sm = __fmaf_rn(-ay1, sv[u], sm);
      sm = __fmaf_rn(-ay3, nv4[u], sm);
      sm = __fmaf_rn(-az1, bv[u], sm);
      sm = __fmaf_rn(-az3, tv[u], sm);
      const float nvv = __fmaf_rn(omega, __fdividef(sm, ax2 + ay2 + az2) - ev[u], ev[u]);
      ev[u] = mv[u] ? nvv : ev[u];
    }
    *reinterpret_cast<float4*>(s.e + ow) = make_float4(ev[0], ev[1], ev[2], ev[3]);
  }
}

// the tile's own rows (both colours) from shared memory to E
__device__ __forceinline__ void tb_store(const DevBlock& B, const Tile& t, const TbSmem& s, float* const E[2]) {
  const Dims& d = B.d;
  const int nq = d.NXH >> 2;
  const int64_t sz = (int64_t)d.NXH * d.NY;
  const int n = t.nj * t.nk * nq;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int a = q % nq, rr = q / nq;
    const int jj = 2 + rr % t.nj, kk = 2 + rr / t.nj;
    const int j = t.j0 - 2 + jj, k = t.k0 - 2 + kk;
    const int64_t pi = (int64_t)d.NXH * (j - 1) + sz * (k - 1) + 4 * a;
#pragma unroll
    for (int c = 0; c < 2; ++c)
      *reinterpret_cast<float4*>(E[c] + pi) = *reinterpret_cast<const float4*>(s.e + s.off(c, jj, kk) + 4 * a);
  }
}

// the tile's rows of E copied to the canonical buffer (an odd sweep count
// leaves the correction in the second buffer)
__device__ __forceinline__ void tb_copy_back(const DevBlock& B, const Tile& t, const float* const E2[2]) {
  const Dims& d = B.d;
  const int nq = d.NXH >> 2;
  const int64_t sz = (int64_t)d.NXH * d.NY;
  const int n = t.nj * t.nk * nq;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int a = q % nq, rr = q / nq;
    const int64_t pi = (int64_t)d.NXH * (t.j0 + rr % t.nj - 1) + sz * (t.k0 + rr / t.nj - 1) + 4 * a;
#pragma unroll
    for (int c = 0; c < 2; ++c)
      *reinterpret_cast<float4*>(B.pcf[c] + pi) = *reinterpret_cast<const float4*>(E2[c] + pi);
  }
}

__global__ void __launch_bounds__(kTbThreads, 1) k_sor_tb(DevBlock B, DcArgs a, GridBar gb, TileMap tm, float* e2) {
  extern __shared__ float4 tb_raw[];
  __shared__ double sh[32];
  const int cta = (int)blockIdx.x;
  const Tile t = my_tile(B.d, tm, cta);
  const TbSmem s = tb_smem(reinterpret_cast<float*>(tb_raw), tm, B.d);
  const int64_t np = B.d.npacked();
  float* const E0[2] = {B.pcf[0], B.pcf[1]};
  float* const E1[2] = {e2, e2 + np};
  BlockStats* st = B.stats;
  tb_zero_pads(s);
  int64_t sweeps = 0;
  double res = 0.0, res_prev = 0.0;
  int inner = a.inner;
  int outer = 0;
  for (;; ++outer) {
    double m = nmax(tile_residual64v<1>(B, t, a.inv_dt), tile_residual64v<0>(B, t, a.inv_dt));
    m = block_max(m, sh);
    if (threadIdx.x == 0) atomic_max_nonneg(&st->slot[outer % 3], m);
    if (!grid_sync(gb)) return;
    res = take_slot(st, outer, cta);
    if (a.dt * res <= a.div_tol || outer >= a.max_outer || non_finite(res)) break;
    inner = next_inner(a, outer, res, res_prev, inner);
    res_prev = res;
    int cur = 0;
    for (int it = 0; it < inner; ++it) {
      const float* const* src = cur ? E1 : E0;
      const float* srcc[2] = {src[0], src[1]};
      tb_load(B, t, s, srcc, it == 0);
      __syncthreads();
      tb_half<1>(B, t, s, 1, a.omega);
      __syncthreads();
      tb_half<0>(B, t, s, 2, a.omega);
      __syncthreads();
      tb_store(B, t, s, cur ? E0 : E1);
      cur ^= 1;
      if (!grid_sync(gb)) return;
    }
    sweeps += inner;
    if (cur) {
      const float* e1c[2] = {E1[0], E1[1]};
      tb_copy_back(B, t, e1c);
      __syncthreads();
    }
    tile_apply4<1>(B, t);
    tile_apply4<0>(B, t);
    if (!grid_sync(gb)) return;
  }
  if (cta == 0 && threadIdx.x == 0) {
    log_solve(a.log, sweeps, outer + 1, B.cnt[C_FLUID], 1);
    st->niter = st->niter + sweeps;
    st->derr2 = a.dt * res;
    st->pad[1] = a.dt * res;
    if (non_finite(res)) set_err(B.err, BCFD_E_NONFINITE);
  }
}

// ---------------------------------------------------------------------------
// Z-marching two-pair FP32 sweeps (variant 5): TMA-fed temporal blocking for
// blocks far larger than L2.  One pass applies four half-sweeps (two sweep
// pairs) while reading the correction from HBM once: each CTA owns a tile of
// rows j0..j0+nj-1 (every h of both colours) and planes k0..k0+nk-1, and
// marches through its planes with the four half-sweeps skewed by one plane
// each (level L = 1..4 at step k works on plane k-L+1; levels 1 and 3 red,
// 2 and 4 black).  The planes in use (k-4 .. k+1) and the one in flight
// (k+2) sit in a ring of seven shared-memory slots, each the plane's rows
// j0-4 .. j0+nj+3 of both colours, filled by two cp.async.bulk.tensor loads
// (TMA) completing on the slot's mbarrier; the tile's rows are recomputed up
// to four rows (and planes) beyond the tile with exactly the operations of
// the owning CTA, so every cell receives the values of four plain
// half-sweeps, bit for bit.  A pass reads one buffer and writes the tile's
// rows of the other (ping-pong), so no CTA's writes race with a neighbour's
// halo reads; passes are separated by the grid barrier.  The right-hand side
// and the masks are pulled into L2 two steps ahead (bulk prefetches) and
// into registers at the start of each step, all four levels' at once, so
// their latencies overlap.  HBM traffic per cell and pass: e 4 B read + 4 B written, rhs 4 B
// and mask 1 B read -- 13 B for two sweep pairs, against 34 B for two plain
// pairs.
// ---------------------------------------------------------------------------
constexpr int kZmThreads = 384;
constexpr int kZmSlots = 7;
constexpr int kZmHalo = 4;
constexpr int kZmGuard = 128;  // bytes before and after the ring

struct ZmArgs {
  int tj, ntj, tk, nzs;  // rows per tile along j, tiles along j; planes per tile along k, tiles along k
  int rows;              // rows of a staged plane (tj + 2 * kZmHalo), the TMA box height
  int slot_floats;       // floats of one colour of one staged plane (a multiple of 32)
  float* e2;             // the second correction buffer: colour c at e2 + c * npacked
};

// the tensor maps of the four correction arrays: [buffer * 2 + colour]
struct ZmMaps {
  CUtensorMap m[4];
};

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait for a slot's load; false once the limit passed
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, parity))
    if (globaltimer_ns() - t0 > limit_ns) return false;
  return true;
}
// rows [y, y + box) of plane z of a packed colour array into shared memory
__device__ __forceinline__ void tma_load_plane(float* dst, const CUtensorMap* map, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

struct ZmRing {
  float* base;      // slot 0, colour 0
  int slot_floats;  // per colour
  int jrow0;        // j of a slot's row 0
  unsigned pbits;   // expected mbarrier parity per slot
  uint64_t* bars;
  __device__ __forceinline__ static int slot(int p) { return (p + 4 * kZmSlots) % kZmSlots; }
  __device__ __forceinline__ float* at(int p, int c) const {
    return base + (size_t)(2 * slot(p) + c) * slot_floats;
  }
};

// the rows and runs of one level at one step (clamped to the interior)
struct ZmSpan {
  int p, ja, n;  // plane, first row, runs (rows x NXH/4); n = 0: nothing to do
};

__device__ __forceinline__ ZmSpan zm_span(const Dims& d, int p, int ja, int jb, bool on) {
  ZmSpan z;
  z.p = p;
  z.ja = max(ja, 2);
  jb = min(jb, d.ny + 1);
  z.n = (on && p >= 2 && p <= d.nz + 1 && z.ja <= jb) ? (jb - z.ja + 1) * (d.NXH >> 2) : 0;
  return z;
}

// the right-hand side and masks of this thread's runs of one level (at most
// kZmRuns runs per thread: the tiling guarantees it), loaded into registers
// before the step's barrier waits so that all their latencies overlap
constexpr int kZmRuns = 2;
template <int C>
__device__ __forceinline__ void zm_fetch(const DevBlock& B, const ZmSpan& z, float4 (&r)[kZmRuns],
                                         uchar4 (&m)[kZmRuns]) {
  const Dims& d = B.d;
  const int nq = d.NXH >> 2;
  const int64_t gz = (int64_t)d.NXH * d.NY * (z.p - 1);
#pragma unroll
  for (int u = 0; u < kZmRuns; ++u) {
    const int q = threadIdx.x + u * blockDim.x;
    if (q < z.n) {
      const int a = q % nq, j = z.ja + q / nq;
      const int64_t pi = gz + (int64_t)d.NXH * (j - 1) + 4 * a;
      r[u] = __ldg(reinterpret_cast<const float4*>(B.rhsf[C] + pi));
      m[u] = *reinterpret_cast<const uchar4*>(B.upd[C] + pi);
    }
  }
}

// one half-sweep of colour C on the level's rows of plane z.p: the arithmetic
// of tile_half32 with the correction read from the ring and the right-hand
// side and masks from registers
template <int C>
__device__ __forceinline__ void zm_level(const DevBlock& B, const ZmRing& R, const ZmSpan& z,
                                         const float4 (&rr)[kZmRuns], const uchar4 (&mm)[kZmRuns], float omega) {
  const Dims& d = B.d;
  const int nq = d.NXH >> 2;
  const int p = z.p;
  const float* __restrict__ om = R.at(p - 1, 1 - C);
  const float* __restrict__ oc = R.at(p, 1 - C);
  const float* __restrict__ op = R.at(p + 1, 1 - C);
  float* __restrict__ own = R.at(p, C);
  const int sy = d.NXH;
#pragma unroll
  for (int uu = 0; uu < kZmRuns; ++uu) {
    const int q = threadIdx.x + uu * blockDim.x;
    if (q >= z.n) break;
    const int a = q % nq, j = z.ja + q / nq;
    const int so = (j - R.jrow0) * sy + 4 * a;
    const uchar4 m = mm[uu];
    const float4 r4 = rr[uu];
    const int par = ((1 + j + p) & 1) != C;
    const float4 c0 = *reinterpret_cast<const float4*>(oc + so);
    const float4 os = *reinterpret_cast<const float4*>(oc + so - sy);
    const float4 on = *reinterpret_cast<const float4*>(oc + so + sy);
    const float4 ob = *reinterpret_cast<const float4*>(om + so);
    const float4 ot = *reinterpret_cast<const float4*>(op + so);
    const float4 e4 = *reinterpret_cast<const float4*>(own + so);
    const float ox = par ? oc[so + 4] : oc[so - 1];
    const float4 cy = B.ayr[j - 2], cz = B.azr[p - 2];
    const float ay1 = cy.x, ay2 = cy.y, ay3 = cy.z;
    const float az1 = cz.x, az2 = cz.y, az3 = cz.z;
    const float4* __restrict__ ar = B.axr + (int64_t)(3 * par) * nq + a;
    const float4 c1 = ar[0], c2 = ar[nq], c3 = ar[2 * nq];
    const float axv1[4] = {c1.x, c1.y, c1.z, c1.w}, axv2[4] = {c2.x, c2.y, c2.z, c2.w},
                axv3[4] = {c3.x, c3.y, c3.z, c3.w};
    const float oxs[6] = {par ? c0.x : ox, c0.x, c0.y, c0.z, c0.w, par ? ox : c0.w};
    const float sv[4] = {os.x, os.y, os.z, os.w}, nv4[4] = {on.x, on.y, on.z, on.w};
    const float bv[4] = {ob.x, ob.y, ob.z, ob.w}, tv[4] = {ot.x, ot.y, ot.z, ot.w};
    const float rv[4] = {r4.x, r4.y, r4.z, r4.w};
    float ev[4] = {e4.x, e4.y, e4.z, e4.w};
    const unsigned char mv[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float left = par ? oxs[u + 1] : oxs[u];
      const float right = par ? oxs[u + 2] : oxs[u + 1];
      const float ax1 = axv1[u], ax2 = axv2[u], ax3 = axv3[u];
      float sm = rv[u];
      sm = __fmaf_rn(-ax1, left, sm);
      sm = __fmaf_rn(-ax3, right, sm);
      sm = __fmaf_rn(-ay1, sv[u], sm);
      sm = __fmaf_rn(-ay3, nv4[u], sm);
      sm = __fmaf_rn(-az1, bv[u], sm);
      sm = __fmaf_rn(-az3, tv[u], sm);
      const float nvv = __fmaf_rn(omega, __fdividef(sm, ax2 + ay2 + az2) - ev[u], ev[u]);
      ev[u] = mv[u] ? nvv : ev[u];
    }
    *reinterpret_cast<float4*>(own + so) = make_float4(ev[0], ev[1], ev[2], ev[3]);
  }
}

// pull rows ja..jb of plane p of colour C's right-hand side and mask into L2
// (bulk prefetches on the copy engine; the byte range is trimmed inward to
// 16-byte boundaries so it never leaves the arrays)
__device__ __forceinline__ void zm_prefetch_l2(const DevBlock& B, int C, const ZmSpan& z) {
  if (z.n <= 0) return;
  const Dims& d = B.d;
  const int rows = z.n / (d.NXH >> 2);
  const int64_t pi = (int64_t)d.NXH * d.NY * (z.p - 1) + (int64_t)d.NXH * (z.ja - 1);
  const char* ranges[2] = {reinterpret_cast<const char*>(B.rhsf[C] + pi),
                           reinterpret_cast<const char*>(B.upd[C] + pi)};
  const int64_t bytes[2] = {(int64_t)rows * d.NXH * 4, (int64_t)rows * d.NXH};
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const uintptr_t a0 = reinterpret_cast<uintptr_t>(ranges[q]);
    const uintptr_t lo = (a0 + 15) & ~(uintptr_t)15, hi = (a0 + (uintptr_t)bytes[q]) & ~(uintptr_t)15;
    if (hi > lo)
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(lo), "r"((unsigned)(hi - lo)) : "memory");
  }
}

// the tile's rows of plane p (both colours) from the ring to E
__device__ __forceinline__ void zm_writeout(const DevBlock& B, const ZmRing& R, const Tile& t, int p,
                                            float* const E[2]) {
  const Dims& d = B.d;
  const int nq = d.NXH >> 2;
  const int per = t.nj * nq, n = 2 * per;
  const int64_t gz = (int64_t)d.NXH * d.NY * (p - 1);
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int c = q / per, rem = q - c * per;
    const int a = rem % nq, j = t.j0 + rem / nq;
    const float4 v = *reinterpret_cast<const float4*>(R.at(p, c) + (j - R.jrow0) * d.NXH + 4 * a);
    *reinterpret_cast<float4*>(E[c] + gz + (int64_t)d.NXH * (j - 1) + 4 * a) = v;
  }
}

// One pass of `nlev` (4, or 2 for an odd final pair) half-sweeps over the
// tile, reading buffer `cur` through the tensor maps and writing the tile's
// rows of the other buffer.  false (on every thread) once a load wait gave up.
__device__ bool zm_pass(const DevBlock& B, const ZmArgs& z, const ZmMaps& maps, ZmRing& R, const Tile& t, int cur,
                        int nlev, float omega, float* const Eout[2], unsigned long long limit_ns) {
  const CUtensorMap* m0 = &maps.m[2 * cur];
  const CUtensorMap* m1 = &maps.m[2 * cur + 1];
  const int y0 = R.jrow0 - 1;  // 0-based row of a slot's row 0
  const int k1 = t.k0 + t.nk - 1;
  const int kb = t.k0 - nlev, ke = k1 + nlev;            // planes loaded
  const int ks = t.k0 - (nlev - 1), kf = k1 + (nlev - 1);  // steps
  const unsigned bytes = 2u * (unsigned)z.rows * (unsigned)B.d.NXH * 4u;
  auto issue = [&](int p) {
    if (threadIdx.x == 0) {
      uint64_t* bar = R.bars + ZmRing::slot(p);
      fence_proxy_async_shared();
      mbar_expect_tx(bar, bytes);
      tma_load_plane(R.at(p, 0), m0, y0, p - 1, bar);
      tma_load_plane(R.at(p, 1), m1, y0, p - 1, bar);
    }
  };
  bool ok = true;
  auto wait = [&](int p) {
    const int s = ZmRing::slot(p);
    ok = mbar_wait(R.bars + s, (R.pbits >> s) & 1u, limit_ns) && ok;
    R.pbits ^= 1u << s;
  };
  auto span = [&](int k, int L) {
    const int sp = nlev - L;  // rows and planes beyond the tile at this level
    const int p = k - L + 1;
    return zm_span(B.d, p, t.j0 - sp, t.j0 + t.nj - 1 + sp, L <= nlev && p >= t.k0 - sp && p <= k1 + sp);
  };
  issue(kb);
  issue(kb + 1);
  issue(kb + 2);
  for (int k = ks; k <= kf; ++k) {
    if (k + 2 <= ke) issue(k + 2);
    if (threadIdx.x == 32) {
      // the right-hand side rows that levels 1 and 2 first touch two steps on
      zm_prefetch_l2(B, 1, span(k + 2, 1));
      zm_prefetch_l2(B, 0, span(k + 2, 2));
    }
    const ZmSpan z1 = span(k, 1), z2 = span(k, 2), z3 = span(k, 3), z4 = span(k, 4);
    float4 r1[kZmRuns], r2[kZmRuns], r3[kZmRuns], r4[kZmRuns];
    uchar4 m1[kZmRuns], m2[kZmRuns], m3[kZmRuns], m4[kZmRuns];
    zm_fetch<1>(B, z1, r1, m1);
    zm_fetch<0>(B, z2, r2, m2);
    zm_fetch<1>(B, z3, r3, m3);
    zm_fetch<0>(B, z4, r4, m4);
    if (k == ks) {
      wait(kb);
      wait(kb + 1);
    }
    wait(k + 1);
    zm_level<1>(B, R, z1, r1, m1, omega);
    if (__syncthreads_or(!ok)) return false;
    zm_level<0>(B, R, z2, r2, m2, omega);
    __syncthreads();
    if (nlev == 4) {
      zm_level<1>(B, R, z3, r3, m3, omega);
      __syncthreads();
      zm_level<0>(B, R, z4, r4, m4, omega);
      __syncthreads();
    }
    const int pw = k - (nlev - 1);
    if (pw >= t.k0 && pw <= k1) zm_writeout(B, R, t, pw, Eout);
  }
  return true;
}

__global__ void __launch_bounds__(kZmThreads, 1) k_sor_zm(DevBlock B, DcArgs a, GridBar gb, ZmArgs z,
                                                          const __grid_constant__ ZmMaps maps) {
  extern __shared__ __align__(128) unsigned char zm_raw[];
  __shared__ __align__(8) uint64_t bars[kZmSlots];
  __shared__ double sh[32];
  const int cta = (int)blockIdx.x;
  Tile t;
  t.a = cta % z.ntj;
  t.b = cta / z.ntj;
  t.j0 = 2 + t.a * z.tj;
  t.k0 = 2 + t.b * z.tk;
  t.nj = min(z.tj, B.d.ny + 2 - t.j0);
  t.nk = min(z.tk, B.d.nz + 2 - t.k0);
  ZmRing R;
  // the ring starts 128-byte aligned in shared memory, after a guard
  const unsigned pad = (128u - (smem_u32(zm_raw) & 127u)) & 127u;
  R.base = reinterpret_cast<float*>(zm_raw + pad + kZmGuard);
  R.slot_floats = z.slot_floats;
  R.jrow0 = t.j0 - kZmHalo;
  R.pbits = 0;
  R.bars = bars;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kZmSlots; ++s) mbar_init(bars + s);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    fence_proxy_async_shared();
  }
  __syncthreads();
  const int64_t np = B.d.npacked();
  float* const E0[2] = {B.pcf[0], B.pcf[1]};
  float* const E1[2] = {z.e2, z.e2 + np};
  BlockStats* st = B.stats;
  int64_t sweeps = 0;
  double res = 0.0, res_prev = 0.0;
  int inner = a.inner;
  int outer = 0;
  for (;; ++outer) {
    double m = nmax(tile_residual64v<1>(B, t, a.inv_dt), tile_residual64v<0>(B, t, a.inv_dt));
    fence_proxy_async_global();
    m = block_max(m, sh);
    if (threadIdx.x == 0) atomic_max_nonneg(&st->slot[outer % 3], m);
    if (!grid_sync(gb)) return;
    res = take_slot(st, outer, cta);
    if (a.dt * res <= a.div_tol || outer >= a.max_outer || non_finite(res)) break;
    inner = next_inner(a, outer, res, res_prev, inner);
    res_prev = res;
    const int passes = (inner + 1) / 2;
    int cur = 0;
    for (int ps = 0; ps < passes; ++ps) {
      const int nlev = (ps == passes - 1 && (inner & 1)) ? 2 : 4;
      if (!zm_pass(B, z, maps, R, t, cur, nlev, a.omega, cur ? E0 : E1, gb.limit_ns)) {
        if (threadIdx.x == 0) {
          atomicCAS(gb.err, 0, BCFD_E_TIMEOUT);
          atomicOr(gb.ctr, kBarAbandon);
        }
        return;
      }
      fence_proxy_async_global();
      cur ^= 1;
      if (!grid_sync(gb)) return;
    }
    sweeps += inner;
    if (cur) {
      const float* e1c[2] = {E1[0], E1[1]};
      tb_copy_back(B, t, e1c);
      __syncthreads();
    }
    tile_apply4<1>(B, t);
    tile_apply4<0>(B, t);
    fence_proxy_async_global();
    if (!grid_sync(gb)) return;
  }
  if (cta == 0 && threadIdx.x == 0) {
    log_solve(a.log, sweeps, outer + 1, B.cnt[C_FLUID], 2);
    st->niter = st->niter + sweeps;
    st->derr2 = a.dt * res;
    st->pad[1] = a.dt * res;
    if (non_finite(res)) set_err(B.err, BCFD_E_NONFINITE);
  }
}

// Several blocks' solves in one cooperative launch: member m owns CTAs
// [cta0, cta0 + its tile count) and has its own barrier, tiles and slots.
constexpr int kMaxSolveBatch = 16;
template <class Args>
struct SolveEntry {
  Args a;
  GridBar gb;
  TileMap tm;
  int id;    // device table index
  int cta0;  // first CTA
};
template <class Args>
struct SolveSet {
  const DevBlock* tab;
  int nb;
  SolveEntry<Args> e[kMaxSolveBatch];
};

template <class Args>
__device__ __forceinline__ int solve_member(const SolveSet<Args>& S) {
  int m = 0;
  for (int q = 1; q < S.nb; ++q)
    if (S.e[q].cta0 <= (int)blockIdx.x) m = q;
  return m;
}

__global__ void __launch_bounds__(kSolveMaxThreads, 2) k_sor64_set(SolveSet<SorArgs> S) {
  __shared__ unsigned long long raw[(sizeof(DevBlock) + 7) / 8];
  const int m = solve_member(S);
  BlockSet bs;
  bs.tab = S.tab;
  bs.ids[0] = S.e[m].id;
  const DevBlock& B = stage_block(bs, 0, raw);
  sor64_body(B, S.e[m].a, S.e[m].gb, S.e[m].tm, (int)blockIdx.x - S.e[m].cta0);
}

__global__ void __launch_bounds__(kDcThreads, 3) k_sor_dc_set(SolveSet<DcArgs> S) {
  __shared__ unsigned long long raw[(sizeof(DevBlock) + 7) / 8];
  const int m = solve_member(S);
  BlockSet bs;
  bs.tab = S.tab;
  bs.ids[0] = S.e[m].id;
  const DevBlock& B = stage_block(bs, 0, raw);
  sor_dc_body(B, S.e[m].a, S.e[m].gb, S.e[m].tm, (int)blockIdx.x - S.e[m].cta0);
}

// dt * max over fluid cells of |b/dt - A pc| (FP64, measurement) -> stats->pad[1]
__global__ void k_resid(DevBlock B, double dt) {
  __shared__ double sh[32];
  const int64_t total = (int64_t)B.d.NXH * B.d.ny * B.d.nz;
  const double m = block_max(nmax(resid_max64<1>(B, total), resid_max64<0>(B, total)), sh);
  if (threadIdx.x == 0) atomic_max_nonneg(&B.stats->pad[1], m * dt);
}

// correctPressure (src/PcorVcor.F90:245-259)
struct CorrectPOp {
  __device__ void run(const DevBlock& B, int cta, int ncta) const {
    const Dims& d = B.d;
    FOR_INTERIOR(B, cta, ncta) {
      INTERIOR_CELL(B);
      if (B.cell[c] != 0) continue;
      B.p[c] = B.p[c] + B.pc[colour_of(i, j, k)][d.pidx(i, j, k)];
    }
  }
};

__device__ __forceinline__ double pc_at(const DevBlock& B, int i, int j, int k) {
  return B.pc[colour_of(i, j, k)][B.d.pidx(i, j, k)];
}

// correctVelocity (src/PcorVcor.F90:261-286)
// correctVelocity's factor dt / (0.5 (delta_i + delta_{i+1})) depends on one
// index only: one value per grid line, computed with the reference's two
// operations, so the per-cell update (factor times the pc difference) rounds
// exactly as the per-cell expression does, without three FP64 divisions per
// cell (GB300 divides at ~61 G/s)
__global__ void k_line_coef(DevBlock B, double dt) {
  const Dims& d = B.d;
  double* lx = const_cast<double*>(B.lcoef);
  double* ly = lx + d.NX;
  double* lz = ly + d.NY;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < d.NX + d.NY + d.NZ; t += gridDim.x * blockDim.x) {
    if (t < d.NX) {
      const int i = t;
      if (i >= 1) lx[i] = dt / (0.5 * (B.dxa[i] + B.dxa[i - 1]));
    } else if (t < d.NX + d.NY) {
      const int j = t - d.NX;
      if (j >= 1) ly[j] = dt / (0.5 * (B.dya[j] + B.dya[j - 1]));
    } else {
      const int k = t - d.NX - d.NY;
      if (k >= 1) lz[k] = dt / (0.5 * (B.dza[k] + B.dza[k - 1]));
    }
  }
}

struct CorrectVOp {
  __device__ void run(const DevBlock& B, int cta, int ncta) const {
    const double* lx = B.lcoef;
    const double* ly = lx + B.d.NX;
    const double* lz = ly + B.d.NY;
    FOR_INTERIOR(B, cta, ncta) {
      INTERIOR_CELL(B);
      if (B.cell[c] != 0) continue;
      const double p0 = pc_at(B, i, j, k);
      B.ut[c] = B.ut[c] - lx[i] * (pc_at(B, i + 1, j, k) - p0);
      B.vt[c] = B.vt[c] - ly[j] * (pc_at(B, i, j + 1, k) - p0);
      B.wt[c] = B.wt[c] - lz[k] * (pc_at(B, i, j, k + 1) - p0);
    }
  }
};

// steady-state error max |ut - u| / dt over the fluid cells (src/PcorVcor.F90:135-153)
struct SteadyOp {
  double dt;
  __device__ void run(const DevBlock& B, int cta, int ncta) const {
    __shared__ double sh[32];
    // max |x| / dt = (max |x|) / dt exactly: a correctly rounded division by
    // dt > 0 is monotone, so one division per CTA gives the per-cell result
    double m = 0.0;
    FOR_INTERIOR(B, cta, ncta) {
      INTERIOR_CELL(B);
      if (B.cell[c] != 0) continue;
      const double eu = fabs((B.ut[c] - B.u[c]));
      const double ev = fabs((B.vt[c] - B.v[c]));
      const double ew = fabs((B.wt[c] - B.w[c]));
      m = nmax(nmax(nmax(m, eu), ev), ew);
    }
    m = block_max(m, sh);
    if (threadIdx.x == 0) atomic_max_nonneg(&B.stats->derr_std_st, m / dt);
  }
};

// max |div| over the fluid cells of (u,v,w) (slot maxdiv) or, right after
// the velocity correction, of (ut,vt,wt) (slot pad[0]); FP64
struct MaxDivOp {
  int tfield;
  __device__ void run(const DevBlock& B, int cta, int ncta) const {
    __shared__ double sh[32];
    const Dims& d = B.d;
    const double* U = tfield ? B.ut : B.u;
    const double* V = tfield ? B.vt : B.v;
    const double* W = tfield ? B.wt : B.w;
    // a measurement (not a reference routine): the divergence with the
    // reciprocal spacings, within an ulp of the divided form, without three
    // FP64 divisions per cell
    const double* rx = B.lcoef + (d.NX + d.NY + d.NZ);
    const double* ry = rx + d.NX;
    const double* rz = ry + d.NY;
    double m = 0.0;
    FOR_INTERIOR(B, cta, ncta) {
      INTERIOR_CELL(B);
      if (B.cell[c] != 0) continue;
      const double dv = (U[c] - U[c - 1]) * rx[i - 1] + (V[c] - V[c - d.NX]) * ry[j - 1] +
                        (W[c] - W[c - (int64_t)d.NX * d.NY]) * rz[k - 1];
      m = nmax(m, fabs(dv));
    }
    m = block_max(m, sh);
    if (threadIdx.x == 0) atomic_max_nonneg(tfield ? &B.stats->pad[0] : &B.stats->maxdiv, m);
  }
};

// u <- ut (to_n) or ut <- u over every point (src/PcorVcor.F90:212-214, 379-397)
struct CopyOp {
  int to_n;
  __device__ void run(const DevBlock& B, int cta, int ncta) const {
    const int64_t n = B.d.npts();
    double *a = to_n ? B.u : B.ut, *b = to_n ? B.v : B.vt, *e = to_n ? B.w : B.wt;
    const double *x = to_n ? B.ut : B.u, *y = to_n ? B.vt : B.v, *z = to_n ? B.wt : B.w;
    for (int64_t t = (int64_t)cta * blockDim.x + threadIdx.x; t < n; t += (int64_t)ncta * blockDim.x) {
      a[t] = x[t];
      b[t] = y[t];
      e[t] = z[t];
    }
  }
};

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

constexpr unsigned kCellCap = 152u * 32u;

int launch_compute_div(const std::vector<HostBlock*>& hbs, bool fast) {
  return launch_op<DivOp, 256>(hbs, DivOp{fast ? 1 : 0}, Extent::Interior, kCellCap);
}
int launch_compute_div(HostBlock* hb) { return launch_compute_div(std::vector<HostBlock*>{hb}, false); }

int launch_correct_pressure(const std::vector<HostBlock*>& hbs) {
  return launch_op<CorrectPOp, 256>(hbs, CorrectPOp{}, Extent::Interior, kCellCap);
}
int launch_correct_pressure(HostBlock* hb) { return launch_correct_pressure(std::vector<HostBlock*>{hb}); }

int launch_correct_velocity(const std::vector<HostBlock*>& hbs, double dt) {
  for (HostBlock* hb : hbs) {
    if (hb->lcoef_dt == dt) continue;
    const Dims& d = hb->d.d;
    k_line_coef<<<grid_for(d.NX + d.NY + d.NZ, 128), 128, 0, stream()>>>(hb->d, dt);
    BCFD_LAUNCHED();
    hb->lcoef_dt = dt;
  }
  return launch_op<CorrectVOp, 256>(hbs, CorrectVOp{}, Extent::Interior, kCellCap);
}
int launch_correct_velocity(HostBlock* hb, double dt) {
  return launch_correct_velocity(std::vector<HostBlock*>{hb}, dt);
}

// warm start: pc keeps its values at the cells the solve updates (the last
// step's correction there, the initial guess) and is 0 everywhere else, as
// after the reference's zeroing (solid cells, block faces, coupling ghosts)
__global__ void k_pc_warm(DevBlock B) {
  const int64_t n = B.d.npacked();
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    if (!B.upd[0][t]) B.pc[0][t] = 0.0;
    if (!B.upd[1][t]) B.pc[1][t] = 0.0;
  }
}

// the relaxation factor a block's FP32 correction sweeps use (the block's
// setting or the default, within [1, kMixedOmegaMax]), before the FP32 rounding
double mixed_omega_of(const HostBlock* hb) {
  const double om = hb->dc_omega > 0 ? hb->dc_omega : mixed_omega_default(hb->d.d);
  return std::min(kMixedOmegaMax, std::max(1.0, om));
}

int launch_zero_poisson(HostBlock* hb, bool warm) {
  const size_t bytes = (size_t)hb->d.d.npacked() * sizeof(double);
  if (warm) {
    k_pc_warm<<<grid_for(hb->d.d.npacked(), 256), 256, 0, stream()>>>(hb->d);
    BCFD_LAUNCHED();
  }
  for (int c = 0; c < 2; ++c) {
    if (!warm) BCFD_CUDA(cudaMemsetAsync(hb->d.pc[c], 0, bytes, stream()));
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

// Tiles for a tiled persistent solve: the smallest tiles (most CTAs) whose
// count fits the co-resident capacity of `fn`, squarest among equal areas.
static TileMap tiles_within(HostBlock* hb, unsigned cap, int global) {
  const Dims& d = hb->d.d;
  cap = std::max(1u, std::min<unsigned>(cap, kMaxTiles));
  TileMap best{d.ny, d.nz, 1, 1, hb->prog, global};
  long barea = (long)d.ny * d.nz, bper = d.ny + d.nz;
  for (int tk = 1; tk <= d.nz; ++tk) {
    const int ntk = (d.nz + tk - 1) / tk;
    if ((unsigned)ntk > cap) continue;
    const int maxntj = (int)(cap / (unsigned)ntk);
    const int tj = (d.ny + maxntj - 1) / maxntj;
    const int ntj = (d.ny + tj - 1) / tj;
    const long area = (long)tj * tk, per = tj + tk;
    if (area < barea || (area == barea && per < bper)) {
      best = TileMap{tj, tk, ntj, ntk, hb->prog, global};
      barea = area;
      bper = per;
    }
  }
  return best;
}

static TileMap choose_tiles(HostBlock* hb, const void* fn, int threads, int global, int ctas_per_sm) {
  unsigned cap = coop_grid(fn, threads, 0, 0xffffffffu);
  if (ctas_per_sm > 0) cap = std::min<unsigned>(cap, (unsigned)(ctas_per_sm * num_sms()));
  return tiles_within(hb, cap, global);
}

// zeroed progress counters, stop-test slots and barrier word for one launch
static int reset_solve_state(HostBlock* hb, const TileMap& tm) {
  BCFD_CUDA(cudaMemsetAsync(hb->prog, 0, (size_t)tm.ntj * tm.ntk * kTileStride * sizeof(unsigned), stream()));
  BCFD_CUDA(cudaMemsetAsync(&hb->d.stats->slot[0], 0, 3 * sizeof(double), stream()));
  BCFD_CUDA(cudaMemsetAsync(hb->bar, 0, 2 * sizeof(unsigned), stream()));
  return 0;
}

int launch_sor(HostBlock* hb, int64_t itmax, double dt, double epsi, double res_tol, int fast) {
  DevBlock& B = hb->d;
  const int64_t np = B.d.npacked();
  k_rhs<<<grid_for(np, 256), 256, 0, stream()>>>(B, dt);
  BCFD_LAUNCHED();
  const int threads = hb->solve_threads > 0 ? hb->solve_threads : 512;
  TileMap tm = choose_tiles(hb, (const void*)k_sor64, threads, hb->solve_sync == 1 ? 1 : 0, hb->solve_ctas_per_sm);
  TRY_R(reset_solve_state(hb, tm));
  const unsigned grid = (unsigned)(tm.ntj * tm.ntk);
  SorArgs a{itmax, epsi, hb->omega, prof_log(), res_tol, dt, hb->sor_rev, fast};
  GridBar gb = make_bar(B.err, grid);
  gb.ctr = reinterpret_cast<unsigned long long*>(hb->bar);
  void* args[] = {(void*)&B, (void*)&a, (void*)&gb, (void*)&tm};
  prof_mark(true);
  BCFD_CUDA(launch_coop((const void*)k_sor64, grid, threads, args));
  prof_mark(false);
  BCFD_LAUNCHED();
  return launch_residual(hb, dt);
}

// the second FP32 correction buffer (both colours, zeroed once) of the
// temporal-blocked and z-marching sweeps
static int ensure_second_buffer(HostBlock* hb) {
  if (hb->pcf2) return 0;
  const int64_t np = hb->d.d.npacked();
  void* p = nullptr;
  if (cudaMalloc(&p, 2 * (size_t)np * sizeof(float)) != cudaSuccess) return BCFD_E_NOMEM;
  hb->allocs.push_back(p);
  hb->pcf2 = static_cast<float*>(p);
  BCFD_CUDA(cudaMemsetAsync(hb->pcf2, 0, 2 * (size_t)np * sizeof(float), stream()));
  lib().gen++;
  return 0;
}

// Temporal-blocked solve: tiles of tj x tk rows with their two halo rows per
// side in shared memory, one CTA of 512 threads per tile, all co-resident.
static size_t tb_bytes(const Dims& d, int tj, int tk) {
  return (size_t)(tj + 4) * (tk + 4) * (d.NXH + 2 * kTbPad) * 18;
}

// the smallest square-ish tiles (the most CTAs, for loads in flight) whose
// count fits one CTA per SM and whose halo'd rows fit in shared memory; 0 when
// the block is too large for this variant
static int tb_tiles(HostBlock* hb, int* tj, int* tk) {
  const Dims& d = hb->d.d;
  int dev = lib().device, smem_max = 0, nsm = num_sms();
  if (cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  const size_t cap = (size_t)smem_max - 1024;  // static shared memory of the kernel
  for (int s = 2; s <= 32; ++s) {
    const int a = std::min(s, d.ny), b = std::min(s, d.nz);
    const int n = ((d.ny + a - 1) / a) * ((d.nz + b - 1) / b);
    if (tb_bytes(d, a, b) <= cap && n <= nsm) {
      *tj = a;
      *tk = b;
      return 1;
    }
  }
  return 0;
}

bool tb_solve_fits(HostBlock* hb) {
  int a, b;
  return tb_tiles(hb, &a, &b) != 0;
}

static int launch_sor_tb(HostBlock* hb, int64_t itmax, double dt, double div_tol) {
  DevBlock& B = hb->d;
  TRY_R(ensure_second_buffer(hb));
  int tj = 0, tk = 0;
  if (!tb_tiles(hb, &tj, &tk)) return BCFD_E_STATE;
  TileMap tm{tj, tk, (B.d.ny + tj - 1) / tj, (B.d.nz + tk - 1) / tk, hb->prog, 1};
  TRY_R(reset_solve_state(hb, tm));
  const size_t smem = tb_bytes(B.d, tj, tk);
  BCFD_CUDA(cudaFuncSetAttribute((const void*)k_sor_tb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const unsigned grid = (unsigned)(tm.ntj * tm.ntk);
  DcArgs a;
  a.inner = hb->dc_inner > 0 ? hb->dc_inner : 64;
  double om = hb->dc_omega > 0 ? hb->dc_omega : mixed_omega_default(B.d);
  a.omega = (float)std::min(kMixedOmegaMax, std::max(1.0, om));
  a.max_outer = itmax / a.inner + 1;
  a.dt = dt;
  a.inv_dt = 1.0 / dt;
  a.div_tol = div_tol;
  a.log = prof_log();
  GridBar gb = make_bar(B.err, grid);
  gb.ctr = reinterpret_cast<unsigned long long*>(hb->bar);
  float* e2 = hb->pcf2;
  void* args[] = {(void*)&B, (void*)&a, (void*)&gb, (void*)&tm, (void*)&e2};
  prof_mark(true);
  BCFD_CUDA(launch_coop((const void*)k_sor_tb, grid, kTbThreads, args, smem));
  prof_mark(false);
  BCFD_LAUNCHED();
  return 0;
}

// Z-marching TMA solve (variant 5): tiles of tj rows x tk planes, one CTA of
// kZmThreads per tile and at most one per SM (the plane ring fills most of
// the shared memory), all co-resident.
static size_t zm_smem_bytes(const Dims& d, int rows) {
  const size_t slot = ((size_t)rows * d.NXH + 31) / 32 * 32;  // floats, 128-byte multiple
  return 128 + 2 * (size_t)kZmGuard + (size_t)kZmSlots * 2 * slot * sizeof(float);
}

// the tiling with the least work per CTA: steps marched (tk + 6 for the
// three planes before and after the tile) x rows handled per step (tj + 8
// loaded, 4 tj + 12 computed, tj written) plus a per-step sync allowance
// worth eight rows, among the tilings whose level-1 rows give no thread more
// than kZmRuns runs; 0 when the block does not fit this variant (a packed
// row wider than one TMA box, or a plane ring beyond shared memory)
static int zm_tiles(HostBlock* hb, ZmArgs* z) {
  const Dims& d = hb->d.d;
  if (d.NXH > 256) return 0;
  int smem_max = 0;
  if (cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, lib().device) != cudaSuccess)
    return 0;
  const size_t cap = (size_t)smem_max - 1024;  // static shared memory of the kernel
  const int nsm = num_sms();
  double best = 0.0;
  int found = 0;
  for (int ntj = 1; ntj <= std::min(d.ny, nsm); ++ntj) {
    const int tj = (d.ny + ntj - 1) / ntj;
    if ((d.ny + tj - 1) / tj != ntj) continue;
    if (zm_smem_bytes(d, tj + 2 * kZmHalo) > cap) continue;
    // every thread holds the right-hand side of at most kZmRuns runs per level
    if ((tj + 2 * (kZmHalo - 1)) * (d.NXH / 4) > kZmRuns * kZmThreads) continue;
    for (int nzs = 1; nzs <= std::min(d.nz, nsm / ntj); ++nzs) {
      const int tk = (d.nz + nzs - 1) / nzs;
      if ((d.nz + tk - 1) / tk != nzs) continue;
      const double cost = (double)(tk + 6) * (6.0 * tj + 28.0);
      if (!found || cost < best) {
        best = cost;
        found = 1;
        z->tj = tj;
        z->ntj = ntj;
        z->tk = tk;
        z->nzs = nzs;
      }
    }
  }
  if (!found) return 0;
  z->rows = z->tj + 2 * kZmHalo;
  z->slot_floats = (int)(((size_t)z->rows * d.NXH + 31) / 32 * 32);
  return 1;
}

bool zm_solve_fits(HostBlock* hb) {
  ZmArgs z{};
  return zm_tiles(hb, &z) != 0;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library)
static PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// one packed colour array (NXH x NY x NZ FP32, x fastest) read in boxes of
// `rows` full rows of one plane; rows outside the array read as zero
static int encode_plane_map(CUtensorMap* m, const float* base, const Dims& d, int rows) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = tmap_encoder();
  if (!fn) return BCFD_E_STATE;
  const cuuint64_t dims[3] = {(cuuint64_t)d.NXH, (cuuint64_t)d.NY, (cuuint64_t)d.NZ};
  const cuuint64_t strides[2] = {(cuuint64_t)d.NXH * sizeof(float), (cuuint64_t)d.NXH * d.NY * sizeof(float)};
  const cuuint32_t box[3] = {(cuuint32_t)d.NXH, (cuuint32_t)rows, 1u};
  const cuuint32_t estride[3] = {1u, 1u, 1u};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estride,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : BCFD_E_STATE;
}

static int launch_sor_zm(HostBlock* hb, int64_t itmax, double dt, double div_tol) {
  DevBlock& B = hb->d;
  ZmArgs z{};
  if (!zm_tiles(hb, &z)) return BCFD_E_STATE;
  TRY_R(ensure_second_buffer(hb));
  z.e2 = hb->pcf2;
  const int64_t np = B.d.npacked();
  ZmMaps maps;
  TRY_R(encode_plane_map(&maps.m[0], B.pcf[0], B.d, z.rows));
  TRY_R(encode_plane_map(&maps.m[1], B.pcf[1], B.d, z.rows));
  TRY_R(encode_plane_map(&maps.m[2], z.e2, B.d, z.rows));
  TRY_R(encode_plane_map(&maps.m[3], z.e2 + np, B.d, z.rows));
  TileMap tm{z.tj, z.tk, z.ntj, z.nzs, hb->prog, 1};
  TRY_R(reset_solve_state(hb, tm));
  const size_t smem = zm_smem_bytes(B.d, z.rows);
  BCFD_CUDA(cudaFuncSetAttribute((const void*)k_sor_zm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const unsigned grid = (unsigned)(z.ntj * z.nzs);
  DcArgs a;
  a.inner = hb->dc_inner > 0 ? hb->dc_inner : 64;
  double om = hb->dc_omega > 0 ? hb->dc_omega : mixed_omega_default(B.d);
  a.omega = (float)std::min(kMixedOmegaMax, std::max(1.0, om));
  a.max_outer = itmax / a.inner + 1;
  a.dt = dt;
  a.inv_dt = 1.0 / dt;
  a.div_tol = div_tol;
  a.log = prof_log();
  GridBar gb = make_bar(B.err, grid);
  gb.ctr = reinterpret_cast<unsigned long long*>(hb->bar);
  void* args[] = {(void*)&B, (void*)&a, (void*)&gb, (void*)&z, (void*)&maps};
  prof_mark(true);
  BCFD_CUDA(launch_coop((const void*)k_sor_zm, grid, kZmThreads, args, smem));
  prof_mark(false);
  BCFD_LAUNCHED();
  return 0;
}

int launch_sor_mixed(HostBlock* hb, int64_t itmax, double dt, double div_tol) {
  DevBlock& B = hb->d;
  const int64_t np = B.d.npacked();
  for (int c = 0; c < 2; ++c) BCFD_CUDA(cudaMemsetAsync(B.pcf[c], 0, np * sizeof(float), stream()));
  if (hb->dc_variant == 4 && tb_solve_fits(hb)) return launch_sor_tb(hb, itmax, dt, div_tol);
  if (hb->dc_variant == 5 && zm_solve_fits(hb)) return launch_sor_zm(hb, itmax, dt, div_tol);
  const int threads = hb->dc_threads > 0 ? std::min(hb->dc_threads, kDcThreads) : kDcThreads;
  // variant 3: point-to-point tile sync; otherwise grid-wide phase barriers
  // four CTAs per SM asked for: the 64-register instantiation
  const void* fn = hb->dc_ctas_per_sm == 4 ? (const void*)k_sor_dc<4> : (const void*)k_sor_dc<3>;
  TileMap tm = choose_tiles(hb, fn, threads, hb->dc_variant == 3 ? 0 : 1, hb->dc_ctas_per_sm);
  TRY_R(reset_solve_state(hb, tm));
  const unsigned grid = (unsigned)(tm.ntj * tm.ntk);
  DcArgs a;
  a.inner = hb->dc_inner > 0 ? hb->dc_inner : 64;
  double om = hb->dc_omega > 0 ? hb->dc_omega : mixed_omega_default(B.d);
  a.omega = (float)std::min(kMixedOmegaMax, std::max(1.0, om));
  a.max_outer = itmax / a.inner + 1;
  a.dt = dt;
  a.inv_dt = 1.0 / dt;
  a.div_tol = div_tol;
  a.log = prof_log();
  GridBar gb = make_bar(B.err, grid);
  gb.ctr = reinterpret_cast<unsigned long long*>(hb->bar);
  void* args[] = {(void*)&B, (void*)&a, (void*)&gb, (void*)&tm};
  prof_mark(true);
  BCFD_CUDA(launch_coop(fn, grid, threads, args));
  prof_mark(false);
  BCFD_LAUNCHED();
  // k_sor_dc records the residual it leaves (stats pad[1]) itself
  return 0;
}

// One cooperative launch for the solves of several blocks (batching on, more
// than one block): the co-resident CTAs are shared out in proportion to the
// blocks' cell counts; each block keeps its own tiles, barrier and slots.
// make(hb, args) fills a block's arguments; returns nonzero to solve that
// block alone (then solo(hb) runs).
template <class Args, class Make, class Solo>
static int launch_solve_set(const std::vector<HostBlock*>& hbs, const void* fn, int threads, int global,
                            Make make, Solo solo) {
  std::vector<HostBlock*> group;
  for (HostBlock* hb : hbs) {
    Args a{};
    if (make(hb, a)) TRY_R(solo(hb));
    else group.push_back(hb);
  }
  if (group.size() == 1 || (!group.empty() && !lib().batch)) {
    for (HostBlock* hb : group) TRY_R(solo(hb));
    return 0;
  }
  if (group.empty()) return 0;
  TRY_R(sync_block_table());
  const unsigned cap_all = std::min<unsigned>(coop_grid(fn, threads, 0, 0xffffffffu), 0x7fffffffu);
  for (size_t g0 = 0; g0 < group.size(); g0 += kMaxSolveBatch) {
    const int nb = (int)std::min<size_t>(kMaxSolveBatch, group.size() - g0);
    double cells = 0;
    for (int m = 0; m < nb; ++m) {
      const Dims& d = group[g0 + m]->d.d;
      cells += (double)d.nx * d.ny * d.nz;
    }
    SolveSet<Args> S{};
    S.tab = lib().dtab;
    S.nb = nb;
    unsigned grid = 0;
    // every member needs at least one CTA: share what is left after that
    const unsigned spare = cap_all > (unsigned)nb ? cap_all - (unsigned)nb : 0u;
    for (int m = 0; m < nb; ++m) {
      HostBlock* hb = group[g0 + m];
      const Dims& d = hb->d.d;
      unsigned cap = 1u + (unsigned)(spare * ((double)d.nx * d.ny * d.nz / cells));
      if (hb->solve_ctas_per_sm > 0) cap = std::min<unsigned>(cap, (unsigned)(hb->solve_ctas_per_sm * num_sms()));
      TileMap tm = tiles_within(hb, cap, global);
      TRY_R(reset_solve_state(hb, tm));
      SolveEntry<Args>& e = S.e[m];
      make(hb, e.a);
      e.tm = tm;
      e.gb = make_bar(hb->d.err, (unsigned)(tm.ntj * tm.ntk));
      e.gb.ctr = reinterpret_cast<unsigned long long*>(hb->bar);
      e.id = hb->index;
      e.cta0 = (int)grid;
      grid += (unsigned)(tm.ntj * tm.ntk);
    }
    void* args[] = {(void*)&S};
    prof_mark(true);
    BCFD_CUDA(launch_coop(fn, grid, threads, args));
    prof_mark(false);
    BCFD_LAUNCHED();
  }
  return 0;
}

int launch_sor_set(const std::vector<HostBlock*>& hbs, int64_t itmax, double dt, double epsi, double res_tol,
                   int fast) {
  if (hbs.size() <= 1 || !lib().batch) {
    for (HostBlock* hb : hbs) TRY_R(launch_sor(hb, itmax, dt, epsi, res_tol, fast));
    return 0;
  }
  const int threads = 512;
  for (HostBlock* hb : hbs) {
    k_rhs<<<grid_for(hb->d.d.npacked(), 256), 256, 0, stream()>>>(hb->d, dt);
    BCFD_LAUNCHED();
  }
  auto make = [&](HostBlock* hb, SorArgs& a) -> int {
    a = SorArgs{itmax, epsi, hb->omega, prof_log(), res_tol, dt, hb->sor_rev, fast};
    // blocks with their own launch shape keep their own launch
    return hb->solve_threads > 0 || hb->solve_sync != 0 || hb->solve_ctas_per_sm > 0;
  };
  // a block solved alone goes through launch_sor (which recomputes b/dt)
  auto solo = [&](HostBlock* hb) -> int { return launch_sor(hb, itmax, dt, epsi, res_tol, fast); };
  TRY_R(launch_solve_set<SorArgs>(hbs, (const void*)k_sor64_set, threads, 0, make, solo));
  for (HostBlock* hb : hbs) TRY_R(launch_residual(hb, dt));
  return 0;
}

int launch_sor_mixed_set(const std::vector<HostBlock*>& hbs, int64_t itmax, double dt, double div_tol) {
  if (hbs.size() <= 1 || !lib().batch) {
    for (HostBlock* hb : hbs) TRY_R(launch_sor_mixed(hb, itmax, dt, div_tol));
    return 0;
  }
  const int threads = kDcThreads;
  for (HostBlock* hb : hbs) {
    if (hb->dc_variant >= 2 || hb->dc_threads > 0 || hb->dc_ctas_per_sm > 0) continue;
    for (int c = 0; c < 2; ++c)
      BCFD_CUDA(cudaMemsetAsync(hb->d.pcf[c], 0, hb->d.d.npacked() * sizeof(float), stream()));
  }
  auto make = [&](HostBlock* hb, DcArgs& a) -> int {
    const Dims& d = hb->d.d;
    a.inner = hb->dc_inner > 0 ? hb->dc_inner : 64;
    const double om = hb->dc_omega > 0 ? hb->dc_omega : mixed_omega_default(d);
    a.omega = (float)std::min(kMixedOmegaMax, std::max(1.0, om));
    a.max_outer = itmax / a.inner + 1;
    a.dt = dt;
    a.inv_dt = 1.0 / dt;
    a.div_tol = div_tol;
    a.log = prof_log();
    return hb->dc_variant >= 2 || hb->dc_threads > 0 || hb->dc_ctas_per_sm > 0;
  };
  auto solo = [&](HostBlock* hb) -> int { return launch_sor_mixed(hb, itmax, dt, div_tol); };
  return launch_solve_set<DcArgs>(hbs, (const void*)k_sor_dc_set, threads, 1, make, solo);
}

int launch_steady_state(const std::vector<HostBlock*>& hbs, double dt) {
  for (HostBlock* hb : hbs)
    BCFD_CUDA(cudaMemsetAsync(&hb->d.stats->derr_std_st, 0, sizeof(double), stream()));
  return launch_op<SteadyOp, 256>(hbs, SteadyOp{dt}, Extent::Interior, 1024);
}
int launch_steady_state(HostBlock* hb, double dt) { return launch_steady_state(std::vector<HostBlock*>{hb}, dt); }

int launch_max_div(const std::vector<HostBlock*>& hbs, bool tfield) {
  for (HostBlock* hb : hbs) {
    double* slot = tfield ? &hb->d.stats->pad[0] : &hb->d.stats->maxdiv;
    BCFD_CUDA(cudaMemsetAsync(slot, 0, sizeof(double), stream()));
  }
  return launch_op<MaxDivOp, 256>(hbs, MaxDivOp{tfield ? 1 : 0}, Extent::Interior, 1024);
}
int launch_max_div(HostBlock* hb, bool tfield) { return launch_max_div(std::vector<HostBlock*>{hb}, tfield); }

int launch_copy_t_to_n(const std::vector<HostBlock*>& hbs) {
  return launch_op<CopyOp, 256>(hbs, CopyOp{1}, Extent::Points, kCellCap);
}
int launch_copy_t_to_n(HostBlock* hb) { return launch_copy_t_to_n(std::vector<HostBlock*>{hb}); }
int launch_copy_n_to_t(HostBlock* hb) {
  return launch_op<CopyOp, 256>(std::vector<HostBlock*>{hb}, CopyOp{0}, Extent::Points, kCellCap);
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
