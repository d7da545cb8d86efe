// Adjoint of the pressure Poisson solve.  The solve of src/PcorVcor.F90
// (REDBLACKSOR_linear) inverts A restricted to the fluid cells, where row
// (i,j,k) of A is the 7-point stencil of the Acx/Acy/Acz line tables
// (src/CoefficientMatrix.f90:10-71).  A is not symmetric on a stretched grid
// or with the coarse block's boundary folding, but its transpose is again a
// 7-point operator of three line tables: in row i the coefficient of i-1 is
// row i-1's right coefficient and that of i+1 is row i+1's left coefficient;
// the diagonal is unchanged.  So the adjoint solve A^T x = r is the same
// persistent red-black SOR kernel run with the transposed tables and the
// colour sweeps in reverse order (black first).  Non-fluid cells are zero
// Dirichlet data for both solves (the adjoint of the boundary coupling is not
// part of this entry point).
#include <cstring>

#include <algorithm>

#include "bcfd_host.h"

namespace bcfd {
namespace {

// transpose of one (n,3) line table
std::vector<double> transpose_line(const std::vector<double>& A, int n) {
  std::vector<double> T(3 * (size_t)n, 0.0);
  for (int i = 2; i <= n + 1; ++i) {
    T[(i - 2)] = i >= 3 ? A[(i - 3) + 2 * (size_t)n] : 0.0;
    T[(i - 2) + n] = A[(i - 2) + (size_t)n];
    T[(i - 2) + 2 * (size_t)n] = i <= n ? A[(i - 1)] : 0.0;
  }
  return T;
}

}  // namespace

// x = A^{-1} r (or A^{-T} r) on the fluid cells, device natural-layout arrays,
// to max|r - A x| <= tol: FP64 SOR, or (lib().adj_precision == 1) FP32 SOR
// sweeps with FP64 defect correction to the same FP64 residual target
int solve_zero_bc_dev(HostBlock* hb, const double* r, double* x, double tol, int64_t itmax, bool transpose) {
  DevBlock& D = hb->d;
  const Dims& d = D.d;
  if (!D.Acx || hb->Acx.empty()) return BCFD_E_STATE;
  const bool mixed = lib().adj_precision == 1;
  const DevBlock keep = D;
  const int keep_rev = hb->sor_rev;
  double* tab = nullptr;
  float* tabf = nullptr;
  int rc = 0;
  if (transpose) {
    const std::vector<double> tx = transpose_line(hb->Acx, d.nx), ty = transpose_line(hb->Acy, d.ny),
                              tz = transpose_line(hb->Acz, d.nz);
    std::vector<double> all(tx);
    all.insert(all.end(), ty.begin(), ty.end());
    all.insert(all.end(), tz.begin(), tz.end());
    if (cudaMalloc(&tab, all.size() * sizeof(double)) != cudaSuccess) return BCFD_E_NOMEM;
    if (h2d(tab, all.data(), all.size() * sizeof(double)) != cudaSuccess) rc = BCFD_E_CUDA;
    D.Acx = tab;
    D.Acy = tab + tx.size();
    D.Acz = tab + tx.size() + ty.size();
    hb->sor_rev = 1;
    if (mixed && !rc) {
      // the FP32 line and sweep tables of the transposed operator
      std::vector<float> f;
      for (double v : all) f.push_back((float)v);
      size_t ox, oy, oz;
      append_sweep_tables(d, tx, ty, tz, f, &ox, &oy, &oz);
      if (cudaMalloc(&tabf, f.size() * sizeof(float)) != cudaSuccess) rc = BCFD_E_NOMEM;
      if (!rc && h2d(tabf, f.data(), f.size() * sizeof(float)) != cudaSuccess) rc = BCFD_E_CUDA;
      if (!rc) {
        D.Acxf = tabf;
        D.Acyf = tabf + tx.size();
        D.Aczf = tabf + tx.size() + ty.size();
        D.axr = reinterpret_cast<const float4*>(tabf + ox);
        D.ayr = reinterpret_cast<const float4*>(tabf + oy);
        D.azr = reinterpret_cast<const float4*>(tabf + oz);
      }
    }
  }
  const size_t pbytes = (size_t)d.npacked() * sizeof(double);
  for (int c = 0; c < 2 && !rc; ++c) {
    if (cudaMemsetAsync(D.pc[c], 0, pbytes, stream()) != cudaSuccess) rc = BCFD_E_CUDA;
    if (!rc && cudaMemsetAsync(D.bpk[c], 0, pbytes, stream()) != cudaSuccess) rc = BCFD_E_CUDA;
  }
  if (!rc && cudaMemsetAsync(&D.stats->niter, 0, sizeof(int64_t), stream()) != cudaSuccess) rc = BCFD_E_CUDA;
  if (!rc) rc = launch_pack(hb, r, D.bpk);
  // residual-target solve of A x = r (deltat = 1)
  if (!rc) rc = mixed ? launch_sor_mixed(hb, itmax, 1.0, tol) : launch_sor(hb, itmax, 1.0, 0.0, tol);
  if (!rc) rc = launch_unpack(hb, D.pc, x);
  if (!rc && cudaStreamSynchronize(stream()) != cudaSuccess) rc = BCFD_E_CUDA;
  D.Acx = keep.Acx;
  D.Acy = keep.Acy;
  D.Acz = keep.Acz;
  D.Acxf = keep.Acxf;
  D.Acyf = keep.Acyf;
  D.Aczf = keep.Aczf;
  D.axr = keep.axr;
  D.ayr = keep.ayr;
  D.azr = keep.azr;
  hb->sor_rev = keep_rev;
  cudaFree(tab);
  cudaFree(tabf);
  if (rc) return rc;
  return take_block_error(hb);
}

namespace {

int solve_zero_bc(HostBlock* hb, const double* r, double* x, double tol, int64_t itmax, bool transpose) {
  const size_t np = (size_t)hb->d.d.npts();
  double* buf = nullptr;
  if (cudaMalloc(&buf, 2 * np * sizeof(double)) != cudaSuccess) return BCFD_E_NOMEM;
  int rc = 0;
  if (h2d(buf, r, np * sizeof(double)) != cudaSuccess) rc = BCFD_E_CUDA;
  if (!rc) rc = solve_zero_bc_dev(hb, buf, buf + np, tol, itmax, transpose);
  if (!rc && d2h(x, buf + np, np * sizeof(double)) != cudaSuccess) rc = BCFD_E_CUDA;
  cudaFree(buf);
  return rc;
}

}  // namespace
}  // namespace bcfd

using namespace bcfd;

extern "C" {

int bcfd_adjoint_set_solver(int precision) {
  LibLock lk;
  if (precision != 0 && precision != 1) return BCFD_E_ARG;
  lib().adj_precision = precision;
  return 0;
}

int bcfd_poisson_solve_zero_bc(bcfd_handle h, const double* r, double* x, double tol, int64_t itmax) {
  LibLock lk;
  HostBlock* hb = get_block(h);
  if (!hb) return BCFD_E_HANDLE;
  if (!r || !x || !(tol > 0.0) || itmax < 1) return BCFD_E_ARG;
  return solve_zero_bc(hb, r, x, tol, itmax, false);
}

int bcfd_momentum_tangent(bcfd_handle h, double deltat, double re, const double* du, const double* dv,
                          const double* dw, const double* dp, double* ut, double* vt, double* wt, double* dut,
                          double* dvt, double* dwt) {
  LibLock lk;
  HostBlock* hb = get_block(h);
  if (!hb) return BCFD_E_HANDLE;
  const double* in[4] = {du, dv, dw, dp};
  double* outh[6] = {ut, vt, wt, dut, dvt, dwt};
  for (const double* p : in)
    if (!p) return BCFD_E_ARG;
  for (double* p : outh)
    if (!p) return BCFD_E_ARG;
  if (!hb->d.ca[0]) return BCFD_E_STATE;
  const size_t np = (size_t)hb->d.d.npts();
  double* buf = nullptr;
  if (cudaMalloc(&buf, 10 * np * sizeof(double)) != cudaSuccess) return BCFD_E_NOMEM;
  int r = 0;
  const double* din[4];
  double* dval[3];
  double* dtan[3];
  for (int q = 0; q < 4 && !r; ++q) {
    din[q] = buf + q * np;
    if (h2d((void*)din[q], in[q], np * sizeof(double)) != cudaSuccess) r = BCFD_E_CUDA;
  }
  for (int q = 0; q < 3; ++q) {
    dval[q] = buf + (4 + q) * np;
    dtan[q] = buf + (7 + q) * np;
  }
  if (!r && cudaMemsetAsync(buf + 4 * np, 0, 6 * np * sizeof(double), stream()) != cudaSuccess) r = BCFD_E_CUDA;
  if (!r) r = launch_momentum_tangent(hb, deltat, re, din, dval, dtan);
  if (!r && cudaStreamSynchronize(stream()) != cudaSuccess) r = BCFD_E_CUDA;
  for (int q = 0; q < 6 && !r; ++q)
    if (d2h(outh[q], buf + (4 + q) * np, np * sizeof(double)) != cudaSuccess)
      r = BCFD_E_CUDA;
  cudaFree(buf);
  if (r) return r;
  return take_block_error(hb);
}

int bcfd_momentum_adjoint(bcfd_handle h, double deltat, double re, const double* utb, const double* vtb,
                          const double* wtb, double* ub, double* vb, double* wb, double* pb) {
  LibLock lk;
  HostBlock* hb = get_block(h);
  if (!hb) return BCFD_E_HANDLE;
  const double* in[3] = {utb, vtb, wtb};
  double* outh[4] = {ub, vb, wb, pb};
  for (const double* p : in)
    if (!p) return BCFD_E_ARG;
  for (double* p : outh)
    if (!p) return BCFD_E_ARG;
  if (!hb->d.ca[0]) return BCFD_E_STATE;
  const size_t np = (size_t)hb->d.d.npts();
  double* buf = nullptr;
  // 3 seeds, 4 adjoints, then the 16-word footprint
  if (cudaMalloc(&buf, 7 * np * sizeof(double) + 64) != cudaSuccess) return BCFD_E_NOMEM;
  int r = 0;
  const double* dsb[3];
  double* dab[4];
  for (int q = 0; q < 3 && !r; ++q) {
    dsb[q] = buf + q * np;
    if (h2d((void*)dsb[q], in[q], np * sizeof(double)) != cudaSuccess) r = BCFD_E_CUDA;
  }
  for (int q = 0; q < 4; ++q) dab[q] = buf + (3 + q) * np;
  if (!r && cudaMemsetAsync(buf + 3 * np, 0, 4 * np * sizeof(double), stream()) != cudaSuccess) r = BCFD_E_CUDA;
  if (!r) r = launch_momentum_adjoint(hb, deltat, re, dsb, dab, (uint32_t*)(buf + 7 * np));
  if (!r && cudaStreamSynchronize(stream()) != cudaSuccess) r = BCFD_E_CUDA;
  for (int q = 0; q < 4 && !r; ++q)
    if (d2h(outh[q], dab[q], np * sizeof(double)) != cudaSuccess) r = BCFD_E_CUDA;
  cudaFree(buf);
  if (r) return r;
  return take_block_error(hb);
}

int bcfd_momentum_adjoint_ts(bcfd_handle h, double deltat, double re, const double* utb, const double* vtb,
                             const double* wtb, double* ub, double* vb, double* wb, double* pb, double* gb) {
  LibLock lk;
  HostBlock* hb = get_block(h);
  if (!hb) return BCFD_E_HANDLE;
  const double* in[3] = {utb, vtb, wtb};
  double* io[4] = {ub, vb, wb, pb};
  for (const double* p : in)
    if (!p) return BCFD_E_ARG;
  for (double* p : io)
    if (!p) return BCFD_E_ARG;
  if (!gb) return BCFD_E_ARG;
  if (!hb->d.ca[0]) return BCFD_E_STATE;
  int64_t cnt[N_COUNT];
  if (d2h(cnt, hb->d.cnt, sizeof(cnt)) != cudaSuccess) return BCFD_E_CUDA;
  const int64_t nts = std::min<int64_t>(cnt[C_TS], hb->d.cap_ib), cap = hb->d.cap_ib;
  const size_t np = (size_t)hb->d.d.npts();
  // 3 seeds, 4 adjoints, the overlay's scratch (7 ints and 14 doubles per
  // point), the ghost adjoint, then the 16-word footprint
  const size_t nd = 7 * np + 14 * np + 14 * (size_t)cap;
  double* buf = nullptr;
  int* last = nullptr;
  if (cudaMalloc(&buf, nd * sizeof(double) + 64) != cudaSuccess) return BCFD_E_NOMEM;
  if (cudaMalloc(&last, 7 * np * sizeof(int)) != cudaSuccess) {
    cudaFree(buf);
    return BCFD_E_NOMEM;
  }
  int r = 0;
  const double* dsb[3];
  double* dab[4];
  for (int q = 0; q < 3 && !r; ++q) {
    dsb[q] = buf + q * np;
    if (h2d((void*)dsb[q], in[q], np * sizeof(double)) != cudaSuccess) r = BCFD_E_CUDA;
  }
  for (int q = 0; q < 4 && !r; ++q) {
    dab[q] = buf + (3 + q) * np;
    if (h2d(dab[q], io[q], np * sizeof(double)) != cudaSuccess) r = BCFD_E_CUDA;
  }
  MomTsAdj ts;
  ts.last = last;
  ts.contrib = buf + 7 * np;
  ts.gb = buf + 21 * np;
  ts.cap = cap;
  if (!r && cudaMemsetAsync(ts.gb, 0, 14 * (size_t)cap * sizeof(double), stream()) != cudaSuccess) r = BCFD_E_CUDA;
  if (!r) r = launch_momentum_adjoint(hb, deltat, re, dsb, dab, (uint32_t*)(buf + nd), &ts);
  if (!r && cudaStreamSynchronize(stream()) != cudaSuccess) r = BCFD_E_CUDA;
  for (int q = 0; q < 4 && !r; ++q)
    if (d2h(io[q], dab[q], np * sizeof(double)) != cudaSuccess) r = BCFD_E_CUDA;
  for (int g = 0; g < 14 && !r && nts > 0; ++g)
    if (d2h(gb + g * nts, ts.gb + g * cap, nts * sizeof(double)) != cudaSuccess) r = BCFD_E_CUDA;
  cudaFree(last);
  cudaFree(buf);
  if (r) return r;
  return take_block_error(hb);
}

int bcfd_forcing_ghost_adjoint(bcfd_handle h, const double* gb, double* ub, double* vb, double* wb, double* pb,
                               double* utb, double* vtb, double* wtb) {
  LibLock lk;
  HostBlock* hb = get_block(h);
  if (!hb) return BCFD_E_HANDLE;
  double* io[7] = {ub, vb, wb, pb, utb, vtb, wtb};
  if (!gb) return BCFD_E_ARG;
  for (double* p : io)
    if (!p) return BCFD_E_ARG;
  if (!hb->has_body || hb->d.ne <= 0) return BCFD_E_STATE;
  int64_t cnt[N_COUNT];
  if (d2h(cnt, hb->d.cnt, sizeof(cnt)) != cudaSuccess) return BCFD_E_CUDA;
  const int64_t nts = std::min<int64_t>(cnt[C_TS], hb->d.cap_ib), cap = hb->d.cap_ib;
  const size_t np = (size_t)hb->d.d.npts(), ntask = 6 * (size_t)cap;
  // 7 adjoint arrays, the ghost adjoint, the task coefficients
  const size_t nd = 7 * np + 14 * (size_t)cap + 8 * ntask + kKinScalars * ntask + kKinScalars;
  double* buf = nullptr;
  void* ibuf = nullptr;
  if (cudaMalloc(&buf, nd * sizeof(double)) != cudaSuccess) return BCFD_E_NOMEM;
  if (cudaMalloc(&ibuf, ntask * (sizeof(int64_t) * 9 + sizeof(int))) != cudaSuccess) {
    cudaFree(buf);
    return BCFD_E_NOMEM;
  }
  int r = 0;
  double* d[7];
  for (int q = 0; q < 7 && !r; ++q) {
    d[q] = buf + q * np;
    if (h2d(d[q], io[q], np * sizeof(double)) != cudaSuccess) r = BCFD_E_CUDA;
  }
  double* dg = buf + 7 * np;
  if (!r && cudaMemsetAsync(dg, 0, 14 * (size_t)cap * sizeof(double), stream()) != cudaSuccess) r = BCFD_E_CUDA;
  for (int g = 0; g < 14 && !r && nts > 0; ++g)
    if (h2d(dg + g * cap, gb + g * nts, nts * sizeof(double)) != cudaSuccess) r = BCFD_E_CUDA;
  ForceCoef fc{};
  fc.coef = dg + 14 * cap;
  fc.kc = fc.coef + 8 * ntask;
  fc.gk = fc.kc + kKinScalars * ntask;
  fc.pos = static_cast<int64_t*>(ibuf);
  fc.tgt = fc.pos + 8 * ntask;
  fc.axis = reinterpret_cast<int*>(fc.tgt + ntask);
  // axis 0 p, 1..3 u/v/w (the t-ghost copies) and ut/vt/wt (the probes)
  const AdjPtrs a{{d[3], d[0], d[1], d[2]}, {d[3], d[4], d[5], d[6]}};
  if (!r) r = launch_ghost_adjoint(hb, 0, a, fc, dg, cap);
  if (!r) r = launch_ghost_adjoint(hb, 1, a, fc, dg, cap);
  if (!r && cudaStreamSynchronize(stream()) != cudaSuccess) r = BCFD_E_CUDA;
  for (int q = 0; q < 7 && !r; ++q)
    if (d2h(io[q], d[q], np * sizeof(double)) != cudaSuccess) r = BCFD_E_CUDA;
  cudaFree(ibuf);
  cudaFree(buf);
  if (r) return r;
  return take_block_error(hb);
}

int bcfd_poisson_solve_adjoint(bcfd_handle h, const double* r, double* x, double tol, int64_t itmax) {
  LibLock lk;
  HostBlock* hb = get_block(h);
  if (!hb) return BCFD_E_HANDLE;
  if (!r || !x || !(tol > 0.0) || itmax < 1) return BCFD_E_ARG;
  return solve_zero_bc(hb, r, x, tol, itmax, true);
}

}  // extern "C"
