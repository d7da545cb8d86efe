// C-ABI entry points of the Bio-CFD GB300 hot path (declared in
// include/biocfd_gb300.h): block registry, device allocation, host mirrors,
// host-side setup tables, and the orchestration of the per-step routines.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "bcfd_host.h"

namespace bcfd {

// ---------------------------------------------------------------------------
// library state
// ---------------------------------------------------------------------------
Lib& lib() {
  static Lib L;
  return L;
}
cudaStream_t stream() { return lib().s; }
int num_sms() { return lib().nsm; }

void report_cuda(cudaError_t e, const char* what, const char* file, int line) {
  std::fprintf(stderr, "biocfd_gb300: CUDA error %s (%s) at %s:%d: %s\n", cudaGetErrorName(e),
               cudaGetErrorString(e), file, line, what);
}

int note_launch(cudaError_t e) {
  if (e != cudaSuccess) {
    report_cuda(e, "kernel launch", __FILE__, __LINE__);
    return BCFD_E_CUDA;
  }
  lib().launches++;
  return 0;
}

HostBlock* get_block(bcfd_handle h) {
  Lib& L = lib();
  if (h < 1 || h > (bcfd_handle)L.blocks.size()) return nullptr;
  return L.blocks[(size_t)(h - 1)];
}
HostInterface* get_iface(bcfd_handle h) {
  Lib& L = lib();
  if (h < 1 || h > (bcfd_handle)L.ifs.size()) return nullptr;
  return L.ifs[(size_t)(h - 1)];
}

unsigned coop_grid(const void* fn, int threads, size_t smem, unsigned want) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
  if (per_sm < 1) per_sm = 1;
  unsigned cap = (unsigned)(per_sm * lib().nsm);
  if (want < 1) want = 1;
  return want < cap ? want : cap;
}

// cooperative launch (all CTAs co-resident) through cudaLaunchKernelEx, which
// stream capture records as a cooperative kernel node
cudaError_t launch_coop(const void* fn, unsigned grid, unsigned block, void** args, size_t smem) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream();
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelExC(&cfg, fn, args);
}

int sync_block_table() {
  Lib& L = lib();
  const size_t n = L.blocks.size();
  std::vector<DevBlock> cur(n);
  for (size_t q = 0; q < n; ++q) {
    if (L.blocks[q]) std::memcpy(&cur[q], &L.blocks[q]->d, sizeof(DevBlock));
    else std::memset(&cur[q], 0, sizeof(DevBlock));
  }
  if (n > L.dtab_cap) {
    if (L.dtab) cudaFree(L.dtab);
    L.dtab = nullptr;
    L.dtab_cap = 0;
    BCFD_CUDA(cudaMalloc(&L.dtab, n * sizeof(DevBlock)));
    L.dtab_cap = n;
    L.htab.clear();
    L.gen++;
  }
  if (cur.size() == L.htab.size() && std::memcmp(cur.data(), L.htab.data(), n * sizeof(DevBlock)) == 0)
    return 0;
  // a captured step must not contain this copy; the step key covers every
  // block view, so a change always ends the capture first
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  BCFD_CUDA(cudaStreamIsCapturing(stream(), &cs));
  if (cs != cudaStreamCaptureStatusNone) return BCFD_E_STATE;
  L.htab = cur;
  BCFD_CUDA(cudaMemcpyAsync(L.dtab, L.htab.data(), n * sizeof(DevBlock), cudaMemcpyHostToDevice, stream()));
  return 0;
}

namespace {
// One grid barrier whose arrival target is one CTA more than the launch has:
// nothing completes it, so every waiting CTA gives up after the wait limit
// (recording BCFD_E_TIMEOUT and setting the abandon bit, which releases the
// others at once).  Exercises the bounded-wait path of the persistent kernels.
__global__ void k_wait_unreachable(GridBar gb) { (void)grid_sync(gb); }
}  // namespace

GridBar make_bar(int* err, unsigned nblocks) {
  GridBar g{};
  g.err = err;
  g.nblocks = nblocks;
  g.limit_ns = lib().wait_limit_ns;
  return g;
}

int64_t* prof_log() { return lib().prof_on ? lib().prof_dev : nullptr; }

void prof_mark(bool /*begin*/) {
  Lib& L = lib();
  if (!L.prof_on) return;
  if (L.prof_used == L.prof_events.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    L.prof_events.push_back(e);
  }
  cudaEventRecord(L.prof_events[L.prof_used++], stream());
}

void phase_mark(int ph) {
  Lib& L = lib();
  if (!L.prof_on) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(stream(), &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
  if (L.phase_used == L.phase_events.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    L.phase_events.push_back(e);
    L.phase_ids.push_back(0);
  }
  L.phase_ids[L.phase_used] = ph;
  cudaEventRecord(L.phase_events[L.phase_used++], stream());
}

int take_block_error(HostBlock* hb) {
  int e = 0;
  BCFD_CUDA(cudaMemcpyAsync(&e, hb->d.err, sizeof(int), cudaMemcpyDeviceToHost, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  if (e) BCFD_CUDA(cudaMemsetAsync(hb->d.err, 0, sizeof(int), stream()));
  return e;
}

// The FP32 sweep tables of line tables Ax/Ay/Az (n,3): the x coefficients
// per float4 run and x-parity, then one float4 (3 coefficients + 0) per y row
// and per z row; 16-byte aligned offsets into f
void append_sweep_tables(const Dims& d, const std::vector<double>& Ax, const std::vector<double>& Ay,
                         const std::vector<double>& Az, std::vector<float>& f, size_t* axr_off, size_t* ayr_off,
                         size_t* azr_off) {
  while (f.size() % 4) f.push_back(0.0f);
  *axr_off = f.size();
  const int nx = d.nx, nq = d.NXH / 4;
  for (int par = 0; par < 2; ++par)
    for (int col = 0; col < 3; ++col)
      for (int run = 0; run < nq; ++run)
        for (int u = 0; u < 4; ++u) {
          const int ic = std::min(std::max(2 * (4 * run + u) + 1 + par, 2), nx + 1);
          f.push_back((float)Ax[(size_t)(ic - 2) + (size_t)col * nx]);
        }
  *ayr_off = f.size();
  for (int j = 0; j < d.ny; ++j)
    for (int col = 0; col < 4; ++col) f.push_back(col < 3 ? (float)Ay[(size_t)j + (size_t)col * d.ny] : 0.0f);
  *azr_off = f.size();
  for (int k = 0; k < d.nz; ++k)
    for (int col = 0; col < 4; ++col) f.push_back(col < 3 ? (float)Az[(size_t)k + (size_t)col * d.nz] : 0.0f);
}

namespace {

template <class T>
int dalloc(HostBlock* hb, T** p, size_t n) {
  if (n == 0) n = 1;
  if (cudaMalloc((void**)p, n * sizeof(T)) != cudaSuccess) return BCFD_E_NOMEM;
  hb->allocs.push_back(*p);
  if (cudaMemsetAsync(*p, 0, n * sizeof(T), stream()) != cudaSuccess) return BCFD_E_CUDA;
  return 0;
}

#define TRY(x) do { int _r = (x); if (_r) return _r; } while (0)

// x1 -> xu, xv/xw/xp (src/ReadInput.f90:310-351 and src/Search.F90:1234-1262)
void derive_staggered(HostBlock* hb) {
  const Dims& d = hb->d.d;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  hb->xu.assign(hb->x1.begin(), hb->x1.end());
  hb->yv.assign(hb->y1.begin(), hb->y1.end());
  hb->zw.assign(hb->z1.begin(), hb->z1.end());
  hb->yu.resize(ny + 2);
  hb->yw.resize(ny + 2);
  hb->yp.resize(ny + 2);
  for (int i = 0; i < ny + 2; ++i) hb->yu[i] = hb->yw[i] = hb->yp[i] = 0.5 * (hb->y1[i] + hb->y1[i + 1]);
  hb->xv.resize(nx + 2);
  hb->xw.resize(nx + 2);
  hb->xp.resize(nx + 2);
  for (int i = 0; i < nx + 2; ++i) hb->xv[i] = hb->xw[i] = hb->xp[i] = 0.5 * (hb->x1[i] + hb->x1[i + 1]);
  hb->zu.resize(nz + 2);
  hb->zv.resize(nz + 2);
  hb->zp.resize(nz + 2);
  for (int i = 0; i < nz + 2; ++i) hb->zu[i] = hb->zv[i] = hb->zp[i] = 0.5 * (hb->z1[i] + hb->z1[i + 1]);
}

// upload all 1-D grids into grid_buf and point the DevBlock at them
int upload_grids(HostBlock* hb) {
  std::vector<const std::vector<double>*> v = {&hb->x1, &hb->y1, &hb->z1, &hb->dxa, &hb->dya, &hb->dza,
                                               &hb->xu, &hb->yu, &hb->zu, &hb->xv, &hb->yv, &hb->zv,
                                               &hb->xw, &hb->yw, &hb->zw, &hb->xp, &hb->yp, &hb->zp};
  size_t tot = 0;
  for (auto* a : v) tot += a->size();
  std::vector<double> h(tot);
  std::vector<size_t> off;
  size_t o = 0;
  for (auto* a : v) {
    off.push_back(o);
    std::copy(a->begin(), a->end(), h.begin() + o);
    o += a->size();
  }
  if (!hb->grid_buf) TRY(dalloc(hb, &hb->grid_buf, tot));
  BCFD_CUDA(cudaMemcpyAsync(hb->grid_buf, h.data(), tot * sizeof(double), cudaMemcpyHostToDevice, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  const double** dst[18] = {&hb->d.x1, &hb->d.y1, &hb->d.z1, &hb->d.dxa, &hb->d.dya, &hb->d.dza,
                            &hb->d.xu, &hb->d.yu, &hb->d.zu, &hb->d.xv, &hb->d.yv, &hb->d.zv,
                            &hb->d.xw, &hb->d.yw, &hb->d.zw, &hb->d.xp, &hb->d.yp, &hb->d.zp};
  for (int q = 0; q < 18; ++q) *dst[q] = hb->grid_buf + off[q];
  std::vector<float> f;
  for (const auto* a : {&hb->dxa, &hb->dya, &hb->dza})
    for (double x : *a) f.push_back((float)x);
  if (!hb->grid_f32) TRY(dalloc(hb, &hb->grid_f32, f.size()));
  BCFD_CUDA(cudaMemcpyAsync(hb->grid_f32, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  hb->d.dxf = hb->grid_f32;
  hb->d.dyf = hb->grid_f32 + hb->dxa.size();
  hb->d.dzf = hb->grid_f32 + hb->dxa.size() + hb->dya.size();
  // per-line tables: correctVelocity's factors (first half, filled per deltat
  // on the device) and the reciprocal spacings (second half, here)
  const size_t nl = hb->dxa.size() + hb->dya.size() + hb->dza.size();
  if (!hb->lcoef) TRY(dalloc(hb, &hb->lcoef, 2 * nl));
  std::vector<double> rec;
  for (const auto* a : {&hb->dxa, &hb->dya, &hb->dza})
    for (double x : *a) rec.push_back(1.0 / x);
  BCFD_CUDA(cudaMemcpyAsync(hb->lcoef + nl, rec.data(), nl * sizeof(double), cudaMemcpyHostToDevice, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  hb->d.lcoef = hb->lcoef;
  hb->lcoef_dt = 0.0;  // the spacings may have changed
  return 0;
}

// ---------------------------------------------------------------------------
// non_uni_coeff (src/NavierStokes.f90:13-250, compute_f/s/ak :915-996).
// Fortran integer powers x**n are repeated products ((x*x)*x, (x*x)*(x*x));
// the real powers x**2.0 / x**3.0 / x**4.0 are x*x / pow(x,3) / pow(x,4).
// ---------------------------------------------------------------------------
inline double q2(double x) { return x * x; }
inline double q3(double x) { return (x * x) * x; }
inline double q4(double x) {
  const double s = x * x;
  return s * s;
}

void coef_column(double t1, double t2, double t3, double* ca, double* ck) {
  double f[9];
  f[1] = t3;
  f[2] = 2.0 * t3 + q2(t3);
  f[3] = 3.0 * t3 + 3.0 * q2(t3) + q3(t3);
  f[4] = 4.0 * t3 + 6.0 * q2(t3) + 4.0 * q3(t3) + q4(t3);
  f[5] = 1.0 / (t1 * t2);
  f[6] = (2.0 * t1 + 1.0) / (q2(t1) * q2(t2));
  f[7] = (3.0 * q2(t1) + 3.0 * t1 + 1.0) / (q3(t1) * q3(t2));
  f[8] = (4.0 * q3(t1) + 6.0 * q2(t1) + 4.0 * t1 + 1.0) / (q4(t1) * q4(t2));
  double s5[8], s6[8], s7[7], s8[7], s9[8], s10[8];
  s5[1] = -1.0 / q4(t2);
  s5[2] = f[4];
  s5[3] = f[4];
  s5[4] = s5[1];
  s5[5] = -(f[1] / q4(t2) + f[4] / t2);
  s5[6] = (f[4] / q2(t2) - f[2] / q4(t2));
  s5[7] = -(f[3] / q4(t2) + f[4] / q3(t2));
  s6[1] = -1.0;
  s6[2] = f[8];
  s6[3] = f[8];
  s6[4] = -1.0;
  s6[5] = (f[5] + f[8]);
  s6[6] = (f[8] - f[6]);
  s6[7] = (f[7] + f[8]);
  s7[1] = -1.0;
  s7[2] = (1.0 + f[4]);
  s7[3] = f[4];
  s7[4] = (f[4] - f[1]);
  s7[5] = (f[4] - f[2]);
  s7[6] = (f[4] - f[3]);
  const double r4 = std::pow(t2, 4.0), r2 = t2 * t2, r3 = std::pow(t2, 3.0);
  s8[1] = -1.0 / r4;
  s8[2] = (f[8] + (1.0 / r4));
  s8[3] = f[8];
  s8[4] = (f[5] / r4 - f[8] / t2);
  s8[5] = (f[8] / r2 - f[6] / r4);
  s8[6] = (f[7] / r4 - f[8] / r3);
  s9[1] = -s6[6] * s5[1];
  s9[2] = s5[6] * s6[1];
  s9[3] = -(s5[4] * s6[6] + s5[6] * s6[2]);
  s9[4] = (s5[6] * s6[4] + s6[6] * s5[2]);
  s9[5] = (s5[6] * s6[3] - s6[6] * s5[3]);
  s9[6] = (s5[6] * s6[5] - s6[6] * s5[5]);
  s9[7] = (s5[6] * s6[7] - s6[6] * s5[7]);
  s10[1] = -s8[5] * s7[1];
  s10[2] = -s8[5] * s7[2];
  s10[3] = s7[5] * s8[1];
  s10[4] = s7[5] * s8[2];
  s10[5] = (s7[5] * s8[3] - s8[5] * s7[3]);
  s10[6] = (s7[5] * s8[4] - s8[5] * s7[4]);
  s10[7] = (s7[5] * s8[6] - s8[5] * s7[6]);
  ca[0] = s9[7] * s10[1] - s10[7] * s9[1];
  ca[1] = s9[7] * s10[2] + s10[7] * s9[3];
  ca[2] = s9[5] * s10[7] - s10[5] * s9[7];
  ca[3] = s9[4] * s10[7] + s10[4] * s9[7];
  ca[4] = s9[7] * s10[3] - s10[7] * s9[2];
  ca[5] = s9[7] * s10[6] - s10[7] * s9[6];
  double ak[8];
  ak[1] = (1.0 + 2.0 * t1) * (t3 + q2(t3)) * t2;
  ak[2] = (1.0 + t1) * (2.0 * t3 + q2(t3));
  ak[3] = (1.0 + t1);
  ak[4] = (1.0 + t1) * q2(1.0 + t3);
  ak[5] = q2(1.0 + t1) * (t3 + q2(t3)) * t2;
  ak[6] = q2(t1) * t2 * (t3 + q2(t3));
  ak[7] = (1.0 + t1) * (t3 + q2(t3)) * t2;
  ck[0] = ak[3];
  ck[1] = -ak[4];
  ck[2] = ak[1] + ak[2];
  ck[3] = -ak[5];
  ck[4] = ak[6];
  ck[5] = ak[7];
}

void build_coefs(HostBlock* hb) {
  const Dims& d = hb->d.d;
  const int n3[3] = {d.nx, d.ny, d.nz};
  const std::vector<double>* del[3] = {&hb->dxa, &hb->dya, &hb->dza};
  const int same[3] = {T_UU, T_VV, T_WW};
  const int cross[3][2] = {{T_UV, T_UW}, {T_VU, T_VW}, {T_WU, T_WV}};
  for (int a = 0; a < 3; ++a) {
    const int n = n3[a];
    const std::vector<double>& D = *del[a];
    auto Dl = [&](int i) { return D[(size_t)(i - 1)]; };  // 1-based
    for (int t : {same[a], cross[a][0], cross[a][1]}) {
      hb->ca[t].assign(6 * (size_t)(n + 2), 0.0);
      hb->ck[t].assign(6 * (size_t)(n + 2), 0.0);
    }
    for (int i = 2; i <= n; ++i) {
      coef_column(Dl(i) / Dl(i - 1), Dl(i + 1) / Dl(i), Dl(i + 2) / Dl(i + 1),
                  &hb->ca[same[a]][6 * (size_t)(i - 1)], &hb->ck[same[a]][6 * (size_t)(i - 1)]);
      const double tt1 = i == 2 ? Dl(i - 1) : 0.5 * (Dl(i - 1) + Dl(i - 2));
      const double tt2 = 0.5 * (Dl(i) + Dl(i - 1));
      const double tt3 = 0.5 * (Dl(i) + Dl(i + 1));
      const double tt4 = 0.5 * (Dl(i + 1) + Dl(i + 2));
      double* c0 = &hb->ca[cross[a][0]][6 * (size_t)(i - 1)];
      double* k0 = &hb->ck[cross[a][0]][6 * (size_t)(i - 1)];
      coef_column(tt2 / tt1, tt3 / tt2, tt4 / tt3, c0, k0);
      std::copy(c0, c0 + 6, &hb->ca[cross[a][1]][6 * (size_t)(i - 1)]);
      std::copy(k0, k0 + 6, &hb->ck[cross[a][1]][6 * (size_t)(i - 1)]);
    }
  }
}

// coefficientMatrix, src/CoefficientMatrix.f90:10-71
void build_poisson_coefs(HostBlock* hb, bool is_coarse) {
  const Dims& d = hb->d.d;
  auto line = [](const std::vector<double>& P, int n, std::vector<double>& A) {
    A.assign(3 * (size_t)n, 0.0);
    for (int i = 2; i <= n + 1; ++i) {
      const double r1 = P[i - 1] - P[i - 2], r2 = P[i] - P[i - 1], rs = r1 + r2;
      A[(i - 2)] = 2.0 / (r1 * rs);
      A[(i - 2) + n] = -2.0 / (r1 * r2);
      A[(i - 2) + 2 * n] = 2.0 / (r2 * rs);
    }
  };
  line(hb->yp, d.ny, hb->Acy);
  line(hb->xp, d.nx, hb->Acx);
  line(hb->zp, d.nz, hb->Acz);
  if (is_coarse) {
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    auto& X = hb->Acx;
    auto& Y = hb->Acy;
    auto& Z = hb->Acz;
    X[0 + nx] = X[0 + nx] - X[0];
    X[0] = 0.0;
    X[(nx - 1) + nx] = X[(nx - 1) + nx] - X[(nx - 1) + 2 * nx];
    X[(nx - 1) + 2 * nx] = 0.0;
    Y[0 + ny] = Y[0 + ny] + Y[0];
    Y[0] = 0.0;
    Y[(ny - 1) + ny] = Y[(ny - 1) + ny] + Y[(ny - 1) + 2 * ny];
    Y[(ny - 1) + 2 * ny] = 0.0;
    Z[0 + nz] = Z[0 + nz] + Z[0];
    Z[0] = 0.0;
    Z[(nz - 1) + nz] = Z[(nz - 1) + nz] + Z[(nz - 1) + 2 * nz];
    Z[(nz - 1) + 2 * nz] = 0.0;
  }
}

int upload_coefs(HostBlock* hb) {
  size_t tot = hb->Acx.size() + hb->Acy.size() + hb->Acz.size();
  for (int t = 0; t < N_TAB; ++t) tot += hb->ca[t].size() + hb->ck[t].size();
  std::vector<double> h;
  h.reserve(tot);
  std::vector<size_t> off;
  auto put = [&](const std::vector<double>& v) {
    off.push_back(h.size());
    h.insert(h.end(), v.begin(), v.end());
  };
  put(hb->Acx);
  put(hb->Acy);
  put(hb->Acz);
  for (int t = 0; t < N_TAB; ++t) put(hb->ca[t]);
  for (int t = 0; t < N_TAB; ++t) put(hb->ck[t]);
  if (hb->coef_buf) {
    cudaFree(hb->coef_buf);
    hb->allocs.erase(std::remove(hb->allocs.begin(), hb->allocs.end(), (void*)hb->coef_buf), hb->allocs.end());
    hb->coef_buf = nullptr;
  }
  TRY(dalloc(hb, &hb->coef_buf, std::max<size_t>(h.size(), 1)));
  BCFD_CUDA(cudaMemcpyAsync(hb->coef_buf, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  hb->d.Acx = hb->coef_buf + off[0];
  hb->d.Acy = hb->coef_buf + off[1];
  hb->d.Acz = hb->coef_buf + off[2];
  {
    std::vector<float> f;
    for (const auto* v : {&hb->Acx, &hb->Acy, &hb->Acz})
      for (double x : *v) f.push_back((float)x);
    std::vector<size_t> foff;
    for (int t = 0; t < 2 * N_TAB; ++t) {
      foff.push_back(f.size());
      for (double x : (t < N_TAB ? hb->ca[t] : hb->ck[t - N_TAB])) f.push_back((float)x);
    }
    size_t axr_off, ayr_off, azr_off;
    append_sweep_tables(hb->d.d, hb->Acx, hb->Acy, hb->Acz, f, &axr_off, &ayr_off, &azr_off);
    if (hb->coef_f32) {
      cudaFree(hb->coef_f32);
      hb->allocs.erase(std::remove(hb->allocs.begin(), hb->allocs.end(), (void*)hb->coef_f32), hb->allocs.end());
      hb->coef_f32 = nullptr;
    }
    TRY(dalloc(hb, &hb->coef_f32, std::max<size_t>(f.size(), 1)));
    BCFD_CUDA(cudaMemcpyAsync(hb->coef_f32, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice, stream()));
    BCFD_CUDA(cudaStreamSynchronize(stream()));
    hb->d.Acxf = hb->coef_f32;
    hb->d.Acyf = hb->coef_f32 + hb->Acx.size();
    hb->d.Aczf = hb->coef_f32 + hb->Acx.size() + hb->Acy.size();
    hb->d.axr = reinterpret_cast<const float4*>(hb->coef_f32 + axr_off);
    hb->d.ayr = reinterpret_cast<const float4*>(hb->coef_f32 + ayr_off);
    hb->d.azr = reinterpret_cast<const float4*>(hb->coef_f32 + azr_off);
    for (int t = 0; t < N_TAB; ++t) {
      hb->d.caf[t] = hb->coef_f32 + foff[t];
      hb->d.ckf[t] = hb->coef_f32 + foff[N_TAB + t];
    }
  }
  for (int t = 0; t < N_TAB; ++t) {
    hb->d.ca[t] = hb->coef_buf + off[3 + t];
    hb->d.ck[t] = hb->coef_buf + off[3 + N_TAB + t];
  }
  return 0;
}

// int64 host tags <-> int8 device tags
int up_tags(const int64_t* src, int8_t* dst, int64_t n) {
  if (!src) return 0;
  std::vector<int8_t> h((size_t)n);
  for (int64_t q = 0; q < n; ++q) h[(size_t)q] = (int8_t)src[q];
  BCFD_CUDA(cudaMemcpyAsync(dst, h.data(), n, cudaMemcpyHostToDevice, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  return 0;
}
int down_tags(const int8_t* src, int64_t* dst, int64_t n) {
  if (!dst) return 0;
  std::vector<int8_t> h((size_t)n);
  BCFD_CUDA(cudaMemcpyAsync(h.data(), src, n, cudaMemcpyDeviceToHost, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  for (int64_t q = 0; q < n; ++q) dst[q] = h[(size_t)q];
  return 0;
}

int upload(double* dst, const double* src, int64_t n) {
  if (!src) return 0;
  BCFD_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, stream()));
  return 0;
}
int download(const double* src, double* dst, int64_t n) {
  if (!dst) return 0;
  BCFD_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, stream()));
  return 0;
}

int alloc_surface(HostBlock* hb, int ne, int nn) {
  DevBlock& D = hb->d;
  if (ne > hb->surf_cap_e) {
    int* p;
    double* f;
    TRY(dalloc(hb, &p, (size_t)ne * 4));
    D.elp1 = p;
    D.elp2 = p + ne;
    D.elp3 = p + 2 * (size_t)ne;
    D.surf_id = p + 3 * (size_t)ne;
    TRY(dalloc(hb, &f, (size_t)ne * 7));
    D.xcent = f;
    D.ycent = f + ne;
    D.zcent = f + 2 * (size_t)ne;
    D.cosA = f + 3 * (size_t)ne;
    D.cosB = f + 4 * (size_t)ne;
    D.cosG = f + 5 * (size_t)ne;
    D.elen = f + 6 * (size_t)ne;
    hb->surf_cap_e = ne;
  }
  if (nn > hb->surf_cap_n) {
    double* f;
    TRY(dalloc(hb, &f, (size_t)nn * 3));
    D.xnode1 = f;
    D.ynode1 = f + nn;
    D.znode1 = f + 2 * (size_t)nn;
    hb->surf_cap_n = nn;
  }
  D.ne = ne;
  D.nn = nn;
  return 0;
}

}  // namespace

// change_block_coords (src/Search.F90:1208-1264): the faces move by whole
// cells, the staggered and centre coordinates follow, the spacings stay
int shift_block_grid(HostBlock* hb, double cx, double cy, double cz) {
  // the search's bound on |node - block centre| holds for the moved centre
  // after growing by the shift (triangle inequality)
  if (hb->node_rmax > 0.0) hb->node_rmax += std::sqrt(cx * cx + cy * cy + cz * cz);
  for (double& x : hb->x1) x = x + cx;
  for (double& y : hb->y1) y = y + cy;
  for (double& z : hb->z1) z = z + cz;
  derive_staggered(hb);
  return upload_grids(hb);
}
}  // namespace bcfd

using namespace bcfd;

#define LOCK() ::bcfd::LibLock _lk
#define GETB(h)                      \
  HostBlock* hb = get_block(h);      \
  if (!hb) return BCFD_E_HANDLE;

extern "C" {

int bcfd_init(int device) {
  LOCK();
  Lib& L = lib();
  if (L.ready) return 0;
  BCFD_CUDA(cudaSetDevice(device));
  cudaDeviceProp prop;
  BCFD_CUDA(cudaGetDeviceProperties(&prop, device));
  L.nsm = prop.multiProcessorCount;
  L.device = device;
  BCFD_CUDA(cudaStreamCreateWithFlags(&L.s, cudaStreamNonBlocking));
  L.ready = true;
  return 0;
}

int bcfd_set_wait_limit_ns(int64_t ns) {
  LOCK();
  if (ns < 0 || ns > 600000000000ll) return BCFD_E_ARG;
  lib().wait_limit_ns = ns == 0 ? kBarrierLimitNs : (uint64_t)ns;
  return 0;
}

int bcfd_check_wait_limit(int* status, double* waited_ms) {
  LOCK();
  if (!lib().ready) return BCFD_E_STATE;
  if (!status) return BCFD_E_ARG;
  // [0] arrival counter (8 bytes), [1] error word
  unsigned long long* w = nullptr;
  BCFD_CUDA(cudaMalloc(&w, 2 * sizeof(unsigned long long)));
  int r = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  auto ck = [&](cudaError_t e) {
    if (e != cudaSuccess && !r) {
      report_cuda(e, "check_wait_limit", __FILE__, __LINE__);
      r = BCFD_E_CUDA;
    }
  };
  ck(cudaMemsetAsync(w, 0, 2 * sizeof(unsigned long long), stream()));
  ck(cudaEventCreate(&e0));
  ck(cudaEventCreate(&e1));
  if (!r) {
    const unsigned ctas = 2;
    GridBar gb = make_bar(reinterpret_cast<int*>(w + 1), ctas + 1);
    gb.ctr = w;
    ck(cudaEventRecord(e0, stream()));
    k_wait_unreachable<<<ctas, 32, 0, stream()>>>(gb);
    r = note_launch();
    ck(cudaEventRecord(e1, stream()));
  }
  int e = 0;
  if (!r) ck(cudaMemcpyAsync(&e, w + 1, sizeof(int), cudaMemcpyDeviceToHost, stream()));
  ck(cudaStreamSynchronize(stream()));
  float ms = 0.0f;
  if (!r) ck(cudaEventElapsedTime(&ms, e0, e1));
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(w);
  if (r) return r;
  *status = e;
  if (waited_ms) *waited_ms = ms;
  return 0;
}

int bcfd_block_set_list_capacity(bcfd_handle h, int64_t cap) {
  LOCK();
  GETB(h);
  if (cap < 0 || cap > hb->cap_ib_alloc) return BCFD_E_ARG;
  hb->d.cap_ib = cap == 0 ? hb->cap_ib_alloc : (int)cap;
  return 0;
}

int bcfd_set_warm_start(int on) {
  LOCK();
  lib().warm_start = on != 0;
  return 0;
}

int bcfd_set_batching(int on) {
  LOCK();
  lib().batch = on != 0;
  return 0;
}

int bcfd_finalize(void) {
  LOCK();
  Lib& L = lib();
  if (!L.ready) return 0;
  cudaStreamSynchronize(L.s);
  if (L.step_graph) cudaGraphExecDestroy(L.step_graph);
  L.step_graph = nullptr;
  L.step_key.clear();
  for (HostBlock* hb : L.blocks)
    if (hb) {
      for (void* p : hb->allocs) cudaFree(p);
      free_search_scratch(hb);
      free_dag_scratch(hb);
      delete hb;
    }
  for (HostInterface* it : L.ifs)
    if (it) {
      if (it->dtab) cudaFree(it->dtab);
      delete it;
    }
  L.blocks.clear();
  if (L.dtab) cudaFree(L.dtab);
  L.dtab = nullptr;
  L.dtab_cap = 0;
  L.htab.clear();
  L.ifs.clear();
  cudaStreamDestroy(L.s);
  L.s = nullptr;
  L.ready = false;
  return 0;
}

int bcfd_synchronize(void) {
  LOCK();
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  return 0;
}

int bcfd_get_stream(void** s) {
  if (!s) return BCFD_E_ARG;
  *s = (void*)lib().s;
  return 0;
}

int64_t bcfd_kernel_launches(void) { return lib().launches; }

const char* bcfd_status_string(int st) {
  switch (st) {
    case BCFD_OK: return "ok";
    case BCFD_E_HANDLE: return "unknown handle";
    case BCFD_E_NOMEM: return "device allocation failed";
    case BCFD_E_NONFINITE: return "non-finite value in a residual or reduction";
    case BCFD_E_NOTFOUND: return "probe bracket not found";
    case BCFD_E_TIMEOUT: return "device-side wait gave up";
    case BCFD_E_ARG: return "invalid argument";
    case BCFD_E_CUDA: return "CUDA runtime error";
    case BCFD_E_STATE: return "call out of order";
    case BCFD_E_CAPACITY: return "list outgrew its device capacity";
    default: return "unknown status";
  }
}

int bcfd_block_create(int64_t nx, int64_t ny, int64_t nz, const double* x1, const double* y1,
                      const double* z1, const double* deltax, const double* deltay,
                      const double* deltaz, bcfd_handle* out) {
  LOCK();
  if (!lib().ready) return BCFD_E_STATE;
  if (nx < 2 || ny < 2 || nz < 2 || !x1 || !y1 || !z1 || !deltax || !deltay || !deltaz || !out)
    return BCFD_E_ARG;
  HostBlock* hb = new HostBlock();
  Dims& d = hb->d.d;
  d.nx = (int)nx;
  d.ny = (int)ny;
  d.nz = (int)nz;
  d.NX = d.nx + 2;
  d.NY = d.ny + 2;
  d.NZ = d.nz + 2;
  // packed row pitch: (NX+1)/2 cells rounded up to 4 so rows start 16-byte
  // aligned (vector loads); the padding slots are never updated
  d.NXH = (((d.NX + 1) / 2) + 3) & ~3;
  const int64_t np = d.npts(), np3 = d.npts3(), npk = d.npacked();
  DevBlock& D = hb->d;
  int r = 0;
  auto A = [&](auto** p, size_t n) {
    if (!r) r = dalloc(hb, p, n);
  };
  A(&D.u, np); A(&D.v, np); A(&D.w, np); A(&D.p, np); A(&D.ut, np); A(&D.vt, np); A(&D.wt, np);
  A(&D.cell, np); A(&D.cell_n, np); A(&D.tsnear, np); A(&D.cell2, np3); A(&D.nodeTag, np3); A(&D.cell_pr, np3);
  for (int c = 0; c < 2; ++c) {
    A(&D.pc[c], npk); A(&D.rhs[c], npk); A(&D.bpk[c], npk); A(&D.upd[c], npk);
    A(&D.pcf[c], npk); A(&D.rhsf[c], npk);
  }
  // IB / TS list capacity: every cell up to 4M cells (a list that outgrows it
  // reports BCFD_E_CAPACITY)
  D.cap_ib = (int)std::max<int64_t>(64, std::min<int64_t>((int64_t)nx * ny * nz, (int64_t)1 << 22));
  hb->cap_ib_alloc = D.cap_ib;
  A(&D.ib_i, D.cap_ib); A(&D.ib_j, D.cap_ib); A(&D.ib_k, D.cap_ib);
  for (int q = 0; q < 7; ++q) { A(&D.nel[q], D.cap_ib); A(&D.nd[q], D.cap_ib); }
  A(&D.ts_idx, D.cap_ib);
  for (int q = 0; q < 14; ++q) A(&D.ghost[q], D.cap_ib);
  A(&D.ibmap, np);
  A(&D.cnt, 16);
  A(&D.err, 1);
  A(&D.scratch, 64);
  A(&D.stats, 1);
  A(&hb->bar, 2);
  A(&hb->prog, (size_t)kMaxTiles * kTileStride);
  A(&hb->kin_dev, 1);
  A(&hb->stage_dev, 1);
  if (r) {
    for (void* p : hb->allocs) cudaFree(p);
    delete hb;
    return r;
  }
  hb->stats = D.stats;
  D.kin = hb->kin_dev;
  for (int q = 0; q < 6; ++q) D.box[q] = q & 1 ? -1 : 0;
  hb->x1.assign(x1, x1 + nx + 3);
  hb->y1.assign(y1, y1 + ny + 3);
  hb->z1.assign(z1, z1 + nz + 3);
  hb->dxa.assign(deltax, deltax + nx + 2);
  hb->dya.assign(deltay, deltay + ny + 2);
  hb->dza.assign(deltaz, deltaz + nz + 2);
  derive_staggered(hb);
  if ((r = upload_grids(hb))) return r;
  hb->dx = hb->dxa[1];
  hb->dy = hb->dya[1];
  hb->dz = hb->dza[1];
  hb->index = (int)lib().blocks.size();
  lib().blocks.push_back(hb);
  *out = (bcfd_handle)lib().blocks.size();
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  return 0;
}

int bcfd_block_destroy(bcfd_handle h) {
  LOCK();
  GETB(h);
  cudaStreamSynchronize(stream());
  for (void* p : hb->allocs) cudaFree(p);
  free_search_scratch(hb);
  free_dag_scratch(hb);
  delete hb;
  lib().blocks[(size_t)(h - 1)] = nullptr;
  return 0;
}

int bcfd_block_set_grid(bcfd_handle h, const double* x1, const double* y1, const double* z1) {
  LOCK();
  GETB(h);
  const Dims& d = hb->d.d;
  if (!x1 || !y1 || !z1) return BCFD_E_ARG;
  hb->x1.assign(x1, x1 + d.nx + 3);
  hb->y1.assign(y1, y1 + d.ny + 3);
  hb->z1.assign(z1, z1 + d.nz + 3);
  derive_staggered(hb);
  return upload_grids(hb);
}

int bcfd_block_set_scalars(bcfd_handle h, double dx, double dy, double dz, double omega) {
  LOCK();
  GETB(h);
  hb->dx = dx;
  hb->dy = dy;
  hb->dz = dz;
  hb->omega = omega;
  return 0;
}

int bcfd_block_set_search_box(bcfd_handle h, int64_t i0, int64_t i1, int64_t j0, int64_t j1,
                              int64_t k0, int64_t k1) {
  LOCK();
  GETB(h);
  const Dims& d = hb->d.d;
  // the tagging loops read x1(i+1) and nodeIdTag(i+1): the box must lie in 1..n+2
  if (i0 < 1 || j0 < 1 || k0 < 1 || i1 > d.nx + 2 || j1 > d.ny + 2 || k1 > d.nz + 2) return BCFD_E_ARG;
  const int64_t b[6] = {i0, i1, j0, j1, k0, k1};
  for (int q = 0; q < 6; ++q) hb->d.box[q] = (int)b[q];
  return 0;
}

int bcfd_block_set_surface(bcfd_handle h, int64_t n_elems, int64_t n_nodes, const int64_t* elp1,
                           const int64_t* elp2, const int64_t* elp3, const int64_t* surf_id,
                           const double* xnode1, const double* ynode1, const double* znode1) {
  LOCK();
  GETB(h);
  if (n_elems < 0 || n_nodes < 0 || (n_elems && (!elp1 || !elp2 || !elp3 || !surf_id)) ||
      (n_nodes && (!xnode1 || !ynode1 || !znode1)))
    return BCFD_E_ARG;
  for (int64_t e = 0; e < n_elems; ++e)
    if (elp1[e] < 1 || elp1[e] > n_nodes || elp2[e] < 1 || elp2[e] > n_nodes || elp3[e] < 1 ||
        elp3[e] > n_nodes)
      return BCFD_E_ARG;
  TRY(alloc_surface(hb, (int)n_elems, (int)n_nodes));
  std::vector<int> ids(4 * (size_t)n_elems);
  for (int64_t e = 0; e < n_elems; ++e) {
    ids[e] = (int)elp1[e];
    ids[n_elems + e] = (int)elp2[e];
    ids[2 * n_elems + e] = (int)elp3[e];
    ids[3 * n_elems + e] = (int)surf_id[e];
  }
  if (n_elems)
    BCFD_CUDA(cudaMemcpyAsync((void*)hb->d.elp1, ids.data(), ids.size() * sizeof(int), cudaMemcpyHostToDevice, stream()));
  hb->elem_host = ids;
  hb->has_body = n_elems > 0;
  // the search's element order: Morton order of the centroids (30-bit code
  // on the centroids' bounding box, ties by index), so that runs of 32
  // consecutive elements are spatially compact; only the pruning of the
  // nearest-element queries depends on it, never a result
  {
    std::vector<double> cx((size_t)n_elems), cy((size_t)n_elems), cz((size_t)n_elems);
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t e = 0; e < n_elems; ++e) {
      const int64_t a0 = elp1[e] - 1, a1 = elp2[e] - 1, a2 = elp3[e] - 1;
      cx[e] = (xnode1[a0] + xnode1[a1] + xnode1[a2]) / 3.0;
      cy[e] = (ynode1[a0] + ynode1[a1] + ynode1[a2]) / 3.0;
      cz[e] = (znode1[a0] + znode1[a1] + znode1[a2]) / 3.0;
      const double c3[3] = {cx[e], cy[e], cz[e]};
      for (int q = 0; q < 3; ++q) {
        lo[q] = std::min(lo[q], c3[q]);
        hi[q] = std::max(hi[q], c3[q]);
      }
    }
    auto spread = [](uint32_t v) {  // 10 bits -> every third bit
      v &= 0x3ffu;
      v = (v | (v << 16)) & 0x30000ffu;
      v = (v | (v << 8)) & 0x300f00fu;
      v = (v | (v << 4)) & 0x30c30c3u;
      v = (v | (v << 2)) & 0x9249249u;
      return v;
    };
    std::vector<std::pair<uint32_t, int>> key((size_t)n_elems);
    for (int64_t e = 0; e < n_elems; ++e) {
      const double c3[3] = {cx[e], cy[e], cz[e]};
      uint32_t g[3];
      for (int q = 0; q < 3; ++q) {
        const double span = hi[q] - lo[q];
        const double t = span > 0.0 ? (c3[q] - lo[q]) / span : 0.0;
        g[q] = (uint32_t)std::min(1023.0, std::max(0.0, std::floor(t * 1023.0)));
      }
      key[(size_t)e] = {spread(g[0]) | (spread(g[1]) << 1) | (spread(g[2]) << 2), (int)e};
    }
    std::sort(key.begin(), key.end());
    hb->elem_perm.resize((size_t)n_elems);
    for (int64_t q = 0; q < n_elems; ++q) hb->elem_perm[(size_t)q] = key[(size_t)q].second;
    hb->elem_perm_gen++;
  }
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  // findDistnode (src/Search.F90:21-47) on the nodes as given, with the node
  // tags readSurfaceMeshGmsh derives from the elements (51/52 first, then 50):
  // mk is the last surface-51 node whose |z| exceeds the running value,
  // mkx1 / mkx2 those of |x| below / above theirs; the running values keep
  // the signed coordinate, as the reference does
  {
    std::vector<int> nid((size_t)n_nodes, 50);
    for (int64_t e = 0; e < n_elems; ++e)
      if (surf_id[e] == 51 || surf_id[e] == 52)
        for (const int64_t* p : {elp1, elp2, elp3}) nid[(size_t)p[e] - 1] = (int)surf_id[e];
    for (int64_t e = 0; e < n_elems; ++e)
      if (surf_id[e] == 50)
        for (const int64_t* p : {elp1, elp2, elp3}) nid[(size_t)p[e] - 1] = 50;
    double dist = 0.0, dist1 = 999999.0, dist2 = 0.0;
    hb->mk = hb->mkx1 = hb->mkx2 = 0;
    for (int64_t i = 0; i < n_nodes; ++i) {
      if (nid[(size_t)i] != 51) continue;
      if (std::fabs(znode1[i]) > dist) dist = znode1[i], hb->mk = i + 1;
      if (std::fabs(xnode1[i]) < dist1) dist1 = xnode1[i], hb->mkx1 = i + 1;
      if (std::fabs(xnode1[i]) > dist2) dist2 = xnode1[i], hb->mkx2 = i + 1;
    }
  }
  return bcfd_block_set_nodes(h, xnode1, ynode1, znode1);
}

int bcfd_block_set_nodes(bcfd_handle h, const double* x, const double* y, const double* z) {
  LOCK();
  GETB(h);
  const int nn = hb->d.nn;
  if (nn == 0) return 0;
  if (!x || !y || !z) return BCFD_E_ARG;
  BCFD_CUDA(cudaMemcpyAsync((void*)hb->d.xnode1, x, nn * sizeof(double), cudaMemcpyHostToDevice, stream()));
  BCFD_CUDA(cudaMemcpyAsync((void*)hb->d.ynode1, y, nn * sizeof(double), cudaMemcpyHostToDevice, stream()));
  BCFD_CUDA(cudaMemcpyAsync((void*)hb->d.znode1, z, nn * sizeof(double), cudaMemcpyHostToDevice, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  const Dims& d = hb->d.d;
  const double cx = 0.5 * (hb->x1[0] + hb->x1[d.nx + 2]), cy = 0.5 * (hb->y1[0] + hb->y1[d.ny + 2]),
               cz = 0.5 * (hb->z1[0] + hb->z1[d.nz + 2]);
  double r2 = 0.0;
  for (int q = 0; q < nn; ++q)
    r2 = std::max(r2, (x[q] - cx) * (x[q] - cx) + (y[q] - cy) * (y[q] - cy) + (z[q] - cz) * (z[q] - cz));
  hb->node_rmax = std::sqrt(r2);
  return 0;
}

// node surface ids from the elements (src/ReadInput.f90:403-420): 50 by
// default; nodes of surface-51/52 elements take that id, then nodes of
// surface-50 elements are set back to 50
static std::vector<int8_t> node_ids(const HostBlock* hb) {
  const int nn = hb->d.nn, ne = hb->d.ne;
  std::vector<int8_t> id((size_t)nn, 50);
  const std::vector<int>& e = hb->elem_host;
  for (int q = 0; q < ne; ++q) {
    const int s = e[3 * (size_t)ne + q];
    if (s == 51 || s == 52)
      for (int c = 0; c < 3; ++c) id[(size_t)e[c * (size_t)ne + q] - 1] = (int8_t)s;
  }
  for (int q = 0; q < ne; ++q)
    if (e[3 * (size_t)ne + q] == 50)
      for (int c = 0; c < 3; ++c) id[(size_t)e[c * (size_t)ne + q] - 1] = 50;
  return id;
}

int bcfd_block_set_body_motion(bcfd_handle h, const double* p) {
  LOCK();
  GETB(h);
  if (!p || hb->d.nn <= 0) return BCFD_E_ARG;
  BodyMotion& m = hb->motion;
  m = BodyMotion{};
  m.on = true;
  m.a0 = p[0];
  m.bfreq = p[1];
  m.yamp = p[2];
  m.xshift = p[3];
  m.yshift = p[4];
  m.zshift = p[5];
  const int nn = hb->d.nn;
  if (!hb->d.xnode0) {
    double* f;
    TRY(dalloc(hb, &f, (size_t)nn * 3));
    hb->d.xnode0 = f;
    hb->d.ynode0 = f + nn;
    hb->d.znode0 = f + 2 * (size_t)nn;
    int8_t* id;
    TRY(dalloc(hb, &id, (size_t)nn));
    hb->d.node_id = id;
  }
  // the nodes given with the surface are the body frame
  BCFD_CUDA(cudaMemcpyAsync((void*)hb->d.xnode0, hb->d.xnode1, nn * sizeof(double), cudaMemcpyDeviceToDevice, stream()));
  BCFD_CUDA(cudaMemcpyAsync((void*)hb->d.ynode0, hb->d.ynode1, nn * sizeof(double), cudaMemcpyDeviceToDevice, stream()));
  BCFD_CUDA(cudaMemcpyAsync((void*)hb->d.znode0, hb->d.znode1, nn * sizeof(double), cudaMemcpyDeviceToDevice, stream()));
  const std::vector<int8_t> id = node_ids(hb);
  BCFD_CUDA(cudaMemcpyAsync((void*)hb->d.node_id, id.data(), id.size(), cudaMemcpyHostToDevice, stream()));
  // bound on the moving nodes' distance from the block centre: body-frame
  // radius, the rotation about the pivot line, and the largest translation
  double r0 = 0.0;
  {
    std::vector<double> x(nn), y(nn), z(nn);
    BCFD_CUDA(cudaMemcpyAsync(x.data(), hb->d.xnode0, nn * sizeof(double), cudaMemcpyDeviceToHost, stream()));
    BCFD_CUDA(cudaMemcpyAsync(y.data(), hb->d.ynode0, nn * sizeof(double), cudaMemcpyDeviceToHost, stream()));
    BCFD_CUDA(cudaMemcpyAsync(z.data(), hb->d.znode0, nn * sizeof(double), cudaMemcpyDeviceToHost, stream()));
    BCFD_CUDA(cudaStreamSynchronize(stream()));
    for (int q = 0; q < nn; ++q) r0 = std::max(r0, std::sqrt(x[q] * x[q] + y[q] * y[q] + z[q] * z[q]));
    hb->node0[0] = std::move(x);
    hb->node0[1] = std::move(y);
    hb->node0[2] = std::move(z);
  }
  hb->node_id_host = id;
  hb->motion_r0 = r0;
  return 0;
}

int bcfd_block_set_body_lag(bcfd_handle h, double lag, double phase_angle) {
  LOCK();
  GETB(h);
  if (!hb->motion.on) return BCFD_E_STATE;
  if (!std::isfinite(lag) || !std::isfinite(phase_angle)) return BCFD_E_ARG;
  hb->motion.lag = lag;
  hb->motion.lag_phase = phase_angle;
  return 0;
}

int bcfd_shift_surface_nodes_initial(bcfd_handle h, double aoa, double piv_pt, int64_t ita, double deltat,
                                     double dxmin, double totime) {
  LOCK();
  GETB(h);
  if (!hb->motion.on) return BCFD_E_STATE;
  return shift_surface_nodes_initial(hb, aoa, piv_pt, ita, deltat, dxmin, totime);
}

int bcfd_compute_surface_variables(bcfd_handle h, double phase_angle, double piv_pt, int64_t ita,
                                   double deltat, double dxmin, double freq, double totime) {
  LOCK();
  GETB(h);
  if (!hb->motion.on) return BCFD_E_STATE;
  return compute_surface_variables(hb, phase_angle, piv_pt, ita, deltat, dxmin, freq, totime);
}

int bcfd_set_motion_inputs(double phase_angle, double piv_pt, double freq, double dxmin, int64_t inor,
                           int64_t ita, double totime) {
  LOCK();
  Lib& L = lib();
  L.phase_angle = phase_angle;
  L.piv_pt = piv_pt;
  L.freq = freq;
  L.dxmin = dxmin;
  L.inor = inor;
  L.ita = ita;
  L.totime = totime;
  return 0;
}

int bcfd_get_time(int64_t* ita, double* totime) {
  LOCK();
  if (ita) *ita = lib().ita;
  if (totime) *totime = lib().totime;
  return 0;
}

int bcfd_block_set_kinematics(bcfd_handle h, const double* k) {
  LOCK();
  GETB(h);
  if (!k) return BCFD_E_ARG;
  Kin& D = hb->kin;
  D.xdot = k[0];
  D.ydot = k[1];
  D.yddot = k[2];
  D.thetaDot1 = k[3];
  D.thetaDDot1 = k[4];
  D.thetaDot2 = k[5];
  D.thetaDDot2 = k[6];
  D.alphaDot = k[7];
  D.piv_x = k[8];
  D.piv_y = k[9];
  D.piv_z = k[10];
  return upload_kin(hb);
}

int bcfd_block_set_flags(bcfd_handle h, int64_t move_check, int64_t blk_mv_tag) {
  LOCK();
  GETB(h);
  if (move_check >= 0) hb->move_check = move_check;
  if (blk_mv_tag >= 0) hb->blk_mv_tag = blk_mv_tag;
  return 0;
}

int bcfd_block_set_role(bcfd_handle h, int is_coarse, int has_body) {
  LOCK();
  GETB(h);
  hb->is_coarse = is_coarse != 0;
  hb->has_body = has_body != 0;
  return 0;
}

int bcfd_block_upload_fields(bcfd_handle h, const double* u, const double* v, const double* w,
                             const double* p, const double* ut, const double* vt, const double* wt) {
  LOCK();
  GETB(h);
  const int64_t n = hb->d.d.npts();
  TRY(upload(hb->d.u, u, n));
  TRY(upload(hb->d.v, v, n));
  TRY(upload(hb->d.w, w, n));
  TRY(upload(hb->d.p, p, n));
  TRY(upload(hb->d.ut, ut, n));
  TRY(upload(hb->d.vt, vt, n));
  TRY(upload(hb->d.wt, wt, n));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  return 0;
}

int bcfd_block_download_fields(bcfd_handle h, double* u, double* v, double* w, double* p,
                               double* ut, double* vt, double* wt) {
  LOCK();
  GETB(h);
  const int64_t n = hb->d.d.npts();
  TRY(download(hb->d.u, u, n));
  TRY(download(hb->d.v, v, n));
  TRY(download(hb->d.w, w, n));
  TRY(download(hb->d.p, p, n));
  TRY(download(hb->d.ut, ut, n));
  TRY(download(hb->d.vt, vt, n));
  TRY(download(hb->d.wt, wt, n));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  return 0;
}

int bcfd_block_upload_tags(bcfd_handle h, const int64_t* cell, const int64_t* cell2,
                           const int64_t* nid, const int64_t* cell_n, const int64_t* cell_pr) {
  LOCK();
  GETB(h);
  const Dims& d = hb->d.d;
  TRY(up_tags(cell, hb->d.cell, d.npts()));
  TRY(up_tags(cell2, hb->d.cell2, d.npts3()));
  TRY(up_tags(nid, hb->d.nodeTag, d.npts3()));
  TRY(up_tags(cell_n, hb->d.cell_n, d.npts()));
  TRY(up_tags(cell_pr, hb->d.cell_pr, d.npts3()));
  return 0;
}

int bcfd_block_download_tags(bcfd_handle h, int64_t* cell, int64_t* cell2, int64_t* nid,
                             int64_t* cell_n, int64_t* cell_pr) {
  LOCK();
  GETB(h);
  const Dims& d = hb->d.d;
  TRY(down_tags(hb->d.cell, cell, d.npts()));
  TRY(down_tags(hb->d.cell2, cell2, d.npts3()));
  TRY(down_tags(hb->d.nodeTag, nid, d.npts3()));
  TRY(down_tags(hb->d.cell_n, cell_n, d.npts()));
  TRY(down_tags(hb->d.cell_pr, cell_pr, d.npts3()));
  return 0;
}

int bcfd_block_get_counts(bcfd_handle h, int64_t* counts) {
  LOCK();
  GETB(h);
  if (!counts) return BCFD_E_ARG;
  BCFD_CUDA(cudaMemcpyAsync(counts, hb->d.cnt, 6 * sizeof(int64_t), cudaMemcpyDeviceToHost, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  return 0;
}

int bcfd_block_get_sor_stats(bcfd_handle h, int64_t* n_iter, double* derr2, double* dss) {
  LOCK();
  GETB(h);
  BlockStats s;
  BCFD_CUDA(cudaMemcpyAsync(&s, hb->d.stats, sizeof(s), cudaMemcpyDeviceToHost, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  if (n_iter) *n_iter = s.niter;
  if (derr2) *derr2 = s.derr2;
  if (dss) *dss = s.derr_std_st;
  return 0;
}

int bcfd_block_set_sor_iter(bcfd_handle h, int64_t n_iter) {
  LOCK();
  GETB(h);
  BCFD_CUDA(cudaMemcpyAsync(&hb->d.stats->niter, &n_iter, sizeof(int64_t), cudaMemcpyHostToDevice, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  return 0;
}

int bcfd_non_uni_coeff(bcfd_handle h) {
  LOCK();
  GETB(h);
  build_coefs(hb);
  if (hb->Acx.empty()) build_poisson_coefs(hb, hb->is_coarse);
  return upload_coefs(hb);
}

int bcfd_coefficient_matrix(bcfd_handle h, int is_coarse) {
  LOCK();
  GETB(h);
  build_poisson_coefs(hb, is_coarse != 0);
  if (hb->ca[0].empty()) build_coefs(hb);
  return upload_coefs(hb);
}

// ---- momentum and boundary conditions ----
int bcfd_ns_momentum_2order(bcfd_handle h, double deltat, double re) {
  LOCK();
  GETB(h);
  if (!hb->d.ca[0]) return BCFD_E_STATE;
  return launch_momentum(hb, deltat, re, false);
}
int bcfd_velocity_bc(bcfd_handle h, double deltat, double uc) {
  LOCK();
  GETB(h);
  return launch_velocity_bc(hb, deltat, uc);
}
int bcfd_solid_cell_bc(bcfd_handle h) {
  LOCK();
  GETB(h);
  return launch_solid_bc(hb, false);
}
int bcfd_solid_cell_bc_move(bcfd_handle h) {
  LOCK();
  GETB(h);
  if (hb->move_check != 1) return 0;
  return launch_solid_bc(hb, true);
}

// The routines below can record a device status (a probe without a bracket,
// a list over capacity, a non-finite residual, a wait that gave up); called
// one at a time they return it, which synchronises the library stream.  The
// whole-step driver reads the status once per step instead.
#define RET_DEV(hb, expr) \
  do {                    \
    TRY(expr);            \
    return take_block_error(hb); \
  } while (0)

// ---- forcing ----
int bcfd_velocity_forcing1(bcfd_handle h) { LOCK(); GETB(h); RET_DEV(hb, launch_forcing_velocity(hb, 0)); }
int bcfd_pressure_forcing1(bcfd_handle h) { LOCK(); GETB(h); RET_DEV(hb, launch_forcing_pressure(hb, 0)); }
int bcfd_velocity_forcing_field(bcfd_handle h) { LOCK(); GETB(h); RET_DEV(hb, launch_forcing_velocity(hb, 1)); }
int bcfd_pressure_forcing_field(bcfd_handle h) { LOCK(); GETB(h); RET_DEV(hb, launch_forcing_pressure(hb, 1)); }
int bcfd_velocity_forcing_ghost(bcfd_handle h) { LOCK(); GETB(h); RET_DEV(hb, launch_forcing_velocity(hb, 2)); }
int bcfd_pressure_forcing_ghost(bcfd_handle h) { LOCK(); GETB(h); RET_DEV(hb, launch_forcing_pressure(hb, 2)); }

// ---- search ----
int bcfd_compute_surface_norm(bcfd_handle h, int64_t inor) {
  LOCK();
  GETB(h);
  hb->inor = inor;
  return launch_surface_norm(hb, inor);
}
int bcfd_tagging_th(bcfd_handle h) {
  LOCK();
  GETB(h);
  TRY(launch_tagging(hb));
  // tagging_th_core ends with the three counts (src/Search.F90:365-380)
  RET_DEV(hb, launch_cellcount(hb, false));
}
int bcfd_selective_retagging_th(bcfd_handle h) {
  LOCK();
  GETB(h);
  if (hb->blk_mv_tag != 0) return 0;
  TRY(launch_retagging(hb));
  RET_DEV(hb, launch_cellcount(hb, false));
}
int bcfd_cellcount_solid(bcfd_handle h) {
  LOCK();
  GETB(h);
  RET_DEV(hb, launch_cellcount(hb, false));
}
int bcfd_cellcount_solid_coarse(bcfd_handle h) {
  LOCK();
  GETB(h);
  RET_DEV(hb, launch_cellcount(hb, true));
}
int bcfd_compute_norm_distance(bcfd_handle h) {
  LOCK();
  GETB(h);
  RET_DEV(hb, launch_norm_distance(hb));
}
int bcfd_find_ts_cells(bcfd_handle h) {
  LOCK();
  GETB(h);
  RET_DEV(hb, launch_find_ts(hb));
}
int bcfd_fine_block_cell(void) {
  LOCK();
  HostBlock* a = get_block(1);
  if (!a) return BCFD_E_HANDLE;
  TRY(launch_fine_block_cell(a, nullptr, true));
  for (HostInterface* it : lib().ifs)
    if (it && it->a == 1) TRY(launch_fine_block_cell(a, it, false));
  return 0;
}

// ---- pressure correction ----
int bcfd_compute_div(bcfd_handle h) { LOCK(); GETB(h); return launch_compute_div(hb); }
int bcfd_correct_pressure(bcfd_handle h) { LOCK(); GETB(h); return launch_correct_pressure(hb); }
int bcfd_correct_velocity(bcfd_handle h, double dt) { LOCK(); GETB(h); return launch_correct_velocity(hb, dt); }
int bcfd_redblack_sor_linear(bcfd_handle h, int64_t itmax, double dt, double epsi) {
  LOCK();
  GETB(h);
  RET_DEV(hb, launch_sor(hb, itmax, dt, epsi));
}
int bcfd_block_sor_sweeps(bcfd_handle h, int64_t n_pairs, int precision) {
  LOCK();
  GETB(h);
  if (n_pairs < 1 || n_pairs > 1000000 || precision < 0 || precision > 2) return BCFD_E_ARG;
  if (precision != 1) {
    // the reference sweeps (0) or the division-free FP64 sweeps (2) from
    // iteration 0, stop test disabled (epsi < 0)
    BCFD_CUDA(cudaMemsetAsync(&hb->d.stats->niter, 0, sizeof(int64_t), stream()));
    TRY(launch_sor(hb, n_pairs - 1, 1.0, -1.0, 0.0, precision == 2));
  } else {
    // one correction of n_pairs FP32 sweep pairs, stop test disabled
    const int keep = hb->dc_inner;
    hb->dc_inner = (int)n_pairs;
    const int r = launch_sor_mixed(hb, 0, 1.0, -1.0);
    hb->dc_inner = keep;
    TRY(r);
  }
  return 0;
}

int bcfd_update_velocity_newv(bcfd_handle h) {
  LOCK();
  GETB(h);
  if (hb->move_check != 1) return 0;
  return launch_copy_n_to_t(hb);
}

int bcfd_max_divergence(bcfd_handle h, double* out) {
  LOCK();
  GETB(h);
  if (!out) return BCFD_E_ARG;
  TRY(launch_max_div(hb, false));
  BCFD_CUDA(cudaMemcpyAsync(out, &hb->d.stats->maxdiv, sizeof(double), cudaMemcpyDeviceToHost, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  return 0;
}

int bcfd_block_get_divergence(bcfd_handle h, double* out) {
  LOCK();
  GETB(h);
  if (!out) return BCFD_E_ARG;
  BCFD_CUDA(cudaMemcpyAsync(out, &hb->d.stats->pad[0], 2 * sizeof(double), cudaMemcpyDeviceToHost, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  return 0;
}

int bcfd_block_set_solve_launch(bcfd_handle h, int threads, int ctas_per_sm, int fp64_sync) {
  LOCK();
  GETB(h);
  if (!(threads == 0 || threads == 128 || threads == 256 || threads == 512) ||
      ctas_per_sm < 0 || ctas_per_sm > 16 || fp64_sync < 0 || fp64_sync > 1)
    return BCFD_E_ARG;
  hb->solve_threads = threads;
  hb->solve_ctas_per_sm = ctas_per_sm;
  hb->solve_sync = fp64_sync;
  hb->dc_threads = threads > 256 ? 256 : threads;
  hb->dc_ctas_per_sm = ctas_per_sm;
  return 0;
}

int bcfd_block_get_solve_launch(bcfd_handle h, int* out) {
  LOCK();
  GETB(h);
  if (!out) return BCFD_E_ARG;
  const int v[6] = {hb->solve_threads, hb->solve_ctas_per_sm, hb->solve_sync,
                    hb->dc_threads,    hb->dc_ctas_per_sm,    hb->dc_variant};
  std::memcpy(out, v, sizeof v);
  return 0;
}

int bcfd_block_get_mixed_omega(bcfd_handle h, double* omega) {
  LOCK();
  GETB(h);
  if (!omega) return BCFD_E_ARG;
  *omega = mixed_omega_of(hb);
  return 0;
}

int bcfd_block_set_mixed_params(bcfd_handle h, int64_t inner_sweeps, double omega, int variant) {
  LOCK();
  GETB(h);
  if (inner_sweeps < 0 || inner_sweeps > 100000 || omega < 0.0 || omega >= 2.0 || variant < 0 || variant > 5 ||
      variant == 2)  // the cluster-resident variant was withdrawn
    return BCFD_E_ARG;
  hb->dc_inner = (int)inner_sweeps;
  hb->dc_omega = omega;
  hb->dc_variant = variant;
  return 0;
}

int bcfd_profile_begin(void) {
  LOCK();
  Lib& L = lib();
  if (!L.ready) return BCFD_E_STATE;
  if (!L.prof_dev) BCFD_CUDA(cudaMalloc(&L.prof_dev, (1 + 4 * kProfLogCap) * sizeof(int64_t)));
  BCFD_CUDA(cudaMemsetAsync(L.prof_dev, 0, sizeof(int64_t), stream()));
  L.prof_used = 0;
  L.phase_used = 0;
  L.prof_on = true;
  L.prof_launch0 = L.launches;
  return 0;
}

int bcfd_profile_phases(double* ms, int n) {
  LOCK();
  if (!ms || n < 0) return BCFD_E_ARG;
  for (int q = 0; q < n && q < PH_COUNT; ++q) ms[q] = lib().phase_ms[q];
  return 0;
}

int bcfd_profile_end(bcfd_profile_report* out) {
  LOCK();
  Lib& L = lib();
  if (!L.prof_on || !out) return BCFD_E_STATE;
  // the window ends at a phase boundary so the last phase is closed
  phase_mark(PH_COUNT);
  L.prof_on = false;
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  std::memset(out, 0, sizeof(*out));
  for (double& v : L.phase_ms) v = 0.0;
  for (size_t q = 0; q + 1 < L.phase_used; ++q) {
    float ms = 0.f;
    BCFD_CUDA(cudaEventElapsedTime(&ms, L.phase_events[q], L.phase_events[q + 1]));
    if (L.phase_ids[q] >= 0 && L.phase_ids[q] < PH_COUNT) L.phase_ms[L.phase_ids[q]] += ms;
  }
  for (size_t q = 0; q + 1 < L.prof_used; q += 2) {
    float ms = 0.f;
    BCFD_CUDA(cudaEventElapsedTime(&ms, L.prof_events[q], L.prof_events[q + 1]));
    out->sor_ms += ms;
    out->sor_launches++;
  }
  int64_t n = 0;
  BCFD_CUDA(d2h(&n, L.prof_dev, sizeof(int64_t)));
  n = std::min<int64_t>(n, (int64_t)kProfLogCap);
  std::vector<int64_t> e(4 * (size_t)std::max<int64_t>(n, 1));
  if (n) BCFD_CUDA(d2h(e.data(), L.prof_dev + 1, 4 * n * sizeof(int64_t)));
  for (int64_t q = 0; q < n; ++q) {
    const double sw = (double)e[4 * q], rp = (double)e[4 * q + 1], fl = (double)e[4 * q + 2];
    out->sor_sweeps += e[4 * q];
    if (e[4 * q + 3] == 0) {
      out->sor_bytes += sw * fl * 33.0;  // 4w + 1, w = 8
    } else if (e[4 * q + 3] == 2) {
      // z-marching sweeps: one pass per two sweep pairs reads e, the rhs
      // and the mask once and writes e once (4 + 4 + 1 + 4 B); the FP64
      // residual and update passes as below
      out->sor_bytes += 0.5 * sw * fl * 13.0 + rp * fl * 29.0 + (rp - 1.0) * fl * 25.0;
    } else {
      // FP32 sweeps 4w + 1 (w = 4); FP64 residual: pc own + neighbours + b/dt
      // read, r written as FP32, mask (8+8+8+4+1); update x += e: pc r/w,
      // e r/w, mask (8+8+4+4+1)
      out->sor_bytes += sw * fl * 17.0 + rp * fl * 29.0 + (rp - 1.0) * fl * 25.0;
    }
  }
  out->kernel_launches = L.launches - L.prof_launch0;
  return 0;
}

int bcfd_stress_calculation(bcfd_handle h, double mu_f, double rho_f, double* out) {
  LOCK();
  GETB(h);
  if (!out) return BCFD_E_ARG;
  TRY(launch_stress(hb, mu_f, rho_f, out));
  return take_block_error(hb);
}

int bcfd_stress_calculation_noalloc(bcfd_handle h, double mu_f, double rho_f, double* out) {
  LOCK();
  GETB(h);
  if (!out) return BCFD_E_ARG;
  TRY(launch_stress_noalloc(hb, mu_f, rho_f, out));
  return take_block_error(hb);
}

}  // extern "C"
