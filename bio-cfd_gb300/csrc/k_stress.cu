// Drag / lift integration over the IB elements (stress_calculation,
// src/StressCalc.f90:14-208), FP64.  Each element's viscous and pressure force
// contributions are computed independently, then summed by one CTA in a fixed
// tree order, so the result is deterministic run to run (the reference's
// OpenACC reduction order is unspecified; its serial build sums in element
// order).
#include <cstdio>

#include "bcfd_host.h"

namespace bcfd {

namespace {

__device__ int fidx(const DevBlock& B, double v, const double* a, int len, int s, int f) {
  for (int i = s; i <= f; ++i) {
    if (i < 1 || i + 1 > len) continue;
    if (v >= a[i - 1] && v < a[i]) return i;
  }
  set_err(B.err, BCFD_E_NOTFOUND);
  return max(1, min(s, len - 1));
}

__device__ __forceinline__ double bil(double x, double y, double x1, double x2, double y1, double y2,
                                      double f0, double f1, double f2, double f3) {
  const double numer = f0 * (x2 - x) * (y2 - y) + f2 * (x2 - x) * (y - y1) +
                       f1 * (x - x1) * (y2 - y) + f3 * (x - x1) * (y - y1);
  return numer / ((x2 - x1) * (y2 - y1));
}

__device__ __forceinline__ double der(double x, double x2, double x1, double p_x, double p_x2,
                                      double p_x1) {
  const double h2 = fabs(x2 - x), h1 = fabs(x1 - x);
  return (h1 * h1 * p_x2 - h2 * h2 * p_x1 + (h2 * h2 - h1 * h1) * p_x) / (h1 * h2 * (h1 + h2) + 1e-16);
}

// compute_value_and_derivatives with the find_index ranges 2..n+1 of StressCalc
__device__ void vad(const DevBlock& B, double x, double y, double z, const double* xg, int nxg,
                    const double* yg, int nyg, const double* zg, int nzg, int off, const double* var,
                    double& val, double d3[3]) {
  const Dims& d = B.d;
  const int i = fidx(B, x, xg, nxg, 2, d.nx + 1), j = fidx(B, y, yg, nyg, 2, d.ny + 1),
            k = fidx(B, z, zg, nzg, 2, d.nz + 1);
  const int ii = i - (off == 1), jj = j - (off == 2), kk = k - (off == 3);
  double f[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) f[q] = var[d.idx(ii + (q & 1), jj + ((q >> 1) & 1), kk + (q >> 2))];
  const double yj = yg[j - 1], yj1 = yg[j], zk = zg[k - 1], zk1 = zg[k], xi = xg[i - 1], xi1 = xg[i];
  const double t11 = bil(y, z, yj, yj1, zk, zk1, f[0], f[2], f[4], f[6]);
  const double t12 = bil(y, z, yj, yj1, zk, zk1, f[1], f[3], f[5], f[7]);
  const double t21 = bil(x, z, xi, xi1, zk, zk1, f[0], f[1], f[4], f[5]);
  const double t22 = bil(x, z, xi, xi1, zk, zk1, f[2], f[3], f[6], f[7]);
  const double t31 = bil(x, y, xi, xi1, yj, yj1, f[0], f[1], f[2], f[3]);
  const double t32 = bil(x, y, xi, xi1, yj, yj1, f[4], f[5], f[6], f[7]);
  val = t11 + (x - xi) * (t12 - t11) / (xi1 - xi);
  d3[0] = der(x, xi1, xi, val, t12, t11);
  d3[1] = der(y, yj1, yj, val, t22, t21);
  d3[2] = der(z, zk1, zk, val, t32, t31);
}

// per element: [viscous drag, pressure drag, viscous lift, pressure lift, area, a_xz, a_yz]
__global__ void k_stress_elem(DevBlock B, double mu_f, double rho_f, double* part) {
  const Dims& d = B.d;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < B.ne; e += gridDim.x * blockDim.x) {
    const double nrm[3] = {B.cosA[e], B.cosB[e], B.cosG[e]};
    const int ic = fidx(B, B.xcent[e], B.x1, d.NX + 1, 2, d.nx + 1);
    const int jc = fidx(B, B.ycent[e], B.y1, d.NY + 1, 2, d.ny + 1);
    const int kc = fidx(B, B.zcent[e], B.z1, d.NZ + 1, 2, d.nz + 1);
    const double dX = B.x1[ic] - B.x1[ic - 1], dY = B.y1[jc] - B.y1[jc - 1], dZ = B.z1[kc] - B.z1[kc - 1];
    const double diag = sqrt(dX * dX + dY * dY + dZ * dZ);
    const double nd = diag;
    const double px = B.xcent[e] + nd * nrm[0], py = B.ycent[e] + nd * nrm[1], pz = B.zcent[e] + nd * nrm[2];
    const int sid = B.surf_id[e];
    const double td = sid == 51 ? B.thetaDot1 : (sid == 52 ? B.thetaDot2 : 0.0);
    const double tdd = sid == 51 ? B.thetaDDot1 : (sid == 52 ? B.thetaDDot2 : 0.0);
    const double us = B.xdot;
    const double vs = -td * (B.zcent[e] - B.piv_z) + B.ydot;
    const double ws = td * (B.ycent[e] - B.piv_y);
    const double ac_z = -(td * td) * (B.zcent[e] - B.piv_z);
    const double ac_y = -(td * td) * (B.ycent[e] - B.piv_y);
    const double at_z = tdd * (B.ycent[e] - B.piv_y);
    const double at_y = -tdd * (B.zcent[e] - B.piv_z);
    const double dpdn = -((ac_z + at_z) * B.cosG[e] + (ac_y + at_y) * B.cosB[e]) - B.yddot * B.cosB[e];
    double val, g[3], ddn[3];
    vad(B, px, py, pz, B.xu, d.NX + 1, B.yu, d.NY, B.zu, d.NZ, 1, B.u, val, g);
    ddn[0] = (2.0 / nd) * (val - us) - (g[0] * nrm[0] + g[1] * nrm[1] + g[2] * nrm[2]);
    vad(B, px, py, pz, B.xv, d.NX, B.yv, d.NY + 1, B.zv, d.NZ, 2, B.v, val, g);
    ddn[1] = (2.0 / nd) * (val - vs) - (g[0] * nrm[0] + g[1] * nrm[1] + g[2] * nrm[2]);
    vad(B, px, py, pz, B.xw, d.NX, B.yw, d.NY, B.zw, d.NZ + 1, 3, B.w, val, g);
    ddn[2] = (2.0 / nd) * (val - ws) - (g[0] * nrm[0] + g[1] * nrm[1] + g[2] * nrm[2]);
    const double alen = B.elen[e];
    const double area = alen / 2.0;
    const double a_yz = 0.5 * fabs(alen * nrm[0]);
    const double a_xz = 0.5 * fabs(alen * nrm[1]);
    const double dd = ddn[0] * nrm[0] + ddn[1] * nrm[1] + ddn[2] * nrm[2];
    const double sh0 = (ddn[0] - dd * nrm[0]) * mu_f * area;
    const double sh1 = (ddn[1] - dd * nrm[1]) * mu_f * area;
    vad(B, px, py, pz, B.xp, d.NX, B.yp, d.NY, B.zp, d.NZ, 0, B.p, val, g);
    const double dpdn_e = g[0] * nrm[0] + g[1] * nrm[1] + g[2] * nrm[2];
    const double cval = val - (dpdn_e + dpdn) * diag * 0.5;
    double* o = part + 7 * (int64_t)e;
    o[0] = sh0;
    o[1] = -cval * area * nrm[0] * rho_f;
    o[2] = sh1;
    o[3] = -cval * area * nrm[1] * rho_f;
    o[4] = area;
    o[5] = a_xz;
    o[6] = a_yz;
  }
}

// fixed-order pairwise reduction by one CTA
__global__ void k_stress_sum(const double* part, int ne, double* out) {
  __shared__ double s[7][256];
  for (int q = 0; q < 7; ++q) {
    double acc = 0.0;
    for (int e = threadIdx.x; e < ne; e += blockDim.x) acc += part[7 * (int64_t)e + q];
    s[q][threadIdx.x] = acc;
  }
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int q = 0; q < 7; ++q) s[q][threadIdx.x] += s[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double aSx = 0.5 * s[5][0], aSy = 0.5 * s[6][0];
    out[0] = 2.0 * (s[0][0] / aSx);
    out[1] = 2.0 * (s[1][0] / aSy);
    out[2] = 2.0 * (s[2][0] / aSx);
    out[3] = 2.0 * (s[3][0] / aSy);
  }
}

}  // namespace

int launch_stress(HostBlock* hb, double mu_f, double rho_f, double* out_host) {
  const int ne = hb->d.ne;
  if (ne <= 0) return BCFD_E_STATE;
  double* part = nullptr;
  double* out = nullptr;
  BCFD_CUDA(cudaMalloc(&part, (size_t)ne * 7 * sizeof(double)));
  BCFD_CUDA(cudaMalloc(&out, 4 * sizeof(double)));
  k_stress_elem<<<grid_for(ne, 128), 128, 0, stream()>>>(hb->d, mu_f, rho_f, part);
  int r = note_launch();
  if (!r) {
    k_stress_sum<<<1, 256, 0, stream()>>>(part, ne, out);
    r = note_launch();
  }
  if (!r) {
    BCFD_CUDA(cudaMemcpyAsync(out_host, out, 4 * sizeof(double), cudaMemcpyDeviceToHost, stream()));
    BCFD_CUDA(cudaStreamSynchronize(stream()));
  }
  cudaFree(part);
  cudaFree(out);
  return r;
}

// ---- allocation-free variant ------------------------------------------------
// The same two kernels, with the per-element partials and the 4 coefficients
// in a fixed device array of this translation unit instead of cudaMalloc'd
// memory.  Nothing in it has to start at zero: k_stress_elem writes all
// 7 * ne partials that k_stress_sum reads, and k_stress_sum writes out[0..3].
// There is one array per device, so two calls that overlap on one device would
// race on it; launch_stress_noalloc runs under the library lock on the library
// stream and synchronises before returning, so calls through it never overlap.
namespace {
constexpr int kStressNoallocMaxElems = BCFD_STRESS_NOALLOC_MAX_ELEMS;
constexpr size_t kStressScratchDoubles = 7 * (size_t)kStressNoallocMaxElems + 4;
static __device__ __align__(256) double g_stress_scratch[kStressScratchDoubles];
constexpr int kMaxDevices = 64;
double* g_stress_scratch_ptr[kMaxDevices] = {};
}  // namespace

// Set-up, once per device with that device current: the address of the
// device array.  The first call on a device does this, so it should come
// before any stream capture begins on that device.  The cached address is
// valid while the device's primary context lives (the library never resets
// the device).
static int stress_scratch(double** out) {
  int dev = -1;
  BCFD_CUDA(cudaGetDevice(&dev));
  // the library stream belongs to the device bcfd_init selected
  if (dev != lib().device) return BCFD_E_STATE;
  if (dev < 0 || dev >= kMaxDevices) return BCFD_E_ARG;
  if (!g_stress_scratch_ptr[dev]) {
    void* p = nullptr;
    BCFD_CUDA(cudaGetSymbolAddress(&p, g_stress_scratch));
    if (!p) return BCFD_E_CUDA;
    g_stress_scratch_ptr[dev] = (double*)p;
  }
  *out = g_stress_scratch_ptr[dev];
  return 0;
}

int launch_stress_noalloc(HostBlock* hb, double mu_f, double rho_f, double* out_host) {
  const int ne = hb->d.ne;
  if (ne <= 0) return BCFD_E_STATE;
  if (ne > kStressNoallocMaxElems) {
    std::fprintf(stderr,
                 "bcfd_stress_calculation_noalloc: block has %d surface elements, more than the "
                 "%d its fixed device scratch holds (use bcfd_stress_calculation)\n",
                 ne, kStressNoallocMaxElems);
    return BCFD_E_CAPACITY;
  }
  double* scratch = nullptr;
  TRY_R(stress_scratch(&scratch));
  double* part = scratch;
  double* out = scratch + 7 * (size_t)kStressNoallocMaxElems;
  k_stress_elem<<<grid_for(ne, 128), 128, 0, stream()>>>(hb->d, mu_f, rho_f, part);
  TRY_R(note_launch());
  k_stress_sum<<<1, 256, 0, stream()>>>(part, ne, out);
  TRY_R(note_launch());
  BCFD_CUDA(cudaMemcpyAsync(out_host, out, 4 * sizeof(double), cudaMemcpyDeviceToHost, stream()));
  BCFD_CUDA(cudaStreamSynchronize(stream()));
  return 0;
}

}  // namespace bcfd
