// Mixed-precision Poisson solve resident in one thread-block cluster.
//
// A 16-CTA cluster (one CTA per SM, ~210 KB of shared memory each) holds the
// whole block's FP32 correction e and its right-hand side r in distributed
// shared memory: CTA c owns a contiguous range of z planes, both colours,
// in the colour-packed layout.  Red and black half-sweeps are separated by
// hardware cluster barriers (barrier.cluster arrive.release / wait.acquire),
// and the z-neighbour planes owned by the adjacent CTAs are read through
// DSMEM.  No global-memory traffic and no software grid barrier remain in the
// inner loop.
//
// Outer defect-correction loop (as k_sor_dc): r = b/dt - A pc in FP64 over
// the block's own planes (pc and the FP64 coefficients read through L2),
// stop when dt * max|r| <= div_tol, else `inner` FP32 sweep pairs on A e = r
// from e = 0 (non-fluid cells hold r = NaN and e = 0) and pc += e in FP64.
//
// Every CTA executes the same sequence of cluster barriers: all loop bounds
// and stop decisions come from cluster-wide reductions that every CTA reads.
#include <cooperative_groups.h>

#include "bcfd_host.h"

namespace cg = cooperative_groups;

namespace bcfd {

namespace {

constexpr int kClusterCtas = 16;
constexpr int kThreads = 1024;

struct ClArgs {
  int64_t max_outer;
  int inner;
  float omega;
  double dt, div_tol;
  int64_t* log;
};

struct Planes {
  int k0, nk;  // first owned plane (1-based k) and count
};

// position t, t + S, ... over (h, j = 2.., k = k0..) of the owned planes
struct PlaneWalk {
  int t, S, k0;
  Walk3 w;
  __device__ PlaneWalk(int t0, int S_, int NXH, int ny, int k0_) : t(t0), S(S_), k0(k0_) {
    w.init(t0, S_, NXH, ny);
  }
  __device__ __forceinline__ void next() {
    t += S;
    w.next();
  }
  __device__ __forceinline__ int h() const { return w.a; }
  __device__ __forceinline__ int j() const { return 2 + w.b; }
  __device__ __forceinline__ int k() const { return k0 + w.c; }
};

__device__ __forceinline__ Planes planes_of(int rank, int nz) {
  const int a = (rank * nz) / kClusterCtas, b = ((rank + 1) * nz) / kClusterCtas;
  return {2 + a, b - a};
}

__global__ void __launch_bounds__(kThreads, 1) k_sor_cluster(DevBlock B, ClArgs a) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const Dims d = B.d;
  const int NXH = d.NXH, NY = d.NY;
  const int plane = NXH * NY;  // floats per colour per plane
  const Planes my = planes_of(rank, d.nz);
  const int nkl_max = (d.nz + kClusterCtas - 1) / kClusterCtas;

  extern __shared__ __align__(16) unsigned char smem[];
  float* cf = reinterpret_cast<float*>(smem);                 // Acxf|Acyf|Aczf
  const int ncoef = 3 * (d.nx + d.ny + d.nz);
  float* e = cf + ((ncoef + 3) & ~3);                          // [2][nkl_max][plane]
  float* r = e + 2 * (size_t)nkl_max * plane;                  // [2][nkl_max][plane]
  double* red = reinterpret_cast<double*>(r + 2 * (size_t)nkl_max * plane);  // [32] + [2] slots

  const float* Axf = cf;
  const float* Ayf = cf + 3 * d.nx;
  const float* Azf = cf + 3 * d.nx + 3 * d.ny;
  for (int q = threadIdx.x; q < 3 * d.nx; q += blockDim.x) cf[q] = B.Acxf[q];
  for (int q = threadIdx.x; q < 3 * d.ny; q += blockDim.x) cf[3 * d.nx + q] = B.Acyf[q];
  for (int q = threadIdx.x; q < 3 * d.nz; q += blockDim.x) cf[3 * d.nx + 3 * d.ny + q] = B.Aczf[q];
  for (int q = threadIdx.x; q < 2 * nkl_max * plane; q += blockDim.x) e[q] = 0.0f;

  // neighbour CTAs' e arrays (DSMEM); planes 1 and nz+2 are zero Dirichlet data
  const float* e_lo = nullptr;
  const float* e_hi = nullptr;
  int lo_nk = 0;
  if (rank > 0) {
    e_lo = cl.map_shared_rank(e, rank - 1);
    lo_nk = planes_of(rank - 1, d.nz).nk;
  }
  if (rank < kClusterCtas - 1) e_hi = cl.map_shared_rank(e, rank + 1);
  cl.sync();

  // e of colour c at packed (h, j) of plane k (1-based); owned, remote or zero
  auto e_at = [&](int c, int h, int j, int k) -> float {
    const int kk = k - my.k0;
    const int off = h + NXH * (j - 1);
    if (kk >= 0 && kk < my.nk) return e[(size_t)(c * nkl_max + kk) * plane + off];
    if (kk == -1 && e_lo && lo_nk > 0) return e_lo[(size_t)(c * nkl_max + lo_nk - 1) * plane + off];
    if (kk == my.nk && e_hi) return e_hi[(size_t)(c * nkl_max) * plane + off];
    return 0.0f;
  };

  const int nrow = d.ny * my.nk;  // interior rows j = 2..ny+1 of the owned planes
  const int64_t sy = NXH, sz = (int64_t)NXH * NY;
  double res = 0.0;
  int64_t outer = 0, sweeps = 0;
  for (;; ++outer) {
    // ---- FP64 residual of the owned planes -> r (FP32), max |r| ----
    double m = 0.0;
    for (int c = 0; c < 2; ++c) {
      const double* own = B.pc[c];
      const double* o = B.pc[1 - c];
      for (PlaneWalk w(threadIdx.x, blockDim.x, NXH, d.ny, my.k0); w.t < nrow * NXH; w.next()) {
        const int h = w.h();
        const int j = w.j(), k = w.k();
        int i = 2 * h + 1;
        if (((i + j + k) & 1) != c) ++i;
        const int64_t pi = h + sy * (j - 1) + sz * (k - 1);
        float* rl = &r[(size_t)(c * nkl_max + (k - my.k0)) * plane + h + NXH * (j - 1)];
        if (!B.upd[c][pi]) {
          *rl = __int_as_float(0x7fc00000);  // NaN marks a cell the sweeps skip
          continue;
        }
        const int64_t row = pi - h;
        double ax = (B.Acx[i - 2 + d.nx] + B.Acy[j - 2 + d.ny] + B.Acz[k - 2 + d.nz]) * __ldcg(own + pi);
        ax = fma(B.Acx[i - 2], __ldcg(o + row + ((i - 2) >> 1)), ax);
        ax = fma(B.Acx[i - 2 + 2 * d.nx], __ldcg(o + row + (i >> 1)), ax);
        ax = fma(B.Acy[j - 2], __ldcg(o + pi - sy), ax);
        ax = fma(B.Acy[j - 2 + 2 * d.ny], __ldcg(o + pi + sy), ax);
        ax = fma(B.Acz[k - 2], __ldcg(o + pi - sz), ax);
        ax = fma(B.Acz[k - 2 + 2 * d.nz], __ldcg(o + pi + sz), ax);
        const double rv = B.rhs[c][pi] - ax;
        *rl = (float)rv;
        m = fmax(m, fabs(rv));
      }
    }
    m = block_max(m, red);
    if (threadIdx.x == 0) red[32] = m;
    cl.sync();
    double cm = 0.0;
    for (int q = 0; q < kClusterCtas; ++q)
      cm = fmax(cm, *cl.map_shared_rank(&red[32], q));
    res = cm;
    if (a.dt * res <= a.div_tol || outer >= a.max_outer || !(res == res)) break;

    // ---- FP32 red-black sweeps on A e = r, e from 0 ----
    for (int it = 0; it < a.inner; ++it) {
#pragma unroll
      for (int c = 1; c >= 0; --c) {
        for (PlaneWalk w(threadIdx.x, blockDim.x, NXH, d.ny, my.k0); w.t < nrow * NXH; w.next()) {
          const int h = w.h();
          const int j = w.j(), k = w.k();
          const size_t lo = (size_t)(c * nkl_max + (k - my.k0)) * plane + h + NXH * (j - 1);
          const float rv = r[lo];
          if (!(rv == rv)) continue;
          int i = 2 * h + 1;
          if (((i + j + k) & 1) != c) ++i;
          const int o = 1 - c;
          const size_t lo_o = (size_t)(o * nkl_max + (k - my.k0)) * plane + NXH * (j - 1);
          float s = rv;
          s = __fmaf_rn(-Axf[i - 2], e[lo_o + ((i - 2) >> 1)], s);
          s = __fmaf_rn(-Axf[i - 2 + 2 * d.nx], e[lo_o + (i >> 1)], s);
          s = __fmaf_rn(-Ayf[j - 2], e[lo_o + h - NXH], s);
          s = __fmaf_rn(-Ayf[j - 2 + 2 * d.ny], e[lo_o + h + NXH], s);
          s = __fmaf_rn(-Azf[k - 2], e_at(o, h, j, k - 1), s);
          s = __fmaf_rn(-Azf[k - 2 + 2 * d.nz], e_at(o, h, j, k + 1), s);
          const float dg = Axf[i - 2 + d.nx] + Ayf[j - 2 + d.ny] + Azf[k - 2 + d.nz];
          const float old = e[lo];
          e[lo] = __fmaf_rn(a.omega, __fdividef(s, dg) - old, old);
        }
        cl.sync();
      }
    }
    sweeps += a.inner;

    // ---- pc += e (FP64), e = 0 ----
    for (int c = 0; c < 2; ++c)
      for (PlaneWalk w(threadIdx.x, blockDim.x, NXH, d.ny, my.k0); w.t < nrow * NXH; w.next()) {
        const int h = w.h();
        const int j = w.j(), k = w.k();
        const size_t lo = (size_t)(c * nkl_max + (k - my.k0)) * plane + h + NXH * (j - 1);
        if (!(r[lo] == r[lo])) continue;
        const int64_t pi = h + sy * (j - 1) + sz * (k - 1);
        B.pc[c][pi] = B.pc[c][pi] + (double)e[lo];
        e[lo] = 0.0f;
      }
    cl.sync();
  }
  if (rank == 0 && threadIdx.x == 0) {
    BlockStats* st = B.stats;
    if (a.log) {
      const unsigned long long s = atomicAdd(reinterpret_cast<unsigned long long*>(a.log), 1ull);
      if (s < kProfLogCap) {
        int64_t* en = a.log + 1 + 4 * s;
        en[0] = sweeps;
        en[1] = outer + 1;
        en[2] = B.cnt[C_FLUID];
        en[3] = 2;
      }
    }
    st->niter = st->niter + sweeps;
    st->derr2 = a.dt * res;
    if (!(res == res)) set_err(B.err, BCFD_E_NONFINITE);
  }
  cl.sync();  // keep every CTA's shared memory alive until remote reads are done
}

size_t cluster_smem_bytes(const Dims& d) {
  const int nkl_max = (d.nz + kClusterCtas - 1) / kClusterCtas;
  const size_t ncoef = (size_t)3 * (d.nx + d.ny + d.nz);
  const size_t plane = (size_t)d.NXH * d.NY;
  return ((ncoef + 3) & ~(size_t)3) * 4 + 4 * plane * nkl_max * 4 + 34 * sizeof(double);
}

}  // namespace

// 1 if the block fits in one cluster's shared memory and the device can run a
// 16-CTA cluster with that much shared memory per CTA
int cluster_solve_fits(HostBlock* hb) {
  static int attr_done = 0;
  const size_t smem = cluster_smem_bytes(hb->d.d);
  if (smem > 227 * 1024 || hb->d.d.nz < kClusterCtas) return 0;
  if (!attr_done) {
    if (cudaFuncSetAttribute(k_sor_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
        cudaFuncSetAttribute(k_sor_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
            cudaSuccess) {
      cudaGetLastError();
      attr_done = -1;
    } else {
      attr_done = 1;
    }
  }
  if (attr_done < 0) return 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kClusterCtas);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kClusterCtas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int nclusters = 0;
  if (cudaOccupancyMaxActiveClusters(&nclusters, k_sor_cluster, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return nclusters >= 1 ? 1 : 0;
}

int launch_sor_cluster(HostBlock* hb, int64_t itmax, double dt, double div_tol, int inner, float omega) {
  DevBlock& B = hb->d;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kClusterCtas);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = cluster_smem_bytes(B.d);
  cfg.stream = stream();
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kClusterCtas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  ClArgs a;
  a.inner = inner;
  a.omega = omega;
  a.max_outer = itmax / inner + 1;
  a.dt = dt;
  a.div_tol = div_tol;
  a.log = prof_log();
  prof_mark(true);
  BCFD_CUDA(cudaLaunchKernelEx(&cfg, k_sor_cluster, B, a));
  prof_mark(false);
  BCFD_LAUNCHED();
  return 0;
}

}  // namespace bcfd
