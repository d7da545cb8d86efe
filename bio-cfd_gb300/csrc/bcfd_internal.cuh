// Internal definitions of the Bio-CFD GB300 hot-path library.
//
// Device data model (one block of the reference's multi-block grid):
//   * cell-centred / staggered fields u,v,w,p,ut,vt,wt are FP64 arrays of
//     NX*NY*NZ = (nx+2)(ny+2)(nz+2) points, x fastest -- byte-identical to the
//     Fortran arrays of Block_t (src/Blocks.f90:42-45), so host<->device copies
//     are plain memcpys;
//   * tags are int8 (the reference stores int64): cell / cell_n on NX*NY*NZ,
//     cell2 / nodeIdTag / cell_pr on (NX+1)(NY+1)(NZ+1);
//   * the Poisson correction pc and the right-hand side b/dt live in a
//     colour-packed red/black layout (one array per colour, NXH*NY*NZ with
//     the row pitch NXH = (NX+1)/2 rounded up to a multiple of 4) so that each
//     SOR half-sweep streams contiguous, 16-byte aligned rows;
//   * 1-D grid arrays keep the reference's 1-based meaning: ptr[i-1] = x(i).
// Every FP64 kernel of the drop-in path is compiled with --fmad=false and
// evaluates its expressions in the reference's order, so it rounds exactly
// like the reference's serial CPU build.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "biocfd_gb300.h"

namespace bcfd {

// ---------------------------------------------------------------------------
// indexing helpers (1-based i,j,k as in the reference)
// ---------------------------------------------------------------------------
struct Dims {
  int nx, ny, nz;  // interior cells
  int NX, NY, NZ;  // nx+2, ny+2, nz+2
  int NXH;         // packed row pitch of one colour: (NX+1)/2 rounded up to 4
  __host__ __device__ int64_t idx(int i, int j, int k) const {
    return (int64_t)(i - 1) + (int64_t)NX * ((int64_t)(j - 1) + (int64_t)NY * (k - 1));
  }
  // (nx+3)^3 arrays (cell2, nodeIdTag, cell_pr)
  __host__ __device__ int64_t idx3(int i, int j, int k) const {
    return (int64_t)(i - 1) + (int64_t)(NX + 1) * ((int64_t)(j - 1) + (int64_t)(NY + 1) * (k - 1));
  }
  // packed colour index of cell (i,j,k): h = (i-1)/2 within row (j,k)
  __host__ __device__ int64_t pidx(int i, int j, int k) const {
    return (int64_t)((i - 1) >> 1) + (int64_t)NXH * ((int64_t)(j - 1) + (int64_t)NY * (k - 1));
  }
  __host__ __device__ int64_t npts() const { return (int64_t)NX * NY * NZ; }
  __host__ __device__ int64_t npts3() const { return (int64_t)(NX + 1) * (NY + 1) * (NZ + 1); }
  __host__ __device__ int64_t npacked() const { return (int64_t)NXH * NY * NZ; }
};

// colour of a cell: 1 = red (i+j+k odd, src/Search.F90:707,724), 0 = black
__host__ __device__ inline int colour_of(int i, int j, int k) { return (i + j + k) & 1; }

// Incremental (a, b, c) coordinates of t = t0, t0 + S, t0 + 2S, ... over an
// n0 x n1 x n2 box in x-fastest order, without a division per step: the
// stride is decomposed once and each step adds it with single carries.
struct Walk3 {
  int a, b, c;
  int da, db, dc, n0, n1;
  __device__ __forceinline__ void init(int t0, int S, int n0_, int n1_) {
    n0 = n0_;
    n1 = n1_;
    a = t0 % n0;
    const int r = t0 / n0;
    b = r % n1;
    c = r / n1;
    da = S % n0;
    const int rs = S / n0;
    db = rs % n1;
    dc = rs / n1;
  }
  __device__ __forceinline__ void next() {
    a += da;
    int carry = a >= n0;
    a -= carry ? n0 : 0;
    b += db + carry;
    carry = b >= n1;
    b -= carry ? n1 : 0;
    c += dc + carry;
  }
};

// Momentum coefficient tables, order of src/NavierStokes.f90:32-40
enum CoefTab { T_UU = 0, T_VV, T_WW, T_UV, T_UW, T_VU, T_VW, T_WU, T_WV, N_TAB };

// Rigid-body kinematic scalars of a block's surface (Block_t's xdot, ydot,
// yddot, thetaDot1/2, thetaDDot1/2, alphaDot and the pivot piv_x/y/z).
struct Kin {
  double xdot, ydot, yddot, thetaDot1, thetaDDot1, thetaDot2, thetaDDot2, alphaDot, piv_x, piv_y, piv_z;
};

// Device view of one block (passed by value to kernels).
struct DevBlock {
  Dims d;
  // 1-D grids (1-based meaning, ptr[i-1])
  const double *x1, *y1, *z1, *dxa, *dya, *dza;
  const double *xu, *yu, *zu, *xv, *yv, *zv, *xw, *yw, *zw, *xp, *yp, *zp;
  // Poisson line coefficients Acx(nx,3) etc., column-major like the reference
  const double *Acx, *Acy, *Acz;
  // the same coefficients rounded to FP32 (mixed-precision sweeps)
  const float *Acxf, *Acyf, *Aczf;
  // Acxf laid out per packed float4 run of the FP32 half-sweep:
  // axr[(3 * par + col) * (NXH / 4) + run] holds column col of the run's 4
  // cells i = 2(4 run + u) + 1 + par (clamped to 2..nx+1)
  const float4* axr;
  // Acyf / Aczf rows as {a1, a2, a3, 0} (one float4 load per run)
  const float4 *ayr, *azr;
  // momentum tables ca/ck(6, n+2), column-major
  const double *ca[N_TAB], *ck[N_TAB];
  // FP32 copies of dxa/dya/dza and ca/ck (FP32 momentum stencil)
  const float *dxf, *dyf, *dzf;
  const float *caf[N_TAB], *ckf[N_TAB];
  // fields
  double *u, *v, *w, *p, *ut, *vt, *wt;
  // tags
  int8_t *cell, *cell_n, *cell2, *nodeTag, *cell_pr;
  uint8_t* tsnear;  // 1 where a cell is within [-3,3]^3 of a TS cell (overlay stencil)
  // colour-packed Poisson arrays: [0] black, [1] red
  double *pc[2], *rhs[2];
  float *pcf[2], *rhsf[2];
  uint8_t* upd[2];  // 1 where the packed cell is a fluid cell updated by SOR
  // surface
  int ne, nn;
  const double *xnode1, *ynode1, *znode1;
  // body-frame nodes and node surface ids (moving bodies only)
  const double *xnode0, *ynode0, *znode0;
  const int8_t* node_id;
  const int *elp1, *elp2, *elp3, *surf_id;
  double *xcent, *ycent, *zcent, *cosA, *cosB, *cosG, *elen;
  // IB / TS lists (capacity cap_ib), counts in cnt[]
  int cap_ib;
  int *ib_i, *ib_j, *ib_k;
  int *nel[7];          // nelp, nelu1, nelu2, nelv1, nelv2, nelw1, nelw2 (1-based element ids)
  double* nd[7];        // pNormDis, u1NormDis, u2NormDis, v1..., w2NormDis
  int* ts_idx;          // index_ts (1-based IB index)
  double* ghost[14];    // p, pt, u2, u2t, v2, v2t, w2, w2t, u1, u1t, v1, v1t, w1, w1t
  int* ibmap;           // NX*NY*NZ: 0-based IB index of a cell or -1
  int64_t* cnt;         // device counts: [0] ib, [1] solid, [2] fluid, [3] red, [4] black, [5] ts
  // search box (tagging_th_core)
  int box[6];
  // kinematics of the block's body (the forcing and stress routines read
  // them); device-resident so that a captured step reads each step's values
  const struct Kin* kin;
  int* err;             // device error word of this block (first error wins)
  double* scratch;      // per-block reduction scratch
  // per-line tables, NX + NY + NZ entries each: correctVelocity's factors
  // deltat / (0.5 (delta_i + delta_{i+1})) along x, y, z (index i, j, k),
  // computed once per deltat with the reference's operations; then the
  // reciprocal spacings 1 / deltax(i) etc. (index i-1, like dxa)
  const double* lcoef;
  double* bpk[2];       // colour-packed divergence b (the reference's Block_t%b)
  struct BlockStats* stats;
};

// Per-block Poisson statistics kept on the device so that a captured step
// needs no host round trip (nIterPcor, derr2, derrStdSt of Block_t).
struct BlockStats {
  int64_t niter;
  double derr2;
  double derr_std_st;
  double slot[3];       // rotating running maxima of the SOR stop test
  double maxdiv;        // max |div u| (diagnostics and the mixed-precision stop)
  double pad[2];
};

enum CountSlot { C_IB = 0, C_SOLID, C_FLUID, C_RED, C_BLACK, C_TS, N_COUNT };

// entries of the solve log of a measurement window ({sweeps, residual
// passes, fluid cells, precision} each, after one counter word)
constexpr unsigned long long kProfLogCap = 4096;
// most CTAs (tiles) of a tiled persistent solve; each tile's phase counter
// sits on its own 128-byte line (kTileStride unsigned words apart)
constexpr unsigned kMaxTiles = 4096;
constexpr unsigned kTileStride = 32;
enum GhostSlot { G_P = 0, G_PT, G_U2, G_U2T, G_V2, G_V2T, G_W2, G_W2T, G_U1, G_U1T, G_V1, G_V1T, G_W1, G_W1T };
enum NelSlot { N_P = 0, N_U1, N_U2, N_V1, N_V2, N_W1, N_W2 };

// device error codes written into DevBlock::err (first error wins)
__device__ inline void set_err(int* err, int code) { atomicCAS(err, 0, code); }

// ---------------------------------------------------------------------------
// bounded grid-wide barrier for cooperative persistent kernels
// ---------------------------------------------------------------------------
// Software grid barrier of a cooperative launch: one monotonic 64-bit arrival
// counter (zeroed before the launch).  The k-th barrier completes when the
// counter reaches k * nblocks; bit 63 set means "abandon": a CTA that gave up
// (timeout or a recorded error) sets it so every waiter leaves at once.
struct GridBar {
  unsigned long long* ctr;
  int* err;          // set to BCFD_E_TIMEOUT when a wait exceeds the limit
  unsigned nblocks;
  unsigned long long limit_ns;  // longest a single wait may last
};
constexpr unsigned long long kBarAbandon = 1ull << 63;

__device__ inline unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ inline unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ inline unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
// relaxed (L1-bypassing, no cache invalidation) loads for polling; an
// acquire fence after the poll succeeds completes the acquire pattern
__device__ inline unsigned ld_relaxed(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ inline unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ inline void st_relaxed(unsigned* p, unsigned v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ inline void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ inline void st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ inline int ld_acquire_i(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

constexpr unsigned long long kBarrierLimitNs = 2000000000ull;  // default: 2 s per wait

// Returns false (on every thread of the CTA) once the barrier was abandoned:
// a wait timed out somewhere, or a CTA saw a recorded error while waiting.
// The caller then leaves its loops and returns.
__device__ inline bool grid_sync(const GridBar& gb) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    const unsigned long long old = atomicAdd(gb.ctr, 1ull);
    if (old & kBarAbandon) {
      ok = 0;
    } else {
      const unsigned long long target = (old / gb.nblocks + 1) * gb.nblocks;
      const unsigned long long t0 = globaltimer_ns();
      unsigned spins = 0;
      for (;;) {
        const unsigned long long v = ld_acquire_u64(gb.ctr);
        if (v & kBarAbandon) { ok = 0; break; }
        if (v >= target) break;
        if (((++spins) & 63u) == 0) {
          if (ld_acquire_i(gb.err) != 0) {
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
      __threadfence();
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// ---------------------------------------------------------------------------
// reductions
// ---------------------------------------------------------------------------
// max that propagates NaN (fmax drops a NaN operand): equal to fmax for
// non-NaN operands, so a reduction of finite values is unchanged, while a NaN
// anywhere reaches the result and the non-finite checks see it
__device__ __forceinline__ double nmax(double a, double b) { return (a > b || a != a) ? a : b; }
// true for NaN and +-Inf
__device__ __forceinline__ bool non_finite(double x) { return !(fabs(x) <= 1.7976931348623157e308); }

__device__ inline double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = nmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
// block-wide max; result valid on thread 0. `sh` needs blockDim.x/32 doubles.
__device__ inline double block_max(double v, double* sh) {
  v = warp_max(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? sh[lane] : 0.0;
    v = warp_max(v);
  }
  return v;
}
// atomic max of a non-negative double through its bit pattern
__device__ inline void atomic_max_nonneg(double* addr, double v) {
  atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------
inline unsigned grid_for(int64_t n, int threads, unsigned cap = 152u * 32u) {
  int64_t g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (unsigned)g;
}

int num_sms();
cudaStream_t stream();

// cooperative launch of a persistent kernel (bounded barrier inside)
cudaError_t launch_coop(const void* fn, unsigned grid, unsigned block, void** args, size_t smem = 0);
// size of a cooperative grid for `fn` (all CTAs co-resident)
unsigned coop_grid(const void* fn, int threads, size_t smem, unsigned want);

// barrier state for persistent kernels (owned by the library)
GridBar make_bar(int* err, unsigned nblocks);

}  // namespace bcfd
