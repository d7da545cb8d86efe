// Marker-to-cell Search of src/Search.F90 on the GPU.
//
// Nearest-element queries (tagging, re-tagging, normal distances) are
// brute force over all surface elements like the reference, but in two
// passes per warp: an FP32 pass over element centroids stored relative to a
// block origin finds the minimum distance d_f; every element whose FP32
// distance lies within a rigorous rounding bound of d_f is then re-evaluated
// with the reference's FP64 expression, and the smallest FP64 distance wins
// with the lowest element index on ties (the strict `<` of the serial loop).
// The result is bit-identical to the reference's argmin at a fraction of the
// FP64 work.  Index lists are built by an order-preserving compaction over
// the (k,j,i) loop order, the order of the reference's serial CPU build.
#include <cstring>

#include "bcfd_host.h"

namespace bcfd {

namespace {

constexpr int kWarps = 8;  // warps per CTA in the query kernels

struct QueryCtx {
  const float4* cf;   // element centroids relative to origin, FP32, in search order
  const int* perm;    // search order -> element index
  const float4* box;  // per chunk of 32 search positions: lo, hi of its FP32 centroids
  int nch;            // chunks
  const double *xc, *yc, *zc;
  int ne;
  double ox, oy, oz;
  float R;            // bound on |coordinate - origin| of queries and centroids
};

constexpr float kFInf = 3.0e38f;

__device__ __forceinline__ float fdist2(float dx, float dy, float dz) {
  return __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
}

// lower bound of fdist2(q - e) over the centroids e of a chunk box [lo, hi]:
// per axis the gap to the box is at most |q - e| in FP32 (rounding is
// monotone), and the same fused squares and sums keep the order
__device__ __forceinline__ float box_lb(const float (&q)[3], float4 lo, float4 hi) {
  const float gx = fmaxf(fmaxf(lo.x - q[0], q[0] - hi.x), 0.0f);
  const float gy = fmaxf(fmaxf(lo.y - q[1], q[1] - hi.y), 0.0f);
  const float gz = fmaxf(fmaxf(lo.z - q[2], q[2] - hi.z), 0.0f);
  return fdist2(gx, gy, gz);
}

__device__ __forceinline__ double sq3(double a, double b, double c) { return a * a + b * b + c * c; }

// Q simultaneous nearest-element queries by one warp; out[q] = 1-based element.
// Pass 1 finds each query's minimum FP32 distance d_f over all elements,
// pass 2 re-evaluates in FP64 every element whose FP32 distance lies within
// a rounding bound of d_f.  Both passes visit only the chunks of 32 elements
// (search order) whose box lower bound can matter: a skipped chunk's elements
// have FP32 distances above the running minimum (pass 1) or above the bound
// (pass 2), so d_f, the candidate set and the FP64 argmin (lowest element
// index on ties) are exactly those of the brute-force loops.
template <int Q>
__device__ void warp_nearest(const QueryCtx& C, const double (&q)[Q][3], int (&out)[Q]) {
  const int lane = threadIdx.x & 31;
  float qf[Q][3];
#pragma unroll
  for (int s = 0; s < Q; ++s) {
    qf[s][0] = (float)(q[s][0] - C.ox);
    qf[s][1] = (float)(q[s][1] - C.oy);
    qf[s][2] = (float)(q[s][2] - C.oz);
  }
  // pass 1, seeds: per query the chunk of least lower bound (lane = chunk)
  float mf[Q];
  int seed[Q];
#pragma unroll
  for (int s = 0; s < Q; ++s) {
    mf[s] = kFInf;
    seed[s] = 0;
  }
  for (int cb = 0; cb < C.nch; cb += 32) {
    const int c = cb + lane;
    if (c < C.nch) {
      const float4 lo = __ldg(C.box + 2 * c), hi = __ldg(C.box + 2 * c + 1);
#pragma unroll
      for (int s = 0; s < Q; ++s) {
        const float lb = box_lb(qf[s], lo, hi);
        if (lb < mf[s]) {
          mf[s] = lb;
          seed[s] = c;
        }
      }
    }
  }
#pragma unroll
  for (int s = 0; s < Q; ++s) {
    float v = mf[s];
    int c = seed[s];
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, v, o);
      const int oc = __shfl_xor_sync(0xffffffffu, c, o);
      if (ov < v || (ov == v && oc < c)) {
        v = ov;
        c = oc;
      }
    }
    seed[s] = c;
    mf[s] = kFInf;
  }
  // one chunk: every query's minimum over its elements (warp-uniform result)
  auto visit1 = [&](int c) {
    const int pos = 32 * c + lane;
    float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
    const bool in = pos < C.ne;
    if (in) e = __ldg(C.cf + pos);
#pragma unroll
    for (int s = 0; s < Q; ++s) {
      float v = in ? fdist2(qf[s][0] - e.x, qf[s][1] - e.y, qf[s][2] - e.z) : kFInf;
      for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
      mf[s] = fminf(mf[s], v);
    }
  };
#pragma unroll
  for (int s = 0; s < Q; ++s) visit1(seed[s]);
  for (int cb = 0; cb < C.nch; cb += 32) {
    const int c = cb + lane;
    bool need = false;
    if (c < C.nch) {
      const float4 lo = __ldg(C.box + 2 * c), hi = __ldg(C.box + 2 * c + 1);
#pragma unroll
      for (int s = 0; s < Q; ++s) need |= box_lb(qf[s], lo, hi) <= mf[s];
    }
    for (unsigned m = __ballot_sync(0xffffffffu, need); m; m &= m - 1) visit1(cb + __ffs(m) - 1);
  }
  float thr[Q];
#pragma unroll
  for (int s = 0; s < Q; ++s) {
    // |d_f - d| <= (3.5 R + 4 d) 2^-24 for coordinates rounded to FP32;
    // keep everything within 8x that bound (plus an absolute floor)
    const float d = sqrtf(mf[s]);
    const float tau = 8.0f * (3.5f * C.R + 4.0f * d + 1e-3f) * 5.9604645e-8f + 1e-12f;
    const float lim = d + 2.0f * tau;
    thr[s] = lim * lim * (1.0f + 1e-6f);
  }
  // pass 2: FP64 distances of the candidates (lowest index on ties)
  double best[Q];
  int bm[Q];
#pragma unroll
  for (int s = 0; s < Q; ++s) {
    best[s] = 1e300;
    bm[s] = 0x7fffffff;
  }
  for (int cb = 0; cb < C.nch; cb += 32) {
    const int c = cb + lane;
    bool need = false;
    if (c < C.nch) {
      const float4 lo = __ldg(C.box + 2 * c), hi = __ldg(C.box + 2 * c + 1);
#pragma unroll
      for (int s = 0; s < Q; ++s) need |= box_lb(qf[s], lo, hi) <= thr[s];
    }
    for (unsigned msk = __ballot_sync(0xffffffffu, need); msk; msk &= msk - 1) {
      const int pos = 32 * (cb + __ffs(msk) - 1) + lane;
      if (pos >= C.ne) continue;
      const float4 e = __ldg(C.cf + pos);
      const int m = __ldg(C.perm + pos);
#pragma unroll
      for (int s = 0; s < Q; ++s) {
        const float dd = fdist2(qf[s][0] - e.x, qf[s][1] - e.y, qf[s][2] - e.z);
        if (dd <= thr[s]) {
          const double d64 = sq3(q[s][0] - __ldg(C.xc + m), q[s][1] - __ldg(C.yc + m), q[s][2] - __ldg(C.zc + m));
          if (d64 < best[s] || (d64 == best[s] && m < bm[s])) {
            best[s] = d64;
            bm[s] = m;
          }
        }
      }
    }
  }
#pragma unroll
  for (int s = 0; s < Q; ++s) {
    double b = best[s];
    int mi = bm[s];
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, b, o);
      const int om = __shfl_xor_sync(0xffffffffu, mi, o);
      if (ob < b || (ob == b && om < mi)) {
        b = ob;
        mi = om;
      }
    }
    out[s] = mi + 1;
  }
}

struct SearchView {
  const float4* cf;
  const int* perm;
  const float4* box;
  const float* org;
};

__device__ __forceinline__ QueryCtx qctx(const DevBlock& B, const SearchView& V) {
  const float* org = V.org;
  QueryCtx C;
  C.cf = V.cf;
  C.perm = V.perm;
  C.box = V.box;
  C.nch = (B.ne + 31) / 32;
  C.xc = B.xcent;
  C.yc = B.ycent;
  C.zc = B.zcent;
  C.ne = B.ne;
  C.ox = org[0];
  C.oy = org[1];
  C.oz = org[2];
  C.R = org[3];
  return C;
}

// computeSurfaceNorm, src/Search.F90:210-258
__global__ void k_surface_norm(DevBlock B, double fin) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < B.ne; n += gridDim.x * blockDim.x) {
    const int a = B.elp1[n] - 1, b = B.elp2[n] - 1, c = B.elp3[n] - 1;
    const double p1x = B.xnode1[a], p1y = B.ynode1[a], p1z = B.znode1[a];
    const double p2x = B.xnode1[b], p2y = B.ynode1[b], p2z = B.znode1[b];
    const double p3x = B.xnode1[c], p3y = B.ynode1[c], p3z = B.znode1[c];
    const double xc = (p2x + p1x + p3x) / 3.0, yc = (p2y + p1y + p3y) / 3.0,
                 zc = (p2z + p1z + p3z) / 3.0;
    B.xcent[n] = xc;
    B.ycent[n] = yc;
    B.zcent[n] = zc;
    const double ca = (p2y - p1y) * (p3z - p1z) - (p3y - p1y) * (p2z - p1z);
    const double cb = (p2z - p1z) * (p3x - p1x) - (p3z - p1z) * (p2x - p1x);
    const double cg = (p2x - p1x) * (p3y - p1y) - (p3x - p1x) * (p2y - p1y);
    const double len = sqrt(ca * ca + cb * cb + cg * cg);
    B.elen[n] = len;
    B.cosA[n] = fin * ca / len;
    B.cosB[n] = fin * cb / len;
    B.cosG[n] = fin * cg / len;
  }
}

// the search's FP32 centroid copies relative to the origin, in search order,
// and the box of each chunk of 32 (one warp per chunk)
__global__ void k_cf_chunks(DevBlock B, float4* cf, const int* perm, float4* box, const float* org) {
  const int lane = threadIdx.x & 31;
  const int nch = (B.ne + 31) / 32;
  const double ox = org[0], oy = org[1], oz = org[2];
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < nch; c += (gridDim.x * blockDim.x) >> 5) {
    const int pos = 32 * c + lane;
    float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
    float lx = kFInf, ly = kFInf, lz = kFInf, hx = -kFInf, hy = -kFInf, hz = -kFInf;
    if (pos < B.ne) {
      const int n = perm[pos];
      e = make_float4((float)(B.xcent[n] - ox), (float)(B.ycent[n] - oy), (float)(B.zcent[n] - oz), 0.0f);
      cf[pos] = e;
      lx = hx = e.x;
      ly = hy = e.y;
      lz = hz = e.z;
    }
    for (int o = 16; o > 0; o >>= 1) {
      lx = fminf(lx, __shfl_xor_sync(0xffffffffu, lx, o));
      ly = fminf(ly, __shfl_xor_sync(0xffffffffu, ly, o));
      lz = fminf(lz, __shfl_xor_sync(0xffffffffu, lz, o));
      hx = fmaxf(hx, __shfl_xor_sync(0xffffffffu, hx, o));
      hy = fmaxf(hy, __shfl_xor_sync(0xffffffffu, hy, o));
      hz = fmaxf(hz, __shfl_xor_sync(0xffffffffu, hz, o));
    }
    if (lane == 0) {
      box[2 * c] = make_float4(lx, ly, lz, 0.0f);
      box[2 * c + 1] = make_float4(hx, hy, hz, 0.0f);
    }
  }
}

// One cell of the nearest-element tagging (src/Search.F90:294-338 and
// :553-591); executed by a whole warp.
__device__ void tag_cell_warp(const DevBlock& B, const QueryCtx& C, int i, int j, int k) {
  const double q[2][3] = {{B.xp[i - 1], B.yp[j - 1], B.zp[k - 1]},
                          {B.x1[i - 1], B.y1[j - 1], B.z1[k - 1]}};
  int nel[2];
  warp_nearest<2>(C, q, nel);
  if ((threadIdx.x & 31) == 0) {
    const Dims& d = B.d;
    const int ec = nel[0] - 1, ep = nel[1] - 1;
    if ((B.x1[i - 1] <= B.xcent[ec] && B.x1[i] >= B.xcent[ec]) &&
        (B.y1[j - 1] <= B.ycent[ec] && B.y1[j] >= B.ycent[ec]) &&
        (B.z1[k - 1] <= B.zcent[ec] && B.z1[k] >= B.zcent[ec]))
      B.cell[d.idx(i, j, k)] = 2;
    const double n2dotn = (B.x1[i - 1] - B.xcent[ep]) * B.cosA[ep] +
                          (B.y1[j - 1] - B.ycent[ep]) * B.cosB[ep] +
                          (B.z1[k - 1] - B.zcent[ep]) * B.cosG[ep];
    B.nodeTag[d.idx3(i, j, k)] = (n2dotn >= -1e-16) ? 0 : 1;
  }
}

// tagging_th_core loop 1 over the search box (one warp per cell)
__global__ void k_tag_box(DevBlock B, SearchView V) {
  const QueryCtx C = qctx(B, V);
  const int bx = B.box[1] - B.box[0] + 1, by = B.box[3] - B.box[2] + 1, bz = B.box[5] - B.box[4] + 1;
  const int64_t n = (int64_t)bx * by * bz;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = warp; t < n; t += nwarps) {
    const int i = B.box[0] + (int)(t % bx);
    const int64_t r = t / bx;
    const int j = B.box[2] + (int)(r % by), k = B.box[4] + (int)(r / by);
    tag_cell_warp(B, C, i, j, k);
  }
}

__device__ __forceinline__ int corner_sum(const DevBlock& B, int i, int j, int k) {
  const Dims& d = B.d;
  const int8_t* t = B.nodeTag;
  return t[d.idx3(i, j, k)] + t[d.idx3(i + 1, j, k)] + t[d.idx3(i, j + 1, k)] +
         t[d.idx3(i + 1, j + 1, k)] + t[d.idx3(i, j, k + 1)] + t[d.idx3(i + 1, j, k + 1)] +
         t[d.idx3(i, j + 1, k + 1)] + t[d.idx3(i + 1, j + 1, k + 1)];
}

// tagging_th_core loop 2: 8-corner solid test over the box
__global__ void k_solid_box(DevBlock B) {
  const int bx = B.box[1] - B.box[0] + 1, by = B.box[3] - B.box[2] + 1, bz = B.box[5] - B.box[4] + 1;
  const int64_t n = (int64_t)bx * by * bz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = B.box[0] + (int)(t % bx);
    const int64_t r = t / bx;
    const int j = B.box[2] + (int)(r % by), k = B.box[4] + (int)(r / by);
    const int64_t c = B.d.idx(i, j, k);
    if (B.cell[c] != 2 && corner_sum(B, i, j, k) == 8) B.cell[c] = 1;
  }
}

// selectiveRetagging_th step 1: clear the IB cells
__global__ void k_clear_ib(DevBlock B) {
  // a count beyond the capacity (BCFD_E_CAPACITY recorded) reads no further
  const int nib = (int)min(B.cnt[C_IB], (int64_t)B.cap_ib);
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nib; n += gridDim.x * blockDim.x)
    B.cell[B.d.idx(B.ib_i[n], B.ib_j[n], B.ib_k[n])] = 0;
}

// mark the 27-neighbourhoods of the IB cells (the union is what the
// reference re-tags; every cell of it gets the same values from any visit)
__global__ void k_mark_nbhd(DevBlock B, uint8_t* mark) {
  const int nib = (int)min(B.cnt[C_IB], (int64_t)B.cap_ib);
  const int64_t n = (int64_t)nib * 27;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int ib = (int)(t / 27), o = (int)(t % 27);
    const int i = B.ib_i[ib] + (o % 3) - 1, j = B.ib_j[ib] + ((o / 3) % 3) - 1,
              k = B.ib_k[ib] + (o / 9) - 1;
    mark[B.d.idx(i, j, k)] = 1;
  }
}

// compact the marked cells (order irrelevant: each is processed independently)
__global__ void k_collect_marked(DevBlock B, const uint8_t* mark, int* list, int* count, int cap) {
  const int64_t n = B.d.npts();
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    if (!mark[t]) continue;
    const int slot = atomicAdd(count, 1);
    if (slot < cap) list[slot] = (int)t;
    else set_err(B.err, BCFD_E_CAPACITY);
  }
}

__device__ __forceinline__ void lin_to_ijk(const Dims& d, int64_t t, int& i, int& j, int& k) {
  i = 1 + (int)(t % d.NX);
  const int64_t r = t / d.NX;
  j = 1 + (int)(r % d.NY);
  k = 1 + (int)(r / d.NY);
}

__global__ void k_retag_cells(DevBlock B, SearchView V, const int* list,
                              const int* count) {
  const QueryCtx C = qctx(B, V);
  const int n = min(*count, (int)B.d.npts());
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int t = warp; t < n; t += nwarps) {
    int i, j, k;
    lin_to_ijk(B.d, list[t], i, j, k);
    tag_cell_warp(B, C, i, j, k);
  }
}

__global__ void k_retag_solid(DevBlock B, const int* list, const int* count) {
  const int n = min(*count, (int)B.d.npts());
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    int i, j, k;
    lin_to_ijk(B.d, list[t], i, j, k);
    const int64_t c = list[t];
    if (B.cell[c] != 2) B.cell[c] = corner_sum(B, i, j, k) == 8 ? 1 : 0;
  }
}

// counts over the interior: ib, solid, fluid, red, black (cellCount_solid)
__global__ void k_count(DevBlock B) {
  __shared__ unsigned long long s[5];
  if (threadIdx.x < 5) s[threadIdx.x] = 0;
  __syncthreads();
  const Dims& d = B.d;
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  unsigned long long a[5] = {0, 0, 0, 0, 0};
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 2 + (int)(t % d.nx);
    const int64_t r = t / d.nx;
    const int j = 2 + (int)(r % d.ny), k = 2 + (int)(r / d.ny);
    const int c = B.cell[d.idx(i, j, k)];
    if (c == 2) a[0]++;
    else if (c == 1) a[1]++;
    else if (c == 0) {
      a[2]++;
      if ((i + j + k) & 1) a[3]++; else a[4]++;
    }
  }
  for (int q = 0; q < 5; ++q) {
    unsigned long long v = a[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&s[q], v);
  }
  __syncthreads();
  if (threadIdx.x < 5 && s[threadIdx.x])
    atomicAdd((unsigned long long*)&B.cnt[threadIdx.x], s[threadIdx.x]);
}

// Order-preserving compaction of the interior cells matching `want` (cell tag
// value) in (k,j,i) order, three passes: per-CTA counts, a scan of the CTA
// counts, ordered scatter with warp ballots.  Writes (i,j,k) into oi/oj/ok
// and, if ibmap != nullptr, the list index into ibmap.
constexpr int kChunk = 2048;  // interior cells per CTA of the compaction

__global__ void k_compact_count(DevBlock B, int want, int* cta_cnt) {
  const Dims& d = B.d;
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  const int64_t beg = (int64_t)blockIdx.x * kChunk;
  int cnt = 0;
  for (int64_t t = beg + threadIdx.x; t < beg + kChunk && t < n; t += blockDim.x) {
    const int i = 2 + (int)(t % d.nx);
    const int64_t r = t / d.nx;
    const int j = 2 + (int)(r % d.ny), k = 2 + (int)(r / d.ny);
    cnt += B.cell[d.idx(i, j, k)] == want;
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  __shared__ int s;
  if (threadIdx.x == 0) s = 0;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) atomicAdd(&s, cnt);
  __syncthreads();
  if (threadIdx.x == 0) cta_cnt[blockIdx.x] = s;
}

// exclusive scan of the CTA counts by one CTA (n <= 1024 * per-thread chunk)
__global__ void k_scan_small(int* a, int n, int64_t* total) {
  __shared__ int part[1024];
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int b = threadIdx.x * per;
  int s = 0;
  for (int q = b; q < b + per && q < n; ++q) s += a[q];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int off = 1; off < (int)blockDim.x; off <<= 1) {
    const int v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = threadIdx.x ? part[threadIdx.x - 1] : 0;
  for (int q = b; q < b + per && q < n; ++q) {
    const int v = a[q];
    a[q] = run;
    run += v;
  }
  if (threadIdx.x == blockDim.x - 1 && total) *total = part[threadIdx.x];
}

__global__ void k_compact_scatter(DevBlock B, int want, const int* cta_off, int* oi, int* oj,
                                  int* ok, int cap, int* ibmap) {
  const Dims& d = B.d;
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  const int64_t beg = (int64_t)blockIdx.x * kChunk;
  __shared__ int wsum[32];
  __shared__ int base;
  if (threadIdx.x == 0) base = cta_off[blockIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t t0 = beg; t0 < beg + kChunk && t0 < n; t0 += blockDim.x) {
    const int64_t t = t0 + threadIdx.x;
    int i = 0, j = 0, k = 0;
    bool hit = false;
    if (t < beg + kChunk && t < n) {
      i = 2 + (int)(t % d.nx);
      const int64_t r = t / d.nx;
      j = 2 + (int)(r % d.ny);
      k = 2 + (int)(r / d.ny);
      hit = B.cell[d.idx(i, j, k)] == want;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) wsum[wid] = __popc(bal);
    __syncthreads();
    int wbase = 0, tot = 0;
    for (int q = 0; q < nw; ++q) {
      if (q < wid) wbase += wsum[q];
      tot += wsum[q];
    }
    if (hit) {
      const int pos = base + wbase + __popc(bal & ((1u << lane) - 1u));
      if (pos < cap) {
        if (oi) {
          oi[pos] = i;
          oj[pos] = j;
          ok[pos] = k;
        }
        if (ibmap) ibmap[d.idx(i, j, k)] = pos;
      } else {
        set_err(B.err, BCFD_E_CAPACITY);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) base += tot;
    __syncthreads();
  }
}

__global__ void k_fill_int(int* a, int64_t n, int v) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    a[t] = v;
}

// computeNormDistance, src/Search.F90:743-861 (one warp per IB cell)
__global__ void k_norm_distance(DevBlock B, SearchView V) {
  const QueryCtx C = qctx(B, V);
  const int nib = (int)min(B.cnt[C_IB], (int64_t)B.cap_ib);
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int n = warp; n < nib; n += nwarps) {
    const int ci = B.ib_i[n], cj = B.ib_j[n], ck = B.ib_k[n];
    const double n1x = B.xp[ci - 1], n2x = B.x1[ci - 1], n3x = B.x1[ci];
    const double n1y = B.yp[cj - 1], n2y = B.y1[cj - 1], n3y = B.y1[cj];
    const double n1z = B.zp[ck - 1], n2z = B.z1[ck - 1], n3z = B.z1[ck];
    const double q[7][3] = {{n1x, n1y, n1z}, {n2x, n1y, n1z}, {n3x, n1y, n1z}, {n1x, n2y, n1z},
                            {n1x, n3y, n1z}, {n1x, n1y, n2z}, {n1x, n1y, n3z}};
    int nel[7];
    warp_nearest<7>(C, q, nel);
    const int lane = threadIdx.x & 31;
    if (lane < 7) {
      // lane s writes query s (no dynamic register indexing of q/nel)
      int e = nel[0];
      double qx = q[0][0], qy = q[0][1], qz = q[0][2];
#pragma unroll
      for (int s = 1; s < 7; ++s)
        if (lane == s) {
          e = nel[s];
          qx = q[s][0];
          qy = q[s][1];
          qz = q[s][2];
        }
      B.nel[lane][n] = e;
      const int m = e - 1;
      B.nd[lane][n] = (qx - B.xcent[m]) * B.cosA[m] + (qy - B.ycent[m]) * B.cosB[m] +
                      (qz - B.zcent[m]) * B.cosG[m];
    }
  }
}

// findTScells, src/Search.F90:434-518: clear interior cell2, mark TS cells.
__global__ void k_ts_mark(DevBlock B) {
  const int nib = (int)min(B.cnt[C_IB], (int64_t)B.cap_ib);
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nib; n += gridDim.x * blockDim.x) {
    const int s = B.surf_id[B.nel[N_P][n] - 1];
    if (s == 51 || s == 52) B.cell2[B.d.idx3(B.ib_i[n], B.ib_j[n], B.ib_k[n])] = 2;
  }
}

__global__ void k_clear_cell2_interior(DevBlock B) {
  const Dims& d = B.d;
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 2 + (int)(t % d.nx);
    const int64_t r = t / d.nx;
    const int j = 2 + (int)(r % d.ny), k = 2 + (int)(r / d.ny);
    B.cell2[d.idx3(i, j, k)] = 0;
  }
}

// ordered TS list over the IB list (one CTA; IB lists are small), zero ghosts
__global__ void k_ts_list(DevBlock B) {
  __shared__ int wsum[32];
  __shared__ int base;
  const int nib = (int)min(B.cnt[C_IB], (int64_t)B.cap_ib);
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int n0 = 0; n0 < nib; n0 += blockDim.x) {
    const int n = n0 + threadIdx.x;
    const bool hit = n < nib && B.cell2[B.d.idx3(B.ib_i[n], B.ib_j[n], B.ib_k[n])] == 2;
    const unsigned bal = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) wsum[wid] = __popc(bal);
    __syncthreads();
    int wb = 0, tot = 0;
    for (int q = 0; q < nw; ++q) {
      if (q < wid) wb += wsum[q];
      tot += wsum[q];
    }
    if (hit) {
      const int pos = base + wb + __popc(bal & ((1u << lane) - 1u));
      B.ts_idx[pos] = n + 1;
#pragma unroll
      for (int g = 0; g < 14; ++g) B.ghost[g][pos] = 0.0;
    }
    __syncthreads();
    if (threadIdx.x == 0) base += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) B.cnt[C_TS] = base;
}

// fine_block_cell marking for one interface (src/Search.F90:878-910)
struct FbcArgs {
  double xs, xe, ys, ye, zs, ze, ci;
};
__global__ void k_fine_block_cell(DevBlock A, FbcArgs f, double dx, double dy, double dz) {
  const Dims& d = A.d;
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 2 + (int)(t % d.nx);
    const int64_t r = t / d.nx;
    const int j = 2 + (int)(r % d.ny), k = 2 + (int)(r / d.ny);
    const double x = A.xp[i - 1], y = A.yp[j - 1], z = A.zp[k - 1];
    if (x >= f.xs + f.ci * dx && x <= f.xe - f.ci * dx && z >= f.zs + f.ci * dz &&
        z <= f.ze - f.ci * dz && y >= f.ys + f.ci * dy && y <= f.ye - f.ci * dy) {
      A.cell_n[d.idx(i, j, k)] = 1;
      A.cell[d.idx(i, j, k)] = 1;
    }
    if (x >= f.xs && x <= f.xe && z >= f.zs && z <= f.ze && y >= f.ys && y <= f.ye)
      A.cell_pr[d.idx3(i, j, k)] = 1;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// per-block search scratch: FP32 centroids, origin/radius, marks, lists
// ---------------------------------------------------------------------------
struct SearchScratch {
  float4* cf = nullptr;   // FP32 centroids in search order
  int* perm = nullptr;    // search order -> element index
  float4* box = nullptr;  // chunk boxes (lo, hi)
  int perm_gen = -1;      // elem_perm_gen of the uploaded perm
  float* org = nullptr;   // [ox, oy, oz, R] on device
  uint8_t* mark = nullptr;
  int* list = nullptr;
  int* count = nullptr;
  int* cta = nullptr;
  int64_t cap_e = 0, npts = 0;
  float org_host[4] = {0, 0, 0, 0};  // last uploaded origin / radius
  bool org_set = false;
};

static SearchScratch& scratch_of(HostBlock* hb) {
  if (!hb->search_scratch) hb->search_scratch = new SearchScratch();
  return *static_cast<SearchScratch*>(hb->search_scratch);
}

void free_search_scratch(HostBlock* hb) {
  if (!hb->search_scratch) return;
  SearchScratch* s = static_cast<SearchScratch*>(hb->search_scratch);
  for (void* p : {(void*)s->cf, (void*)s->perm, (void*)s->box, (void*)s->org, (void*)s->mark, (void*)s->list,
                  (void*)s->count, (void*)s->cta})
    if (p) cudaFree(p);
  delete s;
  hb->search_scratch = nullptr;
}

static int ensure_alloc(HostBlock* hb) {
  SearchScratch& s = scratch_of(hb);
  const int64_t np = hb->d.d.npts();
  if (s.npts != np) {
    if (s.mark) cudaFree(s.mark);
    if (s.list) cudaFree(s.list);
    if (s.count) cudaFree(s.count);
    if (s.cta) cudaFree(s.cta);
    if (s.org) cudaFree(s.org);
    BCFD_CUDA(cudaMalloc(&s.mark, np));
    BCFD_CUDA(cudaMalloc(&s.list, np * sizeof(int)));
    BCFD_CUDA(cudaMalloc(&s.count, sizeof(int)));
    const int64_t nint = (int64_t)hb->d.d.nx * hb->d.d.ny * hb->d.d.nz;
    BCFD_CUDA(cudaMalloc(&s.cta, ((nint + kChunk - 1) / kChunk + 1) * sizeof(int)));
    BCFD_CUDA(cudaMalloc(&s.org, 4 * sizeof(float)));
    s.npts = np;
    s.org_set = false;
    lib().gen++;
  }
  if (s.cap_e < hb->d.ne || !s.cf) {
    if (s.cf) cudaFree(s.cf);
    if (s.perm) cudaFree(s.perm);
    if (s.box) cudaFree(s.box);
    const size_t ne = (size_t)std::max(hb->d.ne, 1), nch = (ne + 31) / 32;
    BCFD_CUDA(cudaMalloc(&s.cf, ne * sizeof(float4)));
    BCFD_CUDA(cudaMalloc(&s.perm, ne * sizeof(int)));
    BCFD_CUDA(cudaMalloc(&s.box, 2 * nch * sizeof(float4)));
    s.cap_e = hb->d.ne;
    s.perm_gen = -1;
    lib().gen++;
  }
  if (s.perm_gen != hb->elem_perm_gen) {
    // the search order (identity when none was set with the surface)
    std::vector<int> perm(hb->elem_perm);
    if ((int)perm.size() != hb->d.ne) {
      perm.resize((size_t)std::max(hb->d.ne, 0));
      for (int q = 0; q < hb->d.ne; ++q) perm[(size_t)q] = q;
    }
    if (!perm.empty()) BCFD_CUDA(h2d(s.perm, perm.data(), perm.size() * sizeof(int)));
    s.perm_gen = hb->elem_perm_gen;
  }
  return 0;
}

static SearchView view_of(const SearchScratch& s) { return SearchView{s.cf, s.perm, s.box, s.org}; }

// origin: centre of the block; R: half diagonal of the padded block
static void origin_of(const HostBlock* hb, float h[4]) {
  const Dims& d = hb->d.d;
  const double x0 = hb->x1[0], x1 = hb->x1[d.nx + 2], y0 = hb->y1[0], y1 = hb->y1[d.ny + 2],
               z0 = hb->z1[0], z1 = hb->z1[d.nz + 2];
  h[0] = (float)(0.5 * (x0 + x1));
  h[1] = (float)(0.5 * (y0 + y1));
  h[2] = (float)(0.5 * (z0 + z1));
  const double R = 0.5 * std::sqrt((x1 - x0) * (x1 - x0) + (y1 - y0) * (y1 - y0) + (z1 - z0) * (z1 - z0));
  // bound on |query - origin| and |centroid - origin| (centroids lie inside
  // the hull of the nodes)
  h[3] = (float)(1.01 * std::max(R, hb->node_rmax) + 1e-6);
}

static int ensure_scratch(HostBlock* hb) {
  TRY_R(ensure_alloc(hb));
  SearchScratch& s = scratch_of(hb);
  float h[4];
  origin_of(hb, h);
  // upload only when it changes (a captured step contains no host copies)
  if (!s.org_set || std::memcmp(h, s.org_host, sizeof(h)) != 0) {
    std::memcpy(s.org_host, h, sizeof(h));
    BCFD_CUDA(cudaMemcpyAsync(s.org, s.org_host, sizeof(h), cudaMemcpyHostToDevice, stream()));
    s.org_set = true;
  }
  return 0;
}

int search_origin_stage(HostBlock* hb, float h[4], float** dev) {
  TRY_R(ensure_alloc(hb));
  SearchScratch& s = scratch_of(hb);
  if (h) {
    origin_of(hb, h);
    std::memcpy(s.org_host, h, 4 * sizeof(float));
    s.org_set = true;
  }
  *dev = s.org;
  return 0;
}

int launch_surface_norm(HostBlock* hb, int64_t inor) {
  if (int r = ensure_scratch(hb)) return r;
  SearchScratch& s = scratch_of(hb);
  if (hb->d.ne <= 0) return 0;
  k_surface_norm<<<grid_for(hb->d.ne, 128), 128, 0, stream()>>>(hb->d, (double)inor);
  BCFD_LAUNCHED();
  const int64_t nch = (hb->d.ne + 31) / 32;
  k_cf_chunks<<<grid_for(nch * 32, 256), 256, 0, stream()>>>(hb->d, s.cf, s.perm, s.box, s.org);
  BCFD_LAUNCHED();
  return 0;
}

int launch_tagging(HostBlock* hb) {
  if (int r = ensure_scratch(hb)) return r;
  SearchScratch& s = scratch_of(hb);
  const Dims& d = hb->d.d;
  BCFD_CUDA(cudaMemsetAsync(hb->d.cell, 0, d.npts(), stream()));
  BCFD_CUDA(cudaMemsetAsync(hb->d.cell2, 0, d.npts3(), stream()));
  BCFD_CUDA(cudaMemsetAsync(hb->d.nodeTag, 0, d.npts3(), stream()));
  const int* b = hb->d.box;
  const int64_t n = (int64_t)(b[1] - b[0] + 1) * (b[3] - b[2] + 1) * (b[5] - b[4] + 1);
  if (n <= 0 || hb->d.ne <= 0) return 0;
  k_tag_box<<<grid_for(n * 32, 32 * kWarps, 152u * 64u), 32 * kWarps, 0, stream()>>>(hb->d, view_of(s));
  BCFD_LAUNCHED();
  k_solid_box<<<grid_for(n, 256), 256, 0, stream()>>>(hb->d);
  BCFD_LAUNCHED();
  return 0;
}

int launch_retagging(HostBlock* hb) {
  if (int r = ensure_scratch(hb)) return r;
  SearchScratch& s = scratch_of(hb);
  const Dims& d = hb->d.d;
  const int cap = hb->d.cap_ib;
  k_clear_ib<<<grid_for(cap, 256), 256, 0, stream()>>>(hb->d);
  BCFD_LAUNCHED();
  BCFD_CUDA(cudaMemsetAsync(s.mark, 0, d.npts(), stream()));
  BCFD_CUDA(cudaMemsetAsync(s.count, 0, sizeof(int), stream()));
  k_mark_nbhd<<<grid_for((int64_t)cap * 27, 256), 256, 0, stream()>>>(hb->d, s.mark);
  BCFD_LAUNCHED();
  k_collect_marked<<<grid_for(d.npts(), 256), 256, 0, stream()>>>(hb->d, s.mark, s.list, s.count,
                                                                   (int)d.npts());
  BCFD_LAUNCHED();
  if (hb->d.ne > 0) {
    k_retag_cells<<<152 * 16, 32 * kWarps, 0, stream()>>>(hb->d, view_of(s), s.list, s.count);
    BCFD_LAUNCHED();
  }
  k_retag_solid<<<grid_for(d.npts(), 256), 256, 0, stream()>>>(hb->d, s.list, s.count);
  BCFD_LAUNCHED();
  return 0;
}

// compaction of cells with tag `want` (0 fluid, 1 solid, 2 IB) into oi/oj/ok
static int compact(HostBlock* hb, int want, int* oi, int* oj, int* ok, int cap, int* ibmap,
                   int64_t* total_dev) {
  SearchScratch& s = scratch_of(hb);
  const Dims& d = hb->d.d;
  const int64_t nint = (int64_t)d.nx * d.ny * d.nz;
  const int nct = (int)((nint + kChunk - 1) / kChunk);
  k_compact_count<<<nct, 256, 0, stream()>>>(hb->d, want, s.cta);
  BCFD_LAUNCHED();
  k_scan_small<<<1, 1024, 0, stream()>>>(s.cta, nct, total_dev);
  BCFD_LAUNCHED();
  k_compact_scatter<<<nct, 256, 0, stream()>>>(hb->d, want, s.cta, oi, oj, ok, cap, ibmap);
  BCFD_LAUNCHED();
  return 0;
}

int launch_cellcount(HostBlock* hb, bool coarse) {
  if (int r = ensure_scratch(hb)) return r;
  const Dims& d = hb->d.d;
  const int64_t nint = (int64_t)d.nx * d.ny * d.nz;
  if (!coarse) {
    BCFD_CUDA(cudaMemsetAsync(hb->d.cnt, 0, 5 * sizeof(int64_t), stream()));
    k_count<<<grid_for(nint, 256, 1024), 256, 0, stream()>>>(hb->d);
    BCFD_LAUNCHED();
    k_fill_int<<<grid_for(d.npts(), 256), 256, 0, stream()>>>(hb->d.ibmap, d.npts(), -1);
    BCFD_LAUNCHED();
    if (int r = compact(hb, 2, hb->d.ib_i, hb->d.ib_j, hb->d.ib_k, hb->d.cap_ib, hb->d.ibmap, nullptr))
      return r;
  } else {
    // cellCount_solid_coarse touches only the fluid / red / black counts
    BCFD_CUDA(cudaMemsetAsync(hb->d.cnt + C_FLUID, 0, 3 * sizeof(int64_t), stream()));
    int64_t* tmp = hb->d.cnt + C_TS + 1;  // scratch slots past the counts
    BCFD_CUDA(cudaMemsetAsync(tmp, 0, 5 * sizeof(int64_t), stream()));
    // reuse k_count into the scratch slots, then copy the fluid/red/black part
    DevBlock t = hb->d;
    t.cnt = tmp;
    k_count<<<grid_for(nint, 256, 1024), 256, 0, stream()>>>(t);
    BCFD_LAUNCHED();
    BCFD_CUDA(cudaMemcpyAsync(hb->d.cnt + C_FLUID, tmp + C_FLUID, 3 * sizeof(int64_t),
                              cudaMemcpyDeviceToDevice, stream()));
  }
  return launch_update_masks(hb);
}

int launch_build_list(HostBlock* hb, int which, int* out_ijk, int64_t cap, int64_t* count_host) {
  // which: 0 fluid, 1 solid, 2 IB (tag value); out_ijk holds 3*cap ints (i | j | k planes)
  if (int r = ensure_scratch(hb)) return r;
  int64_t* tot;
  BCFD_CUDA(cudaMalloc(&tot, sizeof(int64_t)));
  int r = 0;
  cudaError_t e = cudaMemsetAsync(tot, 0, sizeof(int64_t), stream());
  if (e == cudaSuccess) {
    r = compact(hb, which, out_ijk, out_ijk + cap, out_ijk + 2 * cap, (int)cap, nullptr, tot);
    if (r == 0) {
      e = cudaMemcpyAsync(count_host, tot, sizeof(int64_t), cudaMemcpyDeviceToHost, stream());
      if (e == cudaSuccess) e = cudaStreamSynchronize(stream());
    }
  }
  if (e != cudaSuccess) {
    report_cuda(e, "list count to host", __FILE__, __LINE__);
    r = BCFD_E_CUDA;
  }
  cudaFree(tot);
  return r;
}

int launch_norm_distance(HostBlock* hb) {
  if (int r = ensure_scratch(hb)) return r;
  SearchScratch& s = scratch_of(hb);
  if (hb->d.ne <= 0) return 0;
  k_norm_distance<<<152 * 8, 32 * kWarps, 0, stream()>>>(hb->d, view_of(s));
  BCFD_LAUNCHED();
  return 0;
}

// cells whose momentum stencil can read a position of a TS cell (the reach
// of the third-order stencil plus the staggering: [-3,3]^3 around it)
__global__ void k_ts_near(DevBlock B) {
  const Dims& d = B.d;
  const int nts = (int)min(B.cnt[C_TS], (int64_t)B.cap_ib);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)nts * 343;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int nn = (int)(t / 343), o = (int)(t % 343);
    const int bt = B.ts_idx[nn] - 1;
    const int i = B.ib_i[bt] + o % 7 - 3, j = B.ib_j[bt] + (o / 7) % 7 - 3, k = B.ib_k[bt] + o / 49 - 3;
    if (i < 2 || j < 2 || k < 2 || i > d.nx + 1 || j > d.ny + 1 || k > d.nz + 1) continue;
    B.tsnear[d.idx(i, j, k)] = 1;
  }
}

int launch_find_ts(HostBlock* hb) {
  const Dims& d = hb->d.d;
  const int64_t nint = (int64_t)d.nx * d.ny * d.nz;
  k_clear_cell2_interior<<<grid_for(nint, 256), 256, 0, stream()>>>(hb->d);
  BCFD_LAUNCHED();
  k_ts_mark<<<grid_for(hb->d.cap_ib, 256), 256, 0, stream()>>>(hb->d);
  BCFD_LAUNCHED();
  k_ts_list<<<1, 1024, 0, stream()>>>(hb->d);
  BCFD_LAUNCHED();
  BCFD_CUDA(cudaMemsetAsync(hb->d.tsnear, 0, d.npts(), stream()));
  k_ts_near<<<grid_for((int64_t)hb->d.cap_ib * 343, 256, 1024), 256, 0, stream()>>>(hb->d);
  BCFD_LAUNCHED();
  return 0;
}

int launch_fine_block_cell(HostBlock* a, HostInterface* it, bool first) {
  const Dims& d = a->d.d;
  if (first) {
    BCFD_CUDA(cudaMemsetAsync(a->d.cell_n, 0, d.npts(), stream()));
    BCFD_CUDA(cudaMemsetAsync(a->d.cell, 0, d.npts(), stream()));
    BCFD_CUDA(cudaMemsetAsync(a->d.cell_pr, 0, d.npts3(), stream()));
  }
  if (!it) return 0;
  HostBlock* fb = get_block(it->b);
  FbcArgs f{it->box[0], it->box[1], it->box[2], it->box[3], it->box[4], it->box[5],
            fb ? 3.0 : 3.0};
  const int64_t nint = (int64_t)d.nx * d.ny * d.nz;
  k_fine_block_cell<<<grid_for(nint, 256), 256, 0, stream()>>>(a->d, f, a->dx, a->dy, a->dz);
  BCFD_LAUNCHED();
  return 0;
}

}  // namespace bcfd
