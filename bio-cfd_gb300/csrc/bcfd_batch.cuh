// Batched launches over a set of blocks of uneven sizes (one launch per phase
// instead of one per block).  The blocks' device views live in a device table
// (one DevBlock per registered block, refreshed only when one changes).  A
// launch gives every member block a contiguous range of CTAs; each CTA copies
// its block's view into shared memory and runs the same per-block operation
// the single-block launch runs, with (cta, ncta) in place of
// (blockIdx.x, gridDim.x).  A CTA never spans two blocks, so per-CTA
// reductions into a block's statistics stay valid.
#pragma once

#include "bcfd_internal.cuh"

namespace bcfd {

constexpr int kMaxBatch = 32;  // member blocks of one batched launch

struct BlockSet {
  const DevBlock* tab;          // device table, indexed by registration order
  int nb;                       // member blocks
  int ids[kMaxBatch];           // table index of each member
  int cta_off[kMaxBatch + 1];   // first CTA of each member; cta_off[nb] = grid
};

__device__ __forceinline__ int set_member(const BlockSet& s, int cta) {
  int lo = 0, hi = s.nb - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (s.cta_off[mid] <= cta) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// copy member m's view into shared memory (all threads take part)
__device__ __forceinline__ const DevBlock& stage_block(const BlockSet& s, int m, unsigned long long* raw) {
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(s.tab + s.ids[m]);
  constexpr int n8 = (int)(sizeof(DevBlock) / 8);
  for (int q = threadIdx.x; q < n8; q += blockDim.x) raw[q] = src[q];
  __syncthreads();
  return *reinterpret_cast<const DevBlock*>(raw);
}

static_assert(sizeof(DevBlock) % 8 == 0, "DevBlock is copied in 8-byte words");

// one block: the operation over the whole grid
template <class Op, int NT>
__global__ void __launch_bounds__(NT) k_one(DevBlock B, Op op) {
  op.run(B, (int)blockIdx.x, (int)gridDim.x);
}

// a set of blocks: each CTA runs the operation on its member block
template <class Op, int NT>
__global__ void __launch_bounds__(NT) k_set(BlockSet S, Op op) {
  __shared__ unsigned long long raw[(sizeof(DevBlock) + 7) / 8];
  const int m = set_member(S, (int)blockIdx.x);
  const DevBlock& B = stage_block(S, m, raw);
  op.run(B, (int)blockIdx.x - S.cta_off[m], S.cta_off[m + 1] - S.cta_off[m]);
}

// interior cells of a block, grid-stride over this CTA's share: (i, j, k, c)
#define FOR_INTERIOR(B_, cta_, ncta_)                                                  \
  for (int64_t _t = (int64_t)(cta_) * blockDim.x + threadIdx.x,                        \
               _n = (int64_t)(B_).d.nx * (B_).d.ny * (B_).d.nz;                        \
       _t < _n; _t += (int64_t)(ncta_) * blockDim.x)
// (i, j, k) of item _t: 32-bit divisions while the interior count fits them
// (a 64-bit division costs several times as many instructions)
#define INTERIOR_CELL(B_)                                                              \
  int i, j, k;                                                                         \
  if (_n <= 0x7fffffffLL) {                                                            \
    const unsigned _u = (unsigned)_t, _nx = (unsigned)(B_).d.nx, _ny = (unsigned)(B_).d.ny; \
    const unsigned _r = _u / _nx;                                                      \
    i = 2 + (int)(_u - _r * _nx);                                                      \
    k = 2 + (int)(_r / _ny);                                                           \
    j = 2 + (int)(_r - (unsigned)(k - 2) * _ny);                                       \
  } else {                                                                             \
    i = 2 + (int)(_t % (B_).d.nx);                                                     \
    const int64_t _r = _t / (B_).d.nx;                                                 \
    j = 2 + (int)(_r % (B_).d.ny);                                                     \
    k = 2 + (int)(_r / (B_).d.ny);                                                     \
  }                                                                                    \
  const int64_t c = (B_).d.idx(i, j, k)

}  // namespace bcfd
