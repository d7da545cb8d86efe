// Autotuner of the tiled Poisson solves' launch shape.  For each block it
// times short solves (a fixed number of sweep pairs, stop test off) under
// every candidate shape and keeps the fastest: threads per CTA, the cap on
// co-resident CTAs per SM (which sets the tile shape through choose_tiles)
// and the phase synchronisation (grid barrier or neighbour tiles).  None of
// these changes the arithmetic, so the tuned solver computes exactly what the
// untuned one does.  The block's solve state is saved before the trials and
// restored after them; results are cached per block shape.  Blocks whose
// solves would run side by side in one batched launch are tuned alone too;
// then the batched launch of the whole group (default shape) is timed
// against the sum of the members' best launches of their own, and the faster
// is kept, per precision: large blocks that each fill the GPU (and whose
// working sets partly fit L2 when solved one at a time) leave the batch,
// many small blocks stay in it.
#include <cstring>
#include <map>
#include <tuple>

#include "bcfd_host.h"

namespace bcfd {
namespace {

struct Shape {
  int threads, ctas_per_sm, sync;  // sync: FP64 0 neighbour / 1 grid; FP32 variant 1 grid / 3 neighbour,
                                   // 4 temporal-blocked, 5 z-marching TMA
};
struct Tuned {
  Shape fp64, fp32;
  float ms64, ms32;  // trial time of each best shape
};
std::map<std::tuple<int, int, int>, Tuned>& cache() {
  static std::map<std::tuple<int, int, int>, Tuned> c;
  return c;
}

// device copies of what a trial solve overwrites
struct Saved {
  void* buf = nullptr;
  size_t off[5] = {0, 0, 0, 0, 0};
};

int save_state(HostBlock* hb, Saved& s, bool restore) {
  const size_t np = (size_t)hb->d.d.npacked();
  const size_t d8 = np * sizeof(double), f4 = np * sizeof(float);
  // pc[2], rhs[2] (FP64), pcf[2], rhsf[2] (FP32), stats
  const size_t total = 4 * d8 + 4 * f4 + sizeof(BlockStats);
  if (!restore) BCFD_CUDA(cudaMalloc(&s.buf, total));
  char* b = static_cast<char*>(s.buf);
  auto cp = [&](void* dev, size_t at, size_t n) -> int {
    if (restore) BCFD_CUDA(cudaMemcpyAsync(dev, b + at, n, cudaMemcpyDeviceToDevice, stream()));
    else BCFD_CUDA(cudaMemcpyAsync(b + at, dev, n, cudaMemcpyDeviceToDevice, stream()));
    return 0;
  };
  size_t at = 0;
  for (int c = 0; c < 2; ++c) {
    TRY_R(cp(hb->d.pc[c], at, d8));
    at += d8;
    TRY_R(cp(hb->d.rhs[c], at, d8));
    at += d8;
    TRY_R(cp(hb->d.pcf[c], at, f4));
    at += f4;
    TRY_R(cp(hb->d.rhsf[c], at, f4));
    at += f4;
  }
  TRY_R(cp(hb->d.stats, at, sizeof(BlockStats)));
  return 0;
}

// milliseconds of one trial solve (the best of two after a warm-up run)
int time_trial(HostBlock* hb, bool fp32, int pairs, float* ms) {
  cudaEvent_t e0, e1;
  BCFD_CUDA(cudaEventCreate(&e0));
  if (const cudaError_t ee = cudaEventCreate(&e1); ee != cudaSuccess) {
    cudaEventDestroy(e0);
    report_cuda(ee, "cudaEventCreate(&e1)", __FILE__, __LINE__);
    return BCFD_E_CUDA;
  }
  float best = 1e30f;
  int r = 0;
  for (int rep = 0; rep < 3 && !r; ++rep) {
    cudaEventRecord(e0, stream());
    if (fp32) {
      const int keep = hb->dc_inner;
      hb->dc_inner = pairs;
      r = launch_sor_mixed(hb, 0, 1.0, -1.0);
      hb->dc_inner = keep;
    } else {
      if (cudaMemsetAsync(&hb->d.stats->niter, 0, sizeof(int64_t), stream()) != cudaSuccess) r = BCFD_E_CUDA;
      if (!r) r = launch_sor(hb, pairs - 1, 1.0, -1.0);
    }
    cudaEventRecord(e1, stream());
    if (cudaEventSynchronize(e1) != cudaSuccess) r = BCFD_E_CUDA;
    float t = 0.f;
    if (!r && rep > 0 && cudaEventElapsedTime(&t, e0, e1) == cudaSuccess) best = std::min(best, t);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = best;
  return r;
}

// milliseconds of one trial solve of a group of blocks in one batched launch
// (every member in the default shape), the best of two after a warm-up run
int time_group(const std::vector<HostBlock*>& g, bool fp32, int pairs, float* ms) {
  cudaEvent_t e0, e1;
  BCFD_CUDA(cudaEventCreate(&e0));
  if (const cudaError_t ee = cudaEventCreate(&e1); ee != cudaSuccess) {
    cudaEventDestroy(e0);
    report_cuda(ee, "cudaEventCreate(&e1)", __FILE__, __LINE__);
    return BCFD_E_CUDA;
  }
  float best = 1e30f;
  int r = 0;
  for (int rep = 0; rep < 3 && !r; ++rep) {
    cudaEventRecord(e0, stream());
    if (fp32) {
      std::vector<int> keep;
      for (HostBlock* hb : g) keep.push_back(hb->dc_inner), hb->dc_inner = pairs;
      r = launch_sor_mixed_set(g, 0, 1.0, -1.0);
      for (size_t q = 0; q < g.size(); ++q) g[q]->dc_inner = keep[q];
    } else {
      for (HostBlock* hb : g)
        if (!r && cudaMemsetAsync(&hb->d.stats->niter, 0, sizeof(int64_t), stream()) != cudaSuccess) r = BCFD_E_CUDA;
      if (!r) r = launch_sor_set(g, pairs - 1, 1.0, -1.0, 0.0, 0);
    }
    cudaEventRecord(e1, stream());
    if (cudaEventSynchronize(e1) != cudaSuccess) r = BCFD_E_CUDA;
    float t = 0.f;
    if (!r && rep > 0 && cudaEventElapsedTime(&t, e0, e1) == cudaSuccess) best = std::min(best, t);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = best;
  return r;
}

void apply(HostBlock* hb, const Shape& s, bool fp32) {
  if (fp32) {
    hb->dc_threads = s.threads;
    hb->dc_ctas_per_sm = s.ctas_per_sm;
    hb->dc_variant = s.sync;
  } else {
    hb->solve_threads = s.threads;
    hb->solve_ctas_per_sm = s.ctas_per_sm;
    hb->solve_sync = s.sync;
  }
}

int tune_block(HostBlock* hb, Tuned* out) {
  static const Shape c64[] = {{256, 0, 0}, {512, 0, 0}, {256, 0, 1}, {512, 0, 1}, {512, 1, 0}};
  // {256, 4, *} selects the 64-register instantiation of the FP32 solve
  // {512, 0, 4}: the temporal-blocked sweeps (small blocks)
  // {384, 0, 5}: the z-marching TMA sweeps (large blocks)
  static const Shape c32[] = {{128, 0, 1}, {256, 0, 1}, {128, 0, 3}, {256, 0, 3}, {256, 2, 1},
                              {256, 1, 1}, {256, 4, 1}, {256, 4, 3}, {512, 0, 4}, {384, 0, 5}};
  Saved sv;
  if (const int e = save_state(hb, sv, false)) {
    cudaFree(sv.buf);
    return e;
  }
  const int t0 = hb->solve_threads, c0 = hb->solve_ctas_per_sm, s0 = hb->solve_sync, v0 = hb->dc_variant,
            dt0 = hb->dc_threads, dc0 = hb->dc_ctas_per_sm;
  int r = 0;
  float best = 1e30f, best64 = 1e30f;
  Shape b64 = c64[0], b32 = c32[0];
  for (const Shape& s : c64) {
    apply(hb, s, false);
    float ms = 0;
    if ((r = time_trial(hb, false, 5, &ms))) break;
    if (ms < best) best = ms, b64 = s;
  }
  best64 = best;
  best = 1e30f;
  for (const Shape& s : c32) {
    if (r) break;
    if (s.sync == 4 && !tb_solve_fits(hb)) continue;
    if (s.sync == 5 && !zm_solve_fits(hb)) continue;
    apply(hb, s, true);
    float ms = 0;
    if ((r = time_trial(hb, true, 16, &ms))) break;
    if (ms < best) best = ms, b32 = s;
  }
  hb->solve_threads = t0;
  hb->solve_ctas_per_sm = c0;
  hb->solve_sync = s0;
  hb->dc_variant = v0;
  hb->dc_threads = dt0;
  hb->dc_ctas_per_sm = dc0;
  const int rr = save_state(hb, sv, true);
  cudaStreamSynchronize(stream());
  cudaFree(sv.buf);
  if (r) return r;
  if (rr) return rr;
  out->fp64 = b64;
  out->fp32 = b32;
  out->ms64 = best64;
  out->ms32 = best;
  return 0;
}

}  // namespace
}  // namespace bcfd

using namespace bcfd;

extern "C" int bcfd_autotune(int64_t* n_tuned) {
  LibLock lk;
  if (!lib().ready) return BCFD_E_STATE;
  // the blocks other than the first are solved side by side in one batched
  // launch when batching is on and there are several of them
  int others = 0;
  for (size_t q = 1; q < lib().blocks.size(); ++q) others += lib().blocks[q] != nullptr;
  const bool grouped = lib().batch && others > 1;
  int64_t n = 0;
  std::vector<HostBlock*> group;
  std::vector<Tuned> group_t;
  for (size_t q = 0; q < lib().blocks.size(); ++q) {
    HostBlock* hb = lib().blocks[q];
    if (!hb || !hb->d.Acx || !hb->d.Acxf) continue;
    const Dims& d = hb->d.d;
    const auto key = std::make_tuple(d.nx, d.ny, d.nz);
    auto it = cache().find(key);
    Tuned t;
    if (it != cache().end()) {
      t = it->second;
    } else {
      TRY_R(tune_block(hb, &t));
      cache()[key] = t;
      ++n;
    }
    if (q > 0 && grouped) {
      group.push_back(hb);
      group_t.push_back(t);
      continue;
    }
    apply(hb, t.fp64, false);
    apply(hb, t.fp32, true);
  }
  if (!group.empty()) {
    // the group in one batched launch (default shapes: what an earlier call
    // applied is reset first) against its members solved one after the other
    // in their best shapes
    const Shape dflt{0, 0, 0};
    for (HostBlock* hb : group) {
      apply(hb, dflt, true);
      apply(hb, dflt, false);
    }
    std::vector<Saved> sv(group.size());
    std::vector<char> saved(group.size(), 0);  // restore only complete copies
    int r = 0;
    for (size_t q = 0; q < group.size() && !r; ++q) {
      r = save_state(group[q], sv[q], false);
      saved[q] = r == 0;
    }
    float g32 = 0.f, g64 = 0.f;
    if (!r) r = time_group(group, true, 16, &g32);
    if (!r) r = time_group(group, false, 5, &g64);
    int rr = 0;
    for (size_t q = 0; q < group.size(); ++q) {
      if (!saved[q]) continue;
      const int e = save_state(group[q], sv[q], true);
      if (!rr) rr = e;
    }
    cudaStreamSynchronize(stream());
    for (Saved& v : sv) cudaFree(v.buf);
    if (r) return r;
    if (rr) return rr;
    float s32 = 0.f, s64 = 0.f;
    for (const Tuned& t : group_t) s32 += t.ms32, s64 += t.ms64;
    for (size_t q = 0; q < group.size(); ++q) {
      if (s32 < g32) apply(group[q], group_t[q].fp32, true);
      if (s64 < g64) apply(group[q], group_t[q].fp64, false);
    }
  }
  if (n_tuned) *n_tuned = n;
  return 0;
}
