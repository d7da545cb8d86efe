// Arithmetic-rate measurement of the GPU the library runs on: FP64 fused
// multiply-adds, FP64 IEEE divisions and FP32 fused multiply-adds, each as
// chains of independent accumulators over every SM, timed with CUDA events on
// the library stream.  The FP64 kernels of the library (the drop-in stencils
// with their value-dependent divisions, the FP64 sweeps) are bound by these
// rates rather than by HBM on a GPU with a low FP64 rate, and a roofline for
// them needs the measured figure.  No counterpart in the reference.
#include "bcfd_host.h"

namespace bcfd {
namespace {

constexpr int kAcc = 8;      // independent chains per thread
constexpr int kIters = 4096;  // operations per chain

__global__ void k_fma64(double* out, double a, double b) {
  double acc[kAcc];
#pragma unroll
  for (int q = 0; q < kAcc; ++q) acc[q] = threadIdx.x * 1e-9 + q;
  for (int it = 0; it < kIters; ++it)
#pragma unroll
    for (int q = 0; q < kAcc; ++q) acc[q] = fma(acc[q], a, b);
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < kAcc; ++q) s += acc[q];
  if (s == 1.2345) out[0] = s;  // keeps the chains alive
}

__global__ void k_fma32(float* out, float a, float b) {
  float acc[kAcc];
#pragma unroll
  for (int q = 0; q < kAcc; ++q) acc[q] = threadIdx.x * 1e-6f + q;
  for (int it = 0; it < kIters; ++it)
#pragma unroll
    for (int q = 0; q < kAcc; ++q) acc[q] = __fmaf_rn(acc[q], a, b);
  float s = 0.f;
#pragma unroll
  for (int q = 0; q < kAcc; ++q) s += acc[q];
  if (s == 1.2345f) out[0] = s;
}

__global__ void k_div64(double* out, double a) {
  double acc[kAcc];
#pragma unroll
  for (int q = 0; q < kAcc; ++q) acc[q] = 1.0 + threadIdx.x * 1e-9 + q;
  for (int it = 0; it < kIters / 16; ++it)
#pragma unroll
    for (int q = 0; q < kAcc; ++q) acc[q] = a / acc[q] + 1.0;
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < kAcc; ++q) s += acc[q];
  if (s == 1.2345) out[0] = s;
}

}  // namespace
}  // namespace bcfd

using namespace bcfd;

extern "C" int bcfd_measure_alu_rates(double* out) {
  LibLock lk;
  if (!lib().ready) return BCFD_E_STATE;
  if (!out) return BCFD_E_ARG;
  double* sink = nullptr;
  BCFD_CUDA(cudaMalloc(&sink, sizeof(double)));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int r = 0;
  auto ck = [&](cudaError_t e) {
    if (e != cudaSuccess && !r) {
      report_cuda(e, "measure_alu_rates", __FILE__, __LINE__);
      r = BCFD_E_CUDA;
    }
  };
  ck(cudaEventCreate(&e0));
  ck(cudaEventCreate(&e1));
  const unsigned grid = 8u * (unsigned)lib().nsm;
  const int threads = 256;
  const double threads_total = (double)grid * threads;
  // each kernel: one untimed launch, then the best of three timed ones
  auto time_it = [&](auto launch) -> double {
    float best = 1e30f;
    for (int rep = 0; rep < 4 && !r; ++rep) {
      ck(cudaEventRecord(e0, stream()));
      launch();
      r = r ? r : note_launch();
      ck(cudaEventRecord(e1, stream()));
      ck(cudaEventSynchronize(e1));
      float ms = 0.f;
      ck(cudaEventElapsedTime(&ms, e0, e1));
      if (rep > 0) best = std::min(best, ms);
    }
    return (double)best * 1e-3;
  };
  const double t64 = time_it([&] { k_fma64<<<grid, threads, 0, stream()>>>(sink, 0.999999, 1e-7); });
  const double t32 = time_it([&] { k_fma32<<<grid, threads, 0, stream()>>>((float*)sink, 0.9999f, 1e-5f); });
  const double tdv = time_it([&] { k_div64<<<grid, threads, 0, stream()>>>(sink, 0.5); });
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (r) return r;
  // GFLOP/s with an FMA counted as two operations; divisions per second
  out[0] = 2.0 * kAcc * kIters * threads_total / t64 * 1e-9;
  out[1] = (double)kAcc * (kIters / 16) * threads_total / tdv * 1e-9;
  out[2] = 2.0 * kAcc * kIters * threads_total / t32 * 1e-9;
  return 0;
}
