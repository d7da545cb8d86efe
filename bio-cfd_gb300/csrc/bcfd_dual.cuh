// Forward-mode dual numbers with N tangent lanes, for the geometric partials
// of the adjoint through moving bodies: a value and its derivatives with
// respect to N seeded inputs (element centroid and normal, node coordinates).
// Each lane carries the exact derivative of the operations performed on the
// value; branches follow the value, so the derivative is that of the branch
// the forward evaluation took.
#pragma once
#include <cuda_runtime.h>

namespace bcfd {

// the double overloads stay visible beside the dual ones
using ::cos;
using ::fabs;
using ::sin;
using ::sqrt;

template <int N>
struct DualN {
  double v;
  double d[N];
  __host__ __device__ DualN() : v(0.0) {
#pragma unroll
    for (int q = 0; q < N; ++q) d[q] = 0.0;
  }
  __host__ __device__ DualN(double x) : v(x) {
#pragma unroll
    for (int q = 0; q < N; ++q) d[q] = 0.0;
  }
  // an input: value x seeded in lane `lane`
  __host__ __device__ static DualN seed(double x, int lane) {
    DualN r(x);
    r.d[lane] = 1.0;
    return r;
  }
};

template <int N>
__host__ __device__ __forceinline__ DualN<N> operator+(const DualN<N>& a, const DualN<N>& b) {
  DualN<N> r(a.v + b.v);
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = a.d[q] + b.d[q];
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualN<N> operator-(const DualN<N>& a, const DualN<N>& b) {
  DualN<N> r(a.v - b.v);
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = a.d[q] - b.d[q];
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualN<N> operator-(const DualN<N>& a) {
  DualN<N> r(-a.v);
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = -a.d[q];
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualN<N> operator*(const DualN<N>& a, const DualN<N>& b) {
  DualN<N> r(a.v * b.v);
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = a.d[q] * b.v + a.v * b.d[q];
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualN<N> operator/(const DualN<N>& a, const DualN<N>& b) {
  const double iv = 1.0 / b.v;
  DualN<N> r(a.v / b.v);
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = (a.d[q] - r.v * b.d[q]) * iv;
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualN<N> operator+(const DualN<N>& a, double b) { return a + DualN<N>(b); }
template <int N>
__host__ __device__ __forceinline__ DualN<N> operator+(double a, const DualN<N>& b) { return DualN<N>(a) + b; }
template <int N>
__host__ __device__ __forceinline__ DualN<N> operator-(const DualN<N>& a, double b) { return a - DualN<N>(b); }
template <int N>
__host__ __device__ __forceinline__ DualN<N> operator-(double a, const DualN<N>& b) { return DualN<N>(a) - b; }
template <int N>
__host__ __device__ __forceinline__ DualN<N> operator*(const DualN<N>& a, double b) {
  DualN<N> r(a.v * b);
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = a.d[q] * b;
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualN<N> operator*(double a, const DualN<N>& b) { return b * a; }
template <int N>
__host__ __device__ __forceinline__ DualN<N> operator/(const DualN<N>& a, double b) { return a / DualN<N>(b); }
template <int N>
__host__ __device__ __forceinline__ DualN<N> operator/(double a, const DualN<N>& b) { return DualN<N>(a) / b; }
// |x| with the derivative of the branch the value takes (sign(0) = +)
template <int N>
__host__ __device__ __forceinline__ DualN<N> fabs(const DualN<N>& a) { return a.v < 0.0 ? -a : a; }
template <int N>
__host__ __device__ __forceinline__ DualN<N> sqrt(const DualN<N>& a) {
  DualN<N> r(::sqrt(a.v));
  const double h = r.v > 0.0 ? 0.5 / r.v : 0.0;
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = a.d[q] * h;
  return r;
}

template <int N>
__host__ __device__ __forceinline__ DualN<N> sin(const DualN<N>& a) {
  DualN<N> r(::sin(a.v));
  const double c = ::cos(a.v);
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = a.d[q] * c;
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualN<N> cos(const DualN<N>& a) {
  DualN<N> r(::cos(a.v));
  const double sn = -::sin(a.v);
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = a.d[q] * sn;
  return r;
}

}  // namespace bcfd
