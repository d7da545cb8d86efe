// Momentum predictor (nsMomentum2order, src/NavierStokes.f90:252-912) and the
// boundary conditions of src/BoundaryConditions.f90.
//
// One thread per interior cell; non-fluid cells are skipped.  The reference
// loops over the fluid list in (k,j,i) order, and that order matters only next
// to thin-surface (TS) cells: there the loop substitutes ghost values into
// u,v,w,p before a cell's stencil and restores them after it
// (src/NavierStokes.f90:310-490, 860-907), so a cell may read values written
// by earlier cells.  Cells within reach of a TS cell go through a second
// kernel whose reads reproduce that serial order exactly (TsReader below);
// every other cell reads the fields directly.  FP64, compiled without FMA
// contraction, expressions in the reference's evaluation order (T = double);
// the same stencil in FP32 arithmetic serves the mixed-precision path.
#include <type_traits>

#include "bcfd_host.h"

namespace bcfd {

namespace {

struct MomArgs {
  double dt, re;
};

__device__ __forceinline__ bool adj_ok(const int8_t* c, const Dims& d, bool big, int i, int j, int k,
                                       int s) {
  // check_adjacent_cell (src/NavierStokes.f90:1002-1022): false if any of the
  // 6 cells at distance s has tag 2
  auto at = [&](int a, int b, int e) { return big ? c[d.idx3(a, b, e)] : c[d.idx(a, b, e)]; };
  if (at(i - s, j, k) == 2) return false;
  if (at(i + s, j, k) == 2) return false;
  if (at(i, j - s, k) == 2) return false;
  if (at(i, j + s, k) == 2) return false;
  if (at(i, j, k - s) == 2) return false;
  if (at(i, j, k + s) == 2) return false;
  return true;
}

// FP32 number of the mixed path's momentum stencil.  Every divisor of the
// stencil is a grid quantity (spacings, their sums, coefficient-table
// entries, re), so the quotient is taken as a reciprocal times the dividend
// (__fdividef, within 2 ulp of the IEEE quotient) instead of the IEEE
// division's instruction sequence; the stencil's FP32 rounding dominates that
// difference.  The FP64 drop-in stencil keeps IEEE division.
struct FastF {
  float v;
  FastF() = default;
  __device__ __forceinline__ constexpr FastF(float x) : v(x) {}
  __device__ __forceinline__ explicit FastF(double x) : v((float)x) {}
  __device__ __forceinline__ explicit operator double() const { return (double)v; }
};
__device__ __forceinline__ FastF operator+(FastF a, FastF b) { return FastF(a.v + b.v); }
__device__ __forceinline__ FastF operator-(FastF a, FastF b) { return FastF(a.v - b.v); }
__device__ __forceinline__ FastF operator-(FastF a) { return FastF(-a.v); }
__device__ __forceinline__ FastF operator*(FastF a, FastF b) { return FastF(a.v * b.v); }
__device__ __forceinline__ FastF operator/(FastF a, FastF b) { return FastF(__fdividef(a.v, b.v)); }
__device__ __forceinline__ FastF fabs(FastF a) { return FastF(fabsf(a.v)); }

// a grid / coefficient value as T: the FP32 copy for the FP32 stencils, else
// the FP64 table
template <typename T>
__device__ __forceinline__ T grid_t(const double* d64, const float* f32, int q) {
  if constexpr (std::is_same<T, float>::value || std::is_same<T, FastF>::value) return T(f32[q]);
  else return T(d64[q]);
}

// Forward-mode dual number (value, tangent): the stencil evaluated in it gives
// the reference's FP64 value (the value part performs exactly the double
// operations) and the exact derivative of the discrete stencil along the
// input tangent (the tangent-linear model).
struct Dual {
  double v, d;
  __device__ Dual() : v(0.0), d(0.0) {}
  __device__ Dual(double x) : v(x), d(0.0) {}
  __device__ Dual(double x, double dx) : v(x), d(dx) {}
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  const double q = a.v / b.v;
  return Dual(q, (a.d - q * b.d) / b.v);
}
// |x| with the derivative of the branch the value takes (sign(0) = +); the
// global float/double overloads stay visible next to it
using ::fabs;
__device__ __forceinline__ Dual fabs(Dual a) { return a.v < 0.0 ? -a : a; }

// The same with four tangents: one evaluation carries the derivatives along
// four seeds at once.  Each tangent lane performs exactly the operations of
// Dual's tangent on the same operands, so lane l equals the Dual tangent of
// seed l bit for bit.
struct Dual4 {
  double v, d[4];
  __device__ Dual4() : v(0.0), d{0.0, 0.0, 0.0, 0.0} {}
  __device__ Dual4(double x) : v(x), d{0.0, 0.0, 0.0, 0.0} {}
};
__device__ __forceinline__ Dual4 operator+(const Dual4& a, const Dual4& b) {
  Dual4 r(a.v + b.v);
#pragma unroll
  for (int l = 0; l < 4; ++l) r.d[l] = a.d[l] + b.d[l];
  return r;
}
__device__ __forceinline__ Dual4 operator-(const Dual4& a, const Dual4& b) {
  Dual4 r(a.v - b.v);
#pragma unroll
  for (int l = 0; l < 4; ++l) r.d[l] = a.d[l] - b.d[l];
  return r;
}
__device__ __forceinline__ Dual4 operator-(const Dual4& a) {
  Dual4 r(-a.v);
#pragma unroll
  for (int l = 0; l < 4; ++l) r.d[l] = -a.d[l];
  return r;
}
__device__ __forceinline__ Dual4 operator*(const Dual4& a, const Dual4& b) {
  Dual4 r(a.v * b.v);
#pragma unroll
  for (int l = 0; l < 4; ++l) r.d[l] = a.d[l] * b.v + a.v * b.d[l];
  return r;
}
__device__ __forceinline__ Dual4 operator/(const Dual4& a, const Dual4& b) {
  const double q = a.v / b.v;
  Dual4 r(q);
#pragma unroll
  for (int l = 0; l < 4; ++l) r.d[l] = (a.d[l] - q * b.d[l]) / b.v;
  return r;
}
__device__ __forceinline__ Dual4 fabs(const Dual4& a) { return a.v < 0.0 ? -a : a; }

// where a stencil's three results go
struct StoreOut {
  double *ut, *vt, *wt;
  template <typename T>
  __device__ __forceinline__ void put(int q, int64_t c, T val) const {
    (q == 0 ? ut : q == 1 ? vt : wt)[c] = (double)val;
  }
};
struct DualOut {
  double *ut, *vt, *wt, *dut, *dvt, *dwt;
  __device__ __forceinline__ void put(int q, int64_t c, Dual val) const {
    (q == 0 ? ut : q == 1 ? vt : wt)[c] = val.v;
    (q == 0 ? dut : q == 1 ? dvt : dwt)[c] = val.d;
  }
};

// Field reads of the stencil: field f (0 u, 1 v, 2 w, 3 p) at cell (a,b,e),
// linear index x.  The plain reader loads the array.
struct PlainReader {
  const double* f[4];
  __device__ __forceinline__ double get(int q, int, int, int, int64_t x) const { return __ldg(f[q] + x); }
};

// One fluid cell (i,j,k) of nsMomentum2order.  T = double: the reference
// arithmetic (bit-exact drop-in).  T = float: the FP32 momentum stencil of the
// mixed-precision path (fields stay FP64 in HBM; stencil values are rounded to
// FP32 on load, ut/vt/wt stored back as FP64).
template <typename T, class Rd, class Out>
__device__ __forceinline__ void momentum_cell(const DevBlock& B, const MomArgs& a, int i, int j, int k,
                                              int64_t c, const Rd& rd, const Out& out) {
  const T Q25 = T(0.25), HALF = T(0.5), TWO = T(2.0), ONE = T(1.0);
  const Dims& d = B.d;
  const T alpha = ONE;
  const T deltat = T(a.dt), re = T(a.re);
  const int nx_var = d.nx, ny_var = d.ny, nz_var = d.nz;
  const int64_t SX = 1, SY = d.NX, SZ = (int64_t)d.NX * d.NY;
  {
#define u(a, b, e) (T) rd.get(0, i + (a), j + (b), k + (e), c + (a) * SX + (b) * SY + (e) * SZ)
#define v(a, b, e) (T) rd.get(1, i + (a), j + (b), k + (e), c + (a) * SX + (b) * SY + (e) * SZ)
#define w(a, b, e) (T) rd.get(2, i + (a), j + (b), k + (e), c + (a) * SX + (b) * SY + (e) * SZ)
#define p(a, b, e) (T) rd.get(3, i + (a), j + (b), k + (e), c + (a) * SX + (b) * SY + (e) * SZ)
#define DX(q) grid_t<T>(B.dxa, B.dxf, (q) - 1)
#define DY(q) grid_t<T>(B.dya, B.dyf, (q) - 1)
#define DZ(q) grid_t<T>(B.dza, B.dzf, (q) - 1)
#define CA(tab, row, q) grid_t<T>(B.ca[tab], B.caf[tab], ((row) - 1) + 6 * ((q) - 1))
#define CK(tab, row, q) grid_t<T>(B.ck[tab], B.ckf[tab], ((row) - 1) + 6 * ((q) - 1))
    // offsets are relative to (i,j,k): u(-1,0,0) is u(i-1,j,k)
    const T dxr = DX(i + 1), dx = DX(i), dxl = DX(i - 1);
    const T dye = DY(j + 1), dy = DY(j), dyw = DY(j - 1);
    const T dzt = DZ(k + 1), dz = DZ(k), dzb = DZ(k - 1);

    const T u1a = u(-1, 0, 0) + u(0, 0, 0);
    const T u22 = u(-1, 0, 0) - u(0, 0, 0);
    const T u3 = u(0, 0, 0) + u(1, 0, 0);
    const T u4 = u(0, 0, 0) - u(1, 0, 0);
    const T u5 = u(0, -1, 0) + u(0, 0, 0);
    const T u6 = u(0, -1, 0) - u(0, 0, 0);
    const T u7 = u(0, 0, 0) + u(0, 1, 0);
    const T u8 = u(0, 0, 0) - u(0, 1, 0);
    const T u9 = u(0, 0, -1) + u(0, 0, 0);
    const T u10 = u(0, 0, -1) - u(0, 0, 0);
    const T u11 = u(0, 0, 0) + u(0, 0, 1);
    const T u12 = u(0, 0, 0) - u(0, 0, 1);
    const T u13 = u(-1, 0, 0) + u(-1, 1, 0);
    const T u14 = u7;
    const T u15 = u(-1, 0, 0) + u(-1, 0, 1);
    const T u16 = u11;

    const T v1a = v(0, -1, 0) + v(1, -1, 0);
    const T v22 = v(0, 0, 0) + v(1, 0, 0);
    const T v3 = v(-1, 0, 0) + v(0, 0, 0);
    const T v4 = v(-1, 0, 0) - v(0, 0, 0);
    const T v5 = v(0, 0, 0) + v(1, 0, 0);
    const T v6 = v(0, 0, 0) - v(1, 0, 0);
    const T v7 = v(0, -1, 0) + v(0, 0, 0);
    const T v8 = v(0, -1, 0) - v(0, 0, 0);
    const T v9 = v(0, 0, 0) + v(0, 1, 0);
    const T v10 = v(0, 0, 0) - v(0, 1, 0);
    const T v11 = v(0, 0, -1) + v(0, 0, 0);
    const T v12 = v(0, 0, -1) - v(0, 0, 0);
    const T v13 = v(0, 0, 0) + v(0, 0, 1);
    const T v14 = v(0, 0, 0) - v(0, 0, 1);
    const T v15 = v(0, -1, 0) + v(0, -1, 1);
    const T v16 = v13;

    const T w1a = w(0, 0, -1) + w(1, 0, -1);
    const T w22 = w(0, 0, 0) + w(1, 0, 0);
    const T w3 = w(0, 0, -1) + w(0, 1, -1);
    const T w4 = w(0, 0, 0) + w(0, 1, 0);
    const T w5 = w(-1, 0, 0) + w(0, 0, 0);
    const T w6 = w(-1, 0, 0) - w(0, 0, 0);
    const T w7 = w(0, 0, 0) + w(1, 0, 0);
    const T w8 = w(0, 0, 0) - w(1, 0, 0);
    const T w9 = w(0, -1, 0) + w(0, 0, 0);
    const T w10 = w(0, -1, 0) - w(0, 0, 0);
    const T w11 = w(0, 0, 0) + w(0, 1, 0);
    const T w12 = w(0, 0, 0) - w(0, 1, 0);
    const T w13 = w(0, 0, -1) + w(0, 0, 0);
    const T w14 = w(0, 0, -1) - w(0, 0, 0);
    const T w15 = w(0, 0, 0) + w(0, 0, 1);
    const T w16 = w(0, 0, 0) - w(0, 0, 1);

    const T dpdx = (p(0, 0, 0) - p(1, 0, 0)) / (HALF * (dxr + dx));
    const T dpdy = (p(0, 0, 0) - p(0, 1, 0)) / (HALF * (dye + dy));
    const T dpdz = (p(0, 0, 0) - p(0, 0, 1)) / (HALF * (dzt + dz));

    const T dx2xr = dx + dxr, dx2xl = dx + dxl, dy2ye = dy + dye, dy2yw = dy + dyw,
                 dz2zt = dz + dzt, dz2zb = dz + dzb;

    // superset of the three components' third-order index ranges; inside it
    // the distance-2 neighbours exist
    const bool inner = i > 2 && j > 2 && k > 2 && i < nx_var + 1 && j < ny_var + 1 && k < nz_var + 1;
    const bool smooth = inner && adj_ok(B.cell, d, false, i, j, k, 1) && adj_ok(B.cell2, d, true, i, j, k, 2);
    const bool near_ib = !smooth, near_ts2 = false;
    (void)near_ib;

    // ---------------- U momentum ----------------
    {
      const T vu_e = v(1, 0, 0) + (dxr / (dx2xr)) * (v(0, 0, 0) - v(1, 0, 0));
      const T vu_w = v(1, -1, 0) + (dxr / (dx2xr)) * (v(0, -1, 0) - v(1, -1, 0));
      const T v_in_um = HALF * (vu_e + vu_w);
      const T wu_n = w(1, 0, 0) + (dxr / (dx2xr)) * (w(0, 0, 0) - w(1, 0, 0));
      const T wu_s = w(1, 0, -1) + (dxr / (dx2xr)) * (w(0, 0, -1) - w(1, 0, -1));
      const T w_in_um = HALF * (wu_n + wu_s);
      T duudx, dvudy, dwudz;
      const bool third = (i > 2 && i < nx_var && j > 2 && j < ny_var + 1 && k > 2 && k < nz_var + 1) &&
                         !near_ib && !near_ts2;
      if (third) {
        const T ddy = HALF * (DY(j) + DY(j - 1));
        const T ddye = HALF * (DY(j) + DY(j + 1));
        const T ddz = HALF * (DZ(k) + DZ(k - 1));
        const T ddzr = HALF * (DZ(k) + DZ(k + 1));
        duudx = u(0, 0, 0) *
                    (CA(T_UU, 1, i) * u(2, 0, 0) + CA(T_UU, 2, i) * u(1, 0, 0) +
                     CA(T_UU, 3, i) * u(0, 0, 0) + CA(T_UU, 4, i) * u(-1, 0, 0) +
                     CA(T_UU, 5, i) * u(-2, 0, 0)) /
                    (CA(T_UU, 6, i) * DX(i + 1)) +
                fabs(u(0, 0, 0)) *
                    (CK(T_UU, 1, i) * u(2, 0, 0) + CK(T_UU, 2, i) * u(1, 0, 0) +
                     CK(T_UU, 3, i) * u(0, 0, 0) + CK(T_UU, 4, i) * u(-1, 0, 0) +
                     CK(T_UU, 5, i) * u(-2, 0, 0)) /
                    (TWO * CK(T_UU, 6, i) * DX(i));
        dvudy = v_in_um *
                    (CA(T_VU, 1, j) * u(0, 2, 0) + CA(T_VU, 2, j) * u(0, 1, 0) +
                     CA(T_VU, 3, j) * u(0, 0, 0) + CA(T_VU, 4, j) * u(0, -1, 0) +
                     CA(T_VU, 5, j) * u(0, -2, 0)) /
                    (CA(T_VU, 6, j) * ddye) +
                fabs(v_in_um) *
                    (CK(T_VU, 1, j) * u(0, 2, 0) + CK(T_VU, 2, j) * u(0, 1, 0) +
                     CK(T_VU, 3, j) * u(0, 0, 0) + CK(T_VU, 4, j) * u(0, -1, 0) +
                     CK(T_VU, 5, j) * u(0, -2, 0)) /
                    (TWO * CK(T_VU, 6, j) * ddy);
        dwudz = w_in_um *
                    (CA(T_WU, 1, k) * u(0, 0, 2) + CA(T_WU, 2, k) * u(0, 0, 1) +
                     CA(T_WU, 3, k) * u(0, 0, 0) + CA(T_WU, 4, k) * u(0, 0, -1) +
                     CA(T_WU, 5, k) * u(0, 0, -2)) /
                    (CA(T_WU, 6, k) * ddzr) +
                fabs(w_in_um) *
                    (CK(T_WU, 1, k) * u(0, 0, 2) + CK(T_WU, 2, k) * u(0, 0, 1) +
                     CK(T_WU, 3, k) * u(0, 0, 0) + CK(T_WU, 4, k) * u(0, 0, -1) +
                     CK(T_WU, 5, k) * u(0, 0, -2)) /
                    (TWO * CK(T_WU, 6, k) * ddz);
      } else {
        duudx = -Q25 * (u1a * u1a + alpha * fabs(u1a) * u22 - u3 * u3 - alpha * fabs(u3) * u4) / DX(i);
        dvudy = -Q25 * (v1a * u5 + alpha * fabs(v1a) * u6 - v22 * u7 - alpha * fabs(v22) * u8) / DY(j);
        dwudz = -Q25 * (w1a * u9 + alpha * fabs(w1a) * u10 - w22 * u11 - alpha * fabs(w22) * u12) / DZ(k);
      }
      const T d2udx2 = (TWO / dx2xr) * ((-u4 / dxr) + (u22 / dx));
      const T d2udy2 =
          (TWO / (HALF * (dy2ye + dy2yw))) * ((-u8 / (HALF * dy2ye)) + (u6 / (HALF * dy2yw)));
      const T d2udz2 =
          (TWO / (HALF * (dz2zt + dz2zb))) * ((-u12 / (HALF * dz2zt)) + (u10 / (HALF * dz2zb)));
      const T xtt2 = (d2udx2 + d2udy2 + d2udz2) / re;
      const T residu = (-duudx - dvudy - dwudz + xtt2);
      out.put(0, c, u(0, 0, 0) + deltat * (residu + dpdx));
    }
    // ---------------- V momentum ----------------
    {
      const T uv_e = u(0, 1, 0) + (dye / (dy2ye)) * (u(0, 0, 0) - u(0, 1, 0));
      const T uv_w = u(-1, 1, 0) + (dye / (dy2ye)) * (u(-1, 0, 0) - u(-1, 1, 0));
      const T u_in_vm = HALF * (uv_e + uv_w);
      const T wv_n = w(0, 1, 0) + (dye / (dy2ye)) * (w(0, 0, 0) - w(0, 1, 0));
      const T wv_s = w(0, 1, -1) + (dye / (dy2ye)) * (w(0, 0, -1) - w(0, 1, -1));
      const T w_in_vm = HALF * (wv_n + wv_s);
      T duvdx, dvvdy, dwvdz;
      const bool third = (i > 2 && i < nx_var + 1 && j > 2 && j < ny_var && k > 2 && k < nz_var + 1) &&
                         !near_ib && !near_ts2;
      if (third) {
        const T ddx = HALF * (DX(i) + DX(i - 1));
        const T ddxr = HALF * (DX(i) + DX(i + 1));
        const T ddz = HALF * (DZ(k) + DZ(k - 1));
        const T ddzr = HALF * (DZ(k) + DZ(k + 1));
        duvdx = u_in_vm *
                    (CA(T_UW, 1, i) * v(2, 0, 0) + CA(T_UW, 2, i) * v(1, 0, 0) +
                     CA(T_UW, 3, i) * v(0, 0, 0) + CA(T_UW, 4, i) * v(-1, 0, 0) +
                     CA(T_UW, 5, i) * v(-2, 0, 0)) /
                    (CA(T_UW, 6, i) * ddxr) +
                fabs(u_in_vm) *
                    (CK(T_UW, 1, i) * v(2, 0, 0) + CK(T_UW, 2, i) * v(1, 0, 0) +
                     CK(T_UW, 3, i) * v(0, 0, 0) + CK(T_UW, 4, i) * v(-1, 0, 0) +
                     CK(T_UW, 5, i) * v(-2, 0, 0)) /
                    (TWO * CK(T_UW, 6, i) * ddx);
        dvvdy = v(0, 0, 0) *
                    (CA(T_VV, 1, j) * v(0, 2, 0) + CA(T_VV, 2, j) * v(0, 1, 0) +
                     CA(T_VV, 3, j) * v(0, 0, 0) + CA(T_VV, 4, j) * v(0, -1, 0) +
                     CA(T_VV, 5, j) * v(0, -2, 0)) /
                    (CA(T_VV, 6, j) * DY(j + 1)) +
                fabs(v(0, 0, 0)) *
                    (CK(T_VV, 1, j) * v(0, 2, 0) + CK(T_VV, 2, j) * v(0, 1, 0) +
                     CK(T_VV, 3, j) * v(0, 0, 0) + CK(T_VV, 4, j) * v(0, -1, 0) +
                     CK(T_VV, 5, j) * v(0, -2, 0)) /
                    (TWO * CK(T_VV, 6, j) * DY(j));
        dwvdz = w_in_vm *
                    (CA(T_WU, 1, k) * v(0, 0, 2) + CA(T_WU, 2, k) * v(0, 0, 1) +
                     CA(T_WU, 3, k) * v(0, 0, 0) + CA(T_WU, 4, k) * v(0, 0, -1) +
                     CA(T_WU, 5, k) * v(0, 0, -2)) /
                    (CA(T_WU, 6, k) * ddzr) +
                fabs(w_in_vm) *
                    (CK(T_WU, 1, k) * v(0, 0, 2) + CK(T_WU, 2, k) * v(0, 0, 1) +
                     CK(T_WU, 3, k) * v(0, 0, 0) + CK(T_WU, 4, k) * v(0, 0, -1) +
                     CK(T_WU, 5, k) * v(0, 0, -2)) /
                    (TWO * CK(T_WU, 6, k) * ddz);
      } else {
        duvdx = -Q25 * (u13 * v3 + alpha * fabs(u13) * v4 - u14 * v5 - alpha * fabs(u14) * v6) / DX(i);
        dvvdy = -Q25 * (v7 * v7 + alpha * fabs(v7) * v8 - v9 * v9 - alpha * fabs(v9) * v10) / DY(j);
        dwvdz = -Q25 * (w3 * v11 + alpha * fabs(w3) * v12 - w4 * v13 - alpha * fabs(w4) * v14) / DZ(k);
      }
      const T d2vdx2 =
          (TWO / (HALF * (dx2xr + dx2xl))) * ((-v6 / (HALF * dx2xr)) + (v4 / (HALF * dx2xl)));
      const T d2vdy2 = (TWO / dy2ye) * ((-v10 / dye) + (v8 / dy));
      const T d2vdz2 =
          (TWO / (HALF * (dz2zt + dz2zb))) * ((-v14 / (HALF * dz2zt)) + (v12 / (HALF * dz2zb)));
      const T ytt2 = (d2vdx2 + d2vdy2 + d2vdz2) / re;
      const T residv = (-duvdx - dvvdy - dwvdz + ytt2);
      out.put(1, c, v(0, 0, 0) + deltat * (residv + dpdy));
    }
    // ---------------- W momentum ----------------
    {
      const T uw_e = u(0, 0, 1) + (dzt / (dz2zt)) * (u(0, 0, 0) - u(0, 0, 1));
      const T uw_w = u(-1, 0, 1) + (dzt / (dz2zt)) * (u(-1, 0, 0) - u(-1, 0, 1));
      const T u_in_wm = HALF * (uw_e + uw_w);
      const T vw_n = v(0, 0, 1) + (dzt / (dz2zt)) * (v(0, 0, 0) - v(0, 0, 1));
      const T vw_s = v(0, -1, 1) + (dzt / (dz2zt)) * (v(0, -1, 0) - v(0, -1, 1));
      const T v_in_wm = HALF * (vw_n + vw_s);
      T duwdx, dvwdy, dwwdz;
      const bool third = (i > 2 && i < nx_var + 1 && j > 2 && j < ny_var + 1 && k > 2 && k < nz_var) &&
                         !near_ib && !near_ts2;
      if (third) {
        const T ddx = HALF * (DX(i) + DX(i - 1));
        const T ddxr = HALF * (DX(i) + DX(i + 1));
        const T ddy = HALF * (DY(j) + DY(j - 1));
        const T ddye = HALF * (DY(j) + DY(j + 1));
        duwdx = u_in_wm *
                    (CA(T_UW, 1, i) * w(2, 0, 0) + CA(T_UW, 2, i) * w(1, 0, 0) +
                     CA(T_UW, 3, i) * w(0, 0, 0) + CA(T_UW, 4, i) * w(-1, 0, 0) +
                     CA(T_UW, 5, i) * w(-2, 0, 0)) /
                    (CA(T_UW, 6, i) * ddxr) +
                fabs(u_in_wm) *
                    (CK(T_UW, 1, i) * w(2, 0, 0) + CK(T_UW, 2, i) * w(1, 0, 0) +
                     CK(T_UW, 3, i) * w(0, 0, 0) + CK(T_UW, 4, i) * w(-1, 0, 0) +
                     CK(T_UW, 5, i) * w(-2, 0, 0)) /
                    (TWO * CK(T_UW, 6, i) * ddx);
        dvwdy = v_in_wm *
                    (CA(T_VW, 1, j) * w(0, 2, 0) + CA(T_VW, 2, j) * w(0, 1, 0) +
                     CA(T_VW, 3, j) * w(0, 0, 0) + CA(T_VW, 4, j) * w(0, -1, 0) +
                     CA(T_VW, 5, j) * w(0, -2, 0)) /
                    (CA(T_VW, 6, j) * ddye) +
                fabs(v_in_wm) *
                    (CK(T_VW, 1, j) * w(0, 2, 0) + CK(T_VW, 2, j) * w(0, 1, 0) +
                     CK(T_VW, 3, j) * w(0, 0, 0) + CK(T_VW, 4, j) * w(0, -1, 0) +
                     CK(T_VW, 5, j) * w(0, -2, 0)) /
                    (TWO * CK(T_VW, 6, j) * ddy);
        dwwdz = w(0, 0, 0) *
                    (CA(T_WW, 1, k) * w(0, 0, 2) + CA(T_WW, 2, k) * w(0, 0, 1) +
                     CA(T_WW, 3, k) * w(0, 0, 0) + CA(T_WW, 4, k) * w(0, 0, -1) +
                     CA(T_WW, 5, k) * w(0, 0, -2)) /
                    (CA(T_WW, 6, k) * DZ(k + 1)) +
                fabs(w(0, 0, 0)) *
                    (CK(T_WW, 1, k) * w(0, 0, 2) + CK(T_WW, 2, k) * w(0, 0, 1) +
                     CK(T_WW, 3, k) * w(0, 0, 0) + CK(T_WW, 4, k) * w(0, 0, -1) +
                     CK(T_WW, 5, k) * w(0, 0, -2)) /
                    (TWO * CK(T_WW, 6, k) * DZ(k));
      } else {
        duwdx = -HALF * (u15 * w5 + alpha * fabs(u15) * w6 - u16 * w7 - alpha * fabs(u16) * w8) / DX(i);
        dvwdy = -HALF * (v15 * w9 + alpha * fabs(v15) * w10 - v16 * w11 - alpha * fabs(v16) * w12) / DY(j);
        dwwdz = -HALF * (w13 * w13 + alpha * fabs(w13) * w14 - w15 * w15 - alpha * fabs(w15) * w16) / DZ(k);
      }
      const T d2wdx2 =
          (TWO / (HALF * (dx2xr + dx2xl))) * ((-w8 / (HALF * dx2xr)) + (w6 / (HALF * dx2xl)));
      const T d2wdy2 =
          (TWO / (HALF * (dy2ye + dy2yw))) * ((-w12 / (HALF * dy2ye)) + (w10 / (HALF * dy2yw)));
      const T d2wdz2 = (TWO / dz2zt) * ((-w16 / dzt) + (w14 / dz));
      const T ztt2 = (d2wdx2 + d2wdy2 + d2wdz2) / re;
      const T residw = (-duwdx - dvwdy - dwwdz + ztt2);
      out.put(2, c, w(0, 0, 0) + deltat * (residw + dpdz));
    }
#undef u
#undef v
#undef w
#undef p
#undef DX
#undef DY
#undef DZ
#undef CA
#undef CK
  }
}

template <typename T>
struct MomentumOp {
  MomArgs a;
  __device__ void run(const DevBlock& B, int cta, int ncta) const {
    const PlainReader rd{{B.u, B.v, B.w, B.p}};
    FOR_INTERIOR(B, cta, ncta) {
      INTERIOR_CELL(B);
      if (B.cell[c] != 0) continue;
      if (B.tsnear[c]) continue;  // done by MomentumTsOp
      momentum_cell<T>(B, a, i, j, k, c, rd, StoreOut{B.ut, B.vt, B.wt});
    }
  }
};

// ---------------------------------------------------------------------------
// Thin-surface overlay.  Every position the reference substitutes or
// restores is one of a TS cell T's seven own positions; the kind K of the
// position fixes the ghost slot, the element list and the face coordinate of
// its sign test:
//   U2 u(T), U1 u(T-ex), V2 v(T), V1 v(T-ey), W2 w(T), W1 w(T-ez), P p(T).
// A fluid cell F whose +d neighbour is T handles six of them (direction d
// excludes one kind: +x U1, -x U2, +y V1, -y V2, +z W1, -z W2):
//  * before its stencil it writes kind K with ghost_K(nn) for the last TS
//    list entry nn whose sign test at F's own face is negative (the test does
//    not depend on which TS cell is F's neighbour);
//  * after its stencil it restores kind K with tghost_K(n_ts), the saved value
//    of the last TS entry (the index the reference's loop leaves behind).
// So a cell G reads position X as: its own write if it made one, else the
// restore of the latest fluid cell before G (list order = linear index order)
// that restores X, else the original value; and after the loop X holds the
// restore of the latest restorer overall (k_ts_restore).
// ---------------------------------------------------------------------------
enum TsKind { K_U2 = 0, K_U1, K_V2, K_V1, K_W2, K_W1, K_P, N_KIND };

__device__ __forceinline__ int ghost_slot(int K) {
  // ghost[] order: p, pt, u2, u2t, v2, v2t, w2, w2t, u1, u1t, v1, v1t, w1, w1t
  return K == K_P ? G_P : (K & 1) ? (G_U1 + 2 * (K >> 1)) : (G_U2 + 2 * (K >> 1));
}
__device__ __forceinline__ int nel_slot(int K) {
  // nel[] order: p, u1, u2, v1, v2, w1, w2
  return K == K_P ? N_P : (N_U1 + 2 * (K >> 1) + ((K & 1) ? 0 : 1));
}
// the kind direction d (0..5 = +x,-x,+y,-y,+z,-z) does not handle
__device__ __forceinline__ int excluded_kind(int dir) {
  return 2 * (dir >> 1) + ((dir & 1) ? 0 : 1);
}
__device__ __forceinline__ void dir_vec(int dir, int& a, int& b, int& e) {
  const int s = (dir & 1) ? -1 : 1;
  a = (dir >> 1) == 0 ? s : 0;
  b = (dir >> 1) == 1 ? s : 0;
  e = (dir >> 1) == 2 ? s : 0;
}

// latest restorer F (linear index < before) of position kind K of TS cell T;
// updates best / val / kind
__device__ __forceinline__ void latest_restore(const DevBlock& B, int ti, int tj, int tk, int K,
                                               int64_t before, const double* rconst, int64_t& best,
                                               double& val, int& kind) {
  const Dims& d = B.d;
#pragma unroll
  for (int dir = 0; dir < 6; ++dir) {
    if (K == excluded_kind(dir)) continue;
    int a, b, e;
    dir_vec(dir, a, b, e);
    // F's +dir neighbour is T
    const int fi = ti - a, fj = tj - b, fk = tk - e;
    if (fi < 2 || fj < 2 || fk < 2 || fi > d.nx + 1 || fj > d.ny + 1 || fk > d.nz + 1) continue;
    const int64_t lf = d.idx(fi, fj, fk);
    if (lf >= before || lf <= best) continue;
    if (B.cell[lf] != 0) continue;
    best = lf;
    val = rconst[K];
    kind = K;
  }
}

// the (up to two) TS cells and kinds a position of field q belongs to
__device__ __forceinline__ int owners(const DevBlock& B, int q, int xi, int xj, int xk, int ot[2][4]) {
  const Dims& d = B.d;
  int n = 0;
  auto ts = [&](int a, int b, int e) {
    return a >= 1 && b >= 1 && e >= 1 && a <= d.nx + 3 && b <= d.ny + 3 && e <= d.nz + 3 &&
           B.cell2[d.idx3(a, b, e)] == 2;
  };
  if (q == 3) {
    if (ts(xi, xj, xk)) { ot[n][0] = xi; ot[n][1] = xj; ot[n][2] = xk; ot[n][3] = K_P; ++n; }
    return n;
  }
  if (ts(xi, xj, xk)) { ot[n][0] = xi; ot[n][1] = xj; ot[n][2] = xk; ot[n][3] = 2 * q; ++n; }
  const int ai = xi + (q == 0), aj = xj + (q == 1), ak = xk + (q == 2);
  if (ts(ai, aj, ak)) { ot[n][0] = ai; ot[n][1] = aj; ot[n][2] = ak; ot[n][3] = 2 * q + 1; ++n; }
  return n;
}

// One read of position x (field q) by cell G near TS cells, in the
// reference's serial order: the value and where it came from (how 0: the
// array, 1: G's own substitution of kind K, the ghost value of TS entry
// last[K]; 2: the restore of kind K, the t-ghost value of the last entry).
struct TsHit {
  double v;
  int how, K;
};
// not inlined: one copy of the overlay logic serves all ~150 stencil reads
__device__ __noinline__ TsHit ts_read(const DevBlock& B, int gi, int gj, int gk, int64_t glin, const int* last,
                                      const double* rconst, int q, int xi, int xj, int xk, int64_t x) {
  const double* f = q == 0 ? B.u : q == 1 ? B.v : q == 2 ? B.w : B.p;
  const double orig = __ldg(f + x);
  int ot[2][4];
  const int n = owners(B, q, xi, xj, xk, ot);
  if (n == 0) return TsHit{orig, 0, 0};
  // own substitution: T is an axis neighbour of G and the direction handles K
  for (int m = 0; m < n; ++m) {
    const int di = ot[m][0] - gi, dj = ot[m][1] - gj, dk = ot[m][2] - gk;
    const int ad = abs(di) + abs(dj) + abs(dk);
    if (ad != 1) continue;
    const int dir = di ? (di > 0 ? 0 : 1) : dj ? (dj > 0 ? 2 : 3) : (dk > 0 ? 4 : 5);
    const int K = ot[m][3];
    if (K == excluded_kind(dir)) continue;
    if (last[K] >= 0) return TsHit{B.ghost[ghost_slot(K)][last[K]], 1, K};
  }
  int64_t best = -1;
  double val = orig;
  int kind = 0;
  for (int m = 0; m < n; ++m)
    latest_restore(B, ot[m][0], ot[m][1], ot[m][2], ot[m][3], glin, rconst, best, val, kind);
  return best >= 0 ? TsHit{val, 2, kind} : TsHit{orig, 0, 0};
}

// Reads of a cell G near TS cells, in the reference's serial order.
struct TsReader {
  const DevBlock* B;
  int gi, gj, gk;
  int64_t glin;
  int last[N_KIND];      // own substitution: last TS entry with a negative test, -1: none
  double rconst[N_KIND]; // restore value of each kind
  __device__ __forceinline__ double get(int q, int xi, int xj, int xk, int64_t x) const {
    return ts_read(*B, gi, gj, gk, glin, last, rconst, q, xi, xj, xk, x).v;
  }
};

__device__ __forceinline__ void restore_consts(const DevBlock& B, int nts, double* rc) {
#pragma unroll
  for (int K = 0; K < N_KIND; ++K) rc[K] = nts > 0 ? B.ghost[ghost_slot(K) + 1][nts - 1] : 0.0;
}

// sign tests of src/NavierStokes.f90:321-354 for every TS entry: the last
// entry with a negative test, per kind.  The reference's loop keeps the last
// hit, so the entries are visited from the end and each kind stops at its
// first hit: the same entry, the same sign test arithmetic, and usually a few
// entries instead of all of them.
__device__ void own_substitution(const DevBlock& B, int i, int j, int k, int nts, int* last) {
  const double X[N_KIND] = {B.x1[i], B.x1[i - 1], B.xp[i - 1], B.xp[i - 1], B.xp[i - 1], B.xp[i - 1], B.xp[i - 1]};
  const double Y[N_KIND] = {B.yp[j - 1], B.yp[j - 1], B.y1[j], B.y1[j - 1], B.yp[j - 1], B.yp[j - 1], B.yp[j - 1]};
  const double Z[N_KIND] = {B.zp[k - 1], B.zp[k - 1], B.zp[k - 1], B.zp[k - 1], B.z1[k], B.z1[k - 1], B.zp[k - 1]};
#pragma unroll
  for (int K = 0; K < N_KIND; ++K) last[K] = -1;
  unsigned open = (1u << N_KIND) - 1u;  // kinds still without a hit
  for (int nn = nts - 1; nn >= 0 && open; --nn) {
    const int bt = B.ts_idx[nn] - 1;
#pragma unroll
    for (int K = 0; K < N_KIND; ++K) {
      if (!(open & (1u << K))) continue;
      const int e = B.nel[nel_slot(K)][bt] - 1;
      const double t = (X[K] - B.xcent[e]) * B.cosA[e] + (Y[K] - B.ycent[e]) * B.cosB[e] +
                       (Z[K] - B.zcent[e]) * B.cosG[e];
      if (t < 0) {
        last[K] = nn;
        open &= ~(1u << K);
      }
    }
  }
}

template <typename T>
struct MomentumTsOp {
  MomArgs a;
  __device__ void run(const DevBlock& B, int cta, int ncta) const {
  const Dims& d = B.d;
  const int nts = (int)min(B.cnt[C_TS], (int64_t)B.cap_ib);
  FOR_INTERIOR(B, cta, ncta) {
    INTERIOR_CELL(B);
    if (B.cell[c] != 0 || !B.tsnear[c]) continue;
    TsReader rd;
    rd.B = &B;
    rd.gi = i;
    rd.gj = j;
    rd.gk = k;
    rd.glin = c;
    restore_consts(B, nts, rd.rconst);
    const bool adj = !adj_ok(B.cell2, d, true, i, j, k, 1);
    if (adj) {
      own_substitution(B, i, j, k, nts, rd.last);
    } else {
#pragma unroll
      for (int K = 0; K < N_KIND; ++K) rd.last[K] = -1;
    }
    momentum_cell<T>(B, a, i, j, k, c, rd, StoreOut{B.ut, B.vt, B.wt});
  }
  }
};

// tangent-linear stencil: reads (u,v,w,p) and their tangents
struct DualReader {
  const double* f[4];
  const double* df[4];
  __device__ __forceinline__ Dual get(int q, int, int, int, int64_t x) const {
    return Dual(__ldg(f[q] + x), __ldg(df[q] + x));
  }
};

struct MomentumTlmOp {
  MomArgs a;
  const double* du[4];
  double *ut, *vt, *wt, *dut, *dvt, *dwt;
  __device__ void run(const DevBlock& B, int cta, int ncta) const {
    const DualReader rd{{B.u, B.v, B.w, B.p}, {du[0], du[1], du[2], du[3]}};
    const DualOut out{ut, vt, wt, dut, dvt, dwt};
    FOR_INTERIOR(B, cta, ncta) {
      INTERIOR_CELL(B);
      if (B.cell[c] != 0) continue;
      if (B.tsnear[c]) {
        set_err(B.err, BCFD_E_STATE);  // the thin-surface overlay has no tangent model
        continue;
      }
      momentum_cell<Dual>(B, a, i, j, k, c, rd, out);
    }
  }
};

// ---------------------------------------------------------------------------
// Adjoint (reverse mode) of the predictor, as a gather: the adjoint of input
// position X of field f is  sum over fluid cells C that read X, over the
// three outputs q, of  seed_q(C) * dF_q(C)/dX_f.  Each partial is the tangent
// of the dual-number stencil at C seeded with 1 at (f, X), so it is the exact
// transpose of the tangent-linear model, summed in a fixed order (footprint
// offsets ascending, outputs U,V,W): deterministic, no atomics.
// The footprint (the (field, offset) pairs the stencil reads, offsets in
// [-2,2]^3) is collected once per call from the block's own branches.
// ---------------------------------------------------------------------------
constexpr int kFootWords = 16;  // 4 fields x 125 offsets, 4 words per field

struct FootReader {
  const double* f[4];
  uint32_t* m;  // per-thread mask
  int ci, cj, ck;
  int* err;
  __device__ __forceinline__ double get(int q, int ii, int jj, int kk, int64_t x) const {
    const int a = ii - ci, b = jj - cj, e = kk - ck;
    if (a < -2 || a > 2 || b < -2 || b > 2 || e < -2 || e > 2) {
      set_err(err, BCFD_E_STATE);  // a read outside [-2,2]^3 (none in the stencil)
    } else {
      const int o = (a + 2) + 5 * (b + 2) + 25 * (e + 2);
      m[4 * q + (o >> 5)] |= 1u << (o & 31);
    }
    return __ldg(f[q] + x);
  }
};
struct NullOut {
  template <typename T>
  __device__ __forceinline__ void put(int, int64_t, T) const {}
};

// the footprint of a cell near TS cells: its reads go through the overlay,
// so its branches are those of the forward loop
struct FootTsReader {
  const DevBlock* B;
  int gi, gj, gk;
  int64_t glin;
  const int* last;
  const double* rconst;
  uint32_t* m;
  __device__ __forceinline__ double get(int q, int ii, int jj, int kk, int64_t x) const {
    const int a = ii - gi, b = jj - gj, e = kk - gk;
    if (a < -2 || a > 2 || b < -2 || b > 2 || e < -2 || e > 2) {
      set_err(B->err, BCFD_E_STATE);
    } else {
      const int o = (a + 2) + 5 * (b + 2) + 25 * (e + 2);
      m[4 * q + (o >> 5)] |= 1u << (o & 31);
    }
    return ts_read(*B, gi, gj, gk, glin, last, rconst, q, ii, jj, kk, x).v;
  }
};

// ts_last: per point, the own-substitution entries of the cells near TS
// cells (k_ts_last); nullptr: such cells are skipped
__global__ void k_mom_footprint(DevBlock B, MomArgs a, uint32_t* foot, const int* ts_last) {
  uint32_t m[kFootWords];
#pragma unroll
  for (int w = 0; w < kFootWords; ++w) m[w] = 0u;
  const Dims& d = B.d;
  const int nts = (int)min(B.cnt[C_TS], (int64_t)B.cap_ib);
  double rc[N_KIND];
  restore_consts(B, nts, rc);
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 2 + (int)(t % d.nx);
    const int64_t r = t / d.nx;
    const int j = 2 + (int)(r % d.ny), k = 2 + (int)(r / d.ny);
    const int64_t c = d.idx(i, j, k);
    if (B.cell[c] != 0) continue;
    if (B.tsnear[c]) {
      if (!ts_last) continue;
      const FootTsReader rd{&B, i, j, k, c, ts_last + N_KIND * c, rc, m};
      momentum_cell<double>(B, a, i, j, k, c, rd, NullOut{});
      continue;
    }
    const FootReader rd{{B.u, B.v, B.w, B.p}, m, i, j, k, B.err};
    momentum_cell<double>(B, a, i, j, k, c, rd, NullOut{});
  }
#pragma unroll
  for (int w = 0; w < kFootWords; ++w) {
    uint32_t v = m[w];
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) v |= __shfl_xor_sync(0xffffffffu, v, s);
    if ((threadIdx.x & 31) == 0 && v) atomicOr(foot + w, v);
  }
}

// four-lane dual reader: lane f carries the seed 1 at (field f, linear index sx)
struct SeedReader4 {
  const double* f[4];
  int64_t sx;
  __device__ __forceinline__ Dual4 get(int q, int, int, int, int64_t x) const {
    Dual4 r(__ldg(f[q] + x));
    if (x == sx) r.d[q] = 1.0;
    return r;
  }
};
// the same for a cell near TS cells: a read the overlay redirects to a ghost
// or t-ghost value does not depend on the array value at x
struct TsSeedReader4 {
  const DevBlock* B;
  int gi, gj, gk;
  int64_t glin;
  const int* last;
  const double* rconst;
  int64_t sx;
  __device__ __forceinline__ Dual4 get(int q, int xi, int xj, int xk, int64_t x) const {
    const TsHit h = ts_read(*B, gi, gj, gk, glin, last, rconst, q, xi, xj, xk, x);
    Dual4 r(h.v);
    if (h.how == 0 && x == sx) r.d[q] = 1.0;
    return r;
  }
};
// lanes on the ghost scalars a cell near TS cells reads: scalar s (0..6 the
// own substitution of kind s, 7..13 the restore of kind s - 7) is lane
// s - 4 pass of the pass
struct TsGhostReader4 {
  const DevBlock* B;
  int gi, gj, gk;
  int64_t glin;
  const int* last;
  const double* rconst;
  int pass;
  __device__ __forceinline__ Dual4 get(int q, int xi, int xj, int xk, int64_t x) const {
    const TsHit h = ts_read(*B, gi, gj, gk, glin, last, rconst, q, xi, xj, xk, x);
    Dual4 r(h.v);
    if (h.how) {
      const int l = (h.how == 1 ? h.K : N_KIND + h.K) - 4 * pass;
      if (l >= 0 && l < 4) r.d[l] = 1.0;
    }
    return r;
  }
};

// adds seed_q(C) * dF_q(C)/dX_f to field f's sum, for the fields whose
// footprint holds this offset (the others' partials are zero)
struct AdjOut4 {
  const double* sb[3];
  double* acc;
  unsigned fmask;
  __device__ __forceinline__ void put(int q, int64_t c, const Dual4& val) const {
    const double s = __ldg(sb[q] + c);
#pragma unroll
    for (int f = 0; f < 4; ++f)
      if ((fmask >> f) & 1u) acc[f] += s * val.d[f];
  }
};

// One dual evaluation per (point, footprint offset) gives the partials of all
// four fields at that point; each field's sum takes the offsets in ascending
// order and, within one, the outputs U, V, W: the order of one evaluation per
// field and offset, so the sums are those of four single-seed gathers.
__global__ void __launch_bounds__(128) k_mom_adjoint(DevBlock B, MomArgs a, const uint32_t* __restrict__ foot,
                                                     const double* ubar_t, const double* vbar_t,
                                                     const double* wbar_t, double* ub, double* vb, double* wb,
                                                     double* pb, const int* ts_last) {
  const Dims& d = B.d;
  const int64_t n = d.npts();
  const int nts = (int)min(B.cnt[C_TS], (int64_t)B.cap_ib);
  double rc[N_KIND];
  restore_consts(B, nts, rc);
  uint32_t m[kFootWords];
#pragma unroll
  for (int w = 0; w < kFootWords; ++w) m[w] = __ldg(foot + w);
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const int xi = 1 + (int)(x % d.NX);
    const int64_t r = x / d.NX;
    const int xj = 1 + (int)(r % d.NY), xk = 1 + (int)(r / d.NY);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int o = 0; o < 125; ++o) {
      unsigned fmask = 0u;
#pragma unroll
      for (int f = 0; f < 4; ++f) fmask |= ((m[4 * f + (o >> 5)] >> (o & 31)) & 1u) << f;
      if (!fmask) continue;
      const int ci = xi - (o % 5 - 2), cj = xj - ((o / 5) % 5 - 2), ck = xk - (o / 25 - 2);
      if (ci < 2 || ci > d.nx + 1 || cj < 2 || cj > d.ny + 1 || ck < 2 || ck > d.nz + 1) continue;
      const int64_t c = d.idx(ci, cj, ck);
      if (B.cell[c] != 0) continue;
      if (B.tsnear[c]) {
        if (!ts_last) {
          set_err(B.err, BCFD_E_STATE);  // the overlay's entries are needed
          continue;
        }
        const TsSeedReader4 rd{&B, ci, cj, ck, c, ts_last + N_KIND * c, rc, x};
        momentum_cell<Dual4>(B, a, ci, cj, ck, c, rd, AdjOut4{{ubar_t, vbar_t, wbar_t}, acc, fmask});
        continue;
      }
      const SeedReader4 rd{{B.u, B.v, B.w, B.p}, x};
      momentum_cell<Dual4>(B, a, ci, cj, ck, c, rd, AdjOut4{{ubar_t, vbar_t, wbar_t}, acc, fmask});
    }
    ub[x] += acc[0];
    vb[x] += acc[1];
    wb[x] += acc[2];
    pb[x] += acc[3];
  }
}

// u,v,w,p at TS positions after the loop: the restore of the latest restorer
struct TsRestoreOp {
  __device__ void run(const DevBlock& B, int cta, int ncta) const {
  const Dims& d = B.d;
  const int nts = (int)min(B.cnt[C_TS], (int64_t)B.cap_ib);
  double rc[N_KIND];
  restore_consts(B, nts, rc);
  for (int t = cta * blockDim.x + threadIdx.x; t < nts * N_KIND; t += ncta * blockDim.x) {
    const int nn = t / N_KIND, K = t % N_KIND;
    const int bt = B.ts_idx[nn] - 1;
    const int ti = B.ib_i[bt], tj = B.ib_j[bt], tk = B.ib_k[bt];
    const int q = K == K_P ? 3 : K >> 1;
    const int xi = ti - (K == K_U1), xj = tj - (K == K_V1), xk = tk - (K == K_W1);
    int ot[2][4];
    const int n = owners(B, q, xi, xj, xk, ot);
    int64_t best = -1;
    double val = 0.0;
    int kind = 0;
    for (int m = 0; m < n; ++m)
      latest_restore(B, ot[m][0], ot[m][1], ot[m][2], ot[m][3], INT64_MAX, rc, best, val, kind);
    if (best < 0) continue;
    double* f = q == 0 ? B.u : q == 1 ? B.v : q == 2 ? B.w : B.p;
    f[d.idx(xi, xj, xk)] = val;
  }
  }
};

// ---------------------------------------------------------------------------
// Adjoint of the thin-surface overlay.  A cell near TS cells reads, besides
// array values, 14 scalars: the ghost value of kind K of TS entry last[K]
// (its own substitution) and the t-ghost value of kind K of the last TS entry
// (the restore).  Their adjoints go to the ghost arrays' adjoint gb (14
// arrays of cap entries, the ghost[] order); the loop's final restore is
// transposed first.  Sums in a fixed order: one thread per accumulation.
// ---------------------------------------------------------------------------

// the own-substitution entries of every fluid cell near TS cells
__global__ void k_ts_last(DevBlock B, int* last) {
  const Dims& d = B.d;
  const int nts = (int)min(B.cnt[C_TS], (int64_t)B.cap_ib);
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 2 + (int)(t % d.nx);
    const int64_t r = t / d.nx;
    const int j = 2 + (int)(r % d.ny), k = 2 + (int)(r / d.ny);
    const int64_t c = d.idx(i, j, k);
    if (B.cell[c] != 0 || !B.tsnear[c]) continue;
    int l[N_KIND];
    if (!adj_ok(B.cell2, d, true, i, j, k, 1)) {
      own_substitution(B, i, j, k, nts, l);
    } else {
#pragma unroll
      for (int K = 0; K < N_KIND; ++K) l[K] = -1;
    }
#pragma unroll
    for (int K = 0; K < N_KIND; ++K) last[N_KIND * c + K] = l[K];
  }
}

// per fluid cell near TS cells: seed . dF/d(scalar s) for its 14 scalars
__global__ void __launch_bounds__(128) k_mom_ghost_contrib(DevBlock B, MomArgs a, const int* last,
                                                           const double* ubar_t, const double* vbar_t,
                                                           const double* wbar_t, double* contrib) {
  const Dims& d = B.d;
  const int nts = (int)min(B.cnt[C_TS], (int64_t)B.cap_ib);
  double rc[N_KIND];
  restore_consts(B, nts, rc);
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 2 + (int)(t % d.nx);
    const int64_t r = t / d.nx;
    const int j = 2 + (int)(r % d.ny), k = 2 + (int)(r / d.ny);
    const int64_t c = d.idx(i, j, k);
    if (B.cell[c] != 0 || !B.tsnear[c]) continue;
    for (int pass = 0; pass < 4; ++pass) {
      double acc[4] = {0.0, 0.0, 0.0, 0.0};
      const TsGhostReader4 rd{&B, i, j, k, c, last + N_KIND * c, rc, pass};
      momentum_cell<Dual4>(B, a, i, j, k, c, rd, AdjOut4{{ubar_t, vbar_t, wbar_t}, acc, 0xFu});
#pragma unroll
      for (int l = 0; l < 4; ++l)
        if (4 * pass + l < 2 * N_KIND) contrib[2 * N_KIND * c + 4 * pass + l] = acc[l];
    }
  }
}

// the cells near TS cells in list (linear index) order, inside the box of the
// TS cells grown by the stencil's reach: contributions into gb
__global__ void k_mom_ghost_acc(DevBlock B, const int* last, const double* contrib, double* gb, int64_t cap) {
  if (blockIdx.x || threadIdx.x) return;
  const Dims& d = B.d;
  const int nts = (int)min(B.cnt[C_TS], (int64_t)B.cap_ib);
  if (nts <= 0) return;
  int lo[3] = {d.nx + 1, d.ny + 1, d.nz + 1}, hi[3] = {2, 2, 2};
  for (int nn = 0; nn < nts; ++nn) {
    const int bt = B.ts_idx[nn] - 1;
    const int p[3] = {B.ib_i[bt], B.ib_j[bt], B.ib_k[bt]};
    for (int q = 0; q < 3; ++q) {
      lo[q] = min(lo[q], p[q] - 3);
      hi[q] = max(hi[q], p[q] + 3);
    }
  }
  lo[0] = max(lo[0], 2); lo[1] = max(lo[1], 2); lo[2] = max(lo[2], 2);
  hi[0] = min(hi[0], d.nx + 1); hi[1] = min(hi[1], d.ny + 1); hi[2] = min(hi[2], d.nz + 1);
  for (int k = lo[2]; k <= hi[2]; ++k)
    for (int j = lo[1]; j <= hi[1]; ++j)
      for (int i = lo[0]; i <= hi[0]; ++i) {
        const int64_t c = d.idx(i, j, k);
        if (B.cell[c] != 0 || !B.tsnear[c]) continue;
        for (int K = 0; K < N_KIND; ++K) {
          const int l = last[N_KIND * c + K];
          if (l >= 0) gb[ghost_slot(K) * cap + l] += contrib[2 * N_KIND * c + K];
          gb[(ghost_slot(K) + 1) * cap + nts - 1] += contrib[2 * N_KIND * c + N_KIND + K];
        }
      }
}

// the final restore transposed: a restored position's adjoint goes to the
// t-ghost value it received; positions shared by two TS cells are visited
// twice, the second visit adds the zero the first left
__global__ void k_ts_restore_adj(DevBlock B, double* ub, double* vb, double* wb, double* pb, double* gb,
                                 int64_t cap) {
  if (blockIdx.x || threadIdx.x) return;
  const Dims& d = B.d;
  const int nts = (int)min(B.cnt[C_TS], (int64_t)B.cap_ib);
  double rc[N_KIND];
  restore_consts(B, nts, rc);
  for (int t = 0; t < nts * N_KIND; ++t) {
    const int nn = t / N_KIND, K = t % N_KIND;
    const int bt = B.ts_idx[nn] - 1;
    const int ti = B.ib_i[bt], tj = B.ib_j[bt], tk = B.ib_k[bt];
    const int q = K == K_P ? 3 : K >> 1;
    const int xi = ti - (K == K_U1), xj = tj - (K == K_V1), xk = tk - (K == K_W1);
    int ot[2][4];
    const int n = owners(B, q, xi, xj, xk, ot);
    int64_t best = -1;
    double val = 0.0;
    int kind = 0;
    for (int m = 0; m < n; ++m)
      latest_restore(B, ot[m][0], ot[m][1], ot[m][2], ot[m][3], INT64_MAX, rc, best, val, kind);
    if (best < 0) continue;
    double* f = q == 0 ? ub : q == 1 ? vb : q == 2 ? wb : pb;
    const int64_t x = d.idx(xi, xj, xk);
    gb[(ghost_slot(kind) + 1) * cap + nts - 1] += f[x];
    f[x] = 0.0;
  }
}

// velocityBC loop 1 (x faces), src/BoundaryConditions.f90:16-40
__global__ void k_vbc_x(DevBlock B, double deltat, double uc) {
  const Dims& d = B.d;
  const int n = d.ny * d.nz;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int j = 2 + t % d.ny, k = 2 + t / d.ny;
    const int nx = d.nx;
    const int64_t c1 = d.idx(1, j, k), cn = d.idx(nx, j, k), cn1 = d.idx(nx + 1, j, k),
                  cn2 = d.idx(nx + 2, j, k);
    B.ut[c1] = uc;
    B.vt[c1] = -B.vt[cn1];
    B.wt[c1] = -B.wt[cn1];
    B.ut[cn1] = B.u[cn1] - (deltat / B.dxa[nx]) * uc * (B.u[cn1] - B.u[cn]);
    B.vt[cn2] = -B.vt[cn1] + B.v[cn2] + B.v[cn1] -
                (2.0 * deltat / B.dxa[nx + 1]) * uc * (B.v[cn2] - B.v[cn1]);
    B.wt[cn2] = -B.wt[cn1] + B.w[cn2] + B.w[cn1] -
                (2.0 * deltat / B.dxa[nx + 1]) * uc * (B.w[cn2] - B.w[cn1]);
  }
}

// velocityBC loop 2 (y faces), src/BoundaryConditions.f90:42-58
__global__ void k_vbc_y(DevBlock B) {
  const Dims& d = B.d;
  const int n = d.nx * d.nz;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int i = 2 + t % d.nx, k = 2 + t / d.nx;
    const int ny = d.ny;
    B.ut[d.idx(i, 1, k)] = B.ut[d.idx(i, 2, k)];
    B.wt[d.idx(i, 1, k)] = B.wt[d.idx(i, 2, k)];
    B.vt[d.idx(i, 2, k)] = 0.0;
    B.ut[d.idx(i, ny + 2, k)] = B.ut[d.idx(i, ny + 1, k)];
    B.wt[d.idx(i, ny + 2, k)] = B.wt[d.idx(i, ny + 1, k)];
    B.vt[d.idx(i, ny + 1, k)] = 0.0;
  }
}

// velocityBC loop 3 (z faces), src/BoundaryConditions.f90:60-73
__global__ void k_vbc_z(DevBlock B) {
  const Dims& d = B.d;
  const int n = d.nx * d.ny;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int i = 2 + t % d.nx, j = 2 + t / d.nx;
    const int nz = d.nz;
    B.ut[d.idx(i, j, 1)] = B.ut[d.idx(i, j, 2)];
    B.vt[d.idx(i, j, 1)] = B.vt[d.idx(i, j, 2)];
    B.wt[d.idx(i, j, 1)] = 0.0;
    B.ut[d.idx(i, j, nz + 2)] = B.ut[d.idx(i, j, nz + 1)];
    B.vt[d.idx(i, j, nz + 2)] = B.vt[d.idx(i, j, nz + 1)];
    B.wt[d.idx(i, j, nz + 1)] = 0.0;
  }
}

// solidCellBC / solidCellBC_move (src/BoundaryConditions.f90:76-115)
__global__ void k_solid_bc(DevBlock B, int move) {
  const Dims& d = B.d;
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = 2 + (int)(t % d.nx);
    const int64_t r = t / d.nx;
    const int j = 2 + (int)(r % d.ny), k = 2 + (int)(r / d.ny);
    const int64_t c = d.idx(i, j, k);
    if (B.cell[c] != 1) continue;
    B.ut[c] = 0.0;
    B.vt[c] = 0.0;
    B.wt[c] = 0.0;
    B.p[c] = 0.0;
    if (move) {
      B.u[c] = 0.0;
      B.v[c] = 0.0;
      B.w[c] = 0.0;
    }
  }
}

}  // namespace

int launch_momentum(const std::vector<HostBlock*>& hbs, double dt, double re, bool fp32) {
  const MomArgs a{dt, re};
  const unsigned cap = 1u << 20;
  if (fp32) TRY_R((launch_op<MomentumOp<FastF>, 128>(hbs, MomentumOp<FastF>{a}, Extent::Interior, cap)));
  else TRY_R((launch_op<MomentumOp<double>, 128>(hbs, MomentumOp<double>{a}, Extent::Interior, cap)));
  // cells within reach of TS cells (none without surfaces 51/52), then the
  // values the reference's loop leaves at the TS positions
  std::vector<HostBlock*> body;
  for (HostBlock* hb : hbs)
    if (hb->has_body) body.push_back(hb);
  if (body.empty()) return 0;
  if (fp32) TRY_R((launch_op<MomentumTsOp<float>, 128>(body, MomentumTsOp<float>{a}, Extent::Interior, 2048)));
  else TRY_R((launch_op<MomentumTsOp<double>, 128>(body, MomentumTsOp<double>{a}, Extent::Interior, 2048)));
  // up to 7 positions per TS cell: cap_ib * 7 items bound the grid
  std::vector<HostBlock*> one(1);
  for (HostBlock* hb : body) {
    k_one<TsRestoreOp, 128><<<grid_for((int64_t)hb->d.cap_ib * 7, 128, 256), 128, 0, stream()>>>(hb->d, TsRestoreOp{});
    BCFD_LAUNCHED();
  }
  return 0;
}

int launch_momentum(HostBlock* hb, double dt, double re, bool fp32) {
  return launch_momentum(std::vector<HostBlock*>{hb}, dt, re, fp32);
}

int launch_velocity_bc(HostBlock* hb, double dt, double uc) {
  const Dims& d = hb->d.d;
  k_vbc_x<<<grid_for((int64_t)d.ny * d.nz, 128), 128, 0, stream()>>>(hb->d, dt, uc);
  BCFD_LAUNCHED();
  k_vbc_y<<<grid_for((int64_t)d.nx * d.nz, 128), 128, 0, stream()>>>(hb->d);
  BCFD_LAUNCHED();
  k_vbc_z<<<grid_for((int64_t)d.nx * d.ny, 128), 128, 0, stream()>>>(hb->d);
  BCFD_LAUNCHED();
  return 0;
}

int launch_solid_bc(HostBlock* hb, bool move) {
  const int64_t n = (int64_t)hb->d.d.nx * hb->d.d.ny * hb->d.d.nz;
  k_solid_bc<<<grid_for(n, 256), 256, 0, stream()>>>(hb->d, move ? 1 : 0);
  BCFD_LAUNCHED();
  return 0;
}

// tangent-linear model of nsMomentum2order at the block's current (u,v,w,p):
// val = the predictor's ut,vt,wt (bitwise the FP64 stencil), tan = its
// derivative along (du,dv,dw,dp); device arrays of the block's point count
int launch_momentum_tangent(HostBlock* hb, double dt, double re, const double* const du[4], double* const val[3],
                            double* const tan[3]) {
  MomentumTlmOp op{MomArgs{dt, re}, {du[0], du[1], du[2], du[3]}, val[0], val[1], val[2], tan[0], tan[1], tan[2]};
  k_one<MomentumTlmOp, 128><<<grid_for((int64_t)hb->d.d.nx * hb->d.d.ny * hb->d.d.nz, 128, 1u << 20), 128, 0,
                              stream()>>>(hb->d, op);
  BCFD_LAUNCHED();
  return 0;
}


// adjoint of nsMomentum2order at the block's current (u,v,w,p): (ub,vb,wb,pb)
// += J^T (ubar_t, vbar_t, wbar_t), J the predictor's Jacobian on fluid cells;
// foot is 16 words of device scratch.  With ts (a block whose body has
// thin-surface cells) the overlay is transposed too: ab at the positions the
// loop's final restore writes goes to ts->gb first, then the cells near TS
// cells read through the overlay and the ghost scalars' adjoints are added
// to ts->gb (the block's ghost arrays must hold the values the forward step
// read); without it such cells set BCFD_E_STATE.
int launch_momentum_adjoint(HostBlock* hb, double dt, double re, const double* const sb[3], double* const ab[4],
                            uint32_t* foot, const MomTsAdj* ts) {
  const MomArgs a{dt, re};
  const int64_t ni = (int64_t)hb->d.d.nx * hb->d.d.ny * hb->d.d.nz;
  const int* last = nullptr;
  if (ts) {
    k_ts_restore_adj<<<1, 32, 0, stream()>>>(hb->d, ab[0], ab[1], ab[2], ab[3], ts->gb, ts->cap);
    BCFD_LAUNCHED();
    k_ts_last<<<grid_for(ni, 128, 1u << 16), 128, 0, stream()>>>(hb->d, ts->last);
    BCFD_LAUNCHED();
    last = ts->last;
  }
  BCFD_CUDA(cudaMemsetAsync(foot, 0, kFootWords * sizeof(uint32_t), stream()));
  k_mom_footprint<<<grid_for(ni, 128, 1u << 16), 128, 0, stream()>>>(hb->d, a, foot, last);
  BCFD_LAUNCHED();
  k_mom_adjoint<<<grid_for(hb->d.d.npts(), 128, 1u << 20), 128, 0, stream()>>>(
      hb->d, a, foot, sb[0], sb[1], sb[2], ab[0], ab[1], ab[2], ab[3], last);
  BCFD_LAUNCHED();
  if (ts) {
    k_mom_ghost_contrib<<<grid_for(ni, 128, 1u << 16), 128, 0, stream()>>>(hb->d, a, ts->last, sb[0], sb[1], sb[2],
                                                                           ts->contrib);
    BCFD_LAUNCHED();
    k_mom_ghost_acc<<<1, 32, 0, stream()>>>(hb->d, ts->last, ts->contrib, ts->gb, ts->cap);
    BCFD_LAUNCHED();
  }
  return 0;
}

}  // namespace bcfd

