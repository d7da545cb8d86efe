// Inter-block coupling kernels: coarse -> fine face ghosts
// (src/FineInterp_bound.f90), fine -> coarse restriction (src/CoarseInterp.f90)
// and the post-move volume fill (src/FineInterp.f90).
//
// Each interface-table entry (coarse index, fine start, fine end) per axis
// maps a contiguous range of fine points to one coarse donor position; a
// thread owns one entry triple (i,j,k) and visits its <= ratio^3 targets.
// A target belongs to exactly one entry triple, so the edge points visited by
// two face passes receive the same value -- the passes are order-free.
#include "bcfd_host.h"

namespace bcfd {

namespace {

struct Tab {
  const int* t;  // (3, n) column-major, 1-based entries
  int c;         // counter
  __device__ int at(int r, int e) const { return t[(r - 1) + 3 * (e - 1)]; }
};

struct Field {  // a field in natural layout or in the colour-packed layout
  double* nat;
  double* pk0;
  double* pk1;
};

__device__ __forceinline__ double fget(const Dims& d, const Field& f, int i, int j, int k) {
  if (f.nat) return f.nat[d.idx(i, j, k)];
  return (colour_of(i, j, k) ? f.pk1 : f.pk0)[d.pidx(i, j, k)];
}
__device__ __forceinline__ void fset(const Dims& d, const Field& f, int i, int j, int k, double v) {
  if (f.nat) f.nat[d.idx(i, j, k)] = v;
  else (colour_of(i, j, k) ? f.pk1 : f.pk0)[d.pidx(i, j, k)] = v;
}

struct Grids {
  const double *x, *y, *z;
};

__device__ __forceinline__ double bilinear(double x, double y, double x1, double x2, double y1,
                                           double y2, double f0, double f1, double f2, double f3) {
  const double numer = f0 * (x2 - x) * (y2 - y) + f2 * (x2 - x) * (y - y1) +
                       f1 * (x - x1) * (y2 - y) + f3 * (x - x1) * (y - y1);
  const double denom = (x2 - x1) * (y2 - y1);
  return numer / denom;
}
__device__ __forceinline__ double linear(double x, double x0, double x1, double y0, double y1) {
  return y0 + (x - x0) * (y1 - y0) / (x1 - x0);
}

struct FaceArgs {
  Tab tx, ty, tz;
  int comp;          // 0 p, 1 u, 2 v, 3 w
  Grids ga, gb;      // coarse (donor) and fine (target) grids of the component
  Field src, dst, dst2;
  int axis;          // face pass 1..3
};

// the components of one coupling call, each its own arrays (one launch per
// face pass instead of one per component)
struct FaceSet {
  FaceArgs f[4];
};

// trilinear_interpolation of src/FineInterp_bound.f90:554-603 (donors loc+-1).
// SUB: eight threads per table entry, each taking every second fine point
// along each axis of the entry's target range (the points are independent;
// a thread's chain of FP64 divisions is an eighth as long)
template <bool SUB>
__device__ __forceinline__ void face_body(const Dims& da, const Dims& db, const FaceArgs& a) {
  const int sx = a.axis == 1 ? a.tx.c - 1 : 1, sy = a.axis == 2 ? a.ty.c - 1 : 1,
            sz = a.axis == 3 ? a.tz.c - 1 : 1;
  const int nxs = (a.tx.c - 1) / sx + 1, nys = (a.ty.c - 1) / sy + 1, nzs = (a.tz.c - 1) / sz + 1;
  const int n = nxs * nys * nzs;
  const int per = SUB ? 8 : 1;
  for (int64_t tt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; tt < (int64_t)n * per;
       tt += (int64_t)gridDim.x * blockDim.x) {
    const int t = (int)(tt / per), sub = (int)(tt % per);
    const int ox0 = SUB ? (sub & 1) : 0, oy0 = SUB ? ((sub >> 1) & 1) : 0, oz0 = SUB ? (sub >> 2) : 0;
    const int st = SUB ? 2 : 1;
    const int ei = 1 + (t % nxs) * sx, ej = 1 + ((t / nxs) % nys) * sy, ek = 1 + (t / (nxs * nys)) * sz;
    const int vx1 = a.tx.at(2, ei), vx2 = a.tx.at(3, ei);
    const int vy1 = a.ty.at(2, ej), vy2 = a.ty.at(3, ej);
    const int vz1 = a.tz.at(2, ek), vz2 = a.tz.at(3, ek);
    const int i = a.tx.at(1, ei), j = a.ty.at(1, ej), k = a.tz.at(1, ek);
    int vi = i, vj = j, vk = k;
    if (a.comp == 1) vi = i - 1;
    if (a.comp == 2) vj = j - 1;
    if (a.comp == 3) vk = k - 1;
    const double x1 = a.ga.x[i - 2], x2 = a.ga.x[i], y1 = a.ga.y[j - 2], y2 = a.ga.y[j],
                 z1 = a.ga.z[k - 2], z2 = a.ga.z[k];
    const double f0 = fget(da, a.src, vi - 1, vj - 1, vk - 1), f1 = fget(da, a.src, vi + 1, vj - 1, vk - 1),
                 f2 = fget(da, a.src, vi - 1, vj + 1, vk - 1), f3 = fget(da, a.src, vi + 1, vj + 1, vk - 1);
    const double g0 = fget(da, a.src, vi - 1, vj - 1, vk + 1), g1 = fget(da, a.src, vi + 1, vj - 1, vk + 1),
                 g2 = fget(da, a.src, vi - 1, vj + 1, vk + 1), g3 = fget(da, a.src, vi + 1, vj + 1, vk + 1);
    for (int tz = vz1 + oz0; tz <= vz2; tz += st)
      for (int ty = vy1 + oy0; ty <= vy2; ty += st)
        for (int tx = vx1 + ox0; tx <= vx2; tx += st) {
          const double x = a.gb.x[tx - 1], y = a.gb.y[ty - 1], z = a.gb.z[tz - 1];
          const double za = bilinear(x, y, x1, x2, y1, y2, f0, f1, f2, f3);
          const double zb = bilinear(x, y, x1, x2, y1, y2, g0, g1, g2, g3);
          const double r = linear(z, z1, z2, za, zb);
          const int ox = tx - (a.comp == 1), oy = ty - (a.comp == 2), oz = tz - (a.comp == 3);
          fset(db, a.dst, ox, oy, oz, r);
          if (a.dst2.nat || a.dst2.pk0) fset(db, a.dst2, ox, oy, oz, r);
        }
  }
}

__global__ void k_face(Dims da, Dims db, FaceArgs a) { face_body<false>(da, db, a); }

// face pass `axis` of the components S.f[blockIdx.y]
__global__ void k_face_set(Dims da, Dims db, FaceSet S, int axis) {
  FaceArgs a = S.f[blockIdx.y];
  a.axis = axis;
  face_body<true>(da, db, a);
}

// trilinear_interpolation of src/CoarseInterp.f90:447-502 (adjacent donors);
// the target coarse point of entry i is det(1,i); the donor index is the
// middle fine index (start+end-1)/2, or `end` along the staggered axis.
__device__ __forceinline__ void restrict_body(const Dims& da, const Dims& db, const FaceArgs& a, int ci) {
  const int nxs = a.tx.c - 2 * ci + 1, nys = a.ty.c - 2 * ci + 1, nzs = a.tz.c - 2 * ci + 1;
  if (nxs <= 0 || nys <= 0 || nzs <= 0) return;
  const int n = nxs * nys * nzs;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int ei = ci + t % nxs, ej = ci + (t / nxs) % nys, ek = ci + t / (nxs * nys);
    const int tx = a.tx.at(1, ei), ty = a.ty.at(1, ej), tz = a.tz.at(1, ek);
    int lx = (a.tx.at(2, ei) + a.tx.at(3, ei) - 1) / 2;
    int ly = (a.ty.at(2, ej) + a.ty.at(3, ej) - 1) / 2;
    int lz = (a.tz.at(2, ek) + a.tz.at(3, ek) - 1) / 2;
    if (a.comp == 1) lx = a.tx.at(3, ei);
    if (a.comp == 2) ly = a.ty.at(3, ej);
    if (a.comp == 3) lz = a.tz.at(3, ek);
    int ii = lx, jj = ly, kk = lz, vi = lx, vj = ly, vk = lz;
    if (a.comp == 1) { ii = lx - 1; vi = lx - 2; }
    if (a.comp == 2) { jj = ly - 1; vj = ly - 2; }
    if (a.comp == 3) { kk = lz - 1; vk = lz - 2; }
    const double x = a.ga.x[tx - 1], y = a.ga.y[ty - 1], z = a.ga.z[tz - 1];
    const double x1 = a.gb.x[ii - 1], x2 = a.gb.x[ii], y1 = a.gb.y[jj - 1], y2 = a.gb.y[jj],
                 z1 = a.gb.z[kk - 1], z2 = a.gb.z[kk];
    const double za = bilinear(x, y, x1, x2, y1, y2, fget(db, a.src, vi, vj, vk),
                               fget(db, a.src, vi + 1, vj, vk), fget(db, a.src, vi, vj + 1, vk),
                               fget(db, a.src, vi + 1, vj + 1, vk));
    const double zb = bilinear(x, y, x1, x2, y1, y2, fget(db, a.src, vi, vj, vk + 1),
                               fget(db, a.src, vi + 1, vj, vk + 1), fget(db, a.src, vi, vj + 1, vk + 1),
                               fget(db, a.src, vi + 1, vj + 1, vk + 1));
    const double r = linear(z, z1, z2, za, zb);
    const int ox = tx - (a.comp == 1), oy = ty - (a.comp == 2), oz = tz - (a.comp == 3);
    fset(da, a.dst, ox, oy, oz, r);
    if (a.dst2.nat || a.dst2.pk0) fset(da, a.dst2, ox, oy, oz, r);
  }
}

__global__ void k_restrict(Dims da, Dims db, FaceArgs a, int ci) { restrict_body(da, db, a, ci); }
__global__ void k_restrict_set(Dims da, Dims db, FaceSet S, int ci) { restrict_body(da, db, S.f[blockIdx.y], ci); }

// ---------------------------------------------------------------------------
// Adjoints of the coupling (transposed trilinear interpolation).
// ---------------------------------------------------------------------------
// the trilinear weights of k_face for target (x,y,z): corner q = a + 2b + 4c
// of the donor box (a: x+1, b: y+1, c: z+1), in the forward's algebra
__device__ __forceinline__ void face_weights(double x, double y, double z, double x1, double x2, double y1,
                                             double y2, double z1, double z2, double* w) {
  const double den = (x2 - x1) * (y2 - y1);
  const double b00 = (x2 - x) * (y2 - y) / den, b10 = (x - x1) * (y2 - y) / den,
               b01 = (x2 - x) * (y - y1) / den, b11 = (x - x1) * (y - y1) / den;
  const double tz = (z - z1) / (z2 - z1);
  const double za = 1.0 - tz;
  w[0] = b00 * za; w[1] = b10 * za; w[2] = b01 * za; w[3] = b11 * za;
  w[4] = b00 * tz; w[5] = b10 * tz; w[6] = b01 * tz; w[7] = b11 * tz;
}

// Face-fill adjoint, stage 1: every entry triple on the shell (first or last
// entry along some axis: the face passes visit exactly these) sums its
// targets' adjoints times their weights per donor corner, in a fixed order.
// Each target belongs to exactly one entry triple, so it is counted once,
// although the forward's face passes may write it twice (with one value).
__global__ void k_face_adj1(Dims db, FaceArgs a, const double* gbar, double* part) {
  const int cx = a.tx.c, cy = a.ty.c, cz = a.tz.c;
  const int n = cx * cy * cz;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int ei = 1 + t % cx, ej = 1 + (t / cx) % cy, ek = 1 + t / (cx * cy);
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const bool shell = ei == 1 || ei == cx || ej == 1 || ej == cy || ek == 1 || ek == cz;
    if (shell) {
      const int i = a.tx.at(1, ei), j = a.ty.at(1, ej), k = a.tz.at(1, ek);
      const double x1 = a.ga.x[i - 2], x2 = a.ga.x[i], y1 = a.ga.y[j - 2], y2 = a.ga.y[j],
                   z1 = a.ga.z[k - 2], z2 = a.ga.z[k];
      for (int tz = a.tz.at(2, ek); tz <= a.tz.at(3, ek); ++tz)
        for (int ty = a.ty.at(2, ej); ty <= a.ty.at(3, ej); ++ty)
          for (int tx = a.tx.at(2, ei); tx <= a.tx.at(3, ei); ++tx) {
            double w[8];
            face_weights(a.gb.x[tx - 1], a.gb.y[ty - 1], a.gb.z[tz - 1], x1, x2, y1, y2, z1, z2, w);
            const int ox = tx - (a.comp == 1), oy = ty - (a.comp == 2), oz = tz - (a.comp == 3);
            const double g = gbar[db.idx(ox, oy, oz)];
#pragma unroll
            for (int q = 0; q < 8; ++q) acc[q] += w[q] * g;
          }
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) part[8 * (int64_t)t + q] = acc[q];
  }
}

// inverse of an interface table: coarse index -> entry (1-based), 0 if none
__device__ __forceinline__ int entry_of(const Tab& tb, int ci) {
  int lo = 1, hi = tb.c;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    const int v = tb.at(1, mid);
    if (v == ci) return mid;
    if (v < ci) lo = mid + 1;
    else hi = mid - 1;
  }
  return 0;
}

// Face-fill adjoint, stage 2: each coarse point of the donor range gathers
// the partial sums of the (<= 8) entries whose donor box has it as a corner,
// in a fixed corner order, and adds them to cbar.
__global__ void k_face_adj2(Dims da, FaceArgs a, const double* part, double* cbar) {
  const int sh = (a.comp == 1) ? -1 : 0, shy = (a.comp == 2) ? -1 : 0, shz = (a.comp == 3) ? -1 : 0;
  // donor coarse indices span [first centre - 1, last centre + 1]
  const int i0 = a.tx.at(1, 1) + sh - 1, i1 = a.tx.at(1, a.tx.c) + sh + 1;
  const int j0 = a.ty.at(1, 1) + shy - 1, j1 = a.ty.at(1, a.ty.c) + shy + 1;
  const int k0 = a.tz.at(1, 1) + shz - 1, k1 = a.tz.at(1, a.tz.c) + shz + 1;
  const int nx = i1 - i0 + 1, ny = j1 - j0 + 1, nz = k1 - k0 + 1;
  const int cx = a.tx.c, cy = a.ty.c;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nx * ny * nz; t += gridDim.x * blockDim.x) {
    const int di = i0 + t % nx, dj = j0 + (t / nx) % ny, dk = k0 + t / (nx * ny);
    if (di < 1 || dj < 1 || dk < 1 || di > da.NX || dj > da.NY || dk > da.NZ) continue;
    double s = 0.0;
    bool any = false;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      // donor corner q of centre v is v + (2a-1, 2b-1, 2c-1)
      const int vi = di - (2 * (q & 1) - 1), vj = dj - (2 * ((q >> 1) & 1) - 1), vk = dk - (2 * (q >> 2) - 1);
      const int ei = entry_of(a.tx, vi - sh), ej = entry_of(a.ty, vj - shy), ek = entry_of(a.tz, vk - shz);
      if (!ei || !ej || !ek) continue;
      s += part[8 * ((int64_t)(ei - 1) + (int64_t)cx * ((ej - 1) + (int64_t)cy * (ek - 1))) + q];
      any = true;
    }
    if (any) cbar[da.idx(di, dj, dk)] += s;
  }
}

// Restriction adjoint: the donor boxes of different coarse targets are
// disjoint (ratio 2: the donors of entry e lie in its own fine range), so
// the transpose is a plain scatter: fbar[donor] += weight * cbar[target].
__global__ void k_restrict_adj(Dims da, Dims db, FaceArgs a, int ci, const double* cbar, double* fbar) {
  const int nxs = a.tx.c - 2 * ci + 1, nys = a.ty.c - 2 * ci + 1, nzs = a.tz.c - 2 * ci + 1;
  if (nxs <= 0 || nys <= 0 || nzs <= 0) return;
  const int n = nxs * nys * nzs;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int ei = ci + t % nxs, ej = ci + (t / nxs) % nys, ek = ci + t / (nxs * nys);
    const int tx = a.tx.at(1, ei), ty = a.ty.at(1, ej), tz = a.tz.at(1, ek);
    int lx = (a.tx.at(2, ei) + a.tx.at(3, ei) - 1) / 2;
    int ly = (a.ty.at(2, ej) + a.ty.at(3, ej) - 1) / 2;
    int lz = (a.tz.at(2, ek) + a.tz.at(3, ek) - 1) / 2;
    if (a.comp == 1) lx = a.tx.at(3, ei);
    if (a.comp == 2) ly = a.ty.at(3, ej);
    if (a.comp == 3) lz = a.tz.at(3, ek);
    int ii = lx, jj = ly, kk = lz, vi = lx, vj = ly, vk = lz;
    if (a.comp == 1) { ii = lx - 1; vi = lx - 2; }
    if (a.comp == 2) { jj = ly - 1; vj = ly - 2; }
    if (a.comp == 3) { kk = lz - 1; vk = lz - 2; }
    const double x = a.ga.x[tx - 1], y = a.ga.y[ty - 1], z = a.ga.z[tz - 1];
    double w[8];
    face_weights(x, y, z, a.gb.x[ii - 1], a.gb.x[ii], a.gb.y[jj - 1], a.gb.y[jj], a.gb.z[kk - 1], a.gb.z[kk], w);
    const int ox = tx - (a.comp == 1), oy = ty - (a.comp == 2), oz = tz - (a.comp == 3);
    const double c = cbar[da.idx(ox, oy, oz)];
#pragma unroll
    for (int q = 0; q < 8; ++q)
      fbar[db.idx(vi + (q & 1), vj + ((q >> 1) & 1), vk + (q >> 2))] += w[q] * c;
  }
}

// fineUpdate_mv (src/FineInterp.f90:10-281): fine points with cell_n /= 1
__global__ void k_fine_mv(Dims da, Dims db, FaceArgs a, const int8_t* cell_n) {
  const int nxs = a.tx.c - 2, nys = a.ty.c - 2, nzs = a.tz.c - 2;
  if (nxs <= 0 || nys <= 0 || nzs <= 0) return;
  const int n = nxs * nys * nzs;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int ei = 2 + t % nxs, ej = 2 + (t / nxs) % nys, ek = 2 + t / (nxs * nys);
    const int vx1 = a.tx.at(2, ei), vx2 = a.tx.at(3, ei);
    const int vy1 = a.ty.at(2, ej), vy2 = a.ty.at(3, ej);
    const int vz1 = a.tz.at(2, ek), vz2 = a.tz.at(3, ek);
    const int lx = a.tx.at(1, ei), ly = a.ty.at(1, ej), lz = a.tz.at(1, ek);
    const int xm = a.comp == 1 ? lx - 2 : lx - 1, xq = a.comp == 1 ? lx : lx + 1;
    const int ym = a.comp == 2 ? ly - 2 : ly - 1, yq = a.comp == 2 ? ly : ly + 1;
    const int zm = a.comp == 3 ? lz - 2 : lz - 1, zq = a.comp == 3 ? lz : lz + 1;
    for (int q = vz1; q <= vz2; ++q)
      for (int l = vy1; l <= vy2; ++l)
        for (int s = vx1; s <= vx2; ++s) {
          if (cell_n[db.idx(s, l, q)] == 1) continue;
          const double valx = a.gb.x[s - 1], valy = a.gb.y[l - 1], valz = a.gb.z[q - 1];
          const double x1 = a.ga.x[lx - 2], x2 = a.ga.x[lx];
          const double y1 = a.ga.y[ly - 2], y2 = a.ga.y[ly];
          const double z1 = a.ga.z[lz - 2], z2 = a.ga.z[lz];
          const double deno = (x2 - x1) * (y2 - y1);
          const double xtx = (x2 - valx), xxo = (valx - x1);
          const double yty = (y2 - valy), yyo = (valy - y1);
          double f1 = fget(da, a.src, xm, ym, zm), f2 = fget(da, a.src, xq, ym, zm),
                 f3 = fget(da, a.src, xq, yq, zm), f4 = fget(da, a.src, xm, yq, zm);
          double num = (f1 * xtx + f2 * xxo) * yty + (f4 * xtx + f3 * xxo) * yyo;
          const double a1 = (num / deno);
          f1 = fget(da, a.src, xm, ym, zq);
          f2 = fget(da, a.src, xq, ym, zq);
          f3 = fget(da, a.src, xq, yq, zq);
          f4 = fget(da, a.src, xm, yq, zq);
          num = (f1 * xtx + f2 * xxo) * yty + (f4 * xtx + f3 * xxo) * yyo;
          const double a2 = (num / deno);
          const double r = a1 + ((valz - z1) * ((a2 - a1) / (z2 - z1)));
          fset(db, a.dst, s - (a.comp == 1), l - (a.comp == 2), q - (a.comp == 3), r);
        }
  }
}

Grids grids_of(const DevBlock& B, int comp) {
  switch (comp) {
    case 1: return {B.xu, B.yu, B.zu};
    case 2: return {B.xv, B.yv, B.zv};
    case 3: return {B.xw, B.yw, B.zw};
    default: return {B.xp, B.yp, B.zp};
  }
}

// which: 0 = ut/vt/wt (p unused), 1 = pc (+ pco), 2 = u/v/w/p
Field field_of(const DevBlock& B, int comp, int which) {
  if (which == 1) return {nullptr, B.pc[0], B.pc[1]};
  if (which == 0) {
    double* f = comp == 1 ? B.ut : comp == 2 ? B.vt : B.wt;
    return {f, nullptr, nullptr};
  }
  double* f = comp == 0 ? B.p : comp == 1 ? B.u : comp == 2 ? B.v : B.w;
  return {f, nullptr, nullptr};
}

FaceArgs make_args(HostInterface* it, HostBlock* a, HostBlock* b, int comp) {
  FaceArgs f{};
  const int base = 3 * comp;  // px,py,pz | ux,uy,uz | vx.. | wx..
  f.tx = {it->dtab + it->off[base + 0], (int)it->counter[base + 0]};
  f.ty = {it->dtab + it->off[base + 1], (int)it->counter[base + 1]};
  f.tz = {it->dtab + it->off[base + 2], (int)it->counter[base + 2]};
  f.comp = comp;
  f.ga = grids_of(a->d, comp);
  f.gb = grids_of(b->d, comp);
  return f;
}

}  // namespace


// the face fill of several components: one launch per face pass (the
// components write different arrays and read the coarse block only; the
// passes keep their order, so points two passes write get the later value)
int launch_face_fill_set(HostInterface* it, const int* comps, int nc, int which) {
  HostBlock* a = get_block(it->a);
  HostBlock* b = get_block(it->b);
  if (!a || !b) return BCFD_E_HANDLE;
  if (nc < 1 || nc > 4) return BCFD_E_ARG;
  FaceSet S{};
  int n = 0;
  for (int q = 0; q < nc; ++q) {
    FaceArgs& f = S.f[q];
    f = make_args(it, a, b, comps[q]);
    f.src = field_of(a->d, comps[q], which);
    f.dst = field_of(b->d, comps[q], which);
    f.dst2 = Field{nullptr, nullptr, nullptr};
    n = std::max(n, f.tx.c * f.ty.c * f.tz.c);
  }
  for (int axis = 1; axis <= 3; ++axis) {
    const dim3 grid(grid_for(8 * (int64_t)n, 128), (unsigned)nc);
    k_face_set<<<grid, 128, 0, stream()>>>(a->d.d, b->d.d, S, axis);
    BCFD_LAUNCHED();
  }
  return 0;
}

// the restriction of several components in one launch (different arrays)
int launch_restrict_set(HostInterface* it, const int* comps, int nc, int which) {
  HostBlock* a = get_block(it->a);
  HostBlock* b = get_block(it->b);
  if (!a || !b) return BCFD_E_HANDLE;
  if (nc < 1 || nc > 4) return BCFD_E_ARG;
  FaceSet S{};
  int n = 0;
  for (int q = 0; q < nc; ++q) {
    FaceArgs& f = S.f[q];
    f = make_args(it, a, b, comps[q]);
    f.src = field_of(b->d, comps[q], which);
    f.dst = field_of(a->d, comps[q], which);
    f.dst2 = Field{nullptr, nullptr, nullptr};
    n = std::max(n, f.tx.c * f.ty.c * f.tz.c);
  }
  const dim3 grid(grid_for(n, 128), (unsigned)nc);
  k_restrict_set<<<grid, 128, 0, stream()>>>(a->d.d, b->d.d, S, 3);
  BCFD_LAUNCHED();
  return 0;
}


int launch_fine_update_mv(HostInterface* it) {
  HostBlock* a = get_block(it->a);
  HostBlock* b = get_block(it->b);
  if (!a || !b) return BCFD_E_HANDLE;
  for (int comp = 0; comp < 4; ++comp) {
    FaceArgs f = make_args(it, a, b, comp);
    f.src = field_of(a->d, comp, 2);
    f.dst = field_of(b->d, comp, 2);
    const int n = f.tx.c * f.ty.c * f.tz.c;
    k_fine_mv<<<grid_for(n, 128), 128, 0, stream()>>>(a->d.d, b->d.d, f, b->d.cell_n);
    BCFD_LAUNCHED();
  }
  return 0;
}

// Forward and adjoint coupling maps on caller arrays (natural layout, device
// pointers): the face fill f = P c of one component (all three face passes)
// and its transpose c += P^T f; the restriction c = R f and f += R^T c.
int coupling_apply(HostInterface* it, int comp, int op, const double* in, double* out) {
  HostBlock* a = get_block(it->a);
  HostBlock* b = get_block(it->b);
  if (!a || !b) return BCFD_E_HANDLE;
  FaceArgs f = make_args(it, a, b, comp);
  f.dst2 = Field{nullptr, nullptr, nullptr};
  const int n = f.tx.c * f.ty.c * f.tz.c;
  if (op == 0) {  // face fill: coarse in -> fine out
    f.src = Field{const_cast<double*>(in), nullptr, nullptr};
    f.dst = Field{out, nullptr, nullptr};
    for (int axis = 1; axis <= 3; ++axis) {
      f.axis = axis;
      k_face<<<grid_for(n, 128), 128, 0, stream()>>>(a->d.d, b->d.d, f);
      BCFD_LAUNCHED();
    }
  } else if (op == 1) {  // face-fill transpose: fine in -> coarse out (+=)
    double* part = nullptr;
    BCFD_CUDA(cudaMalloc(&part, (size_t)n * 8 * sizeof(double)));
    k_face_adj1<<<grid_for(n, 128), 128, 0, stream()>>>(b->d.d, f, in, part);
    int r = note_launch();
    if (!r) {
      k_face_adj2<<<grid_for((int64_t)(f.tx.c + 4) * (f.ty.c + 4) * (f.tz.c + 4), 128), 128, 0, stream()>>>(
          a->d.d, f, part, out);
      r = note_launch();
    }
    cudaStreamSynchronize(stream());
    cudaFree(part);
    return r;
  } else if (op == 2) {  // restriction: fine in -> coarse out
    f.src = Field{const_cast<double*>(in), nullptr, nullptr};
    f.dst = Field{out, nullptr, nullptr};
    k_restrict<<<grid_for(n, 128), 128, 0, stream()>>>(a->d.d, b->d.d, f, 3);
    BCFD_LAUNCHED();
  } else {  // restriction transpose: coarse in -> fine out (+=)
    k_restrict_adj<<<grid_for(n, 128), 128, 0, stream()>>>(a->d.d, b->d.d, f, 3, in, out);
    BCFD_LAUNCHED();
  }
  return 0;
}

}  // namespace bcfd

