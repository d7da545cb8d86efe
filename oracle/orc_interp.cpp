// ORACLE -- TEST INFRASTRUCTURE ONLY (see orc_core.h).
// Inter-block coupling: interface tables (src/InterfaceDetail.f90), coarse ->
// fine face fill (src/FineInterp_bound.f90), fine -> coarse restriction
// (src/CoarseInterp.f90) and the post-move volume fill (src/FineInterp.f90).
#include <cmath>
#include "orc_core.h"

namespace orc {

// set_interface_detail, src/InterfaceDetail.f90:168-241
void set_interface_detail(const F1& var, real s, real e, int64_t factor, I2& det,
                          int64_t& counter, int64_t starter_in) {
  int64_t starter = starter_in;
  int64_t xx1 = 0, xx2 = 0;
  for (int64_t i = 1; i <= var.size(); ++i)
    if (var(i) > s) {
      xx1 = i;
      break;
    }
  for (int64_t i = xx1; i <= var.size(); ++i)
    if (var(i) > e) {
      xx2 = i - 1;
      break;
    }
  det(1, 1) = xx1 - 1;
  det(2, 1) = starter - 1;
  det(3, 1) = starter - 1;
  int64_t ender = starter + factor - 1;
  counter = 2;
  for (;;) {
    det(1, counter) = xx1;
    det(2, counter) = starter;
    det(3, counter) = ender;
    starter = ender + 1;
    ender = ender + factor;
    counter = counter + 1;
    xx1 = xx1 + 1;
    if (xx1 > xx2) break;
  }
  det(1, counter) = xx2 + 1;
  det(2, counter) = starter;
  det(3, counter) = starter;
}

// interfaceDetail, src/InterfaceDetail.f90:10-165
void interface_detail(Interface& it) {
  Block& a = blk_of(it.a_blk);
  Block& bb = blk_of(it.b_blk);
  const int64_t factor = it.b_msh / it.a_msh;
  const int64_t mx = bb.nx / factor + 3, my = bb.ny / factor + 3, mz = bb.nz / factor + 3;
  for (I2* t : {&it.px, &it.ux, &it.vx, &it.wx}) t->alloc(3, mx);
  for (I2* t : {&it.py, &it.uy, &it.vy, &it.wy}) t->alloc(3, my);
  for (I2* t : {&it.pz, &it.uz, &it.vz, &it.wz}) t->alloc(3, mz);
  set_interface_detail(a.xp, it.xintf_start, it.xintf_end, factor, it.px, it.cxp, 2);
  set_interface_detail(a.yp, it.yintf_start, it.yintf_end, factor, it.py, it.cyp, 2);
  set_interface_detail(a.zp, it.zintf_start, it.zintf_end, factor, it.pz, it.czp, 2);
  set_interface_detail(a.xu, it.xintf_start, it.xintf_end, factor, it.ux, it.cxu, 3);
  set_interface_detail(a.yu, it.yintf_start, it.yintf_end, factor, it.uy, it.cyu, 2);
  set_interface_detail(a.zu, it.zintf_start, it.zintf_end, factor, it.uz, it.czu, 2);
  set_interface_detail(a.xv, it.xintf_start, it.xintf_end, factor, it.vx, it.cxv, 2);
  set_interface_detail(a.yv, it.yintf_start, it.yintf_end, factor, it.vy, it.cyv, 3);
  set_interface_detail(a.zv, it.zintf_start, it.zintf_end, factor, it.vz, it.czv, 2);
  set_interface_detail(a.xw, it.xintf_start, it.xintf_end, factor, it.wx, it.cxw, 2);
  set_interface_detail(a.yw, it.yintf_start, it.yintf_end, factor, it.wy, it.cyw, 2);
  set_interface_detail(a.zw, it.zintf_start, it.zintf_end, factor, it.wz, it.czw, 3);
}

namespace {

// trilinear_interpolation of src/FineInterp_bound.f90:554-603: coarse points
// loc-1 and loc+1 along each axis.
real tri_fine(real x, real y, real z, int64_t i, int64_t j, int64_t k, const F1& xg,
                const F1& yg, const F1& zg, int off, const F3& var) {
  int64_t vi = i, vj = j, vk = k;
  if (off == 1) vi = i - 1;
  if (off == 2) vj = j - 1;
  if (off == 3) vk = k - 1;
  real f[4] = {var(vi - 1, vj - 1, vk - 1), var(vi + 1, vj - 1, vk - 1),
                 var(vi - 1, vj + 1, vk - 1), var(vi + 1, vj + 1, vk - 1)};
  const real z1 = bilinear_interpolation(x, y, xg(i - 1), xg(i + 1), yg(j - 1), yg(j + 1), f);
  real g[4] = {var(vi - 1, vj - 1, vk + 1), var(vi + 1, vj - 1, vk + 1),
                 var(vi - 1, vj + 1, vk + 1), var(vi + 1, vj + 1, vk + 1)};
  const real z2 = bilinear_interpolation(x, y, xg(i - 1), xg(i + 1), yg(j - 1), yg(j + 1), g);
  return linear_interpolation(z, zg(k - 1), zg(k + 1), z1, z2);
}

// trilinear_interpolation of src/CoarseInterp.f90:447-502: adjacent fine points.
real tri_coarse(real x, real y, real z, int64_t i, int64_t j, int64_t k, const F1& xg,
                  const F1& yg, const F1& zg, int off, const F3& var) {
  int64_t ii = i, jj = j, kk = k, vi = i, vj = j, vk = k;
  if (off == 1) { ii = i - 1; vi = i - 2; }
  if (off == 2) { jj = j - 1; vj = j - 2; }
  if (off == 3) { kk = k - 1; vk = k - 2; }
  real f[4] = {var(vi, vj, vk), var(vi + 1, vj, vk), var(vi, vj + 1, vk), var(vi + 1, vj + 1, vk)};
  const real z1 = bilinear_interpolation(x, y, xg(ii), xg(ii + 1), yg(jj), yg(jj + 1), f);
  real g[4] = {var(vi, vj, vk + 1), var(vi + 1, vj, vk + 1), var(vi, vj + 1, vk + 1),
                 var(vi + 1, vj + 1, vk + 1)};
  const real z2 = bilinear_interpolation(x, y, xg(ii), xg(ii + 1), yg(jj), yg(jj + 1), g);
  return linear_interpolation(z, zg(kk), zg(kk + 1), z1, z2);
}

struct CompTab {
  I2 *tx, *ty, *tz;
  int64_t cx, cy, cz;
};

CompTab tabs(Interface& it, int comp) {  // 0 p, 1 u, 2 v, 3 w
  switch (comp) {
    case 0: return {&it.px, &it.py, &it.pz, it.cxp, it.cyp, it.czp};
    case 1: return {&it.ux, &it.uy, &it.uz, it.cxu, it.cyu, it.czu};
    case 2: return {&it.vx, &it.vy, &it.vz, it.cxv, it.cyv, it.czv};
    default: return {&it.wx, &it.wy, &it.wz, it.cxw, it.cyw, it.czw};
  }
}

void comp_grids(Block& b, int comp, const F1*& x, const F1*& y, const F1*& z) {
  switch (comp) {
    case 0: x = &b.xp; y = &b.yp; z = &b.zp; break;
    case 1: x = &b.xu; y = &b.yu; z = &b.zu; break;
    case 2: x = &b.xv; y = &b.yv; z = &b.zv; break;
    default: x = &b.xw; y = &b.yw; z = &b.zw; break;
  }
}

// Coarse -> fine on the six faces of block b_blk (the face-only loops with
// stride counter-1 of src/FineInterp_bound.f90).  dst2 may be null.
void face_fill(Interface& it, int comp, F3& src, F3& dst, F3* dst2) {
  Block& a = blk_of(it.a_blk);
  Block& fb = blk_of(it.b_blk);
  const CompTab t = tabs(it, comp);
  const F1 *ax, *ay, *az, *bx, *by, *bz;
  comp_grids(a, comp, ax, ay, az);
  comp_grids(fb, comp, bx, by, bz);
  for (int axis = 1; axis <= 3; ++axis) {
    int64_t st[3] = {1, 1, 1};
    if (axis == 1) st[0] = t.cx - 1;
    if (axis == 2) st[1] = t.cy - 1;
    if (axis == 3) st[2] = t.cz - 1;
    for (int64_t k = 1; k <= t.cz; k += st[2])
      for (int64_t j = 1; j <= t.cy; j += st[1])
        for (int64_t i = 1; i <= t.cx; i += st[0]) {
          const int64_t vx1 = (*t.tx)(2, i), vx2 = (*t.tx)(3, i);
          const int64_t vy1 = (*t.ty)(2, j), vy2 = (*t.ty)(3, j);
          const int64_t vz1 = (*t.tz)(2, k), vz2 = (*t.tz)(3, k);
          const int64_t lx = (*t.tx)(1, i), ly = (*t.ty)(1, j), lz = (*t.tz)(1, k);
          for (int64_t tz = vz1; tz <= vz2; ++tz)
            for (int64_t ty = vy1; ty <= vy2; ++ty)
              for (int64_t tx = vx1; tx <= vx2; ++tx) {
                const real r =
                    tri_fine((*bx)(tx), (*by)(ty), (*bz)(tz), lx, ly, lz, *ax, *ay, *az, comp, src);
                int64_t ox = tx, oy = ty, oz = tz;
                if (comp == 1) ox = tx - 1;
                if (comp == 2) oy = ty - 1;
                if (comp == 3) oz = tz - 1;
                dst(ox, oy, oz) = r;
                if (dst2) (*dst2)(ox, oy, oz) = r;
              }
        }
  }
}

// Fine -> coarse over the overlap minus cintp on each side (src/CoarseInterp.f90).
void restrict_fill(Interface& it, int comp, F3& src, F3& dst, F3* dst2) {
  Block& a = blk_of(it.a_blk);
  Block& fb = blk_of(it.b_blk);
  const CompTab t = tabs(it, comp);
  const F1 *ax, *ay, *az, *bx, *by, *bz;
  comp_grids(a, comp, ax, ay, az);
  comp_grids(fb, comp, bx, by, bz);
  const int64_t ci = fb.cintp;
  for (int64_t k = ci; k <= t.cz - ci; ++k)
    for (int64_t j = ci; j <= t.cy - ci; ++j)
      for (int64_t i = ci; i <= t.cx - ci; ++i) {
        const int64_t tx = (*t.tx)(1, i), ty = (*t.ty)(1, j), tz = (*t.tz)(1, k);
        // Fortran integer division truncates toward zero; the operands are positive
        int64_t lx = ((*t.tx)(2, i) + (*t.tx)(3, i) - 1) / 2;
        int64_t ly = ((*t.ty)(2, j) + (*t.ty)(3, j) - 1) / 2;
        int64_t lz = ((*t.tz)(2, k) + (*t.tz)(3, k) - 1) / 2;
        if (comp == 1) lx = (*t.tx)(3, i);
        if (comp == 2) ly = (*t.ty)(3, j);
        if (comp == 3) lz = (*t.tz)(3, k);
        const real r =
            tri_coarse((*ax)(tx), (*ay)(ty), (*az)(tz), lx, ly, lz, *bx, *by, *bz, comp, src);
        int64_t ox = tx, oy = ty, oz = tz;
        if (comp == 1) ox = tx - 1;
        if (comp == 2) oy = ty - 1;
        if (comp == 3) oz = tz - 1;
        dst(ox, oy, oz) = r;
        if (dst2) (*dst2)(ox, oy, oz) = r;
      }
}

}  // namespace

// fineUpdate_pc_bd, src/FineInterp_bound.f90:17-107
void fine_update_pc_bd() {
  for (Interface* it : g_interfaces) {
    Block& a = blk_of(it->a_blk);
    Block& b = blk_of(it->b_blk);
    face_fill(*it, 0, a.pc, b.pc, &b.pco);
  }
}

// fineUpdate_newv_bd, src/FineInterp_bound.f90:109-309
void fine_update_newv_bd() {
  for (Interface* it : g_interfaces) {
    Block& a = blk_of(it->a_blk);
    Block& b = blk_of(it->b_blk);
    face_fill(*it, 1, a.ut, b.ut, nullptr);
    face_fill(*it, 2, a.vt, b.vt, nullptr);
    face_fill(*it, 3, a.wt, b.wt, nullptr);
  }
}

// fineUpdate_bd_mv, src/FineInterp_bound.f90:311-544
void fine_update_bd_mv(int64_t g) {
  Interface& it = *g_interfaces[(size_t)(g - 1)];
  Block& a = blk_of(it.a_blk);
  Block& b = blk_of(it.b_blk);
  face_fill(it, 0, a.p, b.p, nullptr);
  face_fill(it, 1, a.u, b.u, nullptr);
  face_fill(it, 2, a.v, b.v, nullptr);
  face_fill(it, 3, a.w, b.w, nullptr);
}

// coarseUpdate, src/CoarseInterp.f90:16-204
void coarse_update() {
  for (Interface* it : g_interfaces) {
    Block& a = blk_of(it->a_blk);
    Block& b = blk_of(it->b_blk);
    restrict_fill(*it, 0, b.p, a.p, nullptr);
    restrict_fill(*it, 1, b.u, a.u, nullptr);
    restrict_fill(*it, 2, b.v, a.v, nullptr);
    restrict_fill(*it, 3, b.w, a.w, nullptr);
  }
}

// coarseUpdate_newv, src/CoarseInterp.f90:206-346
void coarse_update_newv() {
  for (Interface* it : g_interfaces) {
    Block& a = blk_of(it->a_blk);
    Block& b = blk_of(it->b_blk);
    restrict_fill(*it, 1, b.ut, a.ut, nullptr);
    restrict_fill(*it, 2, b.vt, a.vt, nullptr);
    restrict_fill(*it, 3, b.wt, a.wt, nullptr);
  }
}

// coarseUpdate_pc, src/CoarseInterp.f90:347-437
void coarse_update_pc() {
  for (Interface* it : g_interfaces) {
    Block& a = blk_of(it->a_blk);
    Block& b = blk_of(it->b_blk);
    restrict_fill(*it, 0, b.pc, a.pc, &a.pco);
  }
}

// fineUpdate_mv, src/FineInterp.f90:10-281: after a block move, fill the fine
// cells with cell_n /= 1 from the coarse block (bilinear in x-y on the
// loc+-1 z planes, then linear in z).
void fine_update_mv(int64_t g) {
  Interface& it = *g_interfaces[(size_t)(g - 1)];
  Block& a = blk_of(it.a_blk);
  Block& b = blk_of(it.b_blk);
  for (int comp = 0; comp < 4; ++comp) {
    const CompTab t = tabs(it, comp);
    const F1 *ax, *ay, *az, *bx, *by, *bz;
    comp_grids(a, comp, ax, ay, az);
    comp_grids(b, comp, bx, by, bz);
    F3& src = comp == 0 ? a.p : comp == 1 ? a.u : comp == 2 ? a.v : a.w;
    F3& dst = comp == 0 ? b.p : comp == 1 ? b.u : comp == 2 ? b.v : b.w;
    for (int64_t k = 2; k <= t.cz - 1; ++k)
      for (int64_t j = 2; j <= t.cy - 1; ++j)
        for (int64_t i = 2; i <= t.cx - 1; ++i) {
          const int64_t vx1 = (*t.tx)(2, i), vx2 = (*t.tx)(3, i);
          const int64_t vy1 = (*t.ty)(2, j), vy2 = (*t.ty)(3, j);
          const int64_t vz1 = (*t.tz)(2, k), vz2 = (*t.tz)(3, k);
          const int64_t lx = (*t.tx)(1, i), ly = (*t.ty)(1, j), lz = (*t.tz)(1, k);
          // donor offsets: the staggered component's own axis uses loc-2 / loc
          const int64_t xm = comp == 1 ? lx - 2 : lx - 1, xq = comp == 1 ? lx : lx + 1;
          const int64_t ym = comp == 2 ? ly - 2 : ly - 1, yq = comp == 2 ? ly : ly + 1;
          const int64_t zm = comp == 3 ? lz - 2 : lz - 1, zq = comp == 3 ? lz : lz + 1;
          for (int64_t q = vz1; q <= vz2; ++q)
            for (int64_t l = vy1; l <= vy2; ++l)
              for (int64_t s = vx1; s <= vx2; ++s) {
                if (b.cell_n(s, l, q) == 1) continue;
                const real valx = (*bx)(s), valy = (*by)(l), valz = (*bz)(q);
                const real x1 = (*ax)(lx - 1), x2 = (*ax)(lx + 1);
                const real y1 = (*ay)(ly - 1), y2 = (*ay)(ly + 1);
                const real z1 = (*az)(lz - 1), z2 = (*az)(lz + 1);
                const real deno = (x2 - x1) * (y2 - y1);
                const real xtx = (x2 - valx), xxo = (valx - x1);
                const real yty = (y2 - valy), yyo = (valy - y1);
                real f1 = src(xm, ym, zm), f2 = src(xq, ym, zm), f3 = src(xq, yq, zm),
                       f4 = src(xm, yq, zm);
                real num = (f1 * xtx + f2 * xxo) * yty + (f4 * xtx + f3 * xxo) * yyo;
                const real a1 = (num / deno);
                f1 = src(xm, ym, zq);
                f2 = src(xq, ym, zq);
                f3 = src(xq, yq, zq);
                f4 = src(xm, yq, zq);
                num = (f1 * xtx + f2 * xxo) * yty + (f4 * xtx + f3 * xxo) * yyo;
                const real a2 = (num / deno);
                const real r = a1 + ((valz - z1) * ((a2 - a1) / (z2 - z1)));
                int64_t ox = s, oy = l, oz = q;
                if (comp == 1) ox = s - 1;
                if (comp == 2) oy = l - 1;
                if (comp == 3) oz = q - 1;
                dst(ox, oy, oz) = r;
              }
        }
  }
}

}  // namespace orc
