// Test infrastructure, not product code: the serial CPU restatement of the
// reference's fine-block moves, used only as the checker of the GPU path.
//
// block_move_check, change_block_coords, change_block_coords_interfaces,
// change_block_interface (src/Search.F90:997-1461), cellCount_solid_coarse_mv
// (:916-995) and tagging_th_move (:415-432), in the order app/main.F90:178-230
// calls them.  A fine block whose moving surface comes within fixed margins
// of its interface box is shifted by whole cells (a multiple of the refinement
// factor); its fields are moved with it, the interface tables shifted, the
// coarse block re-marked and the fine block re-tagged and refilled from the
// coarse block where it has no old data.
#include <cmath>

#include "orc_core.h"

namespace orc {

namespace {

// the rounding of a move amount to the refinement factor (Search.F90:1043-1058,
// repeated for x and z)
int64_t round_move(int64_t m, int64_t factor) {
  if (std::llabs(m) < factor) return m < 0 ? -factor : factor;
  if (m < 0) return m + std::llabs(m) % factor;
  return m - std::llabs(m) % factor;
}

// first index i in [from, n] with v(i) > s; `fallback` when none
int64_t first_above(const F1& v, int64_t from, int64_t n, real s, int64_t fallback) {
  for (int64_t i = from; i <= n; ++i)
    if (v(i) > s) return i;
  return fallback;
}

}  // namespace

// Search.F90:997-1203
void block_move_check(int64_t& coarse_flcnt_check) {
  for (Interface* itp : g_interfaces) {
    Interface& it = *itp;
    Block& fb = blk_of(it.b_blk);
    // the reference reads ynode1(mk) and xnode1(mkx1) of every fine block;
    // a block without a moving plate has no such nodes (mk = 0, an
    // out-of-bounds read there) and is skipped, as the library does
    if (fb.mk < 1 || fb.mkx1 < 1) continue;
    const real mg1 = (real)fb.cintp * blk_of(1).dx;
    const real marginx = 4.5 * mg1, marginy = 5 * mg1, marginz = 1.52 * mg1;
    const int64_t factor = it.b_msh / it.a_msh;
    const real yval_up = fmax(fb.ynode1(fb.mk), fb.nxty_cent + 0.02);
    const real yval_dw = fmin(fb.ynode1(fb.mk), fb.nxty_cent - 0.02);
    const real xval_lt = fb.xnode1(fb.mkx1);
    fb.move_amty = fb.move_amtx = fb.move_amtz = 0;
    const bool trig = fabs(xval_lt - it.xintf_start) <= marginx ||
                      fabs(fb.piv_z - it.zintf_start) <= marginz ||
                      fabs(fb.piv_z - it.zintf_end) <= marginz ||
                      fabs(yval_dw - it.yintf_start) <= marginy || fabs(yval_up - it.yintf_end) <= marginy;
    if (!trig) continue;
    fb.move_check = 1;
    fb.blk_mv_tag = 1;
    coarse_flcnt_check = 1;
    if (fabs(yval_dw - it.yintf_start) <= marginy || fabs(yval_up - it.yintf_end) <= marginy) {
      fb.move_amty = round_move((int64_t)val(floor((fb.nxty_cent - fb.inity_cent) / fb.dy)), factor);
      fb.inity_cent = fb.nxty_cent;
    }
    if (fabs(xval_lt - it.xintf_start) < marginx) {
      fb.move_amtx = round_move((int64_t)val(floor((fb.nxtx_cent - fb.initx_cent) / fb.dx)) - factor, factor);
      fb.initx_cent = fb.nxtx_cent;
    }
    if (fabs(fb.piv_z - it.zintf_start) < (0.500 - 0.410 - mg1) ||
        fabs(fb.piv_z - it.zintf_end) < (0.600 - 0.500 - mg1)) {
      fb.move_amtz = round_move((int64_t)val(floor((fb.nxtz_cent - fb.initz_cent) / fb.dz)), factor);
      fb.initz_cent = fb.nxtz_cent;
    }
    const real cx = fb.move_amtx * fb.dx, cy = fb.move_amty * fb.dy, cz = fb.move_amtz * fb.dz;
    it.xintf_st_new = fmax(it.xintf_start, it.xintf_start + cx);
    it.xintf_en_new = fmin(it.xintf_end, it.xintf_end + cx);
    it.yintf_st_new = fmax(it.yintf_start, it.yintf_start + cy);
    it.yintf_en_new = fmin(it.yintf_end, it.yintf_end + cy);
    it.zintf_st_new = fmax(it.zintf_start, it.zintf_start + cz);
    it.zintf_en_new = fmin(it.zintf_end, it.zintf_end + cz);
    it.xintf_start = it.xintf_start + cx;
    it.xintf_end = it.xintf_end + cx;
    it.yintf_start = it.yintf_start + cy;
    it.yintf_end = it.yintf_end + cy;
    it.zintf_start = it.zintf_start + cz;
    it.zintf_end = it.zintf_end + cz;
    // the old indices whose centres lie in the overlap of the old and new boxes
    fb.cpy_x_start = first_above(fb.xp, 1, fb.nx + 2, it.xintf_st_new, fb.cpy_x_start);
    fb.cpy_x_end = first_above(fb.xp, fb.cpy_x_start, fb.nx + 2, it.xintf_en_new, fb.cpy_x_end + 1) - 1;
    fb.cpy_y_start = first_above(fb.yp, 1, fb.ny + 2, it.yintf_st_new, fb.cpy_y_start);
    fb.cpy_y_end = first_above(fb.yp, fb.cpy_y_start, fb.ny + 2, it.yintf_en_new, fb.cpy_y_end + 1) - 1;
    fb.cpy_z_start = first_above(fb.zp, 1, fb.nz + 2, it.zintf_st_new, fb.cpy_z_start);
    fb.cpy_z_end = first_above(fb.zp, fb.cpy_z_start, fb.nz + 2, it.zintf_en_new, fb.cpy_z_end + 1) - 1;
    fb.u_dum = fb.u;
    fb.v_dum = fb.v;
    fb.w_dum = fb.w;
    fb.p_dum = fb.p;
  }
}

// Search.F90:1208-1264: the grid shifted by whole cells (spacings unchanged)
void change_block_coords(Block& b) {
  if (b.move_check != 1) return;
  const real cz = b.move_amtz * b.dz, cy = b.move_amty * b.dy, cx = b.move_amtx * b.dx;
  for (int64_t i = 1; i <= b.nx + 3; ++i) b.x1(i) = b.x1(i) + cx;
  for (int64_t i = 1; i <= b.ny + 3; ++i) b.y1(i) = b.y1(i) + cy;
  for (int64_t i = 1; i <= b.nz + 3; ++i) b.z1(i) = b.z1(i) + cz;
  for (int64_t i = 1; i <= b.nx + 3; ++i) b.xu(i) = b.x1(i);
  for (int64_t i = 1; i <= b.ny + 3; ++i) b.yv(i) = b.y1(i);
  for (int64_t i = 1; i <= b.nz + 3; ++i) b.zw(i) = b.z1(i);
  for (int64_t i = 1; i <= b.ny + 2; ++i) {
    b.yu(i) = 0.5 * (b.y1(i) + b.y1(i + 1));
    b.yw(i) = b.yu(i);
    b.yp(i) = b.yu(i);
  }
  for (int64_t i = 1; i <= b.nx + 2; ++i) {
    b.xv(i) = 0.5 * (b.x1(i) + b.x1(i + 1));
    b.xw(i) = b.xv(i);
    b.xp(i) = b.xv(i);
  }
  for (int64_t i = 1; i <= b.nz + 2; ++i) {
    b.zu(i) = 0.5 * (b.z1(i) + b.z1(i + 1));
    b.zv(i) = b.zu(i);
    b.zp(i) = b.zu(i);
  }
}

// Search.F90:1269-1370: cell_n marks the cells with old data, the fields
// move with the grid (zero where there is no old data)
void change_block_coords_interfaces(Interface& it, Block& b) {
  if (b.move_check != 1) return;
  b.cell_n.fill(0);
  for (int64_t k = 1; k <= b.nz + 2; ++k)
    for (int64_t j = 1; j <= b.ny + 2; ++j)
      for (int64_t i = 1; i <= b.nx + 2; ++i)
        if (b.xp(i) > it.xintf_st_new + b.dx && b.xp(i) < it.xintf_en_new - b.dx &&
            b.zp(k) > it.zintf_st_new + b.dz && b.zp(k) < it.zintf_en_new - b.dz &&
            b.yp(j) > it.yintf_st_new + b.dy && b.yp(j) < it.yintf_en_new - b.dy)
          b.cell_n(i, j, k) = 1;
  b.cpy_x_start_mv = first_above(b.xp, 1, b.nx + 2, it.xintf_st_new, b.cpy_x_start_mv);
  b.cpy_x_end_mv = first_above(b.xp, b.cpy_x_start_mv, b.nx + 2, it.xintf_en_new, b.cpy_x_end_mv + 1) - 1;
  b.cpy_y_start_mv = first_above(b.yp, 1, b.ny + 2, it.yintf_st_new, b.cpy_y_start_mv);
  b.cpy_y_end_mv = first_above(b.yp, b.cpy_y_start_mv, b.ny + 2, it.yintf_en_new, b.cpy_y_end_mv + 1) - 1;
  b.cpy_z_start_mv = first_above(b.zp, 1, b.nz + 2, it.zintf_st_new, b.cpy_z_start_mv);
  b.cpy_z_end_mv = first_above(b.zp, b.cpy_z_start_mv, b.nz + 2, it.zintf_en_new, b.cpy_z_end_mv + 1) - 1;
  b.u.fill(0.0);
  b.v.fill(0.0);
  b.w.fill(0.0);
  b.p.fill(0.0);
  int64_t cz = b.cpy_z_start;
  for (int64_t k = b.cpy_z_start_mv; k <= b.cpy_z_end_mv; ++k, ++cz) {
    int64_t cx = b.cpy_x_start;
    for (int64_t i = b.cpy_x_start_mv; i <= b.cpy_x_end_mv; ++i, ++cx) {
      int64_t cy = b.cpy_y_start;
      for (int64_t j = b.cpy_y_start_mv; j <= b.cpy_y_end_mv; ++j, ++cy) {
        b.u(i, j, k) = b.u_dum(cx, cy, cz);
        b.v(i, j, k) = b.v_dum(cx, cy, cz);
        b.w(i, j, k) = b.w_dum(cx, cy, cz);
        b.p(i, j, k) = b.p_dum(cx, cy, cz);
      }
    }
  }
}

// Search.F90:1372-1461: the coarse indices of the interface tables shift by
// the move in coarse cells
void change_block_interface(Interface& it, Block& a, Block& b) {
  (void)a;
  if (b.move_check != 1) return;
  const int64_t factor = it.b_msh / it.a_msh;
  auto shift = [](I2& t, int64_t count, int64_t inc) {
    for (int64_t q = 1; q <= count; ++q) t(1, q) = t(1, q) + inc;
  };
  const int64_t ix = b.move_amtx / factor, iy = b.move_amty / factor, iz = b.move_amtz / factor;
  shift(it.px, it.cxp, ix);
  shift(it.ux, it.cxu, ix);
  shift(it.vx, it.cxv, ix);
  shift(it.wx, it.cxw, ix);
  shift(it.py, it.cyp, iy);
  shift(it.uy, it.cyu, iy);
  shift(it.vy, it.cyv, iy);
  shift(it.wy, it.cyw, iy);
  shift(it.pz, it.czp, iz);
  shift(it.uz, it.czu, iz);
  shift(it.vz, it.czv, iz);
  shift(it.wz, it.czw, iz);
}

// Search.F90:916-995
void cellcount_solid_coarse_mv(int64_t& coarse_flcnt_check) {
  if (coarse_flcnt_check == 1) cellcount_solid_coarse(blk_of(1));
  coarse_flcnt_check = 0;
}

// Search.F90:415-432
void tagging_th_move(Block& b, int64_t id) {
  if (b.move_check != 1) return;
  tagging_th_core(b);
  for (size_t g = 0; g < g_interfaces.size(); ++g) {
    if (g_interfaces[g]->b_blk != id) continue;
    fine_update_mv((int64_t)g + 1);
    fine_update_bd_mv((int64_t)g + 1);
  }
}

}  // namespace orc
