// ORACLE -- TEST INFRASTRUCTURE ONLY (see orc_core.h).
// Marker-to-cell Search of src/Search.F90, restated serially.  The serial
// CPU build fills every index list in (k,j,i) order; the oracle does the same.
#include <cmath>
#include <vector>

#include "orc_core.h"

namespace orc {

// computeSurfaceNorm, src/Search.F90:210-258
void compute_surface_norm(Block& b, int64_t inor) {
  for (int64_t n = 1; n <= b.ibElems; ++n) {
    const real p1x = b.xnode1(b.ibElP1(n)), p1y = b.ynode1(b.ibElP1(n)), p1z = b.znode1(b.ibElP1(n));
    const real p2x = b.xnode1(b.ibElP2(n)), p2y = b.ynode1(b.ibElP2(n)), p2z = b.znode1(b.ibElP2(n));
    const real p3x = b.xnode1(b.ibElP3(n)), p3y = b.ynode1(b.ibElP3(n)), p3z = b.znode1(b.ibElP3(n));
    b.xcent(n) = (p2x + p1x + p3x) / 3.0;
    b.ycent(n) = (p2y + p1y + p3y) / 3.0;
    b.zcent(n) = (p2z + p1z + p3z) / 3.0;
    b.cosAlpha(n) = (p2y - p1y) * (p3z - p1z) - (p3y - p1y) * (p2z - p1z);
    b.cosBeta(n) = (p2z - p1z) * (p3x - p1x) - (p3z - p1z) * (p2x - p1x);
    b.cosGamma(n) = (p2x - p1x) * (p3y - p1y) - (p3x - p1x) * (p2y - p1y);
    const real len = sqrt(b.cosAlpha(n) * b.cosAlpha(n) + b.cosBeta(n) * b.cosBeta(n) +
                                 b.cosGamma(n) * b.cosGamma(n));
    b.element_length(n) = len;
    const real fin = (real)inor;
    b.cosAlpha(n) = fin * b.cosAlpha(n) / len;
    b.cosBeta(n) = fin * b.cosBeta(n) / len;
    b.cosGamma(n) = fin * b.cosGamma(n) / len;
  }
}

namespace {
inline real sq3(real a, real b, real c) { return a * a + b * b + c * c; }

// one cell of the nearest-element tagging (src/Search.F90:294-338 and the
// identical body of selectiveRetagging_th, :553-591)
void tag_cell(Block& b, int64_t i, int64_t j, int64_t k) {
  real minDis = 1e14, minDis1 = 1e14;
  int64_t nel2Cen = 0, nel2Pnt = 0;
  for (int64_t m = 1; m <= b.ibElems; ++m) {
    const real dis_cen = sq3(b.xp(i) - b.xcent(m), b.yp(j) - b.ycent(m), b.zp(k) - b.zcent(m));
    const real dis_pnt = sq3(b.x1(i) - b.xcent(m), b.y1(j) - b.ycent(m), b.z1(k) - b.zcent(m));
    if (dis_cen < minDis) {
      minDis = dis_cen;
      nel2Cen = m;
    }
    if (dis_pnt < minDis1) {
      minDis1 = dis_pnt;
      nel2Pnt = m;
    }
  }
  if ((b.x1(i) <= b.xcent(nel2Cen) && b.x1(i + 1) >= b.xcent(nel2Cen)) &&
      (b.y1(j) <= b.ycent(nel2Cen) && b.y1(j + 1) >= b.ycent(nel2Cen)) &&
      (b.z1(k) <= b.zcent(nel2Cen) && b.z1(k + 1) >= b.zcent(nel2Cen)))
    b.cell(i, j, k) = 2;
  const real n2dotn = (b.x1(i) - b.xcent(nel2Pnt)) * b.cosAlpha(nel2Pnt) +
                        (b.y1(j) - b.ycent(nel2Pnt)) * b.cosBeta(nel2Pnt) +
                        (b.z1(k) - b.zcent(nel2Pnt)) * b.cosGamma(nel2Pnt);
  b.nodeIdTag(i, j, k) = (n2dotn >= -1e-16) ? 0 : 1;
}

int64_t corner_sum(Block& b, int64_t i, int64_t j, int64_t k) {
  const I3& t = b.nodeIdTag;
  return t(i, j, k) + t(i + 1, j, k) + t(i, j + 1, k) + t(i + 1, j + 1, k) + t(i, j, k + 1) +
         t(i + 1, j, k + 1) + t(i, j + 1, k + 1) + t(i + 1, j + 1, k + 1);
}

void count_cells(Block& b) {
  b.ibCellCount = b.solidCellCount = b.fluidCellCount = 0;
  for (int64_t k = 2; k <= b.nz + 1; ++k)
    for (int64_t j = 2; j <= b.ny + 1; ++j)
      for (int64_t i = 2; i <= b.nx + 1; ++i) {
        const int64_t c = b.cell(i, j, k);
        if (c == 1)
          b.solidCellCount++;
        else if (c == 0)
          b.fluidCellCount++;
        else if (c == 2)
          b.ibCellCount++;
      }
}
}  // namespace

// tagging_th_core, src/Search.F90:260-386
void tagging_th_core(Block& b) {
  b.cell.fill(0);
  b.cell2.fill(0);
  b.nodeIdTag.fill(0);
  // each cell's tags depend only on the geometry: parallel over planes
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = b.k_startSearch; k <= b.k_endSearch; ++k)
    for (int64_t j = b.j_startSearch; j <= b.j_endSearch; ++j)
      for (int64_t i = b.i_startSearch; i <= b.i_endSearch; ++i) tag_cell(b, i, j, k);
  for (int64_t k = b.k_startSearch; k <= b.k_endSearch; ++k)
    for (int64_t j = b.j_startSearch; j <= b.j_endSearch; ++j)
      for (int64_t i = b.i_startSearch; i <= b.i_endSearch; ++i)
        if (b.cell(i, j, k) != 2 && corner_sum(b, i, j, k) == 8) b.cell(i, j, k) = 1;
  count_cells(b);
}

// selectiveRetagging_th, src/Search.F90:520-651
void selective_retagging_th(Block& b) {
  if (b.blk_mv_tag != 0) return;
  for (int64_t nn = 1; nn <= b.ibCellCount; ++nn)
    b.cell(b.interceptedIndexPtr(nn, 1), b.interceptedIndexPtr(nn, 2),
           b.interceptedIndexPtr(nn, 3)) = 0;
  // The neighbourhoods of IB cells overlap; a cell's new tags depend only on
  // the geometry and (in the second pass) on its own tag and the node tags of
  // the first pass, so visiting each cell once, in parallel, gives the serial
  // loops' result.
  std::vector<int64_t> cells;
  {
    std::vector<uint8_t> seen((size_t)(b.nx + 2) * (b.ny + 2) * (b.nz + 2), 0);
    for (int64_t nn = 1; nn <= b.ibCellCount; ++nn)
      for (int64_t kp = -1; kp <= 1; ++kp)
        for (int64_t jp = -1; jp <= 1; ++jp)
          for (int64_t ip = -1; ip <= 1; ++ip) {
            const int64_t i = b.interceptedIndexPtr(nn, 1) + ip, j = b.interceptedIndexPtr(nn, 2) + jp,
                          k = b.interceptedIndexPtr(nn, 3) + kp;
            const size_t q = (size_t)((i - 1) + (b.nx + 2) * ((j - 1) + (b.ny + 2) * (k - 1)));
            ORC_CHECK(i >= 1 && i <= b.nx + 2 && j >= 1 && j <= b.ny + 2 && k >= 1 && k <= b.nz + 2,
                      "retag neighbourhood");
            if (!seen[q]) {
              seen[q] = 1;
              cells.push_back((int64_t)q);
            }
          }
  }
  const int64_t nc = (int64_t)cells.size(), sx = b.nx + 2, sy = b.ny + 2;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t c = 0; c < nc; ++c) {
    const int64_t q = cells[(size_t)c];
    tag_cell(b, 1 + q % sx, 1 + (q / sx) % sy, 1 + q / (sx * sy));
  }
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nc; ++c) {
    const int64_t q = cells[(size_t)c];
    const int64_t i = 1 + q % sx, j = 1 + (q / sx) % sy, k = 1 + q / (sx * sy);
    if (b.cell(i, j, k) != 2) b.cell(i, j, k) = corner_sum(b, i, j, k) == 8 ? 1 : 0;
  }
  count_cells(b);
}

// cellCount_solid, src/Search.F90:653-741 (serial order)
void cellcount_solid(Block& b) {
  b.interceptedIndexPtr.alloc(b.ibCellCount, 3);
  b.fluidIndexPtr.alloc(b.fluidCellCount, 3);
  b.solidIndexPtr.alloc(b.solidCellCount, 3);
  int64_t ipt = 0, ipt1 = 0, ipt2 = 0;
  for (int64_t k = 2; k <= b.nz + 1; ++k)
    for (int64_t j = 2; j <= b.ny + 1; ++j)
      for (int64_t i = 2; i <= b.nx + 1; ++i) {
        const int64_t c = b.cell(i, j, k);
        I2* L = nullptr;
        int64_t* cnt = nullptr;
        if (c == 0) {
          L = &b.fluidIndexPtr;
          cnt = &ipt1;
        } else if (c == 1) {
          L = &b.solidIndexPtr;
          cnt = &ipt2;
        } else if (c == 2) {
          L = &b.interceptedIndexPtr;
          cnt = &ipt;
        }
        if (L) {
          ++*cnt;
          (*L)(*cnt, 1) = i;
          (*L)(*cnt, 2) = j;
          (*L)(*cnt, 3) = k;
        }
      }
  int64_t red = 0, black = 0;
  for (int64_t n = 1; n <= b.fluidCellCount; ++n) {
    const int64_t s = b.fluidIndexPtr(n, 1) + b.fluidIndexPtr(n, 2) + b.fluidIndexPtr(n, 3);
    if (s % 2 == 1)
      red++;
    else
      black++;
  }
  b.redCellCount = red;
  b.blackCellCount = black;
  b.redCellIndexPtr.alloc(red, 3);
  b.blackCellIndexPtr.alloc(black, 3);
  int64_t r = 0, bl = 0;
  for (int64_t n = 1; n <= b.fluidCellCount; ++n) {
    const int64_t s = b.fluidIndexPtr(n, 1) + b.fluidIndexPtr(n, 2) + b.fluidIndexPtr(n, 3);
    I2& L = (s % 2 == 1) ? b.redCellIndexPtr : b.blackCellIndexPtr;
    int64_t& c = (s % 2 == 1) ? r : bl;
    ++c;
    for (int d = 1; d <= 3; ++d) L(c, d) = b.fluidIndexPtr(n, d);
  }
}

// cellCount_solid_coarse, src/Search.F90:1463-1532
void cellcount_solid_coarse(Block& b) {
  b.fluidCellCount = 0;
  for (int64_t k = 2; k <= b.nz + 1; ++k)
    for (int64_t j = 2; j <= b.ny + 1; ++j)
      for (int64_t i = 2; i <= b.nx + 1; ++i)
        if (b.cell(i, j, k) == 0) b.fluidCellCount++;
  b.fluidIndexPtr.alloc(b.fluidCellCount, 3);
  int64_t ipt1 = 0;
  for (int64_t k = 2; k <= b.nz + 1; ++k)
    for (int64_t j = 2; j <= b.ny + 1; ++j)
      for (int64_t i = 2; i <= b.nx + 1; ++i)
        if (b.cell(i, j, k) == 0) {
          ++ipt1;
          b.fluidIndexPtr(ipt1, 1) = i;
          b.fluidIndexPtr(ipt1, 2) = j;
          b.fluidIndexPtr(ipt1, 3) = k;
        }
  int64_t red = 0, black = 0;
  for (int64_t n = 1; n <= b.fluidCellCount; ++n) {
    const int64_t s = b.fluidIndexPtr(n, 1) + b.fluidIndexPtr(n, 2) + b.fluidIndexPtr(n, 3);
    if (s % 2 == 1) red++; else black++;
  }
  b.redCellCount = red;
  b.blackCellCount = black;
  b.redCellIndexPtr.alloc(red, 3);
  b.blackCellIndexPtr.alloc(black, 3);
  int64_t r = 0, bl = 0;
  for (int64_t n = 1; n <= b.fluidCellCount; ++n) {
    const int64_t s = b.fluidIndexPtr(n, 1) + b.fluidIndexPtr(n, 2) + b.fluidIndexPtr(n, 3);
    I2& L = (s % 2 == 1) ? b.redCellIndexPtr : b.blackCellIndexPtr;
    int64_t& c = (s % 2 == 1) ? r : bl;
    ++c;
    for (int d = 1; d <= 3; ++d) L(c, d) = b.fluidIndexPtr(n, d);
  }
}

// computeNormDistance, src/Search.F90:743-861
void compute_norm_distance(Block& b) {
  const int64_t nib = b.ibCellCount;
  for (F1* a : {&b.pNormDis, &b.u1NormDis, &b.u2NormDis, &b.v1NormDis, &b.v2NormDis,
                &b.w1NormDis, &b.w2NormDis})
    a->alloc(nib);
  for (I1* a : {&b.nelp, &b.nelu1, &b.nelu2, &b.nelv1, &b.nelv2, &b.nelw1, &b.nelw2}) a->alloc(nib);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t k = 1; k <= nib; ++k) {
    const int64_t ci = b.interceptedIndexPtr(k, 1), cj = b.interceptedIndexPtr(k, 2),
                  ck = b.interceptedIndexPtr(k, 3);
    const real n1x = b.xp(ci), n2x = b.x1(ci), n3x = b.x1(ci + 1);
    const real n1y = b.yp(cj), n2y = b.y1(cj), n3y = b.y1(cj + 1);
    const real n1z = b.zp(ck), n2z = b.z1(ck), n3z = b.z1(ck + 1);
    real md[7] = {1e14, 1e14, 1e14, 1e14, 1e14, 1e14, 1e14};
    int64_t nel[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int64_t m = 1; m <= b.ibElems; ++m) {
      const real cx = b.xcent(m), cy = b.ycent(m), cz = b.zcent(m);
      const real d[7] = {
          sq3(n1x - cx, n1y - cy, n1z - cz), sq3(n2x - cx, n1y - cy, n1z - cz),
          sq3(n3x - cx, n1y - cy, n1z - cz), sq3(n1x - cx, n2y - cy, n1z - cz),
          sq3(n1x - cx, n3y - cy, n1z - cz), sq3(n1x - cx, n1y - cy, n2z - cz),
          sq3(n1x - cx, n1y - cy, n3z - cz)};
      for (int q = 0; q < 7; ++q)
        if (d[q] < md[q]) {
          md[q] = d[q];
          nel[q] = m;
        }
    }
    b.nelp(k) = nel[0];
    b.nelu1(k) = nel[1];
    b.nelu2(k) = nel[2];
    b.nelv1(k) = nel[3];
    b.nelv2(k) = nel[4];
    b.nelw1(k) = nel[5];
    b.nelw2(k) = nel[6];
    auto nd = [&](int64_t e, real x, real y, real z) {
      return (x - b.xcent(e)) * b.cosAlpha(e) + (y - b.ycent(e)) * b.cosBeta(e) +
             (z - b.zcent(e)) * b.cosGamma(e);
    };
    b.pNormDis(k) = nd(nel[0], n1x, n1y, n1z);
    b.u1NormDis(k) = nd(nel[1], n2x, n1y, n1z);
    b.u2NormDis(k) = nd(nel[2], n3x, n1y, n1z);
    b.v1NormDis(k) = nd(nel[3], n1x, n2y, n1z);
    b.v2NormDis(k) = nd(nel[4], n1x, n3y, n1z);
    b.w1NormDis(k) = nd(nel[5], n1x, n1y, n2z);
    b.w2NormDis(k) = nd(nel[6], n1x, n1y, n3z);
  }
}

// findTScells, src/Search.F90:434-518 (serial order of the TS list)
void find_ts_cells(Block& b) {
  for (int64_t k = 2; k <= b.nz + 1; ++k)
    for (int64_t j = 2; j <= b.ny + 1; ++j)
      for (int64_t i = 2; i <= b.nx + 1; ++i) b.cell2(i, j, k) = 0;
  int64_t cnt = 0;
  for (int64_t n = 1; n <= b.ibCellCount; ++n) {
    const int64_t s = b.ibSurfId(b.nelp(n));
    if (s == 51 || s == 52) {
      b.cell2(b.interceptedIndexPtr(n, 1), b.interceptedIndexPtr(n, 2),
              b.interceptedIndexPtr(n, 3)) = 2;
      cnt++;
    }
  }
  b.TSCellCount = cnt;
  b.TSIndexPtr.alloc(cnt, 3);
  b.index_ts.alloc(cnt);
  int64_t ip = 0;
  for (int64_t n = 1; n <= b.ibCellCount; ++n) {
    const int64_t i = b.interceptedIndexPtr(n, 1), j = b.interceptedIndexPtr(n, 2),
                  k = b.interceptedIndexPtr(n, 3);
    if (b.cell2(i, j, k) == 2) {
      ++ip;
      b.TSIndexPtr(ip, 1) = i;
      b.TSIndexPtr(ip, 2) = j;
      b.TSIndexPtr(ip, 3) = k;
      b.index_ts(ip) = n;
    }
  }
  for (F1* a : {&b.u2_ghost, &b.u2t_ghost, &b.v2_ghost, &b.v2t_ghost, &b.p_ghost, &b.pt_ghost,
                &b.u1_ghost, &b.u1t_ghost, &b.v1_ghost, &b.v1t_ghost, &b.w2_ghost, &b.w2t_ghost,
                &b.w1_ghost, &b.w1t_ghost})
    a->alloc(cnt);
}

// fine_block_cell, src/Search.F90:863-914
void fine_block_cell() {
  Block& c = blk_of(1);
  c.cell_n.fill(0);
  c.cell.fill(0);
  c.cell_pr.fill(0);
  for (Interface* itp : g_interfaces) {
    Interface& it = *itp;
    Block& a = blk_of(it.a_blk);
    Block& fb = blk_of(it.b_blk);
    for (int64_t k = 2; k <= a.nz + 1; ++k)
      for (int64_t j = 2; j <= a.ny + 1; ++j)
        for (int64_t i = 2; i <= a.nx + 1; ++i) {
          const real ci = (real)fb.cintp;
          if (a.xp(i) >= it.xintf_start + ci * a.dx && a.xp(i) <= it.xintf_end - ci * a.dx &&
              a.zp(k) >= it.zintf_start + ci * a.dz && a.zp(k) <= it.zintf_end - ci * a.dz &&
              a.yp(j) >= it.yintf_start + ci * a.dy && a.yp(j) <= it.yintf_end - ci * a.dy) {
            a.cell_n(i, j, k) = 1;
            a.cell(i, j, k) = 1;
          }
          if (a.xp(i) >= it.xintf_start && a.xp(i) <= it.xintf_end && a.zp(k) >= it.zintf_start &&
              a.zp(k) <= it.zintf_end && a.yp(j) >= it.yintf_start && a.yp(j) <= it.yintf_end)
            a.cell_pr(i, j, k) = 1;
        }
  }
}

}  // namespace orc
