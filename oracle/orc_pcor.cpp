// ORACLE -- TEST INFRASTRUCTURE ONLY (see orc_core.h).
// Pressure-correction solve of src/PcorVcor.F90, restated serially.
#include <cmath>
#include "orc_core.h"

namespace orc {

// computeDiv, src/PcorVcor.F90:222-243
void compute_div(Block& b) {
#pragma omp parallel for schedule(static)
  for (int64_t n = 1; n <= b.fluidCellCount; ++n) {
    const int64_t i = b.fluidIndexPtr(n, 1), j = b.fluidIndexPtr(n, 2), k = b.fluidIndexPtr(n, 3);
    b.b(i, j, k) = (b.ut(i, j, k) - b.ut(i - 1, j, k)) / b.deltax(i) +
                   (b.vt(i, j, k) - b.vt(i, j - 1, k)) / b.deltay(j) +
                   (b.wt(i, j, k) - b.wt(i, j, k - 1)) / b.deltaz(k);
  }
}

// correctPressure, src/PcorVcor.F90:245-259
void correct_pressure(Block& b) {
#pragma omp parallel for schedule(static)
  for (int64_t n = 1; n <= b.fluidCellCount; ++n) {
    const int64_t i = b.fluidIndexPtr(n, 1), j = b.fluidIndexPtr(n, 2), k = b.fluidIndexPtr(n, 3);
    b.p(i, j, k) = b.p(i, j, k) + b.pc(i, j, k);
  }
}

// correctVelocity, src/PcorVcor.F90:261-286
void correct_velocity(Block& b, real deltat) {
#pragma omp parallel for schedule(static)
  for (int64_t n = 1; n <= b.fluidCellCount; ++n) {
    const int64_t i = b.fluidIndexPtr(n, 1), j = b.fluidIndexPtr(n, 2), k = b.fluidIndexPtr(n, 3);
    b.ut(i, j, k) = b.ut(i, j, k) - deltat / (0.5 * (b.deltax(i + 1) + b.deltax(i))) *
                                        (b.pc(i + 1, j, k) - b.pc(i, j, k));
    b.vt(i, j, k) = b.vt(i, j, k) - deltat / (0.5 * (b.deltay(j + 1) + b.deltay(j))) *
                                        (b.pc(i, j + 1, k) - b.pc(i, j, k));
    b.wt(i, j, k) = b.wt(i, j, k) - deltat / (0.5 * (b.deltaz(k + 1) + b.deltaz(k))) *
                                        (b.pc(i, j, k + 1) - b.pc(i, j, k));
  }
}

// REDBLACKSOR_linear, src/PcorVcor.F90:288-377.  The red sweep reads the old
// iterate pco, the black sweep the updated pc; every 5th iteration the max
// increment over the fluid cells is the stop test; pco <- pc after each sweep
// pair.  Within one sweep every update reads only values that sweep does not
// write (the other colour, pco, b), and a maximum does not depend on the
// order of its operands, so the loops run in parallel (OpenMP) with results
// identical to the serial order.
void redblack_sor_linear(Block& b, int64_t pcItaMax, real deltat, real epsi) {
  const real omega = b.omega;
  real derr4 = 11111.0;
  b.derr2 = 0.0;
  for (;;) {
    b.nIterPcor = b.nIterPcor + 1;
#pragma omp parallel for schedule(static)
    for (int64_t n = 1; n <= b.redCellCount; ++n) {
      const int64_t i = b.redCellIndexPtr(n, 1), j = b.redCellIndexPtr(n, 2),
                    k = b.redCellIndexPtr(n, 3);
      real v = (b.b(i, j, k) / deltat - b.Acx(i - 1, 1) * b.pco(i - 1, j, k) -
                  b.Acx(i - 1, 3) * b.pco(i + 1, j, k) - b.Acy(j - 1, 1) * b.pco(i, j - 1, k) -
                  b.Acy(j - 1, 3) * b.pco(i, j + 1, k) - b.Acz(k - 1, 1) * b.pco(i, j, k - 1) -
                  b.Acz(k - 1, 3) * b.pco(i, j, k + 1)) /
                 (b.Acx(i - 1, 2) + b.Acy(j - 1, 2) + b.Acz(k - 1, 2));
      b.pc(i, j, k) = v;
      b.pc(i, j, k) = (1.0 - omega) * b.pco(i, j, k) + omega * b.pc(i, j, k);
    }
#pragma omp parallel for schedule(static)
    for (int64_t n = 1; n <= b.blackCellCount; ++n) {
      const int64_t i = b.blackCellIndexPtr(n, 1), j = b.blackCellIndexPtr(n, 2),
                    k = b.blackCellIndexPtr(n, 3);
      real v = (b.b(i, j, k) / deltat - b.Acx(i - 1, 1) * b.pc(i - 1, j, k) -
                  b.Acx(i - 1, 3) * b.pc(i + 1, j, k) - b.Acy(j - 1, 1) * b.pc(i, j - 1, k) -
                  b.Acy(j - 1, 3) * b.pc(i, j + 1, k) - b.Acz(k - 1, 1) * b.pc(i, j, k - 1) -
                  b.Acz(k - 1, 3) * b.pc(i, j, k + 1)) /
                 (b.Acx(i - 1, 2) + b.Acy(j - 1, 2) + b.Acz(k - 1, 2));
      b.pc(i, j, k) = v;
      b.pc(i, j, k) = (1.0 - omega) * b.pco(i, j, k) + omega * b.pc(i, j, k);
    }
    if (b.nIterPcor % 5 == 0) {
      double m = 0.0;  // the stop test reads values only
#pragma omp parallel for schedule(static) reduction(max : m)
      for (int64_t n = 1; n <= b.fluidCellCount; ++n) {
        const int64_t i = b.fluidIndexPtr(n, 1), j = b.fluidIndexPtr(n, 2),
                      k = b.fluidIndexPtr(n, 3);
        const double var = val(fabs(b.pc(i, j, k) - b.pco(i, j, k)));
        m = fmax(m, var);
      }
      derr4 = m;
    }
    {
      const size_t nd = b.pc.d.size();
      const real* src = b.pc.d.data();
      real* dst = b.pco.d.data();
#pragma omp parallel for schedule(static)
      for (size_t q = 0; q < nd; ++q) dst[q] = src[q];
    }
    b.derr2 = derr4;
    if (derr4 < epsi || b.nIterPcor > pcItaMax) break;
  }
}

// updateVelocity_newv, src/PcorVcor.F90:379-397
void update_velocity_newv(Block& b) {
  if (b.move_check != 1) return;
  b.ut.d = b.u.d;
  b.vt.d = b.v.d;
  b.wt.d = b.w.d;
}

// poissonSolver, src/PcorVcor.F90:22-220 over blocks start..finish by step.
// Block 1 is the coarse block; the OpenMP regions run their block loops in
// order (the blocks are independent inside each region).
void poisson_solver(int64_t pcItaMax, real epsi, real deltat, real uc, int64_t start,
                    int64_t finish, int64_t step) {
  for (int64_t g = start; g <= finish; g += step) {
    Block& b = blk_of(g);
    b.b.fill(0.0);
    b.pc.fill(0.0);
    b.pco.fill(0.0);
    b.nIterPcor = 0;
    b.derr2 = 0.0;
    b.derrStdSt = 0.0;
  }
  fine_update_newv_bd();
  coarse_update_newv();
  for (int64_t g = start; g <= finish; g += step) {
    compute_div(blk_of(g));
    if (g != 1) redblack_sor_linear(blk_of(g), pcItaMax, deltat, epsi);
  }
  coarse_update_pc();
  for (int64_t g = start; g <= finish; g += step)
    if (g == 1) redblack_sor_linear(blk_of(g), pcItaMax, deltat, epsi);
  fine_update_pc_bd();
  for (int64_t g = start; g <= finish; g += step)
    if (g != 1) redblack_sor_linear(blk_of(g), pcItaMax, deltat, epsi);
  coarse_update_pc();
  for (int64_t g = start; g <= finish; g += step) {
    correct_pressure(blk_of(g));
    correct_velocity(blk_of(g), deltat);
  }
  for (int64_t g = start; g <= finish; g += step)
    if (g == 1) velocity_bc(blk_of(1), deltat, uc);
  for (int64_t g = start; g <= finish; g += step) {
    Block& b = blk_of(g);
    double err_ds = 0.0;  // a statistic: values only
#pragma omp parallel for schedule(static) reduction(max : err_ds)
    for (int64_t n = 1; n <= b.fluidCellCount; ++n) {
      const int64_t i = b.fluidIndexPtr(n, 1), j = b.fluidIndexPtr(n, 2), k = b.fluidIndexPtr(n, 3);
      const double eu = val(fabs((b.ut(i, j, k) - b.u(i, j, k))) / deltat);
      const double ev = val(fabs((b.vt(i, j, k) - b.v(i, j, k))) / deltat);
      const double ew = val(fabs((b.wt(i, j, k) - b.w(i, j, k))) / deltat);
      err_ds = fmax(fmax(fmax(err_ds, eu), ev), ew);
    }
    b.derrStdSt = err_ds;
  }
  for (int64_t g = start; g <= finish; g += step) {
    Block& b = blk_of(g);
    b.u.d = b.ut.d;
    b.v.d = b.vt.d;
    b.w.d = b.wt.d;
  }
  for (size_t g = 1; g <= g_interfaces.size(); ++g) fine_update_bd_mv((int64_t)g);
  coarse_update();
}

}  // namespace orc
