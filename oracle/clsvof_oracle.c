/*
 * clsvof_oracle.c -- CPU restatement of the level-set part of SIMCOFlow's
 * CLSVOF sweeps: X_Sweep (src/Clsvof_Mod.f90:1074-1123) and Y_Sweep
 * (:1191-1244), as the reference's sequential loops over faces, statement
 * by statement (IEEE FP64, built with -ffp-contract=off).
 *
 * TEST INFRASTRUCTURE ONLY: only tests/, smoke() and the CPU-baseline leg of
 * bench.py load it; the product path never calls it.
 * Parity status: UNPINNED against the reference binary (no Fortran compiler
 * here); pinned against a second, pure-Python transcription of the same
 * loops in tests/test_clsvof_oracle.py.
 *
 * Arrays (column-major): (nx,ny) phi, vofS, dx, dy, x, y, temls;
 * (nx+2,ny+2) aE, aW, aN, aS = E/W/N/SEdge_Area(0:nx+1,0:ny+1);
 * ue(0:nx,1:ny) as (nx+1,ny); ve(1:nx,0:ny) as (nx,ny+1).
 */
#include <stddef.h>

#define C1(a, i, j) (a)[(size_t)((i) - 1) + (size_t)((j) - 1) * (size_t)nx]
#define E0(a, i, j) (a)[(size_t)(i) + (size_t)(j) * (size_t)(nx + 2)]
#define UE(i, j) ue[(size_t)(i) + (size_t)((j) - 1) * (size_t)(nx + 1)]
#define VE(i, j) ve[(size_t)((i) - 1) + (size_t)(j) * (size_t)nx]
#define T(i, j) C1(temls, i, j)
#define PHI(i, j) C1(phi, i, j)

/* dir 0: X_Sweep, 1: Y_Sweep */
void oracle_ls_sweep(int dir, int nx, int ny, const double *phi, const double *vofS,
                     const double *dx, const double *dy, const double *x, const double *y,
                     const double *aE, const double *aW, const double *aN, const double *aS,
                     const double *ue, const double *ve, double dtv, double *temls) {
  double l, flux;
  if (dir == 0) {
    for (int j = 1; j <= ny; ++j)
      for (int i = 2; i <= nx - 1; ++i) {
        if (UE(i, j) >= 0.0) l = (PHI(i + 1, j) + PHI(i - 1, j)) / 2.0;
        else if (i <= nx - 2) l = (PHI(i + 2, j) + PHI(i, j)) / 2.0;
        else l = (PHI(i + 1, j) + PHI(i - 1, j)) / 2.0;
        flux = UE(i, j) * l * dtv;
        T(i, j) = T(i, j) - flux * E0(aE, i, j) / C1(dx, i, j);
        T(i + 1, j) = T(i + 1, j) * (1.0 - C1(vofS, i + 1, j)) +
                      flux * E0(aW, i + 1, j) / C1(dx, i + 1, j);
      }
    for (int j = 1; j <= ny; ++j) {
      if (UE(1, j) >= 0.0)
        l = PHI(1, j) + C1(dx, 1, j) / 2.0 * (1.0 - UE(1, j) * dtv / C1(dx, 1, j)) *
                            (PHI(2, j) - PHI(1, j)) / (C1(x, 2, j) - C1(x, 1, j));
      else
        l = PHI(2, j) - C1(dx, 2, j) / 2.0 * (1.0 + UE(1, j) * dtv / C1(dx, 2, j)) *
                            (PHI(3, j) - PHI(1, j)) / (2.0 * C1(dx, 2, j));
      flux = l * UE(1, j) * dtv;
      T(1, j) = T(1, j) - flux * E0(aE, 1, j) / C1(dx, 1, j);
      T(2, j) = T(2, j) + flux * E0(aE, 1, j) / C1(dx, 2, j);
      T(1, j) = T(1, j) + PHI(1, j) * UE(0, j) * dtv * E0(aW, 1, j) / C1(dx, 1, j);
      if (UE(nx, j) > 0.0)
        l = PHI(nx, j) + C1(dx, nx, j) / 2.0 * (1.0 - UE(nx, j) * dtv / C1(dx, nx, j)) *
                             (PHI(nx, j) - PHI(nx - 1, j)) / (C1(x, nx, j) - C1(x, nx - 1, j));
      else
        l = PHI(nx, j) - C1(dx, nx - 1, j) / 2.0 * (1.0 + UE(nx, j) * dtv / C1(dx, nx - 1, j)) *
                             (PHI(nx, j) - PHI(nx - 1, j)) / (C1(x, nx, j) - C1(x, nx - 1, j));
      flux = l * UE(nx, j) * dtv;
      T(nx, j) = T(nx, j) - flux * E0(aE, nx, j) / C1(dx, nx, j);
    }
  } else {
    for (int j = 2; j <= ny - 1; ++j)
      for (int i = 1; i <= nx; ++i) {
        if (VE(i, j) >= 0.0) l = (PHI(i, j + 1) + PHI(i, j - 1)) / 2.0;
        else if (j <= ny - 2) l = (PHI(i, j + 2) + PHI(i, j)) / 2.0;
        else l = (PHI(i, j + 1) + PHI(i, j - 1)) / 2.0;
        flux = l * VE(i, j) * dtv;
        T(i, j) = T(i, j) - flux * E0(aN, i, j) / C1(dy, i, j);
        T(i, j + 1) = T(i, j + 1) * (1.0 - C1(vofS, i, j + 1)) +
                      flux * E0(aS, i, j + 1) / C1(dy, i, j + 1);
      }
    for (int i = 1; i <= nx; ++i) {
      if (VE(i, 1) >= 0.0)
        l = PHI(i, 1) + C1(dy, i, 1) / 2.0 * (1.0 - VE(i, 1) * dtv / C1(dy, i, 1)) *
                            (PHI(i, 2) - PHI(i, 1)) / (C1(y, i, 2) - C1(y, i, 1));
      else
        l = PHI(i, 2) - C1(dy, i, 2) / 2.0 * (1.0 + VE(i, 1) * dtv / C1(dy, i, 2)) *
                            (PHI(i, 3) - PHI(i, 1)) / (C1(y, i, 3) - C1(y, i, 1));
      flux = l * VE(i, 1) * dtv;
      T(i, 1) = T(i, 1) - flux * E0(aN, i, 1) / C1(dy, i, 1);
      T(i, 2) = T(i, 2) + flux * E0(aN, i, 1) / C1(dy, i, 2);
      T(i, 1) = T(i, 1) + PHI(i, 1) * VE(i, 0) * dtv * E0(aS, i, 1) / C1(dy, i, 1);
      if (VE(i, ny) > 0.0)
        l = PHI(i, ny) + C1(dy, i, ny) / 2.0 * (1.0 - VE(i, ny) * dtv / C1(dy, i, ny)) *
                             (PHI(i, ny) - PHI(i, ny - 1)) / (C1(y, i, ny) - C1(y, i, ny - 1));
      else
        l = PHI(i, ny) - C1(dy, i, ny - 1) / 2.0 * (1.0 + VE(i, ny) * dtv / C1(dy, i, ny - 1)) *
                             (PHI(i, ny) - PHI(i, ny - 1)) / (C1(y, i, ny) - C1(y, i, ny - 1));
      flux = l * VE(i, ny) * dtv;
      T(i, ny) = T(i, ny) - flux / C1(dy, i, ny);
    }
  }
}
