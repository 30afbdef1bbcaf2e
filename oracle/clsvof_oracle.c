/*
 * clsvof_oracle.c -- CPU restatement of SIMCOFlow's CLSVOF sweeps after
 * Interface_Reconstruct: the level-set part of X_Sweep
 * (src/Clsvof_Mod.f90:1074-1123) and Y_Sweep (:1191-1244), and their VOF
 * part (:1004-1069, :1141-1189) with the face-flux routines topflux,
 * bottomflux, rightflux, leftflux (:1416-1522), frac (:1371-1404) and
 * CellGeoCal (:2159-2253), as the reference's sequential loops over faces,
 * statement by statement (IEEE FP64, built with -ffp-contract=off).
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
#include <math.h>
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

/* ------------------------------------------------------------------------
 * VOF part of the sweeps.
 * Module constants: vofeps = 1e-14, TolDeno = 1e-24 (src/Clsvof_Mod.f90:10),
 * epsi = 1e-3 (src/StateVariables.f90:28).
 * ---------------------------------------------------------------------- */
static const double VOFEPS = 1e-14, TOLDENO = 1e-24, EPSI = 1e-3;

/* frac (src/Clsvof_Mod.f90:1371-1404): the part of a dx x dy cell where
 * |nx| x + |ny| y + diss <= 0 (origin at the centre). */
double oracle_frac(double nx, double ny, double diss, double dx, double dy) {
  const double slop_eps = 1e-20;
  double tnx = fabs(nx), tny = fabs(ny), xx, yy, totalarea, topvf, rightvf;
  if (diss + 0.5 * (tnx * dx + tny * dy) <= 0.0) return 1.0;
  if (diss - 0.5 * (tnx * dx + tny * dy) >= 0.0) return 0.0;
  if (tnx <= slop_eps) return 0.5 - diss / dy;
  if (tny <= slop_eps) return 0.5 - diss / dx;
  xx = (0.5 * tny * dy - diss) / dx / tnx + 0.5;
  yy = (0.5 * tnx * dx - diss) / dy / tny + 0.5;
  totalarea = 0.5 * xx * yy;
  topvf = 0.0;
  if (yy > 1.0) topvf = ((yy - 1.0) / yy) * ((yy - 1.0) / yy);
  rightvf = 0.0;
  if (xx > 1.0) rightvf = ((xx - 1.0) / xx) * ((xx - 1.0) / xx);
  return totalarea * (1.0 - topvf - rightvf);
}

/* CellGeoCal (src/Clsvof_Mod.f90:2159-2253): solid fraction vols (the cell
 * outside nxs x + nys y + phis >= 0) and the liquid part volf of the rest
 * (nxl x + nyl y + phil <= 0), by the shoelace formula over the clipped
 * polygons.  The polygon arrays are larger than the reference's (6 and 7
 * vertices), which near-collinear rounding can overrun there. */
void oracle_cellgeocal(double nxs, double nys, double phis, double nxl, double nyl, double phil,
                       double dx, double dy, double *vols, double *volf) {
  double node[16][2] = {{0.0}}, nodel[16][2] = {{0.0}}, pdt[16], dpt[4], vol;
  double dx2 = dx / 2.0, dy2 = dy / 2.0;
  int temp = 0, templ = 0; /* 0-based counts */
  dpt[0] = dx2 * nxs - dy2 * nys + phis;
  dpt[1] = -(dx2 * nxs) - dy2 * nys + phis;
  dpt[2] = -(dx2 * nxs) + dy2 * nys + phis;
  dpt[3] = dx2 * nxs + dy2 * nys + phis;
  if (dpt[0] >= 0.0) { node[temp][0] = dx2; node[temp][1] = -dy2; ++temp; }
  if (dpt[0] * dpt[1] < 0.0) { node[temp][0] = (dy2 * nys - phis) / nxs; node[temp][1] = -dy2; ++temp; }
  if (dpt[1] >= 0.0) { node[temp][0] = -dx2; node[temp][1] = -dy2; ++temp; }
  if (dpt[1] * dpt[2] < 0.0) { node[temp][0] = -dx2; node[temp][1] = (dx2 * nxs - phis) / nys; ++temp; }
  if (dpt[2] >= 0.0) { node[temp][0] = -dx2; node[temp][1] = dy2; ++temp; }
  if (dpt[2] * dpt[3] < 0.0) { node[temp][0] = (-(dy2 * nys) - phis) / nxs; node[temp][1] = dy2; ++temp; }
  if (dpt[3] >= 0.0) { node[temp][0] = dx2; node[temp][1] = dy2; ++temp; }
  if (dpt[3] * dpt[0] < 0.0) { node[temp][0] = dx2; node[temp][1] = (-(dx2 * nxs) - phis) / nys; ++temp; }
  node[temp][0] = node[0][0];
  node[temp][1] = node[0][1];
  vol = 0.0;
  for (int k = 0; k < temp; ++k) {
    vol = vol + 0.5 * (node[k][0] * node[k + 1][1] - node[k + 1][0] * node[k][1]);
    pdt[k] = node[k][0] * nxl + node[k][1] * nyl + phil;
  }
  *vols = 1.0 - fabs(vol / (dx * dy));
  pdt[temp] = pdt[0];
  for (int k = 0; k < temp; ++k) {
    if (pdt[k] <= 0.0) { nodel[templ][0] = node[k][0]; nodel[templ][1] = node[k][1]; ++templ; }
    if (pdt[k] * pdt[k + 1] < 0.0) {
      nodel[templ][0] = node[k][0] + (node[k + 1][0] - node[k][0]) * fabs(pdt[k]) /
                                         (fabs(pdt[k]) + fabs(pdt[k + 1]));
      nodel[templ][1] = node[k][1] + (node[k + 1][1] - node[k][1]) * fabs(pdt[k]) /
                                         (fabs(pdt[k]) + fabs(pdt[k + 1]));
      ++templ;
    }
  }
  nodel[templ][0] = nodel[0][0];
  nodel[templ][1] = nodel[0][1];
  vol = 0.0;
  for (int k = 0; k < templ; ++k)
    vol = vol + 0.5 * (nodel[k][0] * nodel[k + 1][1] - nodel[k + 1][0] * nodel[k][1]);
  *volf = fabs(vol / (dx * dy));
}

/* topflux (:1416-1441) */
static double topflux(double nxx, double nyy, double diss, double volf, double nxss, double nyss,
                      double phiss, double vols, double dx, double dy, double vdt) {
  const double eps = 1e-14;
  double flux, volss;
  if (vdt == 0.0) return 0.0;
  if (vols < EPSI) {
    flux = oracle_frac(nxx, nyy, diss - 0.5 * (vdt - dy) * nyy, dx, vdt);
  } else if (vols >= 1.0 - EPSI) {
    return volf;
  } else {
    oracle_cellgeocal(nxss, nyss, phiss - 0.5 * (vdt - dy) * nyss, nxx, nyy,
                      diss - 0.5 * (vdt - dy) * nyy, dx, vdt, &volss, &flux);
    if (volf / (1.0 - vols) >= 1.0 - VOFEPS) flux = 1.0 - volss;
    flux = flux / (1.0 - volss + TOLDENO);
    if (volf + vols > 1.0 - eps) flux = 1.0;
  }
  return flux * vdt;
}

/* bottomflux (:1444-1468) */
static double bottomflux(double nxx, double nyy, double diss, double volf, double nxss,
                         double nyss, double phiss, double vols, double dx, double dy, double vdt) {
  const double eps = 1e-14;
  double flux, volss;
  if (vdt == 0.0) return 0.0;
  if (vols < EPSI) {
    flux = oracle_frac(nxx, nyy, diss + 0.5 * (vdt - dy) * nyy, dx, vdt);
  } else if (vols >= 1.0 - EPSI) {
    return volf;
  } else {
    oracle_cellgeocal(nxss, nyss, phiss + 0.5 * (vdt - dy) * nyss, nxx, nyy,
                      diss + 0.5 * (vdt - dy) * nyy, dx, vdt, &volss, &flux);
    if (volf / (1.0 - vols) >= 1.0 - VOFEPS) flux = 1.0 - volss;
    flux = flux / (1.0 - volss + TOLDENO);
    if (volf + vols > 1.0 - eps) flux = 1.0;
  }
  return flux * vdt;
}

/* rightflux (:1471-1495) */
static double rightflux(double nxx, double nyy, double diss, double volf, double nxss,
                        double nyss, double phiss, double vols, double dx, double dy, double udt) {
  const double eps = 1e-14;
  double flux, volss;
  if (udt == 0.0) return 0.0;
  if (vols < EPSI) {
    flux = oracle_frac(nxx, nyy, diss - 0.5 * (udt - dx) * nxx, udt, dy);
  } else if (vols >= 1.0 - EPSI) {
    return volf;
  } else {
    oracle_cellgeocal(nxss, nyss, phiss - 0.5 * (udt - dx) * nxss, nxx, nyy,
                      diss - 0.5 * (udt - dx) * nxx, udt, dy, &volss, &flux);
    if (volf / (1.0 - vols) >= 1.0 - VOFEPS) flux = 1.0 - volss;
    flux = flux / (1.0 - volss + TOLDENO);
    if (volf + vols > 1.0 - eps) flux = 1.0;
  }
  return flux * udt;
}

/* leftflux (:1498-1522) */
static double leftflux(double nxx, double nyy, double diss, double volf, double nxss,
                       double nyss, double phiss, double vols, double dx, double dy, double udt) {
  const double eps = 1e-14;
  double flux, volss;
  if (udt == 0.0) return 0.0;
  if (vols < EPSI) {
    flux = oracle_frac(nxx, nyy, diss + 0.5 * (udt - dx) * nxx, udt, dy);
  } else if (vols >= 1.0 - EPSI) {
    return volf;
  } else {
    oracle_cellgeocal(nxss, nyss, phiss + 0.5 * (udt - dx) * nxss, nxx, nyy,
                      diss + 0.5 * (udt - dx) * nxx, udt, dy, &volss, &flux);
    if (volf / (1.0 - vols) >= 1.0 - VOFEPS) flux = 1.0 - volss;
    flux = flux / (1.0 - volss + TOLDENO);
    if (volf + vols > 1.0 - eps) flux = 1.0;
  }
  return flux * udt;
}

/* The VOF part of X_Sweep (dir 0, src/Clsvof_Mod.f90:1004-1069) or Y_Sweep
 * (dir 1, :1141-1189) on temvf, after Interface_Reconstruct has produced
 * (nxv, nyv, dis).  vfl is PCell%vof; the solid fraction vflS is PCell%vofS.
 * wave = {Amp0, kw, omew, Depthw, NondiT, k} of X_Sweep's inlet (NULL: no
 * inlet flux). */
void oracle_vof_sweep(int dir, int nx, int ny, const double *vofS, const double *dx,
                      const double *dy, const double *x, const double *y, const double *aE,
                      const double *aW, const double *aN, const double *aS, const double *ue,
                      const double *ve, const double *vfl, const double *nxv, const double *nyv,
                      const double *dis, const double *nxs, const double *nys, const double *phiS,
                      const double *wave, double dtv, double *temvf) {
#define V(a, i, j) C1(a, i, j)
#define TV(i, j) C1(temvf, i, j)
  double flux;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i)
      if (V(vofS, i, j) < 1.0 - VOFEPS) TV(i, j) = TV(i, j) / (1.0 - V(vofS, i, j));
  if (dir == 0) {
    const double xwu = V(x, 1, 1) - V(dx, 1, 1) / 2.0;
    for (int j = 1; j <= ny; ++j) {
      for (int i = 1; i <= nx; ++i) {
        if (UE(i, j) >= 0.0) {
          if (V(vfl, i, j) >= 1.0 - VOFEPS || V(vfl, i, j) <= VOFEPS) {
            flux = V(vfl, i, j) * UE(i, j) * dtv;
            if (V(vfl, i, j) >= 1.0) flux = UE(i, j) * dtv;
            if (V(vfl, i, j) < 0.0) flux = 0.0;
          } else {
            flux = rightflux(V(nxv, i, j), V(nyv, i, j), V(dis, i, j), V(vfl, i, j), V(nxs, i, j),
                             V(nys, i, j), V(phiS, i, j), V(vofS, i, j), V(dx, i, j), V(dy, i, j),
                             UE(i, j) * dtv);
          }
          if (E0(aE, i, j) > 1.0 - VOFEPS && V(vofS, i, j) > 1.0 - VOFEPS)
            flux = 1.0 * UE(i, j) * dtv;
        } else {
          if (i < nx) {
            if (V(vfl, i + 1, j) >= 1.0 - VOFEPS || V(vfl, i + 1, j) <= VOFEPS) {
              flux = V(vfl, i + 1, j) * UE(i, j) * dtv;
              if (V(vfl, i + 1, j) >= 1.0) flux = UE(i, j) * dtv;
              if (V(vfl, i + 1, j) < 0.0) flux = 0.0;
            } else {
              flux = leftflux(V(nxv, i + 1, j), V(nyv, i + 1, j), V(dis, i + 1, j),
                              V(vfl, i + 1, j), V(nxs, i + 1, j), V(nys, i + 1, j),
                              V(phiS, i + 1, j), V(vofS, i + 1, j), V(dx, i + 1, j),
                              V(dy, i + 1, j), -UE(i, j) * dtv);
              flux = -flux;
            }
            if (E0(aW, i + 1, j) > 1.0 - VOFEPS && V(vofS, i + 1, j) > 1.0 - VOFEPS)
              flux = 1.0 * UE(i, j) * dtv;
          } else {
            flux = V(vfl, i, j) * UE(i, j) * dtv;
          }
        }
        TV(i, j) = TV(i, j) - flux * E0(aE, i, j) / V(dx, i, j);
        if (i <= nx - 1)
          TV(i + 1, j) = TV(i + 1, j) * (1.0 - V(vofS, i + 1, j)) +
                         flux * E0(aW, i + 1, j) / V(dx, i + 1, j);
      }
      if (wave) {
        const double etau = wave[0] * sin(wave[1] * xwu - wave[2] * (wave[4] + wave[5] * dtv));
        if (V(y, 1, j) - V(dy, 1, j) / 2.0 < wave[3] + etau) flux = V(vfl, 1, j) * UE(0, j) * dtv;
        else flux = 0.0;
      } else {
        flux = 0.0;
      }
      TV(1, j) = TV(1, j) + flux * E0(aW, 1, j) / V(dx, 1, j);
    }
  } else {
    for (int i = 1; i <= nx; ++i) {
      for (int j = 1; j <= ny; ++j) {
        if (VE(i, j) > 0.0) {
          if (V(vfl, i, j) >= 1.0 - VOFEPS || V(vfl, i, j) <= VOFEPS) {
            flux = V(vfl, i, j) * VE(i, j) * dtv;
            if (V(vfl, i, j) >= 1.0) flux = VE(i, j) * dtv;
            if (V(vfl, i, j) < 0.0) flux = 0.0;
          } else {
            flux = topflux(V(nxv, i, j), V(nyv, i, j), V(dis, i, j), V(vfl, i, j), V(nxs, i, j),
                           V(nys, i, j), V(phiS, i, j), V(vofS, i, j), V(dx, i, j), V(dy, i, j),
                           VE(i, j) * dtv);
          }
          if (E0(aN, i, j) > 1.0 - VOFEPS && V(vofS, i, j) > 1.0 - VOFEPS)
            flux = 1.0 * VE(i, j) * dtv;
        } else {
          if (j < ny) {
            if (V(vfl, i, j + 1) >= 1.0 - VOFEPS || V(vfl, i, j + 1) <= VOFEPS) {
              flux = V(vfl, i, j + 1) * VE(i, j) * dtv;
              if (V(vfl, i, j + 1) >= 1.0) flux = VE(i, j) * dtv;
              if (V(vfl, i, j + 1) < 0.0) flux = 0.0;
            } else {
              flux = bottomflux(V(nxv, i, j + 1), V(nyv, i, j + 1), V(dis, i, j + 1),
                                V(vfl, i, j + 1), V(nxs, i, j + 1), V(nys, i, j + 1),
                                V(phiS, i, j + 1), V(vofS, i, j + 1), V(dx, i, j + 1),
                                V(dy, i, j + 1), -VE(i, j) * dtv);
              flux = -flux;
            }
            if (E0(aS, i, j + 1) > 1.0 - VOFEPS && V(vofS, i, j + 1) > 1.0 - VOFEPS)
              flux = 1.0 * VE(i, j) * dtv;
          } else {
            flux = V(vfl, i, j) * VE(i, j) * dtv;
          }
        }
        TV(i, j) = TV(i, j) - flux * E0(aN, i, j) / V(dy, i, j);
        if (j <= ny - 1)
          TV(i, j + 1) = TV(i, j + 1) * (1.0 - V(vofS, i, j + 1)) +
                         flux * E0(aS, i, j + 1) / V(dy, i, j + 1);
      }
      TV(i, 1) = TV(i, 1) + V(vfl, i, 1) * VE(i, 0) * dtv * E0(aS, i, 1) / V(dy, i, 1);
    }
  }
#undef V
#undef TV
}

/* ------------------------------------------------------------------------
 * Interface_Reconstruct (src/Clsvof_Mod.f90:1250-1321) with
 * Normal_Vector_Irre (:1710-1919), distance (:1323-1369),
 * DistanceFluidCalculate (:1957-2042), zriddr (:2044-2105) and LiqFuncVol
 * (:2107-2155), as the reference's loop over cells (i outer, j inner).
 *
 * The loop's locals nxx, nyy and diss keep their values from one cell to
 * the next: a flagged cell of column 1 or nx (rows 2..ny-1) takes nyy from
 * the cell before it, one of row 1 or ny (columns 2..nx-1) takes nxx, and a
 * three-phase cell whose Ridders bracket fails keeps diss.  Restated as
 * written, with 0 for their values before the first cell.
 * Where the reference pauses for the operator ('pause'), reads outside an
 * array or uses a value never set, this restatement goes on as after the
 * operator's "go" (or with the documented value) and counts the event in
 * *events.
 * Vset is the direction table as Coupled_LS_VOF leaves it (:746-753): its
 * line 747 sets Vset(1,2) = 1 again instead of Vset(2,2), so Vset(1,:) =
 * (0, 1) and Vset(2,:) = (0, 0) (module storage, zero at start).
 * ---------------------------------------------------------------------- */
static const double VSET[8][2] = {{0, 1}, {0, 0}, {-1, 0}, {-1, -1}, {-1, 1}, {1, 0}, {1, -1}, {1, 1}};

typedef struct {
  int nx, ny;
  const double *vfl, *vfls, *phi, *x, *y;
  int *events;
} IrCtx;

#define IRC1(a, i, j) (a)[(size_t)((i) - 1) + (size_t)((j) - 1) * (size_t)c->nx]

/* The direction of Vset most parallel to (vx, vy), then the one-sided pair
 * whose gradient is closer to unit length (:1768-1832 and :1860-1912). */
static void most_parallel(const IrCtx *c, int i, int j, int imv0, double *nxo, double *nyo) {
  const double *phi = c->phi, *x = c->x, *y = c->y;
  const double nuy = 0.075 / 8.0;
  double vx = (IRC1(phi, i + 1, j) - IRC1(phi, i - 1, j)) / (IRC1(x, i + 1, j) - IRC1(x, i - 1, j));
  double vy = (IRC1(phi, i, j + 1) - IRC1(phi, i, j - 1)) / (IRC1(y, i, j + 1) - IRC1(y, i, j - 1));
  double maxv = 0.0, vx1, vx2, vy1, vy2, qv1, qv2;
  int imv = imv0;
  for (int ii = 1; ii <= 8; ++ii) {
    const double a = VSET[ii - 1][0], b = VSET[ii - 1][1];
    const double cp = fabs(a * vx + b * vy) / (sqrt(a * a + b * b) * sqrt(vx * vx + vy * vy));
    if (cp >= maxv) {
      maxv = cp;
      imv = ii;
    }
  }
  if (imv == 0) { /* the reference reads Vset(0,:) outside the table */
    ++*c->events;
    imv = 1;
  }
  const double v11 = -VSET[imv - 1][1], v12 = VSET[imv - 1][0];
  if (v11 == -1) {
    vx1 = (IRC1(phi, i, j) - IRC1(phi, i - 1, j)) / (IRC1(x, i, j) - IRC1(x, i - 1, j));
    vx2 = (IRC1(phi, i + 1, j) - IRC1(phi, i, j)) / (IRC1(x, i + 1, j) - IRC1(x, i, j));
  } else if (v11 == 0) {
    vx1 = (IRC1(phi, i + 1, j) - IRC1(phi, i - 1, j)) / (IRC1(x, i + 1, j) - IRC1(x, i - 1, j));
    vx2 = vx1;
  } else {
    vx1 = (IRC1(phi, i + 1, j) - IRC1(phi, i, j)) / (IRC1(x, i + 1, j) - IRC1(x, i, j));
    vx2 = (IRC1(phi, i, j) - IRC1(phi, i - 1, j)) / (IRC1(x, i, j) - IRC1(x, i - 1, j));
  }
  if (v12 == -1) {
    vy1 = (IRC1(phi, i, j) - IRC1(phi, i, j - 1)) / (IRC1(y, i, j) - IRC1(y, i, j - 1));
    vy2 = (IRC1(phi, i, j + 1) - IRC1(phi, i, j)) / (IRC1(y, i, j + 1) - IRC1(y, i, j));
  } else if (v12 == 0) {
    vy1 = (IRC1(phi, i, j + 1) - IRC1(phi, i, j - 1)) / (IRC1(y, i, j + 1) - IRC1(y, i, j - 1));
    vy2 = vy1;
  } else {
    vy1 = (IRC1(phi, i, j + 1) - IRC1(phi, i, j)) / (IRC1(y, i, j + 1) - IRC1(y, i, j));
    vy2 = (IRC1(phi, i, j) - IRC1(phi, i, j - 1)) / (IRC1(y, i, j) - IRC1(y, i, j - 1));
  }
  qv1 = fabs(1.0 - sqrt(vx1 * vx1 + vy1 * vy1));
  qv2 = fabs(1.0 - sqrt(vx2 * vx2 + vy2 * vy2));
  if (qv1 < qv2 + nuy) {
    *nxo = vx1;
    *nyo = vy1;
  } else {
    *nxo = vx2;
    *nyo = vy2;
  }
}

/* Normal_Vector_Irre (:1710-1919) for 1 < i < nx, 1 < j < ny. */
static void normal_irre(const IrCtx *c, int i, int j, double *nxo, double *nyo) {
  const double *phi = c->phi, *x = c->x, *y = c->y, *vfls = c->vfls;
  const double eta = 0.075;
  const int nx = c->nx, ny = c->ny;
  double vx, vy, q[3];
  int dx, dy;
  if (IRC1(vfls, i, j) >= EPSI) {
    if (IRC1(vfls, i + 1, j) < 1.0 - EPSI && IRC1(vfls, i - 1, j) < 1.0 - EPSI)
      *nxo = (IRC1(phi, i + 1, j) - IRC1(phi, i - 1, j)) / (IRC1(x, i + 1, j) - IRC1(x, i - 1, j));
    else if (IRC1(vfls, i + 1, j) >= 1.0 - EPSI)
      *nxo = (IRC1(phi, i, j) - IRC1(phi, i - 1, j)) / (IRC1(x, i, j) - IRC1(x, i - 1, j));
    else
      *nxo = (IRC1(phi, i + 1, j) - IRC1(phi, i, j)) / (IRC1(x, i + 1, j) - IRC1(x, i, j));
    if (IRC1(vfls, i, j + 1) < 1.0 - EPSI && IRC1(vfls, i, j - 1) < 1.0 - EPSI)
      *nyo = (IRC1(phi, i, j + 1) - IRC1(phi, i, j - 1)) / (IRC1(y, i, j + 1) - IRC1(y, i, j - 1));
    else if (IRC1(vfls, i, j + 1) > 1.0 - EPSI)
      *nyo = (IRC1(phi, i, j) - IRC1(phi, i, j - 1)) / (IRC1(y, i, j) - IRC1(y, i, j - 1));
    else
      *nyo = (IRC1(phi, i, j + 1) - IRC1(phi, i, j)) / (IRC1(y, i, j + 1) - IRC1(y, i, j));
    return;
  }
  if (i >= 3) vx = (IRC1(phi, i, j) - IRC1(phi, i - 2, j)) / (IRC1(x, i, j) - IRC1(x, i - 2, j));
  else vx = (IRC1(phi, i, j) - IRC1(phi, i - 1, j)) / (IRC1(x, i, j) - IRC1(x, i - 1, j));
  vy = (IRC1(phi, i - 1, j + 1) - IRC1(phi, i - 1, j - 1)) /
       (IRC1(y, i - 1, j + 1) - IRC1(y, i - 1, j - 1));
  q[0] = fabs(1.0 - sqrt(vx * vx + vy * vy));
  vx = (IRC1(phi, i + 1, j) - IRC1(phi, i - 1, j)) / (IRC1(x, i + 1, j) - IRC1(x, i - 1, j));
  vy = (IRC1(phi, i, j + 1) - IRC1(phi, i, j - 1)) / (IRC1(y, i, j + 1) - IRC1(y, i, j - 1));
  q[1] = fabs(1.0 - sqrt(vx * vx + vy * vy));
  if (i <= nx - 2) vx = (IRC1(phi, i + 2, j) - IRC1(phi, i, j)) / (IRC1(x, i + 2, j) - IRC1(x, i, j));
  else vx = (IRC1(phi, i + 1, j) - IRC1(phi, i, j)) / (IRC1(x, i + 1, j) - IRC1(x, i, j));
  vy = (IRC1(phi, i + 1, j + 1) - IRC1(phi, i + 1, j - 1)) /
       (IRC1(y, i + 1, j + 1) - IRC1(y, i + 1, j - 1));
  q[2] = fabs(1.0 - sqrt(vx * vx + vy * vy));
  if (q[0] < eta && q[2] >= eta) dx = -1;
  else if (q[0] >= eta && q[2] < eta) dx = 1;
  else if (q[0] < eta && q[1] < eta && q[2] < eta) dx = 0;
  else if (q[0] >= eta && q[1] >= eta && q[2] >= eta) dx = 0;
  else {
    most_parallel(c, i, j, 0, nxo, nyo);
    return;
  }
  if (j >= 3) vy = (IRC1(phi, i, j) - IRC1(phi, i, j - 2)) / (IRC1(y, i, j) - IRC1(y, i, j - 2));
  else vy = (IRC1(phi, i, j) - IRC1(phi, i, j - 1)) / (IRC1(y, i, j) - IRC1(y, i, j - 1));
  vx = (IRC1(phi, i + 1, j - 1) - IRC1(phi, i - 1, j - 1)) /
       (IRC1(x, i + 1, j - 1) - IRC1(x, i - 1, j - 1));
  q[0] = fabs(1.0 - sqrt(vx * vx + vy * vy));
  vx = (IRC1(phi, i + 1, j) - IRC1(phi, i - 1, j)) / (IRC1(x, i + 1, j) - IRC1(x, i - 1, j));
  vy = (IRC1(phi, i, j + 1) - IRC1(phi, i, j - 1)) / (IRC1(y, i, j + 1) - IRC1(y, i, j - 1));
  q[1] = fabs(1.0 - sqrt(vx * vx + vy * vy));
  vx = (IRC1(phi, i + 1, j + 1) - IRC1(phi, i - 1, j + 1)) /
       (IRC1(x, i + 1, j + 1) - IRC1(x, i - 1, j + 1));
  if (j <= ny - 2) vy = (IRC1(phi, i, j + 2) - IRC1(phi, i, j)) / (IRC1(y, i, j + 2) - IRC1(y, i, j));
  else vy = (IRC1(phi, i, j + 1) - IRC1(phi, i, j)) / (IRC1(y, i, j + 1) - IRC1(y, i, j));
  q[2] = fabs(1.0 - sqrt(vx * vx + vy * vy));
  if (q[0] < eta && q[2] >= eta) dy = -1;
  else if (q[0] >= eta && q[2] < eta) dy = 1;
  else if (q[0] < eta && q[1] < eta && q[2] < eta) dy = 0;
  else if (q[0] >= eta && q[1] >= eta && q[2] >= eta) dy = 0;
  else {
    most_parallel(c, i, j, 1, nxo, nyo);
    return;
  }
  if (dx == -1) *nxo = (IRC1(phi, i, j) - IRC1(phi, i - 1, j)) / (IRC1(x, i, j) - IRC1(x, i - 1, j));
  if (dx == 1) *nxo = (IRC1(phi, i + 1, j) - IRC1(phi, i, j)) / (IRC1(x, i + 1, j) - IRC1(x, i, j));
  if (dx == 0)
    *nxo = (IRC1(phi, i + 1, j) - IRC1(phi, i - 1, j)) / (IRC1(x, i + 1, j) - IRC1(x, i - 1, j));
  if (dy == -1) *nyo = (IRC1(phi, i, j) - IRC1(phi, i, j - 1)) / (IRC1(y, i, j) - IRC1(y, i, j - 1));
  if (dy == 1) *nyo = (IRC1(phi, i, j + 1) - IRC1(phi, i, j)) / (IRC1(y, i, j + 1) - IRC1(y, i, j));
  if (dy == 0)
    *nyo = (IRC1(phi, i, j + 1) - IRC1(phi, i, j - 1)) / (IRC1(y, i, j + 1) - IRC1(y, i, j - 1));
}

/* distance (:1323-1369): the PLIC line distance of a two-phase cell. */
double oracle_plic_distance(double v, double dx, double dy, double nxx, double nyy) {
  const double slop_eps = 1e-20, equal_eps = 1e-20;
  double nx = fabs(nxx), ny = fabs(nyy), dll, dul, dlr, dur, vful, vflr, t;
  if (nx < slop_eps) return (0.5 - v) * dy;
  if (ny < slop_eps) return (0.5 - v) * dx;
  dll = 0.5 * (nx * dx + ny * dy);
  dul = 0.5 * (nx * dx - ny * dy);
  dlr = -dul;
  dur = -dll;
  vful = oracle_frac(nx, ny, dul, dx, dy);
  vflr = oracle_frac(nx, ny, dlr, dx, dy);
  if (v <= vful && v <= vflr) {
    if (vful > vflr) {
      t = vful; vful = vflr; vflr = t;
      t = dul; dul = dlr; dlr = t;
    }
    return dll - sqrt(((dul - dll) * (dul - dll)) * v / vful);
  } else if (v >= vful && v >= vflr) {
    if (vflr < vful) {
      t = vful; vful = vflr; vflr = t;
      t = dul; dul = dlr; dlr = t;
    }
    return dur + sqrt((dlr - dur) * (dlr - dur) * (1.0 - v) / (1.0 - vflr));
  }
  if (fabs(vflr - vful) < equal_eps) return 0.5 * (dul + dlr);
  t = (v - vful) / (vflr - vful);
  return dlr * t + dul * (1.0 - t);
}

/* LiqFuncVol (:2107-2155): volf minus the liquid part of the polygon node
 * (closed, zero-padded to 6 entries) below the line through xf. */
static double liq_func_vol(const double node[9][2], double nxf, double nyf, double volf,
                           double dx, double dy, const double *xf, int *events) {
  double pdt[9], nodel[20][2], vol;
  const double phil = -(nxf * xf[0] + nyf * xf[1]);
  int temp = 0, templ = 0;
  for (int k = 1; k <= 6; ++k)
    if (fabs(node[k - 1][0]) > 1e-14 || fabs(node[k - 1][1]) > 1e-14) temp = k;
  for (int k = 1; k <= temp - 1; ++k) pdt[k - 1] = node[k - 1][0] * nxf + node[k - 1][1] * nyf + phil;
  if (temp == 0) { /* the reference pauses and then reads pdt(0) */
    ++*events;
    return volf - 0.0;
  }
  pdt[temp - 1] = pdt[0];
  for (int k = 1; k <= temp - 1; ++k) {
    if (pdt[k - 1] <= 0.0) {
      nodel[templ][0] = node[k - 1][0];
      nodel[templ][1] = node[k - 1][1];
      ++templ;
    }
    if (pdt[k - 1] * pdt[k] < 0.0) {
      nodel[templ][0] = node[k - 1][0] + (node[k][0] - node[k - 1][0]) * fabs(pdt[k - 1]) /
                                             (fabs(pdt[k - 1]) + fabs(pdt[k]));
      nodel[templ][1] = node[k - 1][1] + (node[k][1] - node[k - 1][1]) * fabs(pdt[k - 1]) /
                                             (fabs(pdt[k - 1]) + fabs(pdt[k]));
      ++templ;
    }
  }
  nodel[templ][0] = templ ? nodel[0][0] : 0.0;
  nodel[templ][1] = templ ? nodel[0][1] : 0.0;
  vol = 0.0;
  for (int k = 0; k < templ; ++k)
    vol = vol + 0.5 * (nodel[k][0] * nodel[k + 1][1] - nodel[k + 1][0] * nodel[k][1]);
  return volf - fabs(vol / (dx * dy));
}

/* DistanceFluidCalculate + zriddr (:1957-2105).  Returns 1 and sets *phif
 * when the reference assigns phif, 0 when it leaves it unchanged. */
int oracle_dfc(double nxss, double nyss, double phiss, double nxf, double nyf, double volf,
               double dx, double dy, double *phif, int *events) {
  double node[9][2] = {{0.0}}, dpt[4], maxv[2] = {0.0, 0.0}, minv[2] = {0.0, 0.0};
  const double dx2 = dx / 2.0, dy2 = dy / 2.0, tol = 1e-14, unused = -1.11e-30;
  int temp = 0;
  dpt[0] = dx2 * nxss - dy2 * nyss + phiss;
  dpt[1] = -(dx2 * nxss) - dy2 * nyss + phiss;
  dpt[2] = -(dx2 * nxss) + dy2 * nyss + phiss;
  dpt[3] = dx2 * nxss + dy2 * nyss + phiss;
  if (dpt[0] >= 0.0) { node[temp][0] = dx2; node[temp][1] = -dy2; ++temp; }
  if (dpt[0] * dpt[1] < 0.0) { node[temp][0] = (dy2 * nyss - phiss) / nxss; node[temp][1] = -dy2; ++temp; }
  if (dpt[1] >= 0.0) { node[temp][0] = -dx2; node[temp][1] = -dy2; ++temp; }
  if (dpt[1] * dpt[2] < 0.0) { node[temp][0] = -dx2; node[temp][1] = (dx2 * nxss - phiss) / nyss; ++temp; }
  if (dpt[2] >= 0.0) { node[temp][0] = -dx2; node[temp][1] = dy2; ++temp; }
  if (dpt[2] * dpt[3] < 0.0) { node[temp][0] = (-(dy2 * nyss) - phiss) / nxss; node[temp][1] = dy2; ++temp; }
  if (dpt[3] >= 0.0) { node[temp][0] = dx2; node[temp][1] = dy2; ++temp; }
  if (dpt[3] * dpt[0] < 0.0) { node[temp][0] = dx2; node[temp][1] = (-(dx2 * nxss) - phiss) / nyss; ++temp; }
  node[temp][0] = node[0][0];
  node[temp][1] = node[0][1];
  {
    double maxdis = -2.0 * sqrt(dx * dx + dy * dy), mindis = 2.0 * sqrt(dx * dx + dy * dy);
    for (int k = 0; k < temp; ++k) {
      const double d23 = nxf * node[k][0] + nyf * node[k][1];
      if (d23 > maxdis) { maxdis = d23; maxv[0] = node[k][0]; maxv[1] = node[k][1]; }
      if (d23 < mindis) { mindis = d23; minv[0] = node[k][0]; minv[1] = node[k][1]; }
    }
  }
  maxv[0] = maxv[0] + maxv[0] * nxf * EPSI;
  maxv[1] = maxv[1] + maxv[1] * nyf * EPSI;
  minv[0] = minv[0] - minv[0] * nxf * EPSI;
  minv[1] = minv[1] - minv[1] * nyf * EPSI;
  if (temp == 0 || (fabs(node[0][0]) < 1e-14 && fabs(node[0][1]) < 1e-14)) ++*events; /* pause */
  /* zriddr(x1 = minv, x2 = maxv) */
  double fl = liq_func_vol(node, nxf, nyf, volf, dx, dy, minv, events);
  double fh = liq_func_vol(node, nxf, nyf, volf, dx, dy, maxv, events);
  if ((fl > tol && fh < -tol) || (fl < -tol && fh > tol)) {
    double xl[2] = {minv[0], minv[1]}, xh[2] = {maxv[0], maxv[1]}, ans[2] = {unused, unused};
    double xm[2], xnew[2], fm, fnew, s;
    for (int iter = 1; iter <= 1000; ++iter) {
      xm[0] = 0.5 * (xl[0] + xh[0]);
      xm[1] = 0.5 * (xl[1] + xh[1]);
      fm = liq_func_vol(node, nxf, nyf, volf, dx, dy, xm, events);
      s = sqrt(fm * fm - fl * fh);
      if (s == 0.0) ++*events; /* pause */
      const double sg = copysign(1.0, fl - fh);
      xnew[0] = xm[0] + (xm[0] - xl[0]) * sg * fm / s;
      xnew[1] = xm[1] + (xm[1] - xl[1]) * sg * fm / s;
      if (sqrt((xnew[0] - ans[0]) * (xnew[0] - ans[0]) + (xnew[1] - ans[1]) * (xnew[1] - ans[1])) <=
          tol) {
        *phif = -(nxf * ans[0] + nyf * ans[1]);
        return 1;
      }
      ans[0] = xnew[0];
      ans[1] = xnew[1];
      fnew = liq_func_vol(node, nxf, nyf, volf, dx, dy, ans, events);
      if (fabs(fnew) <= tol) {
        *phif = -(nxf * ans[0] + nyf * ans[1]);
        return 1;
      }
      if (copysign(fm, fnew) != fm) {
        xl[0] = xm[0]; xl[1] = xm[1]; fl = fm;
        xh[0] = ans[0]; xh[1] = ans[1]; fh = fnew;
      } else if (copysign(fl, fnew) != fl) {
        xh[0] = ans[0]; xh[1] = ans[1]; fh = fnew;
      } else if (copysign(fh, fnew) != fh) {
        xl[0] = ans[0]; xl[1] = ans[1]; fl = fnew;
      } else {
        ++*events; /* pause */
      }
      if (sqrt((xh[0] - xl[0]) * (xh[0] - xl[0]) + (xh[1] - xl[1]) * (xh[1] - xl[1])) <= tol) {
        *phif = -(nxf * ans[0] + nyf * ans[1]);
        return 1;
      }
    }
    *phif = -(nxf * ans[0] + nyf * ans[1]);
    return 1;
  }
  if (fl < tol && fl > -tol) {
    *phif = -(nxf * minv[0] + nyf * minv[1]);
    return 1;
  }
  if (fh < tol && fh > -tol) {
    *phif = -(nxf * maxv[0] + nyf * maxv[1]);
    return 1;
  }
  return 0;
}

/* Interface_Reconstruct (:1250-1321) with UpdateNorVec = 1; nx, ny >= 3.
 * Outputs (nx,ny) nxv, nyv, dis.  Returns the number of events. */
int oracle_interface_reconstruct(int nx, int ny, const double *vfl, const double *vfls,
                                 const double *phi, const double *nxs, const double *nys,
                                 const double *phis, const double *x, const double *y,
                                 const double *dx, const double *dy, double *nxv, double *nyv,
                                 double *dis) {
  int events = 0;
  IrCtx ctx = {nx, ny, vfl, vfls, phi, x, y, &events};
  const IrCtx *c = &ctx;
  double nxx = 0.0, nyy = 0.0, diss = 0.0, temp;
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j) {
      const double v = C1(vfl, i, j), s = C1(vfls, i, j);
      int flag = 0;
      if (v >= VOFEPS && v < (1.0 - VOFEPS - s) && s < EPSI) flag = 1;
      if (v >= VOFEPS && v < (1.0 - VOFEPS - s) && s >= EPSI && s < 1.0 - EPSI) flag = 2;
      if (flag) {
        if (i > 1 && i < nx && j > 1 && j < ny) {
          normal_irre(c, i, j, &nxx, &nyy);
        } else {
          if (i == 1)
            nxx = (IRC1(phi, i + 1, j) - IRC1(phi, i, j)) / (IRC1(x, i + 1, j) - IRC1(x, i, j));
          else if (i == nx)
            nxx = (IRC1(phi, i, j) - IRC1(phi, i - 1, j)) / (IRC1(x, i, j) - IRC1(x, i - 1, j));
          if (j == 1)
            nyy = (IRC1(phi, i, j + 1) - IRC1(phi, i, j)) / (IRC1(y, i, j + 1) - IRC1(y, i, j));
          else if (j == ny)
            nyy = (IRC1(phi, i, j) - IRC1(phi, i, j - 1)) / (IRC1(y, i, j) - IRC1(y, i, j - 1));
        }
        temp = sqrt(nxx * nxx + nyy * nyy);
        if (temp < 1e-14) {
          nxx = 0.0;
          nyy = 1.0;
        } else {
          nxx = nxx / temp;
          nyy = nyy / temp;
        }
        if (flag == 1)
          diss = oracle_plic_distance(v, C1(dx, i, j), C1(dy, i, j), nxx, nyy);
        else
          oracle_dfc(C1(nxs, i, j), C1(nys, i, j), C1(phis, i, j), nxx, nyy, v, C1(dx, i, j),
                     C1(dy, i, j), &diss, &events);
      } else {
        nxx = 0.0;
        nyy = 1.0;
        if (1.0 - s > VOFEPS) diss = (0.5 - v / (1.0 - s)) * C1(dy, i, j);
        else diss = (0.0 - v) * C1(dy, i, j);
      }
      C1(nxv, i, j) = nxx;
      C1(nyv, i, j) = nyy;
      C1(dis, i, j) = diss;
    }
  return events;
}

/* ------------------------------------------------------------------------
 * Redistance (src/Clsvof_Mod.f90:1525-1708) with isinsiderect (:1921-1955):
 * phi rebuilt as the distance to the PLIC interface within band_width = 4
 * cells of every interface cell (module parameter, :9), the rest of phi
 * set to +-5 sqrt(dx^2 + dy^2) outside the band.  The reference's scatter
 * from each interface cell (i outer, j inner) is restated as written.
 * dmin1 / dmax1 are fmin / fmax; the 'pause' checks count events.
 * ---------------------------------------------------------------------- */
static int inside_rect(double xp, double yp, double dx, double dy) {
  const double x1 = -0.5 * dx, y1 = 0.5 * dy, x2 = 0.5 * dx, y2 = 0.5 * dy;
  const double x3 = 0.5 * dx, y3 = -0.5 * dy, x4 = -0.5 * dx, y4 = -0.5 * dy;
  const double b1 = sqrt((x1 - xp) * (x1 - xp) + (y1 - yp) * (y1 - yp));
  const double b2 = sqrt((x2 - xp) * (x2 - xp) + (y2 - yp) * (y2 - yp));
  const double b3 = sqrt((x3 - xp) * (x3 - xp) + (y3 - yp) * (y3 - yp));
  const double b4 = sqrt((x4 - xp) * (x4 - xp) + (y4 - yp) * (y4 - yp));
  const double u1 = 0.5 * (dx + b1 + b2), u2 = 0.5 * (dy + b2 + b3);
  const double u3 = 0.5 * (dx + b3 + b4), u4 = 0.5 * (dy + b4 + b1);
  const double area = dx * dy;
  const double a1 = sqrt(u1 * (u1 - dx) * (u1 - b1) * (u1 - b2));
  const double a2 = sqrt(u2 * (u2 - dy) * (u2 - b2) * (u2 - b3));
  const double a3 = sqrt(u3 * (u3 - dx) * (u3 - b3) * (u3 - b4));
  const double a4 = sqrt(u4 * (u4 - dy) * (u4 - b4) * (u4 - b1));
  const double sum = a1 + a2 + a3 + a4;
  return fabs(sum - area) < 1e-10;
}

int oracle_redistance(int nx, int ny, const double *vfl, const double *vfls, const double *nxs,
                      const double *nys, const double *phis, const double *x, const double *y,
                      const double *dx, const double *dy, const double *nxx1,
                      const double *nyy1, const double *diss1, double *phi, double *phiaux,
                      int *fix) {
  const int band = 4;
  const double tol = 1e-24;
  int events = 0;
  for (size_t k = 0; k < (size_t)nx * ny; ++k) {
    fix[k] = 0;
    phiaux[k] = 1e4;
  }
#define RA(a, i, j) C1(a, i, j)
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j) {
      if (!((0.0 + VOFEPS) < RA(vfl, i, j) && RA(vfl, i, j) < (1.0 - VOFEPS - RA(vfls, i, j))))
        continue;
      RA(phiaux, i, j) = RA(diss1, i, j);
      RA(fix, i, j) = 1;
      const double dxs = RA(dx, i, j), dys = RA(dy, i, j);
      const double nxs_ = RA(nxs, i, j), nys_ = RA(nys, i, j), phs = RA(phis, i, j);
      const double n1 = RA(nxx1, i, j), n2 = RA(nyy1, i, j), d1 = RA(diss1, i, j);
      for (int ii = -band; ii <= band; ++ii)
        for (int jj = -band; jj <= band; ++jj) {
          const int p = i + ii, q = j + jj;
          if (!(p >= 1 && p <= nx && q >= 1 && q <= ny)) continue;
          const double vT = RA(vfl, p, q), sT = RA(vfls, p, q);
          if (!(vT < 0.0 + VOFEPS || vT >= 1.0 - VOFEPS - sT)) continue;
          double *pa = &RA(phiaux, p, q);
          RA(fix, p, q) = 1;
          const int l = ii < -1 ? -1 : (ii > 1 ? 1 : ii), m = jj < -1 ? -1 : (jj > 1 ? 1 : jj);
          double xv = dxs * (double)l / 2.0, yv = dys * (double)m / 2.0;
          double dvs = nxs_ * xv + nys_ * yv + phs;
          if (dvs < 0.0) {
            if (fabs(yv) < VOFEPS) {
              yv = dys / 2.0;
              dvs = nxs_ * xv + nys_ * yv + phs;
              if (dvs < 0.0) {
                yv = -dys / 2.0;
                dvs = nxs_ * xv + nys_ * yv + phs;
                if (dvs < 0.0) {
                  xv = dxs * (0.0 - (double)l) / 2.0;
                  dvs = nxs_ * xv + nys_ * yv + phs;
                  if (dvs < 0.0) yv = dys / 2.0;
                }
              }
            } else if (fabs(xv) < VOFEPS) {
              xv = dxs / 2.0;
              dvs = nxs_ * xv + nys_ * yv + phs;
              if (dvs < 0.0) {
                xv = -dxs / 2.0;
                dvs = nxs_ * xv + nys_ * yv + phs;
                if (dvs < 0.0) {
                  yv = dys * (0.0 - (double)m) / 2.0;
                  dvs = nxs_ * xv + nys_ * yv + phs;
                  if (dvs < 0.0) xv = dxs / 2.0;
                }
              }
            } else {
              yv = dys * (0.0 - (double)m) / 2.0;
              dvs = nxs_ * xv + nys_ * yv + phs;
              if (dvs < 0.0) {
                xv = dxs * (0.0 - (double)l) / 2.0;
                yv = dys * (double)m / 2.0;
                dvs = nxs_ * xv + nys_ * yv + phs;
                if (dvs < 0.0) yv = dys * (0.0 - (double)m) / 2.0;
              }
            }
          }
          const double rx = RA(x, p, q) - RA(x, i, j), ry = RA(y, p, q) - RA(y, i, j);
          const double dv = n1 * xv + n2 * yv + d1;
          double deuc;
          if (dv * copysign(1.0, RA(phi, p, q)) <= 0.0) {
            deuc = sqrt((rx - xv) * (rx - xv) + (ry - yv) * (ry - yv));
            if (sT < EPSI) {
              *pa = copysign(1.0, 0.5 - vT) * fmin(deuc, fabs(*pa));
            } else {
              if (fabs(deuc) < fabs(*pa) && vT >= 1.0 - VOFEPS - sT) *pa = -fabs(deuc);
              if (fabs(deuc) < fabs(*pa) && vT < VOFEPS) *pa = fabs(deuc);
            }
          } else {
            const double dij1 = n1 * rx + n2 * ry + d1;
            const double xp = rx - dij1 * n1, yp = ry - dij1 * n2;
            const int pointp = inside_rect(xp, yp, dxs, dys);
            if (pointp && sT < EPSI) {
              deuc = sqrt((rx - xp) * (rx - xp) + (ry - yp) * (ry - yp));
              *pa = copysign(1.0, 0.5 - vT) * fmin(deuc, fabs(*pa));
            } else if (pointp && sT >= EPSI && sT < 1.0 - EPSI) {
              deuc = sqrt((rx - xp) * (rx - xp) + (ry - yp) * (ry - yp));
              if (fabs(deuc) < fabs(*pa) && vT >= 1.0 - VOFEPS - sT) *pa = -fabs(deuc);
              if (fabs(deuc) < fabs(*pa) && vT < VOFEPS) *pa = fabs(deuc);
            } else if (sT >= 1.0 - EPSI) {
              if (RA(vfls, i, j) < EPSI) {
                deuc = sqrt((rx - xp) * (rx - xp) + (ry - yp) * (ry - yp));
                if (fabs(deuc) < fabs(*pa)) *pa = copysign(1.0, dij1) * deuc;
              }
            } else {
              const double xoff = fmax(fabs(xp) - 0.5 * dxs, 0.0);
              const double yoff = fmax(fabs(yp) - 0.5 * dys, 0.0);
              const double xfc = copysign(1.0, xp) * 0.5 * dxs, yfc = copysign(1.0, yp) * 0.5 * dys;
              double xs, ys;
              if (xoff * fabs(n1 + tol) >= yoff * fabs(n2 + tol)) {
                xs = xfc;
                ys = (d1 + n1 * xs) / (-n2 + tol);
              } else {
                ys = yfc;
                xs = (d1 + n2 * ys) / (-n1 + tol);
              }
              deuc = sqrt((rx - xs) * (rx - xs) + (ry - ys) * (ry - ys));
              const double dvs2 = nxs_ * xs + nys_ * ys + phs;
              if (dvs2 >= 0.0) {
                if (sT < EPSI) {
                  *pa = copysign(1.0, 0.5 - vT) * fmin(deuc, fabs(*pa));
                } else {
                  if (fabs(deuc) < fabs(*pa) && vT >= 1.0 - VOFEPS - sT) *pa = -fabs(deuc);
                  if (fabs(deuc) < fabs(*pa) && vT < VOFEPS) *pa = fabs(deuc);
                }
              }
            }
          }
          if (*pa > 9.999e3) RA(fix, p, q) = 0;
        }
    }
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j) {
      const double v = RA(vfl, i, j), s = RA(vfls, i, j);
      const double h = sqrt(RA(dx, i, j) * RA(dx, i, j) + RA(dy, i, j) * RA(dy, i, j));
      if (RA(fix, i, j) == 1) {
        if (RA(phiaux, i, j) > 1e3) ++events; /* pause */
        RA(phi, i, j) = RA(phiaux, i, j);
      } else {
        if (v <= VOFEPS) RA(phi, i, j) = (double)(band + 1) * h;
        else if (v >= (1.0 - VOFEPS - s)) RA(phi, i, j) = -(double)(band + 1) * h;
      }
      if (v < VOFEPS && RA(phi, i, j) < -VOFEPS && s < 1.0 - EPSI) ++events; /* pause */
    }
#undef RA
  return events;
}

/* ------------------------------------------------------------------------
 * Coupled_LS_VOF (src/Clsvof_Mod.f90:730-959) with a fixed solid: nv = 6
 * sub-steps of dtv = dt/6, each an X_Sweep then a Y_Sweep (odd k) or the
 * reverse (even k) with Coupled_LS_VOF's updates after each sweep and
 * Boundary_Condition (:961-973) between them, then Boundary_Condition,
 * Interface_Reconstruct and Redistance.  ObjectMovement and
 * SolidVolumeFraction, which move the solid body between sub-steps, are
 * the caller's: here the solid fields stay as given.
 * wave = {Amp0, kw, omew, Depthw, NondiT} (the X inlet; NULL: no inflow);
 * vfl, phi in/out; nxv, nyv, dis out (the last reconstruction: PCell%nx,
 * PCell%ny and the distance Redistance used).  Returns the events of the
 * reconstructions and of Redistance.
 * ---------------------------------------------------------------------- */
static void boundary_condition(int nx, int ny, double *v) {
  for (int i = 1; i <= nx; ++i) {
    C1(v, i, 1) = C1(v, i, 2);
    C1(v, i, ny) = C1(v, i, ny - 1);
  }
  for (int j = 1; j <= ny; ++j) {
    C1(v, 1, j) = C1(v, 2, j);
    C1(v, nx, j) = C1(v, nx - 1, j);
  }
}

int oracle_clsvof_step(int nx, int ny, const double *vofS, const double *nxs, const double *nys,
                       const double *phiS, const double *dx, const double *dy, const double *x,
                       const double *y, const double *aE, const double *aW, const double *aN,
                       const double *aS, const double *ue, const double *ve, const double *wave,
                       double dt, double *vfl, double *phi, double *nxv, double *nyv,
                       double *dis, double *work) {
  const int nv = 6;
  const size_t n1 = (size_t)nx * ny;
  double *tvx = work, *tvy = work + n1, *tlx = work + 2 * n1, *tly = work + 3 * n1;
  double *aux = work + 4 * n1;
  int *fix = (int *)(work + 5 * n1);
  const double dtv = dt / (double)nv;
  int events = 0;
  double w[6];
#define REC() events += oracle_interface_reconstruct(nx, ny, vfl, vofS, phi, nxs, nys, phiS, x, y, \
                                                     dx, dy, nxv, nyv, dis)
#define XSWEEP(k)                                                                          \
  do {                                                                                     \
    REC();                                                                                 \
    if (wave) {                                                                            \
      for (int q = 0; q < 5; ++q) w[q] = wave[q];                                          \
      w[5] = (double)(k);                                                                  \
    }                                                                                      \
    oracle_vof_sweep(0, nx, ny, vofS, dx, dy, x, y, aE, aW, aN, aS, ue, ve, vfl, nxv, nyv, \
                     dis, nxs, nys, phiS, wave ? w : NULL, dtv, tvx);                      \
    oracle_ls_sweep(0, nx, ny, phi, vofS, dx, dy, x, y, aE, aW, aN, aS, ue, ve, dtv, tlx);  \
  } while (0)
#define YSWEEP()                                                                           \
  do {                                                                                     \
    REC();                                                                                 \
    oracle_vof_sweep(1, nx, ny, vofS, dx, dy, x, y, aE, aW, aN, aS, ue, ve, vfl, nxv, nyv, \
                     dis, nxs, nys, phiS, NULL, dtv, tvy);                                 \
    oracle_ls_sweep(1, nx, ny, phi, vofS, dx, dy, x, y, aE, aW, aN, aS, ue, ve, dtv, tly);  \
  } while (0)
  for (int k = 1; k <= nv; ++k) {
    if (k % 2 == 1) {
      for (size_t c = 0; c < n1; ++c) { tvx[c] = vfl[c]; tlx[c] = phi[c]; }
      XSWEEP(k);
      for (int i = 1; i <= nx; ++i)
        for (int j = 1; j <= ny; ++j) {
          const double den = (1.0 - C1(vofS, i, j) + TOLDENO) -
                             dtv / C1(dx, i, j) * (UE(i, j) * E0(aE, i, j) - UE(i - 1, j) * E0(aW, i, j));
          C1(tvx, i, j) = C1(tvx, i, j) / den;
          C1(tlx, i, j) = C1(tlx, i, j) / den;
          C1(vfl, i, j) = C1(tvx, i, j) * (1.0 - C1(vofS, i, j));
          C1(phi, i, j) = C1(tlx, i, j);
          if (C1(vfl, i, j) >= 1.0 - VOFEPS - C1(vofS, i, j)) C1(vfl, i, j) = 1.0 - C1(vofS, i, j);
          if (C1(vfl, i, j) < VOFEPS) C1(vfl, i, j) = 0.0;
        }
      boundary_condition(nx, ny, vfl);
      boundary_condition(nx, ny, phi);
      for (size_t c = 0; c < n1; ++c) { tvy[c] = vfl[c]; tly[c] = phi[c]; }
      YSWEEP();
      for (int i = 1; i <= nx; ++i)
        for (int j = 1; j <= ny; ++j) {
          const double dd = VE(i, j) * E0(aN, i, j) - VE(i, j - 1) * E0(aS, i, j);
          C1(tvy, i, j) = C1(tvy, i, j) + dtv / C1(dy, i, j) * C1(tvx, i, j) * dd;
          C1(tly, i, j) = C1(tly, i, j) + dtv / C1(dy, i, j) * C1(tlx, i, j) * dd;
          C1(vfl, i, j) = C1(tvy, i, j);
          if (C1(vofS, i, j) < 1.0 - EPSI) C1(phi, i, j) = C1(tly, i, j) / (1.0 - C1(vofS, i, j));
        }
    } else {
      for (size_t c = 0; c < n1; ++c) { tvy[c] = vfl[c]; tly[c] = phi[c]; }
      YSWEEP();
      for (int i = 1; i <= nx; ++i)
        for (int j = 1; j <= ny; ++j) {
          const double den = (1.0 - C1(vofS, i, j) + TOLDENO) -
                             dtv / C1(dy, i, j) * (VE(i, j) * E0(aN, i, j) - VE(i, j - 1) * E0(aS, i, j));
          C1(tvy, i, j) = C1(tvy, i, j) / den;
          C1(tly, i, j) = C1(tly, i, j) / den;
          C1(vfl, i, j) = C1(tvy, i, j) * (1.0 - C1(vofS, i, j));
          C1(phi, i, j) = C1(tly, i, j);
          if (C1(vfl, i, j) >= 1.0 - VOFEPS - C1(vofS, i, j)) C1(vfl, i, j) = 1.0 - C1(vofS, i, j);
          if (C1(vfl, i, j) < VOFEPS) C1(vfl, i, j) = 0.0;
        }
      boundary_condition(nx, ny, vfl);
      boundary_condition(nx, ny, phi);
      for (size_t c = 0; c < n1; ++c) { tvx[c] = vfl[c]; tlx[c] = phi[c]; }
      XSWEEP(k);
      for (int i = 1; i <= nx; ++i)
        for (int j = 1; j <= ny; ++j) {
          const double dd = UE(i, j) * E0(aE, i, j) - UE(i - 1, j) * E0(aW, i, j);
          C1(tvx, i, j) = C1(tvx, i, j) + dtv / C1(dx, i, j) * C1(tvy, i, j) * dd;
          C1(tlx, i, j) = C1(tlx, i, j) + dtv / C1(dx, i, j) * C1(tly, i, j) * dd;
          C1(vfl, i, j) = C1(tvx, i, j);
          if (C1(vofS, i, j) < 1.0 - EPSI) C1(phi, i, j) = C1(tlx, i, j) / (1.0 - C1(vofS, i, j));
        }
    }
    boundary_condition(nx, ny, vfl);
    boundary_condition(nx, ny, phi);
    REC();
    events += oracle_redistance(nx, ny, vfl, vofS, nxs, nys, phiS, x, y, dx, dy, nxv, nyv, dis,
                                phi, aux, fix);
  }
#undef REC
#undef XSWEEP
#undef YSWEEP
  return events;
}
