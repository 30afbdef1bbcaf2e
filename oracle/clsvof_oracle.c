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
