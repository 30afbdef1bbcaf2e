/*
 * mom_oracle.c -- CPU restatement of the implicit part of SIMCOFlow's
 * momentum predictor (one velocity component per call): SetMatrix
 * (src/PredictorUV_mod.f90:622-768), SetVectors (:770-845), the HYPRE solve
 * (:507-513, :530-536), DeltaGetValues (:847-885), the pressure-gradient
 * update and the Dp boundary copies (:517-522, :540-545, :552-562) and
 * PredictorVelocityBoundaryCondition (:563, :2199-2213).
 *
 * TEST INFRASTRUCTURE ONLY (see scf_oracle.c): only tests/, smoke() and the
 * CPU-baseline leg of bench.py load it; the product path never calls it.
 * Parity status: UNPINNED, for the same reason as the projection oracle (the
 * Fortran + HYPRE reference cannot be built here and ships no golden data).
 *
 * Operation order follows the Fortran expressions left to right; compile
 * with -ffp-contract=off.  Arrays (Fortran layouts, column-major):
 *   F1(a,i,j)  (1:nx,1:ny)            dx, dy, vof, vofS, WlLh, delh, flux, GradP
 *   F0(a,i,j)  (0:nx+1,0:ny+1)        Posnu, EtaE, EtaN, u, v, Dp, Pred
 *   FE(a,i,j)  (1:nx+1,1:ny)          DifFluxEW, EDFluxEW (this component)
 *   FN(a,i,j)  (1:nx,1:ny+1)          DifFluxNS, EDFluxNS (this component)
 *   CWE (1:ny,2), CSN (1:nx,2), matr (1:nx,1:ny,5): S, W, P, E, N.
 * The component is iu = 1, iv = 0 for u and iu = 0, iv = 1 for v.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define F1(a, i, j) (a)[(size_t)((i)-1) + (size_t)((j)-1) * (size_t)nx]
#define F0(a, i, j) (a)[(size_t)(i) + (size_t)(j) * (size_t)(nx + 2)]
#define FE(a, i, j) (a)[(size_t)((i)-1) + (size_t)((j)-1) * (size_t)(nx + 1)]
#define FN(a, i, j) (a)[(size_t)((i)-1) + (size_t)((j)-1) * (size_t)nx]
#define MT(f, i, j) matr[(size_t)((i)-1) + (size_t)((j)-1) * (size_t)nx + (size_t)((f)-1) * (size_t)nx * (size_t)ny]
#define CWE(j, k) cwe[(size_t)((j)-1) + (size_t)((k)-1) * (size_t)ny]
#define CSN(i, k) csn[(size_t)((i)-1) + (size_t)((k)-1) * (size_t)nx]

/* cst: dt, BetaVis, nua, nuw, nuref, Rey (src/StateVariables.f90:26-28) */
int oracle_mom_matrix(int nx, int ny, int iu, int iv, const double *dx, const double *dy,
                      const int32_t *posnu, const double *vof, const double *vofS,
                      const double *etaE, const double *etaN, const double *wllh,
                      const double *delh, const double *difEW, const double *difNS,
                      const double *edEW, const double *edNS, const double *cst, double *Dp,
                      double *cwe, double *csn, double *matr) {
  const double dt = cst[0], BetaVis = cst[1], nua = cst[2], nuw = cst[3], nuref = cst[4],
               Rey = cst[5];
  int bad = 0;
  for (int i = 1; i <= nx - iu; ++i)
    for (int j = 1; j <= ny - iv; ++j) {
      if (F0(posnu, i, j) == -1) continue;
      for (int f = 1; f <= 5; ++f) MT(f, i, j) = 0.0;
      const double VofAF = 1.0 - F1(vofS, i, j);
      double De = (1.0 - BetaVis) * FE(difEW, i + 1, j) / VofAF;
      double Dw = (1.0 - BetaVis) * FE(difEW, i, j) / VofAF;
      double Dn = (1.0 - BetaVis) * FN(difNS, i, j + 1) / VofAF;
      const double Ds = (1.0 - BetaVis) * FN(difNS, i, j) / VofAF;
      const double Fep = FE(edEW, i + 1, j) * (1.0 - F0(etaE, i, j)) / VofAF;
      const double Fem = FE(edEW, i + 1, j) * F0(etaE, i, j) / VofAF;
      const double Fwp = FE(edEW, i, j) * F0(etaE, i - 1, j) / VofAF;
      const double Fwm = FE(edEW, i, j) * (1.0 - F0(etaE, i - 1, j)) / VofAF;
      const double Fnp = FN(edNS, i, j + 1) * (1.0 - F0(etaN, i, j)) / VofAF;
      const double Fnm = FN(edNS, i, j + 1) * F0(etaN, i, j) / VofAF;
      const double Fsp = FN(edNS, i, j) * F0(etaN, i, j - 1) / VofAF;
      const double Fsm = FN(edNS, i, j) * (1.0 - F0(etaN, i, j - 1)) / VofAF;
      if (iu == 1) {
        if (j == ny) Dn = 0.0;
        if (i == nx - iu) De = 0.0;
        if (i == 1) Dw = 0.0;
      } else if (j == ny - iv) {
        Dn = 0.0;
      }
      double aE = De, aW = Dw, aN = Dn, aS = Ds;
      if (i == 1) CWE(j, 1) = aW;
      if (i == nx - iu) CWE(j, 2) = aE;
      if (j == 1) CSN(i, 1) = aS;
      if (j == ny - iv) CSN(i, 2) = aN;
      const double rv = F1(vof, i, j) / (1.0 - F1(vofS, i, j));
      double aP = F1(dx, i, j) * F1(dy, i, j) / dt + aE + aW + aN + aS +
                  ((1.0 - rv) * nua / nuref + rv * nuw / nuref) / Rey * F1(wllh, i, j) /
                      F1(delh, i, j) / VofAF;
      aP = aP + Fep - Fwp + Fnp - Fsp;
      aE = aE - Fem;
      aW = aW + Fwm;
      aN = aN - Fnm;
      aS = aS + Fsm;
      F0(Dp, i, j) = F1(dx, i, j) * F1(dy, i, j) / (aP - aE - aW - aN - aS);
      if (j > 1 && F0(posnu, i, j - 1) != -1) MT(1, i, j) = -aS;
      if (i > 1 && F0(posnu, i - 1, j) != -1) MT(2, i, j) = -aW;
      if (isnan(aP) || fabs(aP) > 1.0e20) bad = 1;
      MT(3, i, j) = aP;
      if (i < nx && F0(posnu, i + 1, j) != -1) MT(4, i, j) = -aE;
      if (j < ny && F0(posnu, i, j + 1) != -1) MT(5, i, j) = -aN;
    }
  return bad ? -1 : 0;
}

/* Right-hand side of the active cells (rhm, (1:nx,1:ny); 0 elsewhere in the
 * loop range).  u and v are the old velocities (0:nx+1,0:ny+1).  The
 * reference adds CSN(j,2) (row index j, not i) on the top row; every CSN(.,2)
 * this call sets is the zeroed top diffusion coefficient, and elements it
 * does not set are undefined in the reference: both read as +0 here. */
void oracle_mom_vectors(int nx, int ny, int iu, int iv, const int32_t *posnu, const double *dx,
                        const double *dy, const double *flux, const double *cwe,
                        const double *csn, const double *u, const double *v, double Fr,
                        double *rhm) {
  const double diu = (double)iu, div_ = (double)iv;
  for (int i = 1; i <= nx - iu; ++i)
    for (int j = 1; j <= ny - iv; ++j) {
      F1(rhm, i, j) = 0.0;
      if (F0(posnu, i, j) == -1) continue;
      double r = 0.0;
      if (iu == 1) {
        r = r - F1(flux, i, j);
      } else {
        r = r - F1(flux, i, j);
        r = r - 1.0 / (Fr * Fr) * F1(dx, i, j) * F1(dy, i, j);
      }
      if (i == 1) r = r + CWE(j, 1) * (diu * F0(u, i - 1, j) + div_ * F0(v, i - 1, j));
      if (i == nx - iu) r = r + CWE(j, 2) * (diu * F0(u, i + 1, j) + div_ * F0(v, i + 1, j));
      if (j == 1) r = r + CSN(i, 1) * (diu * F0(u, i, j - 1) + div_ * F0(v, i, j - 1));
      if (j == ny - iv) r = r + 0.0 * (diu * F0(u, i, j + 1) + div_ * F0(v, i, j + 1));
      F1(rhm, i, j) = r;
    }
}

/* DeltaGetValues, the pressure-gradient update of the solved component and
 * its boundary copies.  x: solution by unknown number (Posnu). */
void oracle_mom_finish(int nx, int ny, int iu, int iv, const int32_t *posnu, const double *x,
                       const double *gradp, const double *dx, const double *dy, double dt,
                       double *pred, double *Dp) {
  for (int i = 1; i <= nx - iu; ++i)
    for (int j = 1; j <= ny - iv; ++j) {
      const int32_t k = F0(posnu, i, j);
      F0(pred, i, j) = k != -1 ? x[k] : 0.0;
    }
  for (int i = 1; i <= nx - iu; ++i)
    for (int j = 1; j <= ny - iv; ++j)
      F0(pred, i, j) = F0(pred, i, j) + dt * F1(gradp, i, j) / F1(dx, i, j) / F1(dy, i, j);
  if (iu == 1) {
    for (int j = 0; j <= ny + 1; ++j) F0(Dp, 0, j) = F0(Dp, 1, j);
    for (int j = 0; j <= ny + 1; ++j) F0(Dp, nx, j) = F0(Dp, nx - 1, j);
    for (int j = 0; j <= ny + 1; ++j) F0(Dp, nx + 1, j) = F0(Dp, nx, j);
    for (int i = 0; i <= nx + 1; ++i) F0(Dp, i, 0) = F0(Dp, i, 1);
    for (int i = 0; i <= nx + 1; ++i) F0(Dp, i, ny + 1) = F0(Dp, i, ny);
  } else {
    for (int j = 0; j <= ny + 1; ++j) F0(Dp, 0, j) = F0(Dp, 1, j);
    for (int j = 0; j <= ny + 1; ++j) F0(Dp, nx + 1, j) = F0(Dp, nx, j);
    for (int i = 0; i <= nx + 1; ++i) F0(Dp, i, 0) = F0(Dp, i, 1);
    for (int i = 0; i <= nx + 1; ++i) F0(Dp, i, ny) = F0(Dp, i, ny - 1);
    for (int i = 0; i <= nx + 1; ++i) F0(Dp, i, ny + 1) = F0(Dp, i, ny);
    /* PredictorVelocityBoundaryCondition: open top */
    for (int i = 1; i <= nx; ++i) F0(pred, i, ny) = F0(pred, i, ny - 1);
  }
}

/* CPU baseline solver for the same system: BiCGStab with the diagonal as
 * preconditioner on the 5-point operator held in matr, unknowns in grid
 * order (cells outside the system stay 0).  Returns the iterations taken
 * (-1: breakdown or no convergence within maxit); *relres the final
 * ||b - A x|| / ||b||.  OpenMP over rows. */
static void mom_apply(int nx, int ny, int iu, int iv, const int32_t *posnu,
                      const double *matr, const double *p, double *q) {
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny - iv; ++j)
    for (int i = 1; i <= nx - iu; ++i) {
      if (F0(posnu, i, j) == -1) { F1(q, i, j) = 0.0; continue; }
      double s = MT(3, i, j) * F1(p, i, j);
      if (j > 1) s += MT(1, i, j) * F1(p, i, j - 1);
      if (i > 1) s += MT(2, i, j) * F1(p, i - 1, j);
      if (i < nx) s += MT(4, i, j) * F1(p, i + 1, j);
      if (j < ny) s += MT(5, i, j) * F1(p, i, j + 1);
      F1(q, i, j) = s;
    }
}
static double mom_dot(size_t n, const double *a, const double *b) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (size_t k = 0; k < n; ++k) s += a[k] * b[k];
  return s;
}
int oracle_mom_bicgstab(int nx, int ny, int iu, int iv, const int32_t *posnu,
                        const double *matr, const double *rhm, double rtol, int maxit,
                        double *xg, double *relres) {
  const size_t n = (size_t)nx * ny;
  double *r = calloc(n, 8), *rh = calloc(n, 8), *p = calloc(n, 8), *vv = calloc(n, 8),
         *s = calloc(n, 8), *t = calloc(n, 8), *y = calloc(n, 8), *z = calloc(n, 8),
         *di = calloc(n, 8);
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const int act = i <= nx - iu && j <= ny - iv && F0(posnu, i, j) != -1;
      F1(di, i, j) = act ? 1.0 / MT(3, i, j) : 0.0;
      F1(xg, i, j) = 0.0;
      F1(r, i, j) = act ? F1(rhm, i, j) : 0.0;
      F1(rh, i, j) = F1(r, i, j);
    }
  const double bn = sqrt(mom_dot(n, r, r));
  double rho = 1.0, alpha = 1.0, omega = 1.0, rn = bn;
  int it = 0, ok = bn == 0.0;
  for (; !ok && it < maxit; ++it) {
    const double rho1 = mom_dot(n, rh, r);
    if (rho1 == 0.0) break;
    const double beta = (rho1 / rho) * (alpha / omega);
    rho = rho1;
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n; ++k) {
      p[k] = r[k] + beta * (p[k] - omega * vv[k]);
      y[k] = di[k] * p[k];
    }
    mom_apply(nx, ny, iu, iv, posnu, matr, y, vv);
    alpha = rho / mom_dot(n, rh, vv);
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n; ++k) {
      s[k] = r[k] - alpha * vv[k];
      z[k] = di[k] * s[k];
    }
    mom_apply(nx, ny, iu, iv, posnu, matr, z, t);
    const double tt = mom_dot(n, t, t);
    omega = tt > 0.0 ? mom_dot(n, t, s) / tt : 0.0;
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n; ++k) {
      xg[k] += alpha * y[k] + omega * z[k];
      r[k] = s[k] - omega * t[k];
    }
    rn = sqrt(mom_dot(n, r, r));
    if (rn <= rtol * bn) { ok = 1; ++it; break; }
    if (omega == 0.0) break;
  }
  *relres = bn > 0.0 ? rn / bn : 0.0;
  free(r); free(rh); free(p); free(vv); free(s); free(t); free(y); free(z); free(di);
  return ok ? it : -1;
}
