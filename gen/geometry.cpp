// geometry.cpp -- host-side builder of the cut-cell geometry that the
// projection consumes (the input side of the path).
//
// In SIMCOFlow these fields are produced on the CPU every time step by
//   Initial_Grid / InitialUVGrid      src/Mesh_Mod.f90:54-175
//   Initial_Clsvof (solid/liquid)     src/Clsvof_Mod.f90:39-400, frac :1371-1404
//   Grid_Preprocess -> Cell_Geo_Cal,  src/Cutcell_Mod.f90:18-300
//     Edge_Geo_Cal, DefineMomentumExchangeCell, NumberExternalCell
//                                     src/Cutcell_Mod.f90:302-397
// This file restates those steps for synthetic solids (circles and rotated
// rectangles given by signed distance) and a sinusoidal free surface, so that
// seeded workloads can be built at full size.  Loops that the reference runs
// in a fixed order and whose result depends on that order (solid-face zeroing
// and the degenerate-cell rule) are kept in that order.
//
// Output layouts are the reference's Fortran layouts: column-major, i fastest,
// (1:nx,1:ny) or (0:nx+1,0:ny+1).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "scf_geom.h"

namespace {

constexpr double kEpsi = 1.0e-3;     // src/StateVariables.f90:26
constexpr double kEpsiF = 1.0e-2;    // src/StateVariables.f90:26
constexpr double kVofEps = 1.0e-14;  // src/Clsvof_Mod.f90:10
constexpr double kRoundoff = 1.0e-24;

struct F1 {  // (1:nx,1:ny)
  double* a; int nx;
  double& operator()(int i, int j) const { return a[(size_t)(i - 1) + (size_t)(j - 1) * nx]; }
};
struct F0 {  // (0:nx+1,0:ny+1)
  double* a; int nx;
  double& operator()(int i, int j) const { return a[(size_t)i + (size_t)j * (nx + 2)]; }
};
struct I1 {
  int32_t* a; int nx;
  int32_t& operator()(int i, int j) const { return a[(size_t)(i - 1) + (size_t)(j - 1) * nx]; }
};
struct I0 {
  int32_t* a; int nx;
  int32_t& operator()(int i, int j) const { return a[(size_t)i + (size_t)j * (nx + 2)]; }
};

// frac: area fraction of the cell where nx*x+ny*y+diss < 0 (the solid side
// of a linear level set), src/Clsvof_Mod.f90:1371-1404.
double frac(double nx, double ny, double diss, double dx, double dy) {
  const double slop_eps = 1.0e-20;
  double tnx = std::fabs(nx), tny = std::fabs(ny);
  if (diss + 0.5 * (tnx * dx + tny * dy) <= 0.0) return 1.0;
  if (diss - 0.5 * (tnx * dx + tny * dy) >= 0.0) return 0.0;
  if (tnx <= slop_eps) return 0.5 - diss / dy;
  if (tny <= slop_eps) return 0.5 - diss / dx;
  double xx = (0.5 * tny * dy - diss) / dx / tnx + 0.5;
  double yy = (0.5 * tnx * dx - diss) / dy / tny + 0.5;
  double totalarea = 0.5 * xx * yy;
  double topvf = 0.0, rightvf = 0.0;
  if (yy > 1.0) topvf = std::pow((yy - 1.0) / yy, 2.0);
  if (xx > 1.0) rightvf = std::pow((xx - 1.0) / xx, 2.0);
  return totalarea * (1.0 - topvf - rightvf);
}

// Edge_Geo_Cal, src/Cutcell_Mod.f90:302-337: solid fraction of the edge
// Pt1-Pt2 under the linear level set (>= 1e-14 is fluid).
double edge_solid(double p1x, double p1y, double p2x, double p2y, double nxx, double nyy,
                  double diss) {
  double l1 = nxx * p1x + nyy * p1y + diss;
  double l2 = nxx * p2x + nyy * p2y + diss;
  const double epsil = 1.0e-14;
  if (l1 >= epsil && l2 >= epsil) return 0.0;
  if (l1 < epsil && l2 < epsil) return 1.0;
  if (l1 >= epsil && l2 < epsil) return std::fabs(l2) / (std::fabs(l1) + std::fabs(l2));
  return std::fabs(l1) / (std::fabs(l1) + std::fabs(l2));
}

// signed distance (positive in the fluid) and outward unit normal of one solid
void solid_sd(const scf_solid& s, double x, double y, double* phi, double* nx, double* ny) {
  if (s.kind == SCF_SOLID_CIRCLE) {
    double dx = x - s.cx, dy = y - s.cy;
    double r = std::sqrt(dx * dx + dy * dy);
    *phi = r - s.r;
    if (r > 0.0) { *nx = dx / r; *ny = dy / r; }
    else { *nx = 0.0; *ny = 1.0; }
    return;
  }
  // rotated rectangle: local coordinates q = R^T (p - c)
  double c = std::cos(s.angle), sn = std::sin(s.angle);
  double px = x - s.cx, py = y - s.cy;
  double qx = c * px + sn * py, qy = -sn * px + c * py;
  double dx = std::fabs(qx) - s.hw, dy = std::fabs(qy) - s.hh;
  double sx = qx >= 0.0 ? 1.0 : -1.0, sy = qy >= 0.0 ? 1.0 : -1.0;
  double lnx, lny;
  if (dx > 0.0 && dy > 0.0) {
    double d = std::sqrt(dx * dx + dy * dy);
    *phi = d; lnx = sx * dx / d; lny = sy * dy / d;
  } else if (dx > dy) {
    *phi = dx; lnx = sx; lny = 0.0;
  } else {
    *phi = dy; lnx = 0.0; lny = sy;
  }
  *nx = c * lnx - sn * lny;
  *ny = sn * lnx + c * lny;
}

void solid_levelset(int nsolid, const scf_solid* solids, double x, double y, double* phi,
                    double* nx, double* ny) {
  *phi = 1.0e30; *nx = 0.0; *ny = 1.0;
  for (int k = 0; k < nsolid; ++k) {
    double p, a, b;
    solid_sd(solids[k], x, y, &p, &a, &b);
    if (p < *phi) { *phi = p; *nx = a; *ny = b; }
  }
}

double surf_h(const scf_surface& s, double x) {
  double h = s.y0;
  for (int m = 0; m < s.nmodes; ++m) h += s.amp[m] * std::sin(s.k[m] * x + s.phase[m]);
  return h;
}
double surf_dh(const scf_surface& s, double x) {
  double d = 0.0;
  for (int m = 0; m < s.nmodes; ++m) d += s.amp[m] * s.k[m] * std::cos(s.k[m] * x + s.phase[m]);
  return d;
}

// Newton crossing of the horizontal line y=yl with the surface,
// as in src/Clsvof_Mod.f90:89-96 and :120-127.
double newton_cross(const scf_surface& s, double yl, double x0, double tolc) {
  double x = x0, tol = 1.0;
  for (int it = 0; it < 200 && tol > tolc; ++it) {
    double fx = yl - surf_h(s, x);
    double dfx = -surf_dh(s, x);
    if (dfx == 0.0) break;
    tol = std::fabs(fx / dfx);
    x = x - fx / dfx;
  }
  return x;
}

// liquid volume fraction and level set of one cell for the sinusoidal
// surface, src/Clsvof_Mod.f90:58-178 (polygon of the air side, shoelace area)
void liquid_cell(const scf_surface& s, double xc, double yc, double dxc, double dyc,
                 double* vof, double* phi) {
  double dx2 = dxc / 2.0, dy2 = dyc / 2.0;
  double dpt[5];
  dpt[1] = yc - dy2 - surf_h(s, xc + dx2);
  dpt[2] = yc - dy2 - surf_h(s, xc - dx2);
  dpt[3] = yc + dy2 - surf_h(s, xc - dx2);
  dpt[4] = yc + dy2 - surf_h(s, xc + dx2);
  double node[10][2], cut[3][2];
  int temp = 0, templ = 0;
  if (dpt[1] >= 0.0) { node[temp][0] = dx2; node[temp][1] = -dy2; temp++; }
  if (dpt[1] * dpt[2] < 0.0) {
    double x0 = xc - dx2 + dxc * std::fabs(dpt[2]) / (std::fabs(dpt[2]) + std::fabs(dpt[1]));
    double xcr = newton_cross(s, yc - dy2, x0, 1.0e-12);
    node[temp][0] = xcr - xc; node[temp][1] = -dy2;
    if (templ < 2) { cut[templ][0] = node[temp][0]; cut[templ][1] = node[temp][1]; }
    templ++; temp++;
  }
  if (dpt[2] >= 0.0) { node[temp][0] = -dx2; node[temp][1] = -dy2; temp++; }
  if (dpt[2] * dpt[3] < 0.0) {
    node[temp][0] = -dx2; node[temp][1] = surf_h(s, -dx2 + xc) - yc;
    if (templ < 2) { cut[templ][0] = node[temp][0]; cut[templ][1] = node[temp][1]; }
    templ++; temp++;
  }
  if (dpt[3] >= 0.0) { node[temp][0] = -dx2; node[temp][1] = dy2; temp++; }
  if (dpt[3] * dpt[4] < 0.0) {
    double x0 = xc - dx2 + dxc * std::fabs(dpt[3]) / (std::fabs(dpt[3]) + std::fabs(dpt[4]));
    double xcr = newton_cross(s, yc + dy2, x0, 1.0e-13);
    node[temp][0] = xcr - xc; node[temp][1] = dy2;
    if (templ < 2) { cut[templ][0] = node[temp][0]; cut[templ][1] = node[temp][1]; }
    templ++; temp++;
  }
  if (dpt[4] >= 0.0) { node[temp][0] = dx2; node[temp][1] = dy2; temp++; }
  if (dpt[4] * dpt[1] < 0.0) {
    node[temp][0] = dx2; node[temp][1] = surf_h(s, dx2 + xc) - yc;
    if (templ < 2) { cut[templ][0] = node[temp][0]; cut[templ][1] = node[temp][1]; }
    templ++; temp++;
  }
  double vol = 0.0;
  if (temp > 0) {
    node[temp][0] = node[0][0]; node[temp][1] = node[0][1];
    for (int k = 0; k < temp; ++k)
      vol = vol + 0.5 * (node[k][0] * node[k + 1][1] - node[k + 1][0] * node[k][1]);
  }
  vol = 1.0 - std::fabs(vol / (dxc * dyc));
  double dis;
  if (templ == 2) {
    double nxx = cut[1][1] - cut[0][1];
    double nyy = cut[1][0] - cut[0][0];
    double nxy = std::sqrt(nxx * nxx + nyy * nyy);
    dis = std::fabs(cut[1][0] * cut[0][1] - cut[0][0] * cut[1][1]) / nxy *
          std::copysign(1.0, 0.5 - vol);
  } else {
    dis = yc - surf_h(s, xc);
  }
  *vof = vol;
  *phi = dis;
}

// One staggered family (P, U or V cells): solid fractions from the level set
// at the family's cell centres with the family's spacings; Initial_Clsvof
// clamps (:311-313) followed by the Cell_Geo_Cal clamp (Cutcell :217-218).
void solid_fraction(int nx, int ny, const double* xc, const double* yc, const double* dxc,
                    const double* dyc, int nsolid, const scf_solid* solids, double* vofS,
                    double* phiS, double* nxS, double* nyS) {
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t k = (size_t)(i - 1) + (size_t)(j - 1) * nx;
      double p, a, b;
      solid_levelset(nsolid, solids, xc[k], yc[k], &p, &a, &b);
      double v = frac(a, b, p, dxc[k], dyc[k]);
      if (v < kVofEps) v = 0.0;
      if (v >= 1.0 - kVofEps) v = 1.0;
      vofS[k] = v;
      if (phiS) phiS[k] = p;
      if (nxS) nxS[k] = a;
      if (nyS) nyS[k] = b;
    }
}

}  // namespace

extern "C" {

// Initial_Grid 1-D spacing, src/Mesh_Mod.f90:54-137 (one axis):
// npts = cells+1 face coordinates from s0 to s1; if nonuniform, a uniform
// band [r0,r1] with nrec points and geometric growth outside it (ratio
// found by Newton-Raphson, :191-204).
int scf_geom_axis(int npts, double s0, double s1, int nonuniform, double r0, double r1, int nrec,
                  double* out) {
  if (npts < 2 || !out) return -1;
  if (!nonuniform) {
    double d = (s1 - s0) / (double)(npts - 1);
    for (int j = 0; j < npts; ++j) out[j] = s0 + d * (double)j;
    return 0;
  }
  auto newton = [](double dl, double d, int n) {
    double beta = 1.001, tol = 1.0;
    for (int it = 0; it < 200 && tol > 1.0e-14; ++it) {
      double fx = d * (std::pow(beta, n + 1) - beta) / (beta - 1.0) - dl;
      double dfx = d * (n * std::pow(beta, n + 1) - (n + 1) * std::pow(beta, n) + 1.0) /
                   std::pow(beta - 1.0, 2.0);
      tol = std::fabs(fx / dfx);
      beta = beta - fx / dfx;
    }
    return beta;
  };
  double d = (r1 - r0) / (double)(nrec - 1);
  int ns = (int)((double)(npts - nrec) * std::fabs(r0 - s0) / (std::fabs(r0 - s0) + std::fabs(s1 - r1)));
  int ne = (npts - nrec) - ns;
  std::vector<double> y(npts + 2);
  // 1-based as in the reference
  double beta = newton(r0 - s0, d, ns);
  y[1] = s0;
  for (int j = 2; j <= 2 + ns; ++j) y[j] = y[j - 1] + d * std::pow(beta, ns - (j - 2));
  for (int j = ns + 2; j <= ns + nrec; ++j) y[j] = y[j - 1] + d;
  beta = newton(s1 - r1, d, ne);
  for (int j = ns + nrec + 1; j <= npts; ++j) y[j] = y[j - 1] + d * std::pow(beta, j - (ns + nrec));
  for (int j = 0; j < npts; ++j) out[j] = y[j + 1];
  return 0;
}

int scf_geom_build(int nx, int ny, const double* xf, const double* yf, int nsolid,
                   const scf_solid* solids, const scf_surface* surf, int icorprob,
                   const scf_geom_out* o) {
  if (nx < 3 || ny < 3 || !xf || !yf || !o || (nsolid > 0 && !solids) || !surf) return -1;
  const size_t n1 = (size_t)nx * ny;
  // --- grids: Initial_Grid / InitialUVGrid (Mesh_Mod :128-175) ---
  std::vector<double> px(n1), py(n1), pdx(n1), pdy(n1);
  std::vector<double> ux(n1), uy(n1), udx(n1), udy(n1), vx(n1), vy(n1), vdx(n1), vdy(n1);
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t k = (size_t)(i - 1) + (size_t)(j - 1) * nx;
      px[k] = 0.5 * (xf[i] + xf[i - 1]);
      pdx[k] = xf[i] - xf[i - 1];
      py[k] = 0.5 * (yf[j] + yf[j - 1]);
      pdy[k] = yf[j] - yf[j - 1];
    }
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t k = (size_t)(i - 1) + (size_t)(j - 1) * nx;
      ux[k] = px[k] + 0.5 * pdx[k];
      uy[k] = py[k];
      udy[k] = pdy[k];
      udx[k] = (i < nx) ? px[k + 1] - px[k] : pdx[k];
      vx[k] = px[k];
      vy[k] = py[k] + 0.5 * pdy[k];
      vdx[k] = pdx[k];
      vdy[k] = (j < ny) ? py[k + nx] - py[k] : pdy[k];
    }
  if (o->x) std::memcpy(o->x, px.data(), n1 * sizeof(double));
  if (o->y) std::memcpy(o->y, py.data(), n1 * sizeof(double));
  if (o->dx) std::memcpy(o->dx, pdx.data(), n1 * sizeof(double));
  if (o->dy) std::memcpy(o->dy, pdy.data(), n1 * sizeof(double));
  if (o->dxU) std::memcpy(o->dxU, udx.data(), n1 * sizeof(double));
  if (o->dyV) std::memcpy(o->dyV, vdy.data(), n1 * sizeof(double));

  // --- solid fractions of the three families (Initial_Clsvof x3, Main.f90:212-214) ---
  std::vector<double> vofS(n1), phiS(n1), nxS(n1), nyS(n1), vofSU(n1), vofSV(n1);
  solid_fraction(nx, ny, px.data(), py.data(), pdx.data(), pdy.data(), nsolid, solids,
                 vofS.data(), phiS.data(), nxS.data(), nyS.data());
  solid_fraction(nx, ny, ux.data(), uy.data(), udx.data(), udy.data(), nsolid, solids,
                 vofSU.data(), nullptr, nullptr, nullptr);
  solid_fraction(nx, ny, vx.data(), vy.data(), vdx.data(), vdy.data(), nsolid, solids,
                 vofSV.data(), nullptr, nullptr, nullptr);
  if (o->vofS_in) std::memcpy(o->vofS_in, vofS.data(), n1 * sizeof(double));
  if (o->nxS_in) std::memcpy(o->nxS_in, nxS.data(), n1 * sizeof(double));
  if (o->nyS_in) std::memcpy(o->nyS_in, nyS.data(), n1 * sizeof(double));
  if (o->vofS_u_in) std::memcpy(o->vofS_u_in, vofSU.data(), n1 * sizeof(double));
  if (o->vofS_v_in) std::memcpy(o->vofS_v_in, vofSV.data(), n1 * sizeof(double));

  // --- liquid fraction and level set of the P cells ---
  std::vector<double> vof(n1), phi(n1);
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t k = (size_t)(i - 1) + (size_t)(j - 1) * nx;
      double vv, pp;
      liquid_cell(*surf, px[k], py[k], pdx[k], pdy[k], &vv, &pp);
      vof[k] = vv * (1.0 - vofS[k]);  // Clsvof :394
      phi[k] = pp;
    }

  // --- Cell_Geo_Cal for the P cells (Cutcell :34-300) ---
  const size_t n0 = (size_t)(nx + 2) * (ny + 2);
  std::vector<double> aE(n0, 0.0), aW(n0, 0.0), aN(n0, 0.0), aS(n0, 0.0), wl(n1, 0.0);
  F0 E{aE.data(), nx}, W{aW.data(), nx}, N{aN.data(), nx}, S{aS.data(), nx};
  F1 VS{vofS.data(), nx}, WL{wl.data(), nx}, DX{pdx.data(), nx}, DY{pdy.data(), nx};
  F1 NXS{nxS.data(), nx}, NYS{nyS.data(), nx}, PHS{phiS.data(), nx};
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j) {
      double dx = DX(i, j), dy = DY(i, j);
      // Pt(ii,jj) = (-dx*(0.5-ii), -dy*(0.5-jj))
      double x0 = -dx * 0.5, x1 = dx * 0.5, y0 = -dy * 0.5, y1 = dy * 0.5;
      double a = NXS(i, j), b = NYS(i, j), p = PHS(i, j);
      W(i, j) = edge_solid(x0, y0, x0, y1, a, b, p);
      N(i, j) = edge_solid(x0, y1, x1, y1, a, b, p);
      E(i, j) = edge_solid(x1, y1, x1, y0, a, b, p);
      S(i, j) = edge_solid(x1, y0, x0, y0, a, b, p);
    }
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j)
      WL(i, j) = std::sqrt(std::pow((E(i, j) - W(i, j)) * DX(i, j), 2.0) +
                           std::pow((N(i, j) - S(i, j)) * DY(i, j), 2.0));
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j) {
      W(i, j) = 1.0 - W(i, j); E(i, j) = 1.0 - E(i, j);
      N(i, j) = 1.0 - N(i, j); S(i, j) = 1.0 - S(i, j);
    }
  // harmonic averaging of interior shared faces (:161-204)
  for (int i = 2; i <= nx - 1; ++i)
    for (int j = 2; j <= ny - 1; ++j) {
      double av = 2.0 * N(i, j) * S(i, j + 1) / (N(i, j) + S(i, j + 1) + kRoundoff);
      N(i, j) = av; S(i, j + 1) = av;
      av = 2.0 * E(i, j) * W(i + 1, j) / (E(i, j) + W(i + 1, j) + kRoundoff);
      E(i, j) = av; W(i + 1, j) = av;
    }
  // solid cells and degenerate cells, in the reference's order (:215-244)
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j) {
      if (VS(i, j) > 1.0 - kEpsi) {
        VS(i, j) = 1.0;
        W(i, j) = 0.0; E(i, j) = 0.0; N(i, j) = 0.0; S(i, j) = 0.0;
        E(i - 1, j) = 0.0; N(i, j - 1) = 0.0; W(i + 1, j) = 0.0; S(i, j + 1) = 0.0;
      }
      if ((W(i, j) + E(i, j) < kRoundoff || S(i, j) + N(i, j) < kRoundoff) &&
          VS(i, j) < 1.0 - kEpsi) {
        VS(i, j) = 1.0;
        W(i, j) = 0.0; E(i, j) = 0.0; N(i, j) = 0.0; S(i, j) = 0.0;
        E(i - 1, j) = 0.0; N(i, j - 1) = 0.0; W(i + 1, j) = 0.0; S(i, j + 1) = 0.0;
      }
    }
  // wall length of fully solid cells (:245-258)
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j)
      if (std::fabs(VS(i, j) - 1.0) < kRoundoff) {
        if (W(i, j) == 0.0 || E(i, j) == 0.0) WL(i, j) = DY(i, j);
        if (N(i, j) == 0.0 || S(i, j) == 0.0) WL(i, j) = DX(i, j);
      }
  // corner correction of the P cells when ICorProb is set (:259-285, Main.f90:204)
  if (icorprob) {
    for (int i = 1; i <= nx; ++i)
      for (int j = 1; j <= ny - 4; ++j) {
        if (VS(i, j) > -kEpsi && VS(i, j) < kEpsi) {
          if (VS(i, j + 1) > 0.6 - kEpsi && VS(i, j + 1) < 0.6 + kEpsi) {
            if (VS(i, j + 2) > 0.6 - kEpsi && VS(i, j + 2) < 0.6 + kEpsi) {
              N(i, j) = 0.40; S(i, j + 1) = 0.4;
              WL(i, j) = 0.6 * DX(i, j); NYS(i, j) = -1.0; NXS(i, j) = 0.0;
            }
          }
          if (VS(i, j + 1) > 1.0 - kEpsi && VS(i, j + 1) < 1.0 + kEpsi) {
            WL(i, j) = DX(i, j); NYS(i, j) = -1.0; NXS(i, j) = 0.0;
          }
        }
      }
  }
  // U and V families: Cell_Geo_Cal clamp only (their apertures are not used
  // by the projection; they carry MsCe so no degenerate rule applies)
  for (size_t k = 0; k < n1; ++k) {
    if (vofSU[k] > 1.0 - kEpsi) vofSU[k] = 1.0;
    if (vofSV[k] > 1.0 - kEpsi) vofSV[k] = 1.0;
  }
  F1 VSU{vofSU.data(), nx}, VSV{vofSV.data(), nx};
  // DefineMomentumExchangeCell (:360-397)
  std::vector<int32_t> moexU(n1, 0), moexV(n1, 0);
  I1 MU{moexU.data(), nx}, MV{moexV.data(), nx};
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j) {
      MU(i, j) = 0; MV(i, j) = 0;
      if (VSU(i, j) >= kEpsi && VSU(i, j) < 1.0 - kEpsi) {
        if (i < nx) {
          if (VS(i, j) >= 1.0 - kEpsi || VS(i + 1, j) >= 1.0 - kEpsi || E(i, j) < kEpsiF) {
            MU(i, j) = 1; E(i, j) = 0.0; W(i + 1, j) = 0.0;
          }
        } else if (VS(i, j) >= 1.0 - kEpsi) {
          MU(i, j) = 1;
        }
      }
      if (VSV(i, j) >= kEpsi && VSV(i, j) < 1.0 - kEpsi) {
        if (j < ny) {
          if (VS(i, j) >= 1.0 - kEpsi || VS(i, j + 1) >= 1.0 - kEpsi || N(i, j) < kEpsiF) {
            MV(i, j) = 1; N(i, j) = 0.0; S(i, j + 1) = 0.0;
          }
        } else if (VS(i, j) >= 1.0 - kEpsi) {
          MV(i, j) = 1;
        }
      }
    }
  // NumberExternalCell (:340-358): j fastest; cells outside the numbered
  // range are -1 here (the reference leaves them unset)
  std::vector<int32_t> pnp(n0, -1), pnu(n0, -1), pnv(n0, -1);
  I0 PN{pnp.data(), nx}, UN{pnu.data(), nx}, VN{pnv.data(), nx};
  int32_t ctr = 0;
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j) PN(i, j) = VS(i, j) < 1.0 - kEpsi ? ctr++ : -1;
  int next = ctr;
  ctr = 0;
  for (int i = 1; i <= nx - 1; ++i)
    for (int j = 1; j <= ny; ++j) UN(i, j) = VSU(i, j) < 1.0 - kEpsi ? ctr++ : -1;
  ctr = 0;
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny - 1; ++j) VN(i, j) = VSV(i, j) < 1.0 - kEpsi ? ctr++ : -1;

  auto put = [](double* dst, const std::vector<double>& src) {
    if (dst) std::memcpy(dst, src.data(), src.size() * sizeof(double));
  };
  auto puti = [](int32_t* dst, const std::vector<int32_t>& src) {
    if (dst) std::memcpy(dst, src.data(), src.size() * sizeof(int32_t));
  };
  put(o->vof, vof); put(o->phi, phi); put(o->vofS, vofS); put(o->phiS, phiS);
  put(o->nxS, nxS); put(o->nyS, nyS); put(o->WlLh, wl);
  put(o->aE, aE); put(o->aW, aW); put(o->aN, aN); put(o->aS, aS);
  puti(o->posnu_p, pnp); puti(o->posnu_u, pnu); puti(o->posnu_v, pnv);
  puti(o->moex_u, moexU); puti(o->moex_v, moexV);
  put(o->vofS_u, vofSU); put(o->vofS_v, vofSV);
  return next;  // number of pressure unknowns (ExtCell+1)
}

}  // extern "C"
