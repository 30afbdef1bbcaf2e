// scf_clsvof.cu -- the CLSVOF sweeps after Interface_Reconstruct
// (include/scf_clsvof.h): the level-set part of X_Sweep
// (src/Clsvof_Mod.f90:1074-1123) and Y_Sweep (:1191-1244), and their VOF part
// (:1004-1069, :1141-1189) with the face-flux routines topflux, bottomflux,
// rightflux, leftflux (:1416-1522), frac (:1371-1404) and CellGeoCal
// (:2159-2253).
//
// The reference walks the faces of each row (column) in order; face f
// subtracts its flux from cell f and scales cell f+1 by (1 - vofS) before
// adding the flux to it, and a second loop applies the first and last
// faces.  So every cell ends as a fixed expression of at most two face
// fluxes, which the kernels evaluate for each cell:
//   cell 1:          (t - f1 E1/d1) + phi1 u0 dtv W1/d1
//   cell 2:          (t - f2 E2/d2) + f1 E1/d2
//   cells 3..n-1:    (t (1 - s) + f(i-1) Wi/di) - fi Ei/di
//   cell n:          (t (1 - s) + f(n-1) Wn/dn) - fn En/dn     (Y: - fn/dn)
// The VOF update has the same shape (every face applied to both of its
// cells), after the division of temvf by (1 - vofS); its cell 1 gets the
// inflow through face 0 (X: the wave inlet, Y: vof ve(0) dtv) last.  Face
// fluxes read only the sweep's inputs, never temvf, so they can be
// evaluated in any order.
// Compiled with -fmad=false: the operations and their order are the
// reference's, so results are bit-identical to the sequential loops.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "../../include/scf_clsvof.h"
#include "../../include/scf_proj.h"
#include "scf_internal.cuh"

namespace scf {
namespace {

// The kernels' FP64 division and square root: the correctly rounded
// integer-pipe forms of the library (identical results to IEEE '/' and
// sqrt; GB300's FP64 pipe is what bounds these kernels).
__device__ __forceinline__ double dv(double a, double b) { return div_rn(a, b); }
__device__ __forceinline__ double sq(double x) { return sqrt_rn(x); }
// The FP64 pipe's division, for the geometric flux routines: their chains of
// dependent divisions run faster there than on the longer integer-pipe form.
__device__ __forceinline__ double dvh(double a, double b) { return __ddiv_rn(a, b); }

struct LsIn {
  int nx, ny;
  double dtv;
  const double *phi, *vofS, *dx, *dy, *x, *y, *aE, *aW, *aN, *aS, *ue, *ve;
};

// Along one row (X) or column (Y): n cells, element k (1-based) of a
// (nx,ny) array at base + (k-1)*st; of an edge array at ebase + k*est.
struct Line {
  const double *phi, *d, *c, *s;  // phi, dx (dy), x (y), vofS
  const double *lo, *hi;          // W and E (S and N) apertures, at k
  const double *vel;              // ue (ve) at face k, k = 0..n
  long long st, est, vst;
  int n;
  __device__ double P(int k) const { return phi[(k - 1) * st]; }
  __device__ double D(int k) const { return d[(k - 1) * st]; }
  __device__ double C(int k) const { return c[(k - 1) * st]; }
  __device__ double S(int k) const { return s[(k - 1) * st]; }
  __device__ double Lo(int k) const { return lo[k * est]; }
  __device__ double Hi(int k) const { return hi[k * est]; }
  __device__ double V(int k) const { return vel[k * vst]; }
};

// flux through face f (the high face of cell f), f = 1..n
template <int DIR>
__device__ double face_flux(const Line& L, int f, double dtv) {
  const int n = L.n;
  const double u = L.V(f);
  double l;
  if (f == 1) {
    if (u >= 0.0)
      l = L.P(1) + dv(L.D(1) * 0.5 * (1.0 - dv(u * dtv, L.D(1))) * (L.P(2) - L.P(1)),
                      L.C(2) - L.C(1));
    else if (DIR == SCF_LS_X)
      l = L.P(2) - dv(L.D(2) * 0.5 * (1.0 + dv(u * dtv, L.D(2))) * (L.P(3) - L.P(1)),
                      2.0 * L.D(2));
    else
      l = L.P(2) - dv(L.D(2) * 0.5 * (1.0 + dv(u * dtv, L.D(2))) * (L.P(3) - L.P(1)),
                      L.C(3) - L.C(1));
    return l * u * dtv;
  }
  if (f == n) {
    if (u > 0.0)
      l = L.P(n) + dv(L.D(n) * 0.5 * (1.0 - dv(u * dtv, L.D(n))) * (L.P(n) - L.P(n - 1)),
                      L.C(n) - L.C(n - 1));
    else
      l = L.P(n) - dv(L.D(n - 1) * 0.5 * (1.0 + dv(u * dtv, L.D(n - 1))) *
                          (L.P(n) - L.P(n - 1)),
                      L.C(n) - L.C(n - 1));
    return l * u * dtv;
  }
  if (u >= 0.0) l = (L.P(f + 1) + L.P(f - 1)) * 0.5;
  else if (f <= n - 2) l = (L.P(f + 2) + L.P(f)) * 0.5;
  else l = (L.P(f + 1) + L.P(f - 1)) * 0.5;
  return DIR == SCF_LS_X ? u * l * dtv : l * u * dtv;
}

// The level-set value of cell idx (0-based (i0, j0)) after the sweep.
template <int DIR>
__device__ double ls_cell(const LsIn& in, long long idx, int i0, int j0, double t) {
  const int nx = in.nx, ny = in.ny;
  Line L;
  const long long e0 = (long long)(i0 + 1) + (long long)(j0 + 1) * (nx + 2);  // (i,j) of an edge array
  int k;
  if (DIR == SCF_LS_X) {
    const long long r = (long long)j0 * nx;
    L = {in.phi + r, in.dx + r, in.x + r, in.vofS + r, in.aW + e0 - (i0 + 1),
         in.aE + e0 - (i0 + 1), in.ue + (long long)j0 * (nx + 1), 1, 1, 1, nx};
    k = i0 + 1;
  } else {
    const long long c = i0;
    L = {in.phi + c, in.dy + c, in.y + c, in.vofS + c, in.aS + e0 - (long long)(j0 + 1) * (nx + 2),
         in.aN + e0 - (long long)(j0 + 1) * (nx + 2), in.ve + c, nx, nx + 2, nx, ny};
    k = j0 + 1;
  }
  (void)idx;
  const int n = L.n;
  const double dtv = in.dtv;
  if (k == 1) {
    t = t - dv(face_flux<DIR>(L, 1, dtv) * L.Hi(1), L.D(1));
    t = t + dv(L.P(1) * L.V(0) * dtv * L.Lo(1), L.D(1));
  } else if (k == 2) {
    t = t - dv(face_flux<DIR>(L, 2, dtv) * L.Hi(2), L.D(2));
    t = t + dv(face_flux<DIR>(L, 1, dtv) * L.Hi(1), L.D(2));
  } else {
    t = t * (1.0 - L.S(k)) + dv(face_flux<DIR>(L, k - 1, dtv) * L.Lo(k), L.D(k));
    if (k < n || DIR == SCF_LS_X) t = t - dv(face_flux<DIR>(L, k, dtv) * L.Hi(k), L.D(k));
    else t = t - dv(face_flux<DIR>(L, k, dtv), L.D(k));
  }
  return t;
}

// ---------------------------------------------------------------------------
// VOF part.  vofeps = 1e-14, TolDeno = 1e-24 (src/Clsvof_Mod.f90:10),
// epsi = 1e-3 (src/StateVariables.f90:28).
// ---------------------------------------------------------------------------
constexpr double kVofEps = 1e-14, kTolDeno = 1e-24, kEpsi = 1e-3;

// frac: the part of a dx x dy cell where |nx| x + |ny| y + diss <= 0.
__device__ double frac_part(double nx, double ny, double diss, double dx, double dy) {
  const double tnx = fabs(nx), tny = fabs(ny);
  if (diss + 0.5 * (tnx * dx + tny * dy) <= 0.0) return 1.0;
  if (diss - 0.5 * (tnx * dx + tny * dy) >= 0.0) return 0.0;
  if (tnx <= 1e-20) return 0.5 - dvh(diss, dy);
  if (tny <= 1e-20) return 0.5 - dvh(diss, dx);
  const double xx = dvh(dvh(0.5 * tny * dy - diss, dx), tnx) + 0.5;
  const double yy = dvh(dvh(0.5 * tnx * dx - diss, dy), tny) + 0.5;
  const double total = 0.5 * xx * yy;
  double top = 0.0, right = 0.0;
  if (yy > 1.0) {
    const double r = dvh(yy - 1.0, yy);
    top = r * r;
  }
  if (xx > 1.0) {
    const double r = dvh(xx - 1.0, xx);
    right = r * r;
  }
  return total * (1.0 - top - right);
}

// CellGeoCal: the solid fraction vols (the cell outside nxs x + nys y +
// phis >= 0) and the liquid part volf (nxl x + nyl y + phil <= 0) of the
// rest, by the shoelace formula over the clipped polygon.  At most five
// vertices (three corners and two cuts) bound the non-solid part; the
// liquid polygon keeps every vertex its sign tests give (up to ten).
__device__ void cell_geo(double nxs, double nys, double phis, double nxl, double nyl, double phil,
                         double dx, double dy, double& vols, double& volf) {
  double px[8], py[8], pd[8];  // at most 8 puts below (5 in exact arithmetic)
  const double dx2 = dx * 0.5, dy2 = dy * 0.5;
  const double d0 = dx2 * nxs - dy2 * nys + phis, d1 = -(dx2 * nxs) - dy2 * nys + phis;
  const double d2 = -(dx2 * nxs) + dy2 * nys + phis, d3 = dx2 * nxs + dy2 * nys + phis;
  int m = 0;
  auto put = [&](double a, double b) {
    px[m] = a;
    py[m] = b;
    ++m;
  };
  if (d0 >= 0.0) put(dx2, -dy2);
  if (d0 * d1 < 0.0) put(dvh(dy2 * nys - phis, nxs), -dy2);
  if (d1 >= 0.0) put(-dx2, -dy2);
  if (d1 * d2 < 0.0) put(-dx2, dvh(dx2 * nxs - phis, nys));
  if (d2 >= 0.0) put(-dx2, dy2);
  if (d2 * d3 < 0.0) put(dvh(-(dy2 * nys) - phis, nxs), dy2);
  if (d3 >= 0.0) put(dx2, dy2);
  if (d3 * d0 < 0.0) put(dx2, dvh(-(dx2 * nxs) - phis, nys));
  double vol = 0.0;
  for (int k = 0; k < m; ++k) {
    const int k1 = k + 1 < m ? k + 1 : 0;
    vol = vol + 0.5 * (px[k] * py[k1] - px[k1] * py[k]);
    pd[k] = px[k] * nxl + py[k] * nyl + phil;
  }
  vols = 1.0 - fabs(dvh(vol, dx * dy));
  // liquid polygon, streamed: keep its first vertex and the previous one
  double fx = 0.0, fy = 0.0, lx = 0.0, ly = 0.0;
  int ml = 0;
  vol = 0.0;
  auto add = [&](double a, double b) {
    if (ml == 0) {
      fx = a;
      fy = b;
    } else {
      vol = vol + 0.5 * (lx * b - a * ly);
    }
    lx = a;
    ly = b;
    ++ml;
  };
  for (int k = 0; k < m; ++k) {
    const int k1 = k + 1 < m ? k + 1 : 0;
    if (pd[k] <= 0.0) add(px[k], py[k]);
    if (pd[k] * pd[k1] < 0.0) {
      const double w = fabs(pd[k]), ws = fabs(pd[k]) + fabs(pd[k1]);
      add(px[k] + dvh((px[k1] - px[k]) * w, ws), py[k] + dvh((py[k1] - py[k]) * w, ws));
    }
  }
  if (ml > 0) vol = vol + 0.5 * (lx * fy - fx * ly);
  volf = fabs(dvh(vol, dx * dy));
}

// The inputs of one cell's upwind flux.
struct VofCell {
  double vof, nxv, nyv, dis, nxs, nys, phiS, vofS, dx, dy;
};

// topflux (DIR Y, SIDE -1), bottomflux (Y, +1), rightflux (X, -1),
// leftflux (X, +1) with the face displacement vdt.
template <int DIR, int SIDE>
__device__ double face_geo(const VofCell& c, double vdt) {
  if (vdt == 0.0) return 0.0;
  const double h = DIR == SCF_LS_X ? c.dx : c.dy;
  const double nl = DIR == SCF_LS_X ? c.nxv : c.nyv;
  const double sh = 0.5 * (vdt - h);
  const double dl = SIDE < 0 ? c.dis - sh * nl : c.dis + sh * nl;
  const double sx = DIR == SCF_LS_X ? vdt : c.dx, sy = DIR == SCF_LS_X ? c.dy : vdt;
  double flux;
  if (c.vofS < kEpsi) {
    flux = frac_part(c.nxv, c.nyv, dl, sx, sy);
  } else if (c.vofS >= 1.0 - kEpsi) {
    return c.vof;
  } else {
    const double ns = DIR == SCF_LS_X ? c.nxs : c.nys;
    const double ds = SIDE < 0 ? c.phiS - sh * ns : c.phiS + sh * ns;
    double volss;
    cell_geo(c.nxs, c.nys, ds, c.nxv, c.nyv, dl, sx, sy, volss, flux);
    if (dvh(c.vof, 1.0 - c.vofS) >= 1.0 - kVofEps) flux = 1.0 - volss;
    flux = dvh(flux, 1.0 - volss + kTolDeno);
    if (c.vof + c.vofS > 1.0 - 1e-14) flux = 1.0;
  }
  return flux * vdt;
}

struct VofIn {
  int nx, ny;
  double dtv, level;  // level: Depthw + etau of the X inlet (-inf: no inflow)
  const double *vofS, *dx, *dy, *y, *aE, *aW, *aN, *aS, *ue, *ve;
  const double *vof, *nxv, *nyv, *dis, *nxs, *nys, *phiS;
};

// One row (X) or column (Y) of the VOF inputs.
struct VLine {
  const VofIn* in;
  long long c0, st;         // element k (1-based) of an (nx,ny) array: c0 + (k-1)*st
  const double *lo, *hi;    // W and E (S and N) apertures at k*est
  const double* vel;        // ue (ve) at face k, k = 0..n, stride vst
  long long est, vst;
  int n;
  __device__ long long at(int k) const { return c0 + (k - 1) * st; }
  __device__ double F(int k) const { return in->vof[at(k)]; }
  __device__ double S(int k) const { return in->vofS[at(k)]; }
  __device__ double D(int k) const { return DIR_X ? in->dx[at(k)] : in->dy[at(k)]; }
  __device__ double Lo(int k) const { return lo[k * est]; }
  __device__ double Hi(int k) const { return hi[k * est]; }
  __device__ double V(int k) const { return vel[k * vst]; }
  __device__ VofCell cell(int k) const {
    const long long a = at(k);
    return {in->vof[a], in->nxv[a], in->nyv[a], in->dis[a], in->nxs[a],
            in->nys[a], in->phiS[a], in->vofS[a], in->dx[a], in->dy[a]};
  }
  bool DIR_X;
};

// Flux carried by the upwind cell c of a face with velocity u (SIDE -1: c
// is the face's low cell, +1: its high cell).
template <int DIR, int SIDE>
__device__ double upwind_flux(const VLine& L, int c, double u, double dtv) {
  const double vf = L.F(c);
  if (vf >= 1.0 - kVofEps || vf <= kVofEps) {
    double fl = vf * u * dtv;
    if (vf >= 1.0) fl = u * dtv;
    if (vf < 0.0) fl = 0.0;
    return fl;
  }
  const VofCell cc = L.cell(c);
  if (SIDE < 0) return face_geo<DIR, -1>(cc, u * dtv);
  return -face_geo<DIR, +1>(cc, -u * dtv);
}

// VOF flux through face f (the high face of cell f), f = 1..n.
template <int DIR>
__device__ double vof_face(const VLine& L, int f, double dtv) {
  const double u = L.V(f);
  double flux;
  if (DIR == SCF_LS_X ? u >= 0.0 : u > 0.0) {
    flux = upwind_flux<DIR, -1>(L, f, u, dtv);
    if (L.Hi(f) > 1.0 - kVofEps && L.S(f) > 1.0 - kVofEps) flux = u * dtv;
  } else if (f < L.n) {
    flux = upwind_flux<DIR, +1>(L, f + 1, u, dtv);
    if (L.Lo(f + 1) > 1.0 - kVofEps && L.S(f + 1) > 1.0 - kVofEps) flux = u * dtv;
  } else {
    flux = L.F(f) * u * dtv;
  }
  return flux;
}

constexpr int kSwTx = 32, kSwTy = 8;

// One thread per cell of a 32 x 8 tile.  Each thread evaluates the VOF flux
// of its cell's high face; the low face's comes from the neighbouring
// thread through shared memory (the tile's first column (X) or row (Y)
// evaluates it itself), so a face is evaluated about once.
template <int DIR, bool LS>
__global__ void __launch_bounds__(kSwTx* kSwTy)
    k_clsvof_sweep(VofIn vin, LsIn lin, double* __restrict__ temvf, double* __restrict__ temls) {
  __shared__ double face[kSwTy][kSwTx];
  const int nx = vin.nx, ny = vin.ny;
  const double dtv = vin.dtv;
  const int i0 = blockIdx.x * kSwTx + threadIdx.x, j0 = blockIdx.y * kSwTy + threadIdx.y;
  const bool live = i0 < nx && j0 < ny;
  VLine L;
  int k = 0;
  double fhi = 0.0;
  if (live) {
    L.in = &vin;
    const long long e0 = (long long)(i0 + 1) + (long long)(j0 + 1) * (nx + 2);
    if (DIR == SCF_LS_X) {
      L.c0 = (long long)j0 * nx;
      L.st = 1;
      L.lo = vin.aW + e0 - (i0 + 1);
      L.hi = vin.aE + e0 - (i0 + 1);
      L.vel = vin.ue + (long long)j0 * (nx + 1);
      L.est = 1;
      L.vst = 1;
      L.n = nx;
      L.DIR_X = true;
      k = i0 + 1;
    } else {
      L.c0 = i0;
      L.st = nx;
      L.lo = vin.aS + e0 - (long long)(j0 + 1) * (nx + 2);
      L.hi = vin.aN + e0 - (long long)(j0 + 1) * (nx + 2);
      L.vel = vin.ve + i0;
      L.est = nx + 2;
      L.vst = nx;
      L.n = ny;
      L.DIR_X = false;
      k = j0 + 1;
    }
    fhi = vof_face<DIR>(L, k, dtv);
  }
  face[threadIdx.y][threadIdx.x] = fhi;
  __syncthreads();
  if (!live) return;
  const long long idx = (long long)i0 + (long long)j0 * nx;
  double t = temvf[idx];
  const double s = L.S(k);
  if (s < 1.0 - kVofEps) t = dv(t, 1.0 - s);
  if (k == 1) {
    t = t - dv(fhi * L.Hi(1), L.D(1));
    if (DIR == SCF_LS_X) {
      double fin = 0.0;
      if (vin.y[idx] - vin.dy[idx] * 0.5 < vin.level) fin = L.F(1) * L.V(0) * dtv;
      t = t + dv(fin * L.Lo(1), L.D(1));
    } else {
      t = t + dv(L.F(1) * L.V(0) * dtv * L.Lo(1), L.D(1));
    }
  } else {
    double flo;
    if (DIR == SCF_LS_X ? threadIdx.x > 0 : threadIdx.y > 0)
      flo = DIR == SCF_LS_X ? face[threadIdx.y][threadIdx.x - 1] : face[threadIdx.y - 1][threadIdx.x];
    else
      flo = vof_face<DIR>(L, k - 1, dtv);
    t = t * (1.0 - s) + dv(flo * L.Lo(k), L.D(k));
    t = t - dv(fhi * L.Hi(k), L.D(k));
  }
  temvf[idx] = t;
  if (LS) temls[idx] = ls_cell<DIR>(lin, idx, i0, j0, temls[idx]);
}

template <int DIR>
__global__ void k_ls_sweep(LsIn in, double* temls) {
  const int nx = in.nx, ny = in.ny;
  const long long total = (long long)nx * ny;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x)
    temls[idx] = ls_cell<DIR>(in, idx, (int)(idx % nx), (int)(idx / nx), temls[idx]);
}

// ---------------------------------------------------------------------------
// Interface_Reconstruct (src/Clsvof_Mod.f90:1250-1321) with
// Normal_Vector_Irre (:1710-1919), distance (:1323-1369),
// DistanceFluidCalculate (:1957-2042), zriddr (:2044-2105) and LiqFuncVol
// (:2107-2155).
//
// The reference loops over cells (i outer, j inner) and its locals nxx,
// nyy, diss carry from one cell to the next.  Only three cases read a
// carried value: a flagged cell of column 1 or nx (rows 2..ny-1) takes nyy
// from the cell before it (j-1), one of row 1 or ny (columns 2..nx-1) takes
// nxx from the cell before it (row ny: (i, ny-1); row 1: (i-1, ny)), and a
// three-phase cell whose Ridders bracket fails keeps diss.  Each of those
// values is the carrying cell's output, so the kernels run in passes:
//   1. every cell that reads no carried normal (interior, corners, and
//      unflagged boundary cells);
//   2. row ny, then 3. row 1 (reading the outputs of passes 1 and 2);
//   4. columns 1 and nx: a flagged cell walks back to the nearest unflagged
//      cell (or row 1) and replays the short chain of nyy;
//   5. cells whose bracket failed copy dis from the nearest earlier cell
//      (loop order) whose dis was assigned.
// Each pass writes only its own cells.  Where the reference pauses for the
// operator, reads outside an array or uses a value never set, the kernels go
// on as after the operator's "go" (or with the documented value) and count
// the event.
// ---------------------------------------------------------------------------
// Vset as Coupled_LS_VOF leaves it (:746-753: its line 747 sets Vset(1,2)
// again instead of Vset(2,2)).
__constant__ double kVset[8][2] = {{0, 1}, {0, 0}, {-1, 0}, {-1, -1},
                                   {-1, 1}, {1, 0}, {1, -1}, {1, 1}};

struct IrIn {
  int nx, ny;
  const double *vof, *vofS, *phi, *nxs, *nys, *phiS, *x, *y, *dx, *dy;
  double *nxv, *nyv, *dis;
  unsigned char* failed;
  int* events;
  int *list, *count;  // the interface cells of pass 1 (scratch)
  __device__ long long at(int i, int j) const { return (long long)(i - 1) + (long long)(j - 1) * nx; }
  __device__ double P(int i, int j) const { return phi[at(i, j)]; }
  __device__ double S(int i, int j) const { return vofS[at(i, j)]; }
  __device__ double gx(int a, int b, int j) const {
    return dv(phi[at(a, j)] - phi[at(b, j)], x[at(a, j)] - x[at(b, j)]);
  }
  __device__ double gy(int i, int a, int b) const {
    return dv(phi[at(i, a)] - phi[at(i, b)], y[at(i, a)] - y[at(i, b)]);
  }
  __device__ int flag(int i, int j) const {
    const double v = vof[at(i, j)], s = vofS[at(i, j)];
    int f = 0;
    if (v >= kVofEps && v < (1.0 - kVofEps - s) && s < kEpsi) f = 1;
    if (v >= kVofEps && v < (1.0 - kVofEps - s) && s >= kEpsi && s < 1.0 - kEpsi) f = 2;
    return f;
  }
};

__device__ double unit_dev(double vx, double vy) { return fabs(1.0 - sq(vx * vx + vy * vy)); }

// The direction of Vset most parallel to the central gradient, then the
// one-sided pair closer to unit length (:1768-1832, :1860-1912).
__device__ void most_parallel(const IrIn& c, int i, int j, int imv, double& nxo, double& nyo) {
  const double vx = c.gx(i + 1, i - 1, j), vy = c.gy(i, j + 1, j - 1);
  double maxv = 0.0;
  for (int ii = 1; ii <= 8; ++ii) {
    const double a = kVset[ii - 1][0], b = kVset[ii - 1][1];
    const double cp = dv(fabs(a * vx + b * vy), sq(a * a + b * b) * sq(vx * vx + vy * vy));
    if (cp >= maxv) {
      maxv = cp;
      imv = ii;
    }
  }
  if (imv == 0) {  // the reference reads Vset(0,:), outside the table
    atomicAdd(c.events, 1);
    imv = 1;
  }
  const double v11 = -kVset[imv - 1][1], v12 = kVset[imv - 1][0];
  double vx1, vx2, vy1, vy2;
  if (v11 == -1) {
    vx1 = c.gx(i, i - 1, j);
    vx2 = c.gx(i + 1, i, j);
  } else if (v11 == 0) {
    vx1 = vx2 = c.gx(i + 1, i - 1, j);
  } else {
    vx1 = c.gx(i + 1, i, j);
    vx2 = c.gx(i, i - 1, j);
  }
  if (v12 == -1) {
    vy1 = c.gy(i, j, j - 1);
    vy2 = c.gy(i, j + 1, j);
  } else if (v12 == 0) {
    vy1 = vy2 = c.gy(i, j + 1, j - 1);
  } else {
    vy1 = c.gy(i, j + 1, j);
    vy2 = c.gy(i, j, j - 1);
  }
  if (unit_dev(vx1, vy1) < unit_dev(vx2, vy2) + 0.075 / 8.0) {
    nxo = vx1;
    nyo = vy1;
  } else {
    nxo = vx2;
    nyo = vy2;
  }
}

__device__ int one_sided(double qm, double q0, double qp) {
  const double eta = 0.075;
  if (qm < eta && qp >= eta) return -1;
  if (qm >= eta && qp < eta) return 1;
  if (qm < eta && q0 < eta && qp < eta) return 0;
  if (qm >= eta && q0 >= eta && qp >= eta) return 0;
  return 2;  // none: the most-parallel rule
}

// Normal_Vector_Irre for 1 < i < nx, 1 < j < ny.
__device__ void normal_irre(const IrIn& c, int i, int j, double& nxo, double& nyo) {
  const int nx = c.nx, ny = c.ny;
  if (c.S(i, j) >= kEpsi) {
    if (c.S(i + 1, j) < 1.0 - kEpsi && c.S(i - 1, j) < 1.0 - kEpsi) nxo = c.gx(i + 1, i - 1, j);
    else if (c.S(i + 1, j) >= 1.0 - kEpsi) nxo = c.gx(i, i - 1, j);
    else nxo = c.gx(i + 1, i, j);
    if (c.S(i, j + 1) < 1.0 - kEpsi && c.S(i, j - 1) < 1.0 - kEpsi) nyo = c.gy(i, j + 1, j - 1);
    else if (c.S(i, j + 1) > 1.0 - kEpsi) nyo = c.gy(i, j, j - 1);
    else nyo = c.gy(i, j + 1, j);
    return;
  }
  double qm = unit_dev(i >= 3 ? c.gx(i, i - 2, j) : c.gx(i, i - 1, j), c.gy(i - 1, j + 1, j - 1));
  const double q0 = unit_dev(c.gx(i + 1, i - 1, j), c.gy(i, j + 1, j - 1));
  double qp = unit_dev(i <= nx - 2 ? c.gx(i + 2, i, j) : c.gx(i + 1, i, j),
                       c.gy(i + 1, j + 1, j - 1));
  const int dx = one_sided(qm, q0, qp);
  if (dx == 2) {
    most_parallel(c, i, j, 0, nxo, nyo);
    return;
  }
  qm = unit_dev(c.gx(i + 1, i - 1, j - 1), j >= 3 ? c.gy(i, j, j - 2) : c.gy(i, j, j - 1));
  qp = unit_dev(c.gx(i + 1, i - 1, j + 1), j <= ny - 2 ? c.gy(i, j + 2, j) : c.gy(i, j + 1, j));
  const int dy = one_sided(qm, q0, qp);
  if (dy == 2) {
    most_parallel(c, i, j, 1, nxo, nyo);
    return;
  }
  nxo = dx == -1 ? c.gx(i, i - 1, j) : dx == 1 ? c.gx(i + 1, i, j) : c.gx(i + 1, i - 1, j);
  nyo = dy == -1 ? c.gy(i, j, j - 1) : dy == 1 ? c.gy(i, j + 1, j) : c.gy(i, j + 1, j - 1);
}

// distance: the PLIC line distance of a two-phase cell.
__device__ double plic_distance(double v, double dx, double dy, double nxx, double nyy) {
  const double nx = fabs(nxx), ny = fabs(nyy);
  if (nx < 1e-20) return (0.5 - v) * dy;
  if (ny < 1e-20) return (0.5 - v) * dx;
  const double dll = 0.5 * (nx * dx + ny * dy), dur = -dll;
  double dul = 0.5 * (nx * dx - ny * dy), dlr = -dul;
  double vful = frac_part(nx, ny, dul, dx, dy), vflr = frac_part(nx, ny, dlr, dx, dy);
  if (v <= vful && v <= vflr) {
    if (vful > vflr) {
      double t = vful; vful = vflr; vflr = t;
      t = dul; dul = dlr; dlr = t;
    }
    return dll - sq(dv(((dul - dll) * (dul - dll)) * v, vful));
  }
  if (v >= vful && v >= vflr) {
    if (vflr < vful) {
      double t = vful; vful = vflr; vflr = t;
      t = dul; dul = dlr; dlr = t;
    }
    return dur + sq(dv((dlr - dur) * (dlr - dur) * (1.0 - v), 1.0 - vflr));
  }
  if (fabs(vflr - vful) < 1e-20) return 0.5 * (dul + dlr);
  const double t = dv(v - vful, vflr - vful);
  return dlr * t + dul * (1.0 - t);
}

// LiqFuncVol: volf minus the liquid part (below the line through xf) of
// the closed polygon node, zero-padded; its vertex count is found as the
// reference finds it, from the last non-zero entry of the first six.
__device__ double liq_func_vol(const double (&node)[9][2], double nxf, double nyf, double volf,
                               double dx, double dy, double xf0, double xf1, int* events) {
  const double phil = -(nxf * xf0 + nyf * xf1);
  int temp = 0;
  for (int k = 1; k <= 6; ++k)
    if (fabs(node[k - 1][0]) > 1e-14 || fabs(node[k - 1][1]) > 1e-14) temp = k;
  if (temp == 0) {  // the reference pauses and then reads pdt(0)
    atomicAdd(events, 1);
    return volf - 0.0;
  }
  const int m = temp - 1;  // vertices; node[m] closes the polygon
  double fx = 0.0, fy = 0.0, lx = 0.0, ly = 0.0, vol = 0.0;
  int ml = 0;
  auto add = [&](double a, double b) {
    if (ml == 0) {
      fx = a;
      fy = b;
    } else {
      vol = vol + 0.5 * (lx * b - a * ly);
    }
    lx = a;
    ly = b;
    ++ml;
  };
  double pk = m > 0 ? node[0][0] * nxf + node[0][1] * nyf + phil : 0.0;
  const double p0 = pk;
  for (int k = 0; k < m; ++k) {
    const double pn = k + 1 < m ? node[k + 1][0] * nxf + node[k + 1][1] * nyf + phil : p0;
    if (pk <= 0.0) add(node[k][0], node[k][1]);
    if (pk * pn < 0.0) {
      const double w = fabs(pk), ws = fabs(pk) + fabs(pn);
      add(node[k][0] + dv((node[k + 1][0] - node[k][0]) * w, ws),
          node[k][1] + dv((node[k + 1][1] - node[k][1]) * w, ws));
    }
    pk = pn;
  }
  if (ml > 0) vol = vol + 0.5 * (lx * fy - fx * ly);
  return volf - fabs(dv(vol, dx * dy));
}

// DistanceFluidCalculate + zriddr: true when the reference assigns phif.
__device__ bool fluid_distance(double nxss, double nyss, double phiss, double nxf, double nyf,
                               double volf, double dx, double dy, double& phif, int* events) {
  double node[9][2];
  for (int k = 0; k < 9; ++k) node[k][0] = node[k][1] = 0.0;
  const double dx2 = dx * 0.5, dy2 = dy * 0.5, tol = 1e-14, unused = -1.11e-30;
  const double d0 = dx2 * nxss - dy2 * nyss + phiss, d1 = -(dx2 * nxss) - dy2 * nyss + phiss;
  const double d2 = -(dx2 * nxss) + dy2 * nyss + phiss, d3 = dx2 * nxss + dy2 * nyss + phiss;
  int m = 0;
  auto put = [&](double a, double b) {
    node[m][0] = a;
    node[m][1] = b;
    ++m;
  };
  if (d0 >= 0.0) put(dx2, -dy2);
  if (d0 * d1 < 0.0) put(dv(dy2 * nyss - phiss, nxss), -dy2);
  if (d1 >= 0.0) put(-dx2, -dy2);
  if (d1 * d2 < 0.0) put(-dx2, dv(dx2 * nxss - phiss, nyss));
  if (d2 >= 0.0) put(-dx2, dy2);
  if (d2 * d3 < 0.0) put(dv(-(dy2 * nyss) - phiss, nxss), dy2);
  if (d3 >= 0.0) put(dx2, dy2);
  if (d3 * d0 < 0.0) put(dx2, dv(-(dx2 * nxss) - phiss, nyss));
  node[m][0] = node[0][0];  // m <= 8 above, so node[m] is in bounds
  node[m][1] = node[0][1];
  double mx0 = 0.0, mx1 = 0.0, mn0 = 0.0, mn1 = 0.0;
  {
    double maxd = -2.0 * sq(dx * dx + dy * dy), mind = 2.0 * sq(dx * dx + dy * dy);
    for (int k = 0; k < m; ++k) {
      const double t = nxf * node[k][0] + nyf * node[k][1];
      if (t > maxd) {
        maxd = t;
        mx0 = node[k][0];
        mx1 = node[k][1];
      }
      if (t < mind) {
        mind = t;
        mn0 = node[k][0];
        mn1 = node[k][1];
      }
    }
  }
  mx0 = mx0 + mx0 * nxf * kEpsi;
  mx1 = mx1 + mx1 * nyf * kEpsi;
  mn0 = mn0 - mn0 * nxf * kEpsi;
  mn1 = mn1 - mn1 * nyf * kEpsi;
  if (m == 0 || (fabs(node[0][0]) < 1e-14 && fabs(node[0][1]) < 1e-14)) atomicAdd(events, 1);
  double fl = liq_func_vol(node, nxf, nyf, volf, dx, dy, mn0, mn1, events);
  double fh = liq_func_vol(node, nxf, nyf, volf, dx, dy, mx0, mx1, events);
  if ((fl > tol && fh < -tol) || (fl < -tol && fh > tol)) {
    double xl0 = mn0, xl1 = mn1, xh0 = mx0, xh1 = mx1, a0 = unused, a1 = unused;
    for (int iter = 1; iter <= 1000; ++iter) {
      const double xm0 = 0.5 * (xl0 + xh0), xm1 = 0.5 * (xl1 + xh1);
      const double fm = liq_func_vol(node, nxf, nyf, volf, dx, dy, xm0, xm1, events);
      const double s = sq(fm * fm - fl * fh);
      if (s == 0.0) atomicAdd(events, 1);
      const double sg = copysign(1.0, fl - fh);
      const double xn0 = xm0 + dv((xm0 - xl0) * sg * fm, s);
      const double xn1 = xm1 + dv((xm1 - xl1) * sg * fm, s);
      if (sq((xn0 - a0) * (xn0 - a0) + (xn1 - a1) * (xn1 - a1)) <= tol) {
        phif = -(nxf * a0 + nyf * a1);
        return true;
      }
      a0 = xn0;
      a1 = xn1;
      const double fnew = liq_func_vol(node, nxf, nyf, volf, dx, dy, a0, a1, events);
      if (fabs(fnew) <= tol) {
        phif = -(nxf * a0 + nyf * a1);
        return true;
      }
      if (copysign(fm, fnew) != fm) {
        xl0 = xm0; xl1 = xm1; fl = fm;
        xh0 = a0; xh1 = a1; fh = fnew;
      } else if (copysign(fl, fnew) != fl) {
        xh0 = a0; xh1 = a1; fh = fnew;
      } else if (copysign(fh, fnew) != fh) {
        xl0 = a0; xl1 = a1; fl = fnew;
      } else {
        atomicAdd(events, 1);
      }
      if (sq((xh0 - xl0) * (xh0 - xl0) + (xh1 - xl1) * (xh1 - xl1)) <= tol) {
        phif = -(nxf * a0 + nyf * a1);
        return true;
      }
    }
    phif = -(nxf * a0 + nyf * a1);
    return true;
  }
  if (fl < tol && fl > -tol) {
    phif = -(nxf * mn0 + nyf * mn1);
    return true;
  }
  if (fh < tol && fh > -tol) {
    phif = -(nxf * mx0 + nyf * mx1);
    return true;
  }
  return false;
}

// The reference's body for cell (i, j) with the carried values nxx, nyy
// (read only where the body reads them); writes nxv, nyv, dis and the
// failed flag.
__device__ void ir_cell(const IrIn& c, int i, int j, double nxx, double nyy) {
  const long long a = c.at(i, j);
  const int nx = c.nx, ny = c.ny, flag = c.flag(i, j);
  const double v = c.vof[a], s = c.vofS[a];
  double diss = 0.0;
  bool assigned = true;
  if (flag) {
    if (i > 1 && i < nx && j > 1 && j < ny) {
      normal_irre(c, i, j, nxx, nyy);
    } else {
      if (i == 1) nxx = c.gx(i + 1, i, j);
      else if (i == nx) nxx = c.gx(i, i - 1, j);
      if (j == 1) nyy = c.gy(i, j + 1, j);
      else if (j == ny) nyy = c.gy(i, j, j - 1);
    }
    const double t = sq(nxx * nxx + nyy * nyy);
    if (t < 1e-14) {
      nxx = 0.0;
      nyy = 1.0;
    } else {
      nxx = dv(nxx, t);
      nyy = dv(nyy, t);
    }
    if (flag == 1)
      diss = plic_distance(v, c.dx[a], c.dy[a], nxx, nyy);
    else
      assigned = fluid_distance(c.nxs[a], c.nys[a], c.phiS[a], nxx, nyy, v, c.dx[a], c.dy[a],
                                diss, c.events);
  } else {
    nxx = 0.0;
    nyy = 1.0;
    if (1.0 - s > kVofEps) diss = (0.5 - dv(v, 1.0 - s)) * c.dy[a];
    else diss = (0.0 - v) * c.dy[a];
  }
  c.nxv[a] = nxx;
  c.nyv[a] = nyy;
  c.dis[a] = diss;
  c.failed[a] = assigned ? 0 : 1;
}

// Pass 1: every cell whose body reads no carried normal component.
// Unflagged cells take (0, 1) and the flat-interface distance here; the
// flagged cells of pass 1 go to a list for k_ir_flagged, so that this
// pass over every cell stays light (few registers, full occupancy).
__global__ void k_ir_main(IrIn c) {
  const long long total = (long long)c.nx * c.ny;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx % c.nx) + 1, j = (int)(idx / c.nx) + 1;
    if (c.flag(i, j)) {
      const bool edge_i = i == 1 || i == c.nx, edge_j = j == 1 || j == c.ny;
      if (edge_i == edge_j) c.list[atomicAdd(c.count, 1)] = (int)idx;  // else: a later pass
      continue;
    }
    const double v = c.vof[idx], s = c.vofS[idx];
    c.nxv[idx] = 0.0;
    c.nyv[idx] = 1.0;
    c.dis[idx] = 1.0 - s > kVofEps ? (0.5 - dv(v, 1.0 - s)) * c.dy[idx] : (0.0 - v) * c.dy[idx];
    c.failed[idx] = 0;
  }
}

// Pass 1's interface cells (interior cells and corners).
__global__ void k_ir_flagged(IrIn c) {
  const int n = *c.count;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int idx = c.list[k];
    ir_cell(c, idx % c.nx + 1, idx / c.nx + 1, 0.0, 0.0);
  }
}

// Passes 2 and 3: flagged cells of row ny (ROW 0) or row 1 (ROW 1),
// columns 2..nx-1, with nxx carried from the cell before.
template <int ROW>
__global__ void k_ir_row(IrIn c) {
  for (int i = 2 + blockIdx.x * blockDim.x + threadIdx.x; i <= c.nx - 1;
       i += gridDim.x * blockDim.x) {
    const int j = ROW == 0 ? c.ny : 1;
    if (!c.flag(i, j)) continue;
    const double nxx = ROW == 0 ? c.nxv[c.at(i, c.ny - 1)] : c.nxv[c.at(i - 1, c.ny)];
    ir_cell(c, i, j, nxx, 0.0);
  }
}

// Pass 4: flagged cells of columns 1 and nx, rows 2..ny-1: nyy carried down
// the column from the nearest unflagged cell (or row 1).
__global__ void k_ir_sides(IrIn c) {
  const int rows = c.ny - 2;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 2 * rows; t += gridDim.x * blockDim.x) {
    const int i = t < rows ? 1 : c.nx, j = 2 + (t < rows ? t : t - rows);
    if (!c.flag(i, j)) continue;
    int j0 = j - 1;
    while (j0 > 1 && c.flag(i, j0)) --j0;
    double nyy = c.nyv[c.at(i, j0)];
    for (int jj = j0 + 1; jj < j; ++jj) {  // flagged cells between: their normalised nyy
      const double nxx = i == 1 ? c.gx(i + 1, i, jj) : c.gx(i, i - 1, jj);
      const double tt = sq(nxx * nxx + nyy * nyy);
      nyy = tt < 1e-14 ? 1.0 : dv(nyy, tt);
    }
    ir_cell(c, i, j, 0.0, nyy);
  }
}

// Pass 5: a cell whose Ridders bracket failed keeps diss from the cell
// before it in the loop order (i outer, j inner): copy the nearest earlier
// assigned dis (0 before the first cell).
__global__ void k_ir_carry_dis(IrIn c) {
  const long long total = (long long)c.nx * c.ny;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    if (!c.failed[idx]) continue;
    int i = (int)(idx % c.nx) + 1, j = (int)(idx / c.nx) + 1;
    double d = 0.0;
    for (;;) {
      if (j > 1) --j;
      else if (i > 1) {
        --i;
        j = c.ny;
      } else {
        atomicAdd(c.events, 1);  // the reference's diss before any cell: never set
        break;
      }
      if (!c.failed[c.at(i, j)]) {
        d = c.dis[c.at(i, j)];
        break;
      }
    }
    c.dis[idx] = d;
  }
}

// ---------------------------------------------------------------------------
// Redistance (src/Clsvof_Mod.f90:1525-1708) with isinsiderect (:1921-1955).
// The reference scatters from every interface cell S (i outer, j inner) to
// the full or empty cells T within band_width = 4 cells, each update reading
// the value T holds so far.  Interface cells are never targets, so every
// target here gathers its sources itself, in the reference's order, and
// applies the same updates to the same running value: the result is the
// scatter's, bit for bit.  dmin1 / dmax1 are fmin / fmax.
// ---------------------------------------------------------------------------
constexpr int kBand = 4;

struct RdIn {
  int nx, ny;
  const double *vof, *vofS, *nxs, *nys, *phiS, *x, *y, *dx, *dy, *nxv, *nyv, *dis;
  double* phi;
  int* events;
  __device__ long long at(int i, int j) const { return (long long)(i - 1) + (long long)(j - 1) * nx; }
  __device__ bool source(int i, int j) const {
    const double v = vof[at(i, j)];
    return (0.0 + kVofEps) < v && v < (1.0 - kVofEps - vofS[at(i, j)]);
  }
};

__device__ bool inside_rect(double xp, double yp, double dx, double dy) {
  const double x1 = -0.5 * dx, y1 = 0.5 * dy, x2 = 0.5 * dx, y2 = 0.5 * dy;
  const double x3 = 0.5 * dx, y3 = -0.5 * dy, x4 = -0.5 * dx, y4 = -0.5 * dy;
  const double b1 = sq((x1 - xp) * (x1 - xp) + (y1 - yp) * (y1 - yp));
  const double b2 = sq((x2 - xp) * (x2 - xp) + (y2 - yp) * (y2 - yp));
  const double b3 = sq((x3 - xp) * (x3 - xp) + (y3 - yp) * (y3 - yp));
  const double b4 = sq((x4 - xp) * (x4 - xp) + (y4 - yp) * (y4 - yp));
  const double u1 = 0.5 * (dx + b1 + b2), u2 = 0.5 * (dy + b2 + b3);
  const double u3 = 0.5 * (dx + b3 + b4), u4 = 0.5 * (dy + b4 + b1);
  const double a1 = sq(u1 * (u1 - dx) * (u1 - b1) * (u1 - b2));
  const double a2 = sq(u2 * (u2 - dy) * (u2 - b2) * (u2 - b3));
  const double a3 = sq(u3 * (u3 - dx) * (u3 - b3) * (u3 - b4));
  const double a4 = sq(u4 * (u4 - dy) * (u4 - b4) * (u4 - b1));
  return fabs(a1 + a2 + a3 + a4 - dx * dy) < 1e-10;
}

// The reference's two guarded assignments for a target inside a cut cell.
__device__ double closer(double pa, double deuc, double vT, double sT) {
  if (fabs(deuc) < fabs(pa) && vT >= 1.0 - kVofEps - sT) pa = -fabs(deuc);
  if (fabs(deuc) < fabs(pa) && vT < kVofEps) pa = fabs(deuc);
  return pa;
}

// The reference's work for target T from source S = (i, j), T at offset
// (ii, jj) (:1551-1676): the distance candidate deuc and which of its three
// update rules applies, handed to emit(rule, deuc, dij1):
//   1  T outside the solid (vofS < epsi): pa = sign(0.5 - vof(T)) min(deuc, |pa|)
//   2  T cut by the solid, or any T when the segment test passes: the two
//      guarded assignments of closer()
//   3  T inside the solid, from a source without solid: pa = sign(dij1) deuc
//      when deuc < |pa|.
template <typename Emit>
__device__ void rd_pair(const RdIn& c, int i, int j, int ii, int jj, double vT, double sT,
                        double phiT, double xT, double yT, Emit&& emit) {
  const double tol = 1e-24;
  const long long a = c.at(i, j);
  const double dxs = c.dx[a], dys = c.dy[a], nxs = c.nxs[a], nys = c.nys[a], phs = c.phiS[a];
  const double n1 = c.nxv[a], n2 = c.nyv[a], d1 = c.dis[a];
  auto solid = [&](double px, double py) { return nxs * px + nys * py + phs; };
  const int l = ii < -1 ? -1 : (ii > 1 ? 1 : ii), m = jj < -1 ? -1 : (jj > 1 ? 1 : jj);
  double xv = dxs * (double)l * 0.5, yv = dys * (double)m * 0.5;
  if (solid(xv, yv) < 0.0) {
    if (fabs(yv) < kVofEps) {
      yv = dys * 0.5;
      if (solid(xv, yv) < 0.0) {
        yv = -dys * 0.5;
        if (solid(xv, yv) < 0.0) {
          xv = dxs * (0.0 - (double)l) * 0.5;
          if (solid(xv, yv) < 0.0) yv = dys * 0.5;
        }
      }
    } else if (fabs(xv) < kVofEps) {
      xv = dxs * 0.5;
      if (solid(xv, yv) < 0.0) {
        xv = -dxs * 0.5;
        if (solid(xv, yv) < 0.0) {
          yv = dys * (0.0 - (double)m) * 0.5;
          if (solid(xv, yv) < 0.0) xv = dxs * 0.5;
        }
      }
    } else {
      yv = dys * (0.0 - (double)m) * 0.5;
      if (solid(xv, yv) < 0.0) {
        xv = dxs * (0.0 - (double)l) * 0.5;
        yv = dys * (double)m * 0.5;
        if (solid(xv, yv) < 0.0) yv = dys * (0.0 - (double)m) * 0.5;
      }
    }
  }
  const double rx = xT - c.x[a], ry = yT - c.y[a];
  const double dvl = n1 * xv + n2 * yv + d1;
  if (dvl * copysign(1.0, phiT) <= 0.0) {
    emit(sT < kEpsi ? 1 : 2, sq((rx - xv) * (rx - xv) + (ry - yv) * (ry - yv)), 0.0);
    return;
  }
  const double dij1 = n1 * rx + n2 * ry + d1;
  const double xp = rx - dij1 * n1, yp = ry - dij1 * n2;
  const bool in = inside_rect(xp, yp, dxs, dys);
  if (in && sT < kEpsi) {
    emit(1, sq((rx - xp) * (rx - xp) + (ry - yp) * (ry - yp)), 0.0);
    return;
  }
  if (in && sT >= kEpsi && sT < 1.0 - kEpsi) {
    emit(2, sq((rx - xp) * (rx - xp) + (ry - yp) * (ry - yp)), 0.0);
    return;
  }
  if (sT >= 1.0 - kEpsi) {
    if (c.vofS[a] < kEpsi) emit(3, sq((rx - xp) * (rx - xp) + (ry - yp) * (ry - yp)), dij1);
    return;
  }
  const double xoff = fmax(fabs(xp) - 0.5 * dxs, 0.0), yoff = fmax(fabs(yp) - 0.5 * dys, 0.0);
  const double xfc = copysign(1.0, xp) * 0.5 * dxs, yfc = copysign(1.0, yp) * 0.5 * dys;
  double xs, ys;
  if (xoff * fabs(n1 + tol) >= yoff * fabs(n2 + tol)) {
    xs = xfc;
    ys = dv(d1 + n1 * xs, -n2 + tol);
  } else {
    ys = yfc;
    xs = dv(d1 + n2 * ys, -n1 + tol);
  }
  const double deuc = sq((rx - xs) * (rx - xs) + (ry - ys) * (ry - ys));
  if (solid(xs, ys) >= 0.0) emit(sT < kEpsi ? 1 : 2, deuc, 0.0);
}

// T is a target (full or empty), S a source (interface cell): disjoint sets.
__device__ bool rd_target(double vT, double sT) {
  return vT < 0.0 + kVofEps || vT >= 1.0 - kVofEps - sT;
}

// Rules 1 and 2 reduce to a minimum of deuc with a sign fixed by T, so a
// target's result does not depend on the order of its sources; rule 3 takes
// the sign of the first source (in the reference's order) reaching the
// minimum, and targets inside the solid (the only ones it applies to) keep
// the sequential order.  The pair pass: one thread per (source, offset)
// pair, the minimum by an atomic on the distance's bits (non-negative
// doubles order like their bit patterns).  key = ~0: no candidate.
// flags bit 0: a source within the band; bit 1: a rule-1 update ran.
__global__ void k_rd_sources(RdIn c, int* list, int* count) {
  const long long total = (long long)c.nx * c.ny;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx % c.nx) + 1, j = (int)(idx / c.nx) + 1;
    if (c.source(i, j)) list[atomicAdd(count, 1)] = (int)idx;
  }
}

__global__ void k_rd_pairs(RdIn c, const int* list, const int* count, unsigned long long* key,
                           unsigned* flags) {
  const long long work = (long long)(*count) * 81;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < work;
       w += (long long)gridDim.x * blockDim.x) {
    const int sidx = list[w / 81], o = (int)(w % 81);
    const int i = sidx % c.nx + 1, j = sidx / c.nx + 1;
    const int ii = o / 9 - kBand, jj = o % 9 - kBand;
    const int p = i + ii, q = j + jj;
    if (p < 1 || p > c.nx || q < 1 || q > c.ny) continue;
    const long long t = c.at(p, q);
    const double vT = c.vof[t], sT = c.vofS[t];
    if (!rd_target(vT, sT)) continue;
    atomicOr(&flags[t], 1u);
    if (sT >= 1.0 - kEpsi) continue;  // inside the solid: the sequential path
    rd_pair(c, i, j, ii, jj, vT, sT, c.phi[t], c.x[t], c.y[t],
            [&](int rule, double deuc, double) {
              if (rule == 1) {
                atomicOr(&flags[t], 2u);
                if (deuc == deuc)
                  atomicMin(&key[t], (unsigned long long)__double_as_longlong(deuc));
              } else if (deuc < 1e4) {  // rule 2: an update needs deuc < |pa| <= 1e4
                atomicMin(&key[t], (unsigned long long)__double_as_longlong(deuc));
              }
            });
  }
}

constexpr int kRdTx = 32, kRdTy = 8;

// One thread per cell (i fastest within a 32 x 8 tile).  Sources take their
// PLIC distance; targets outside the solid read the pair pass's minimum;
// targets inside the solid run their sources in the reference's order (the
// source flags of the tile and its 4-cell halo staged in shared memory).
__global__ void __launch_bounds__(kRdTx* kRdTy)
    k_redistance(RdIn c, const unsigned long long* key, const unsigned* flags) {
  __shared__ unsigned char src[kRdTy + 2 * kBand][kRdTx + 2 * kBand];
  const int i0 = blockIdx.x * kRdTx, j0 = blockIdx.y * kRdTy;
  const int tid = threadIdx.y * kRdTx + threadIdx.x;
  for (int k = tid; k < (kRdTx + 2 * kBand) * (kRdTy + 2 * kBand); k += kRdTx * kRdTy) {
    const int ti = k % (kRdTx + 2 * kBand), tj = k / (kRdTx + 2 * kBand);
    const int i = i0 + ti - kBand + 1, j = j0 + tj - kBand + 1;  // 1-based
    src[tj][ti] = (i >= 1 && i <= c.nx && j >= 1 && j <= c.ny && c.source(i, j)) ? 1 : 0;
  }
  __syncthreads();
  const int p = i0 + threadIdx.x + 1, q = j0 + threadIdx.y + 1;
  if (p > c.nx || q > c.ny) return;
  const long long t = c.at(p, q);
  const double vT = c.vof[t], sT = c.vofS[t];
  const double h = sq(c.dx[t] * c.dx[t] + c.dy[t] * c.dy[t]);
  double out = c.phi[t];
  bool fix = false;
  double pa = 1e4;
  if (src[threadIdx.y + kBand][threadIdx.x + kBand]) {
    pa = c.dis[t];
    fix = true;
  } else if (rd_target(vT, sT) && (flags[t] & 1u)) {
    if (sT >= 1.0 - kEpsi) {
      const double phiT = out, xT = c.x[t], yT = c.y[t];
      for (int di = -kBand; di <= kBand; ++di)  // sources in the reference's order
        for (int dj = -kBand; dj <= kBand; ++dj) {
          if (!src[threadIdx.y + kBand + dj][threadIdx.x + kBand + di]) continue;
          rd_pair(c, p + di, q + dj, -di, -dj, vT, sT, phiT, xT, yT,
                  [&](int rule, double deuc, double dij1) {
                    if (rule == 1) pa = copysign(1.0, 0.5 - vT) * fmin(deuc, fabs(pa));
                    else if (rule == 2) pa = closer(pa, deuc, vT, sT);
                    else if (fabs(deuc) < fabs(pa)) pa = copysign(1.0, dij1) * deuc;
                  });
        }
    } else {
      const unsigned long long k = key[t];
      const double mn = k == ~0ull ? 1e4 : __longlong_as_double((long long)k);
      if (sT < kEpsi) {  // rule 1
        if (flags[t] & 2u) pa = copysign(1.0, 0.5 - vT) * fmin(mn, 1e4);
      } else if (k != ~0ull) {  // rule 2: the smallest deuc below 1e4, signed by T
        pa = vT >= 1.0 - kVofEps - sT ? -mn : mn;
      }
    }
    fix = !(pa > 9.999e3);
  }
  if (fix) {
    if (pa > 1e3) atomicAdd(c.events, 1);  // the reference pauses here
    out = pa;
  } else {
    if (vT <= kVofEps) out = (double)(kBand + 1) * h;
    else if (vT >= (1.0 - kVofEps - sT)) out = -(double)(kBand + 1) * h;
  }
  if (vT < kVofEps && out < -kVofEps && sT < 1.0 - kEpsi) atomicAdd(c.events, 1);
  c.phi[t] = out;
}

// ---------------------------------------------------------------------------
// Coupled_LS_VOF (src/Clsvof_Mod.f90:730-959) between the sweeps: the
// updates after the first and the second sweep of a sub-step and
// Boundary_Condition (:961-973).
// ---------------------------------------------------------------------------
struct StepIn {
  int nx, ny;
  double dtv;
  const double *vofS, *dx, *dy, *aE, *aW, *aN, *aS, *ue, *ve;
  __device__ double vel(int dir, int i, int j) const {  // ue(i,j) / ve(i,j), 1-based cells
    return dir == SCF_LS_X ? ue[(long long)i + (long long)(j - 1) * (nx + 1)]
                           : ve[(long long)(i - 1) + (long long)j * nx];
  }
  __device__ double edge(const double* a, int i, int j) const {
    return a[(long long)i + (long long)j * (nx + 2)];
  }
  // ue(i,j) E - ue(i-1,j) W  (X),  ve(i,j) N - ve(i,j-1) S  (Y)
  __device__ double div(int dir, int i, int j) const {
    return dir == SCF_LS_X ? vel(dir, i, j) * edge(aE, i, j) - vel(dir, i - 1, j) * edge(aW, i, j)
                           : vel(dir, i, j) * edge(aN, i, j) - vel(dir, i, j - 1) * edge(aS, i, j);
  }
};

// After the first sweep of a sub-step (direction DIR): temvf and temls
// divided by the cell's net outflow factor; vof (clipped) and phi from them.
template <int DIR>
__global__ void k_after_first(StepIn c, double* tv, double* tl, double* vof, double* phi) {
  const long long total = (long long)c.nx * c.ny;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx % c.nx) + 1, j = (int)(idx / c.nx) + 1;
    const double s = c.vofS[idx], h = DIR == SCF_LS_X ? c.dx[idx] : c.dy[idx];
    const double den = (1.0 - s + kTolDeno) - dv(c.dtv, h) * c.div(DIR, i, j);
    const double a = dv(tv[idx], den), b = dv(tl[idx], den);
    tv[idx] = a;
    tl[idx] = b;
    double v = a * (1.0 - s);
    if (v >= 1.0 - kVofEps - s) v = 1.0 - s;
    if (v < kVofEps) v = 0.0;
    vof[idx] = v;
    phi[idx] = b;
  }
}

// After the second sweep (direction DIR): the first sweep's values (t1v,
// t1l) times this direction's net outflow added; vof and phi from them.
template <int DIR>
__global__ void k_after_second(StepIn c, const double* t1v, const double* t1l, double* tv,
                               double* tl, double* vof, double* phi) {
  const long long total = (long long)c.nx * c.ny;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx % c.nx) + 1, j = (int)(idx / c.nx) + 1;
    const double s = c.vofS[idx], h = DIR == SCF_LS_X ? c.dx[idx] : c.dy[idx];
    const double d = c.div(DIR, i, j);
    const double a = tv[idx] + dv(c.dtv, h) * t1v[idx] * d;
    const double b = tl[idx] + dv(c.dtv, h) * t1l[idx] * d;
    tv[idx] = a;
    tl[idx] = b;
    vof[idx] = a;
    if (s < 1.0 - kEpsi) phi[idx] = dv(b, 1.0 - s);
  }
}

// Boundary_Condition on two fields: rows 1 and ny copy rows 2 and ny-1,
// then columns 1 and nx copy columns 2 and nx-1 (the corners so take the
// diagonal interior cell).  Reads interior cells only.
__global__ void k_boundary(int nx, int ny, double* a, double* b) {
  const int per = 2 * nx + 2 * (ny - 2);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 2 * per; t += gridDim.x * blockDim.x) {
    double* v = t < per ? a : b;
    const int e = t < per ? t : t - per;
    int i, j;
    if (e < nx) { i = e + 1; j = 1; }
    else if (e < 2 * nx) { i = e - nx + 1; j = ny; }
    else if (e < 2 * nx + ny - 2) { i = 1; j = e - 2 * nx + 2; }
    else { i = nx; j = e - (2 * nx + ny - 2) + 2; }
    const int si = i == 1 ? 2 : (i == nx ? nx - 1 : i);
    const int sj = j == 1 ? 2 : (j == ny ? ny - 1 : j);
    v[(long long)(i - 1) + (long long)(j - 1) * nx] = v[(long long)(si - 1) + (long long)(sj - 1) * nx];
  }
}

}  // namespace
}  // namespace scf

using namespace scf;

namespace {

// One sweep call: ncnt input arrays (host or device), outputs temvf and/or
// temls (in/out), one kernel.
template <typename Launch>
int run_sweep(int n_in, const double* const* arr, const size_t* cnt, double* const* outs,
              int n_out, size_t n1, bool dev, int device, double* ms, Launch&& launch) {
  const auto t0 = std::chrono::steady_clock::now();
  if (cudaSetDevice(device) != cudaSuccess) return SCF_ERR_CUDA;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return SCF_ERR_CUDA;
  void* mem = nullptr;
  int rc = SCF_OK;
  const double* d[32];
  double* o[2] = {outs[0], n_out > 1 ? outs[1] : nullptr};
  do {
    if (!dev) {
      size_t tot = n1 * n_out;
      for (int a = 0; a < n_in; ++a) tot += cnt[a];
      if (cudaMalloc(&mem, tot * 8) != cudaSuccess) {
        rc = SCF_ERR_NOMEM;
        break;
      }
      double* p = static_cast<double*>(mem);
      for (int a = 0; a < n_in && rc == SCF_OK; ++a) {
        if (cudaMemcpyAsync(p, arr[a], cnt[a] * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
          rc = SCF_ERR_CUDA;
        d[a] = p;
        p += cnt[a];
      }
      for (int b = 0; b < n_out && rc == SCF_OK; ++b) {
        if (cudaMemcpyAsync(p, outs[b], n1 * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
          rc = SCF_ERR_CUDA;
        o[b] = p;
        p += n1;
      }
      if (rc) break;
    } else {
      for (int a = 0; a < n_in; ++a) d[a] = arr[a];
    }
    launch(d, o, s);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    for (int b = 0; b < n_out && !dev && rc == SCF_OK; ++b)
      if (cudaMemcpyAsync(outs[b], o[b], n1 * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        rc = SCF_ERR_CUDA;
  } while (false);
  if (cudaStreamSynchronize(s) != cudaSuccess && rc == SCF_OK) rc = SCF_ERR_CUDA;
  if (mem) cudaFree(mem);
  cudaStreamDestroy(s);
  if (ms)
    *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

unsigned grid_for(size_t n1) {
  return (unsigned)((n1 + 255) / 256 < 152 * 8 ? (n1 + 255) / 256 : 152 * 8);
}

}  // namespace

extern "C" int scf_ls_sweep(int dir, int nx, int ny, const scf_ls_fields* f, double dtv,
                            double* temls, int flags, int device, double* ms) {
  if ((dir != SCF_LS_X && dir != SCF_LS_Y) || nx < 3 || ny < 3 || !f || !temls)
    return SCF_ERR_ARG;
  const double* arr[12] = {f->phi, f->vofS, f->dx, f->dy, f->x,  f->y,
                           f->aE,  f->aW,   f->aN, f->aS, f->ue, f->ve};
  for (auto a : arr)
    if (!a) return SCF_ERR_ARG;
  const size_t n1 = (size_t)nx * ny, n0 = (size_t)(nx + 2) * (ny + 2);
  const size_t cnt[12] = {n1, n1, n1, n1, n1, n1, n0, n0, n0, n0, (size_t)(nx + 1) * ny,
                          (size_t)nx * (ny + 1)};
  double* outs[1] = {temls};
  return run_sweep(12, arr, cnt, outs, 1, n1, (flags & SCF_LS_DEVICE_PTRS) != 0, device, ms,
                   [&](const double* const* d, double* const* o, cudaStream_t s) {
                     const LsIn in{nx,   ny,   dtv,  d[0], d[1], d[2],  d[3],
                                   d[4], d[5], d[6], d[7], d[8], d[9], d[10], d[11]};
                     if (dir == SCF_LS_X) k_ls_sweep<SCF_LS_X><<<grid_for(n1), 256, 0, s>>>(in, o[0]);
                     else k_ls_sweep<SCF_LS_Y><<<grid_for(n1), 256, 0, s>>>(in, o[0]);
                   });
}

extern "C" int scf_clsvof_sweep(int dir, int nx, int ny, const scf_ls_fields* f,
                                const scf_vof_fields* v, const scf_vof_wave* wave, double dtv,
                                double* temvf, double* temls, int flags, int device, double* ms) {
  if ((dir != SCF_LS_X && dir != SCF_LS_Y) || nx < 1 || ny < 1 || !f || !v || !temvf)
    return SCF_ERR_ARG;
  const bool ls = temls != nullptr;
  if (ls && (nx < 3 || ny < 3)) return SCF_ERR_ARG;
  if ((ny + kSwTy - 1) / kSwTy > 65535) return SCF_ERR_ARG;  // grid rows
  // inputs: the level-set fields (phi only with temls), then the VOF fields
  const double* arr[19] = {f->phi, f->vofS, f->dx, f->dy, f->x, f->y, f->aE, f->aW, f->aN,
                           f->aS,  f->ue,   f->ve, v->vof, v->nx, v->ny, v->dis, v->nxs,
                           v->nys, v->phiS};
  for (int a = 0; a < 19; ++a)
    if (!arr[a] && (a != 0 || ls)) return SCF_ERR_ARG;
  const bool dev = (flags & SCF_LS_DEVICE_PTRS) != 0;
  const size_t n1 = (size_t)nx * ny, n0 = (size_t)(nx + 2) * (ny + 2);
  size_t cnt[19] = {n1, n1, n1, n1, n1, n1, n0, n0, n0, n0, (size_t)(nx + 1) * ny,
                    (size_t)nx * (ny + 1), n1, n1, n1, n1, n1, n1, n1};
  // X inlet: Depthw + etau, etau = Amp0 sin(kw xwu - omew (NondiT + k dtv)),
  // xwu = x(1,1) - dx(1,1)/2 (src/Clsvof_Mod.f90:1005, 1057-1068), on the host
  double level = -INFINITY;
  if (dir == SCF_LS_X && wave) {
    double x11 = 0.0, dx11 = 0.0;
    if (dev) {
      if (cudaSetDevice(device) != cudaSuccess ||
          cudaMemcpy(&x11, f->x, 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
          cudaMemcpy(&dx11, f->dx, 8, cudaMemcpyDeviceToHost) != cudaSuccess)
        return SCF_ERR_CUDA;
    } else {
      x11 = f->x[0];
      dx11 = f->dx[0];
    }
    const double xwu = x11 - dx11 / 2.0;
    const double etau =
        wave->amp0 * std::sin(wave->kw * xwu - wave->omew * (wave->nondit + (double)wave->k * dtv));
    level = wave->depthw + etau;
  }
  // without temls, phi is not read: stand in another array of the same size
  if (!ls) arr[0] = arr[1];
  double* outs[2] = {temvf, temls};
  return run_sweep(19, arr, cnt, outs, ls ? 2 : 1, n1, dev, device, ms,
                   [&](const double* const* d, double* const* o, cudaStream_t s) {
                     const LsIn lin{nx,   ny,   dtv,  d[0], d[1], d[2],  d[3],
                                    d[4], d[5], d[6], d[7], d[8], d[9], d[10], d[11]};
                     const VofIn vin{nx,    ny,    dtv,   level, d[1],  d[2],  d[3],
                                     d[5],  d[6],  d[7],  d[8],  d[9],  d[10], d[11],
                                     d[12], d[13], d[14], d[15], d[16], d[17], d[18]};
                     const dim3 g((unsigned)((nx + kSwTx - 1) / kSwTx),
                                  (unsigned)((ny + kSwTy - 1) / kSwTy)),
                         b(kSwTx, kSwTy);
                     if (dir == SCF_LS_X) {
                       if (ls) k_clsvof_sweep<SCF_LS_X, true><<<g, b, 0, s>>>(vin, lin, o[0], o[1]);
                       else k_clsvof_sweep<SCF_LS_X, false><<<g, b, 0, s>>>(vin, lin, o[0], o[1]);
                     } else {
                       if (ls) k_clsvof_sweep<SCF_LS_Y, true><<<g, b, 0, s>>>(vin, lin, o[0], o[1]);
                       else k_clsvof_sweep<SCF_LS_Y, false><<<g, b, 0, s>>>(vin, lin, o[0], o[1]);
                     }
                   });
}

extern "C" int scf_interface_reconstruct(int nx, int ny, const scf_ir_fields* f, double* nxv,
                                         double* nyv, double* dis, int* events, int flags,
                                         int device, double* ms) {
  if (nx < 3 || ny < 3 || !f || !nxv || !nyv || !dis) return SCF_ERR_ARG;
  const double* arr[10] = {f->vof, f->vofS, f->phi, f->nxs, f->nys,
                           f->phiS, f->x, f->y, f->dx, f->dy};
  for (auto a : arr)
    if (!a) return SCF_ERR_ARG;
  const auto t0 = std::chrono::steady_clock::now();
  if (cudaSetDevice(device) != cudaSuccess) return SCF_ERR_CUDA;
  const bool dev = (flags & SCF_LS_DEVICE_PTRS) != 0;
  const size_t n1 = (size_t)nx * ny;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return SCF_ERR_CUDA;
  void* mem = nullptr;
  int rc = SCF_OK;
  // scratch: the event counter (16 B), the failed flags (n1 B); host mode
  // adds the 10 inputs and 3 outputs
  // scratch: the event counter and the list count (16 B), the failed flags
  // (n1 B), the list (n1 ints); host mode adds the 10 inputs and 3 outputs
  const size_t flags_b = ((n1 + 15) / 16) * 16;
  const size_t scratch = 16 + flags_b + ((n1 * 4 + 15) / 16) * 16;
  const size_t bytes = scratch + (dev ? 0 : 13 * n1 * 8);
  int h_events = 0;
  do {
    if (cudaMalloc(&mem, bytes) != cudaSuccess) {
      rc = SCF_ERR_NOMEM;
      break;
    }
    char* base = static_cast<char*>(mem);
    int* d_events = reinterpret_cast<int*>(base);
    unsigned char* failed = reinterpret_cast<unsigned char*>(base + 16);
    int* list = reinterpret_cast<int*>(base + 16 + flags_b);
    const double* d[10];
    double* o[3] = {nxv, nyv, dis};
    if (cudaMemsetAsync(d_events, 0, 16, s) != cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    if (!dev) {
      double* p = reinterpret_cast<double*>(base + scratch);
      for (int a = 0; a < 10 && rc == SCF_OK; ++a) {
        if (cudaMemcpyAsync(p, arr[a], n1 * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
          rc = SCF_ERR_CUDA;
        d[a] = p;
        p += n1;
      }
      for (int b = 0; b < 3; ++b) {
        o[b] = p;
        p += n1;
      }
      if (rc) break;
    } else {
      for (int a = 0; a < 10; ++a) d[a] = arr[a];
    }
    const IrIn in{nx,   ny,   d[0], d[1], d[2], d[3], d[4], d[5], d[6],   d[7],
                  d[8], d[9], o[0], o[1], o[2], failed, d_events, list, d_events + 2};
    const unsigned g = grid_for(n1);
    k_ir_main<<<g, 256, 0, s>>>(in);
    k_ir_flagged<<<152 * 2, 128, 0, s>>>(in);
    note_launch();
    note_launch();
    const unsigned gr = (unsigned)((nx + 127) / 128), gs = (unsigned)((2 * ny + 127) / 128);
    k_ir_row<0><<<gr, 128, 0, s>>>(in);
    note_launch();
    k_ir_row<1><<<gr, 128, 0, s>>>(in);
    note_launch();
    k_ir_sides<<<gs, 128, 0, s>>>(in);
    note_launch();
    k_ir_carry_dis<<<g, 256, 0, s>>>(in);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    if (cudaMemcpyAsync(&h_events, d_events, sizeof(int), cudaMemcpyDeviceToHost, s) !=
        cudaSuccess)
      rc = SCF_ERR_CUDA;
    for (int b = 0; b < 3 && !dev && rc == SCF_OK; ++b) {
      double* hb = b == 0 ? nxv : b == 1 ? nyv : dis;
      if (cudaMemcpyAsync(hb, o[b], n1 * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        rc = SCF_ERR_CUDA;
    }
  } while (false);
  if (cudaStreamSynchronize(s) != cudaSuccess && rc == SCF_OK) rc = SCF_ERR_CUDA;
  if (mem) cudaFree(mem);
  cudaStreamDestroy(s);
  if (events) *events = h_events;
  if (ms)
    *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

namespace {

// Redistance's scratch: the per-cell minimum key (8 B), flags (4 B) and
// source list (4 B), and the source count.
size_t rd_scratch_bytes(size_t n1) { return 16 + n1 * 16; }

cudaError_t launch_redistance(const RdIn& in, void* scratch, size_t n1, cudaStream_t s) {
  char* b = static_cast<char*>(scratch);
  int* count = reinterpret_cast<int*>(b);
  unsigned long long* key = reinterpret_cast<unsigned long long*>(b + 16);
  unsigned* flags = reinterpret_cast<unsigned*>(b + 16 + n1 * 8);
  int* list = reinterpret_cast<int*>(b + 16 + n1 * 12);
  cudaError_t e = cudaMemsetAsync(count, 0, 16, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(key, 0xff, n1 * 8, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, n1 * 4, s);
  if (e != cudaSuccess) return e;
  k_rd_sources<<<grid_for(n1), 256, 0, s>>>(in, list, count);
  k_rd_pairs<<<152 * 8, 256, 0, s>>>(in, list, count, key, flags);
  const dim3 grid((unsigned)((in.nx + kRdTx - 1) / kRdTx), (unsigned)((in.ny + kRdTy - 1) / kRdTy));
  k_redistance<<<grid, dim3(kRdTx, kRdTy), 0, s>>>(in, key, flags);
  for (int q = 0; q < 3; ++q) note_launch();
  return cudaGetLastError();
}

}  // namespace

extern "C" int scf_redistance(int nx, int ny, const scf_rd_fields* f, double* phi, int* events,
                              int flags, int device, double* ms) {
  if (nx < 1 || ny < 1 || !f || !phi) return SCF_ERR_ARG;
  if ((ny + kRdTy - 1) / kRdTy > 65535) return SCF_ERR_ARG;  // grid rows
  const double* arr[12] = {f->vof, f->vofS, f->nxs, f->nys, f->phiS, f->x,
                           f->y,   f->dx,   f->dy,  f->nx,  f->ny,   f->dis};
  for (auto a : arr)
    if (!a) return SCF_ERR_ARG;
  const auto t0 = std::chrono::steady_clock::now();
  if (cudaSetDevice(device) != cudaSuccess) return SCF_ERR_CUDA;
  const bool dev = (flags & SCF_LS_DEVICE_PTRS) != 0;
  const size_t n1 = (size_t)nx * ny;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return SCF_ERR_CUDA;
  void* mem = nullptr;
  int rc = SCF_OK, h_events = 0;
  const size_t bytes = 16 + rd_scratch_bytes(n1) + (dev ? 0 : 13 * n1 * 8);
  do {
    if (cudaMalloc(&mem, bytes) != cudaSuccess) {
      rc = SCF_ERR_NOMEM;
      break;
    }
    int* d_events = static_cast<int*>(mem);
    if (cudaMemsetAsync(d_events, 0, 16, s) != cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    void* rd_scratch = static_cast<char*>(mem) + 16;
    const double* d[12];
    double* dphi = phi;
    if (!dev) {
      double* p = reinterpret_cast<double*>(static_cast<char*>(mem) + 16 + rd_scratch_bytes(n1));
      for (int a = 0; a < 12 && rc == SCF_OK; ++a) {
        if (cudaMemcpyAsync(p, arr[a], n1 * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
          rc = SCF_ERR_CUDA;
        d[a] = p;
        p += n1;
      }
      dphi = p;
      if (rc == SCF_OK &&
          cudaMemcpyAsync(dphi, phi, n1 * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
        rc = SCF_ERR_CUDA;
      if (rc) break;
    } else {
      for (int a = 0; a < 12; ++a) d[a] = arr[a];
    }
    const RdIn in{nx,   ny,   d[0], d[1], d[2],  d[3],  d[4], d[5],
                  d[6], d[7], d[8], d[9], d[10], d[11], dphi, d_events};
    if (launch_redistance(in, rd_scratch, n1, s) != cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    if (cudaGetLastError() != cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    if (cudaMemcpyAsync(&h_events, d_events, sizeof(int), cudaMemcpyDeviceToHost, s) !=
        cudaSuccess)
      rc = SCF_ERR_CUDA;
    if (rc == SCF_OK && !dev &&
        cudaMemcpyAsync(phi, dphi, n1 * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess)
      rc = SCF_ERR_CUDA;
  } while (false);
  if (cudaStreamSynchronize(s) != cudaSuccess && rc == SCF_OK) rc = SCF_ERR_CUDA;
  if (mem) cudaFree(mem);
  cudaStreamDestroy(s);
  if (events) *events = h_events;
  if (ms)
    *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

namespace {

void launch_reconstruct(const IrIn& in, size_t n1, cudaStream_t s) {
  const unsigned g = grid_for(n1);
  const unsigned gr = (unsigned)((in.nx + 127) / 128), gs = (unsigned)((2 * in.ny + 127) / 128);
  cudaMemsetAsync(in.count, 0, sizeof(int), s);
  k_ir_main<<<g, 256, 0, s>>>(in);
  k_ir_flagged<<<152 * 2, 128, 0, s>>>(in);
  k_ir_row<0><<<gr, 128, 0, s>>>(in);
  k_ir_row<1><<<gr, 128, 0, s>>>(in);
  k_ir_sides<<<gs, 128, 0, s>>>(in);
  k_ir_carry_dis<<<g, 256, 0, s>>>(in);
  for (int q = 0; q < 6; ++q) note_launch();
}

}  // namespace

extern "C" int scf_clsvof_step(int nx, int ny, const scf_clsvof_fields* f,
                               const scf_vof_wave* wave, double dt, double* vof, double* phi,
                               double* nxv, double* nyv, double* dis, int* events, int flags,
                               int device, double* ms) {
  if (nx < 3 || ny < 3 || !f || !vof || !phi || !nxv || !nyv || !dis) return SCF_ERR_ARG;
  if ((ny + kSwTy - 1) / kSwTy > 65535) return SCF_ERR_ARG;
  const double* arr[14] = {f->vofS, f->nxs, f->nys, f->phiS, f->x,  f->y,  f->dx,
                           f->dy,   f->aE,  f->aW,  f->aN,   f->aS, f->ue, f->ve};
  for (auto a : arr)
    if (!a) return SCF_ERR_ARG;
  const auto t0 = std::chrono::steady_clock::now();
  if (cudaSetDevice(device) != cudaSuccess) return SCF_ERR_CUDA;
  const bool dev = (flags & SCF_LS_DEVICE_PTRS) != 0;
  const size_t n1 = (size_t)nx * ny, n0 = (size_t)(nx + 2) * (ny + 2);
  const size_t cnt[14] = {n1, n1, n1, n1, n1, n1, n1, n1, n0, n0, n0, n0,
                          (size_t)(nx + 1) * ny, (size_t)nx * (ny + 1)};
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return SCF_ERR_CUDA;
  void* mem = nullptr;
  int rc = SCF_OK, h_events = 0;
  // scratch: events (16 B), failed flags, 4 sweep fields; host mode adds the
  // 14 inputs and the 5 in/out fields
  const size_t flags_b = ((n1 + 15) / 16) * 16;
  size_t in_n = 0;
  for (size_t c : cnt) in_n += c;
  const size_t bytes =
      16 + flags_b + rd_scratch_bytes(n1) + 4 * n1 * 8 + (dev ? 0 : (in_n + 5 * n1) * 8);
  do {
    if (cudaMalloc(&mem, bytes) != cudaSuccess) {
      rc = SCF_ERR_NOMEM;
      break;
    }
    char* base = static_cast<char*>(mem);
    int* d_events = reinterpret_cast<int*>(base);
    unsigned char* failed = reinterpret_cast<unsigned char*>(base + 16);
    void* rd_scratch = base + 16 + flags_b;
    double* w = reinterpret_cast<double*>(base + 16 + flags_b + rd_scratch_bytes(n1));
    double *tvx = w, *tvy = w + n1, *tlx = w + 2 * n1, *tly = w + 3 * n1;
    double* p = w + 4 * n1;
    const double* d[14];
    double* io[5] = {vof, phi, nxv, nyv, dis};
    if (cudaMemsetAsync(d_events, 0, 16, s) != cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    if (!dev) {
      for (int a = 0; a < 14 && rc == SCF_OK; ++a) {
        if (cudaMemcpyAsync(p, arr[a], cnt[a] * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
          rc = SCF_ERR_CUDA;
        d[a] = p;
        p += cnt[a];
      }
      for (int b = 0; b < 5 && rc == SCF_OK; ++b) {
        if (b < 2 && cudaMemcpyAsync(p, io[b], n1 * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
          rc = SCF_ERR_CUDA;
        io[b] = p;
        p += n1;
      }
      if (rc) break;
    } else {
      for (int a = 0; a < 14; ++a) d[a] = arr[a];
    }
    double* dvof = io[0];
    double* dp = io[1];
    // the X inlet's level per sub-step, on the host as in X_Sweep
    double x11 = 0.0, dx11 = 0.0;
    if (wave) {
      if (dev) {
        if (cudaMemcpy(&x11, f->x, 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(&dx11, f->dx, 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
          rc = SCF_ERR_CUDA;
          break;
        }
      } else {
        x11 = f->x[0];
        dx11 = f->dx[0];
      }
    }
    const int nv = 6;
    const double dtv = dt / (double)nv;
    // the reconstruction's list shares Redistance's source list (never in use together)
    int* ir_list = reinterpret_cast<int*>(static_cast<char*>(rd_scratch) + 16 + n1 * 12);
    const IrIn irc{nx,   ny,   dvof,  d[0],  dp,    d[1],   d[2],     d[3],    d[4],        d[5],
                   d[6], d[7], io[2], io[3], io[4], failed, d_events, ir_list, d_events + 2};
    const LsIn lin{nx,   ny,   dtv,  dp,   d[0],  d[6],  d[7],  d[4],
                   d[5], d[8], d[9], d[10], d[11], d[12], d[13]};
    const StepIn st{nx, ny, dtv, d[0], d[6], d[7], d[8], d[9], d[10], d[11], d[12], d[13]};
    const dim3 gsw((unsigned)((nx + kSwTx - 1) / kSwTx), (unsigned)((ny + kSwTy - 1) / kSwTy)),
        bsw(kSwTx, kSwTy);
    const unsigned g = grid_for(n1);
    const unsigned gb = (unsigned)((2 * (2 * nx + 2 * (ny - 2)) + 255) / 256);
    auto sweep = [&](int dir, int k, double* tv, double* tl) {
      launch_reconstruct(irc, n1, s);
      double level = -INFINITY;
      if (dir == SCF_LS_X && wave) {
        const double xwu = x11 - dx11 / 2.0;
        level = wave->depthw +
                wave->amp0 * std::sin(wave->kw * xwu - wave->omew * (wave->nondit + (double)k * dtv));
      }
      const VofIn vin{nx,    ny,    dtv,   level, d[0],  d[6],  d[7],  d[5],  d[8],  d[9], d[10],
                      d[11], d[12], d[13], dvof,    io[2], io[3], io[4], d[1],  d[2],  d[3]};
      if (dir == SCF_LS_X) k_clsvof_sweep<SCF_LS_X, true><<<gsw, bsw, 0, s>>>(vin, lin, tv, tl);
      else k_clsvof_sweep<SCF_LS_Y, true><<<gsw, bsw, 0, s>>>(vin, lin, tv, tl);
      note_launch();
    };
    for (int k = 1; k <= nv && rc == SCF_OK; ++k) {
      const int first = k % 2 == 1 ? SCF_LS_X : SCF_LS_Y;
      double *tv1 = first == SCF_LS_X ? tvx : tvy, *tl1 = first == SCF_LS_X ? tlx : tly;
      double *tv2 = first == SCF_LS_X ? tvy : tvx, *tl2 = first == SCF_LS_X ? tly : tlx;
      if (cudaMemcpyAsync(tv1, dvof, n1 * 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
          cudaMemcpyAsync(tl1, dp, n1 * 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
        rc = SCF_ERR_CUDA;
        break;
      }
      sweep(first, k, tv1, tl1);
      if (first == SCF_LS_X) k_after_first<SCF_LS_X><<<g, 256, 0, s>>>(st, tv1, tl1, dvof, dp);
      else k_after_first<SCF_LS_Y><<<g, 256, 0, s>>>(st, tv1, tl1, dvof, dp);
      k_boundary<<<gb, 256, 0, s>>>(nx, ny, dvof, dp);
      note_launch();
      note_launch();
      if (cudaMemcpyAsync(tv2, dvof, n1 * 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
          cudaMemcpyAsync(tl2, dp, n1 * 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
        rc = SCF_ERR_CUDA;
        break;
      }
      const int second = first == SCF_LS_X ? SCF_LS_Y : SCF_LS_X;
      sweep(second, k, tv2, tl2);
      if (second == SCF_LS_Y)
        k_after_second<SCF_LS_Y><<<g, 256, 0, s>>>(st, tv1, tl1, tv2, tl2, dvof, dp);
      else
        k_after_second<SCF_LS_X><<<g, 256, 0, s>>>(st, tv1, tl1, tv2, tl2, dvof, dp);
      k_boundary<<<gb, 256, 0, s>>>(nx, ny, dvof, dp);
      note_launch();
      note_launch();
      launch_reconstruct(irc, n1, s);
      const RdIn rd{nx,   ny,   dvof,   d[0], d[1],  d[2],  d[3],  d[4],
                    d[5], d[6], d[7], io[2], io[3], io[4], dp,    d_events};
      if (launch_redistance(rd, rd_scratch, n1, s) != cudaSuccess) {
        rc = SCF_ERR_CUDA;
        break;
      }
    }
    if (rc) break;
    if (cudaGetLastError() != cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    if (cudaMemcpyAsync(&h_events, d_events, sizeof(int), cudaMemcpyDeviceToHost, s) !=
        cudaSuccess)
      rc = SCF_ERR_CUDA;
    double* host_out[5] = {vof, phi, nxv, nyv, dis};
    for (int b = 0; b < 5 && !dev && rc == SCF_OK; ++b)
      if (cudaMemcpyAsync(host_out[b], io[b], n1 * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        rc = SCF_ERR_CUDA;
  } while (false);
  if (cudaStreamSynchronize(s) != cudaSuccess && rc == SCF_OK) rc = SCF_ERR_CUDA;
  if (mem) cudaFree(mem);
  cudaStreamDestroy(s);
  if (events) *events = h_events;
  if (ms)
    *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}
