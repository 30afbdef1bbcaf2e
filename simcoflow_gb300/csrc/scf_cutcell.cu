// scf_cutcell.cu -- the per-step cut-cell geometry of all three cell families
// on the GPU (include/scf_cutcell.h): Grid_Preprocess and NewCellFace
// (src/Cutcell_Mod.f90:18-725).
//
// Every loop of those routines that touches each element from one iteration
// only runs as one thread per cell; the P family's order-dependent
// solid/degenerate-cell rule, exchange cells and numbering come from the
// projection's geometry pipeline (geometry_build, scf_geom.cu).  This file
// is compiled without FMA contraction (-fmad=false): every expression rounds
// each multiply and add on its own, in the reference's order, so plain C++
// arithmetic here is the reference's IEEE FP64 arithmetic.
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/scf_cutcell.h"
#include "../../include/scf_proj.h"
#include "scf_geom_gpu.cuh"
#include "scf_internal.cuh"

namespace scf {
namespace {

constexpr double kEpsF = 1.0e-2, kRnd = 1.0e-24;  // epsiF, Roundoff (kEpsi = epsi)

// device views of one family
struct Fam {
  int nx, ny;
  const double *dx, *dy, *x, *y, *phiS;  // grid and raw level set (nx,ny)
  double *vofS, *nxS, *nyS;              // (nx,ny), changed by the rules
  double *aE, *aW, *aN, *aS;             // (nx+2,ny+2)
  double *FCE, *FCN;                     // (nx+2,ny+2,2)
  double *FCW, *FCS;                     // (nx,ny,2) scratch
  double *cent;                          // (nx,ny,2)
  double *WlLh, *delh;                   // (nx,ny)
  int32_t *posnu, *moex, *msce;          // (nx+2,ny+2), (nx,ny), (nx,ny,2)
  double *SxE, *EtaE, *AlE, *DAlE, *SyN, *EtaN, *AlN, *DAlN;  // (nx+2,ny+2)
  int is_p;
};

// index helpers (1-based i, j as in the reference)
__device__ __forceinline__ size_t I1(const Fam& f, int i, int j) {
  return (size_t)(i - 1) + (size_t)(j - 1) * f.nx;
}
__device__ __forceinline__ size_t I0(const Fam& f, int i, int j) {
  return (size_t)i + (size_t)j * (f.nx + 2);
}
__device__ __forceinline__ size_t N0(const Fam& f) { return (size_t)(f.nx + 2) * (f.ny + 2); }
__device__ __forceinline__ size_t N1(const Fam& f) { return (size_t)f.nx * f.ny; }
// FCE / FCN component k (0: x, 1: y) at (i,j); Cell_Cent / FCW / FCS / MsCe
__device__ __forceinline__ double& FC(double* a, const Fam& f, int i, int j, int k) {
  return a[I0(f, i, j) + k * N0(f)];
}
__device__ __forceinline__ double& C2(double* a, const Fam& f, int i, int j, int k) {
  return a[I1(f, i, j) + k * N1(f)];
}

// IEEE division on the integer pipe (bit-identical; GB300's FP64 pipe is slow).
// Halvings are written as products with 0.5, which round identically.
__device__ __forceinline__ double dv(double a, double b) { return div_rn(a, b); }
// sqrt(x) with the common x = 0 (open or closed cells) taken without the FP64 pipe
__device__ __forceinline__ double sqrt0(double x) { return x == 0.0 ? x : sqrt(x); }

// l >= 1e-14 and l < 1e-14 (both false for NaN) by the bit pattern, on the
// integer pipe: for non-NaN doubles and a positive constant the signed
// 64-bit patterns order like the values
constexpr long long kE14 = 0x3d06849b86a12b9bll;  // 1.0e-14
__device__ __forceinline__ bool nan_bits(long long u) {
  return (u & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
}
__device__ __forceinline__ bool ge14(double l) {
  const long long u = __double_as_longlong(l);
  return !nan_bits(u) && u >= kE14;
}
__device__ __forceinline__ bool lt14(double l) {
  const long long u = __double_as_longlong(l);
  return !nan_bits(u) && u < kE14;
}

// Edge_Geo_Cal (:302-337) from the level set at the edge's ends l1 (p1) and
// l2 (p2): solid fraction of the edge and the centre of its solid part.
// (mx, my) is the edge's midpoint 0.5*(p1+p2), given exactly by the caller.
__device__ void edge(double p1x, double p1y, double p2x, double p2y, double l1, double l2,
                     double mx, double my, double* area, double* fx, double* fy) {
  *fx = mx;
  *fy = my;
  const bool g1 = ge14(l1), g2 = ge14(l2), s1 = lt14(l1), s2 = lt14(l2);
  if (g1 && g2) {
    *area = 0.0;
  } else if (s1 && s2) {
    *area = 1.0;
  } else if (g1 && s2) {
    *area = dv(fabs(l2), fabs(l1) + fabs(l2));
    if (fabs(p1x - p2x) <= 1.0e-10) *fy = p2y - 0.5 * *area * (p2y - p1y);
    else *fx = p2x - 0.5 * *area * (p2x - p1x);
  } else if (s1 && g2) {
    *area = dv(fabs(l1), fabs(l1) + fabs(l2));
    if (fabs(p1x - p2x) <= 1.0e-10) *fy = p1y - 0.5 * *area * (p1y - p2y);
    else *fx = p1x - 0.5 * *area * (p1x - p2x);
  } else {
    *area = 0.0;  // a NaN level set
  }
}

#define CELL_LOOP(f)                                       \
  const int i = blockIdx.x * 32 + threadIdx.x + 1;        \
  const int j = blockIdx.y * 8 + threadIdx.y + 1;         \
  if (i > (f).nx || j > (f).ny) return;

// bit-exact equality of two doubles on the integer pipe
__device__ __forceinline__ bool same(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b);
}

// Cell_Geo_Cal (:45-89): edge fractions, solid-part face centres, WlLh from
// the solid fractions; Cell_Cent = 0.  Exact rewrites of the reference's
// expressions: the corners are (-h, -k), (-h, k), (h, k), (h, -k) with
// h = dx*0.5, k = dy*0.5 (the reference's -dx*(0.5-ii) for ii = 0, 1); a
// product with -h is the negated product with h, so the level set at each
// corner is +-(a h) +- (b k) + phiS, evaluated once per corner (the
// reference evaluates it once per edge through the corner, the same
// expression); the midpoints of the edges are the corners' shared
// coordinate and 0 (-k + k = +0); WlLh is +0 when the opposite fractions are
// equal.
__global__ void k_cg_edges(Fam f) {
  CELL_LOOP(f)
  const double dx = f.dx[I1(f, i, j)], dy = f.dy[I1(f, i, j)];
  const double a = f.nxS[I1(f, i, j)], b = f.nyS[I1(f, i, j)], p = f.phiS[I1(f, i, j)];
  const double h = dx * 0.5, k = dy * 0.5;
  const double x0 = -h, x1 = h, y0 = -k, y1 = k;
  const double ah = a * h, bk = b * k;
  const double l00 = -ah + -bk + p, l01 = -ah + bk + p;
  const double l11 = ah + bk + p, l10 = ah + -bk + p;
  double W, N, E, S, fx, fy;
  edge(x0, y0, x0, y1, l00, l01, x0, 0.0, &W, &fx, &fy);
  C2(f.FCW, f, i, j, 0) = fx; C2(f.FCW, f, i, j, 1) = fy;
  edge(x0, y1, x1, y1, l01, l11, 0.0, y1, &N, &fx, &fy);
  FC(f.FCN, f, i, j, 0) = fx; FC(f.FCN, f, i, j, 1) = fy;
  edge(x1, y1, x1, y0, l11, l10, x1, 0.0, &E, &fx, &fy);
  FC(f.FCE, f, i, j, 0) = fx; FC(f.FCE, f, i, j, 1) = fy;
  edge(x1, y0, x0, y0, l10, l00, 0.0, y0, &S, &fx, &fy);
  C2(f.FCS, f, i, j, 0) = fx; C2(f.FCS, f, i, j, 1) = fy;
  f.aW[I0(f, i, j)] = W; f.aN[I0(f, i, j)] = N; f.aE[I0(f, i, j)] = E; f.aS[I0(f, i, j)] = S;
  double wl = 0.0;
  if (!same(E, W) || !same(N, S) || nan_bits(__double_as_longlong(E)) ||
      nan_bits(__double_as_longlong(N))) {
    const double ta = (E - W) * dx, tb = (N - S) * dy;
    wl = sqrt0(ta * ta + tb * tb);
  }
  f.WlLh[I1(f, i, j)] = wl;
  C2(f.cent, f, i, j, 0) = 0.0;
  C2(f.cent, f, i, j, 1) = 0.0;
  if (f.delh) f.delh[I1(f, i, j)] = 0.0;
}

// ghost face centres (:91-104 for the columns j = 1..ny)
__global__ void k_cg_ghost_cols(Fam f) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > f.ny) return;
  const int nx = f.nx;
  const double dx1 = f.dx[I1(f, 1, 1)], dxn = f.dx[I1(f, nx, 1)];
  double* const arr[2] = {f.FCE, f.FCN};
  for (int q = 0; q < 2; ++q) {
    double* a = arr[q];
    FC(a, f, 0, j, 0) = FC(a, f, 1, j, 0) - dx1;
    FC(a, f, 0, j, 1) = FC(a, f, 1, j, 1);
    FC(a, f, nx + 1, j, 0) = FC(a, f, nx, j, 0) + dxn;
    FC(a, f, nx + 1, j, 1) = FC(a, f, nx, j, 1);
  }
}

// ghost face centres (:103-112 for the rows, i = 0..nx+1; FCN's from FCE's)
__global__ void k_cg_ghost_rows(Fam f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > f.nx + 1) return;
  const int ny = f.ny;
  const double dy1 = f.dy[I1(f, 1, 1)], dyn = f.dy[I1(f, 1, ny)];
  const double e10 = FC(f.FCE, f, i, 1, 0), e11 = FC(f.FCE, f, i, 1, 1);
  const double en0 = FC(f.FCE, f, i, ny, 0), en1 = FC(f.FCE, f, i, ny, 1);
  FC(f.FCE, f, i, 0, 0) = e10;
  FC(f.FCE, f, i, 0, 1) = e11 - dy1;
  FC(f.FCE, f, i, ny + 1, 0) = en0;
  FC(f.FCE, f, i, ny + 1, 1) = en1 + dyn;
  FC(f.FCN, f, i, 0, 0) = e10;
  FC(f.FCN, f, i, 0, 1) = e11 - dy1;
  FC(f.FCN, f, i, ny + 1, 0) = en0;
  FC(f.FCN, f, i, ny + 1, 1) = en1 + dyn;
}

// (:114-153) open fractions and the open parts' face centres.  |c| < epsi
// and a < epsiF on the bit patterns (integer pipe; a is never NaN here, an
// open fraction in [0, 1]); 1 - 0 and 1 - 1 without the FP64 pipe.
constexpr long long kEpsiBits = 0x3f50624dd2f1a9fcll;   // 1.0e-3
constexpr long long kEpsFBits = 0x3f847ae147ae147bll;   // 1.0e-2
__device__ __forceinline__ double open_centre(double c, double a, double h) {
  if (__double_as_longlong(a) < kEpsFBits) return 0.0;  // a >= 0: a < epsiF
  const long long cb = __double_as_longlong(c) & 0x7fffffffffffffffll;
  if (cb < kEpsiBits) return 0.0;  // |c| < epsi (NaN c takes the formula, as in IEEE)
  return (0.5 - a * 0.5) * copysign(1.0, -c) * h;
}
__device__ __forceinline__ double one_minus(double x) {
  if (same(x, 0.0)) return 1.0;
  if (same(x, 1.0)) return 0.0;
  return 1.0 - x;
}
__global__ void k_cg_open(Fam f) {
  CELL_LOOP(f)
  const double dx = f.dx[I1(f, i, j)], dy = f.dy[I1(f, i, j)];
  const size_t k = I0(f, i, j);
  const double W = one_minus(f.aW[k]), E = one_minus(f.aE[k]), N = one_minus(f.aN[k]),
               S = one_minus(f.aS[k]);
  f.aW[k] = W; f.aE[k] = E; f.aN[k] = N; f.aS[k] = S;
  FC(f.FCE, f, i, j, 1) = open_centre(FC(f.FCE, f, i, j, 1), E, dy);
  C2(f.FCW, f, i, j, 1) = open_centre(C2(f.FCW, f, i, j, 1), W, dy);
  FC(f.FCN, f, i, j, 0) = open_centre(FC(f.FCN, f, i, j, 0), N, dx);
  C2(f.FCS, f, i, j, 0) = open_centre(C2(f.FCS, f, i, j, 0), S, dx);
}

// (:155-203) faces shared by two inner cells: harmonic mean of the open
// fractions, weighted face centres; each thread owns its cell's north and
// east faces
// (a*u + b*v) / (u + v + 1e-24) for the open fractions u, v of a shared
// face: two fully open faces (u = v = 1) give (a + b) / 2 exactly (1e-24 is
// far below an ulp of 2), without the division
__device__ __forceinline__ double wmean(double a, double u, double b, double v) {
  if (u == 1.0 && v == 1.0) return (a + b) * 0.5;
  return dv(a * u + b * v, u + v + kRnd);
}
__device__ __forceinline__ double hmean(double u, double v) {
  if (u == 1.0 && v == 1.0) return 1.0;  // 2 / (2 + 1e-24) rounds to 1
  return dv(2.0 * u * v, u + v + kRnd);
}
__global__ void k_cg_average(Fam f) {
  CELL_LOOP(f)
  if (i < 2 || i > f.nx - 1 || j < 2 || j > f.ny - 1) return;
  const size_t k = I0(f, i, j), kn = I0(f, i, j + 1), ke = I0(f, i + 1, j);
  const double N = f.aN[k], Sn = f.aS[kn];
  double av = hmean(N, Sn);
  const double n0 = wmean(FC(f.FCN, f, i, j, 0), N, C2(f.FCS, f, i, j + 1, 0), Sn);
  double n1 = wmean(FC(f.FCN, f, i, j, 1), N,
                    C2(f.FCS, f, i, j + 1, 1) + (f.y[I1(f, i, j + 1)] - f.y[I1(f, i, j)]), Sn);
  if (N < kEpsF && Sn < kEpsF) n1 = f.dy[I1(f, i, j)] * 0.5;
  FC(f.FCN, f, i, j, 0) = n0;
  FC(f.FCN, f, i, j, 1) = n1;
  f.aN[k] = av;
  f.aS[kn] = av;
  const double E = f.aE[k], We = f.aW[ke];
  av = hmean(E, We);
  double e0 = wmean(FC(f.FCE, f, i, j, 0), E,
                    C2(f.FCW, f, i + 1, j, 0) + (f.x[I1(f, i + 1, j)] - f.x[I1(f, i, j)]), We);
  const double e1 = wmean(FC(f.FCE, f, i, j, 1), E, C2(f.FCW, f, i + 1, j, 1), We);
  if (E < kEpsF && We < kEpsF) e0 = f.dx[I1(f, i, j)] * 0.5;
  FC(f.FCE, f, i, j, 0) = e0;
  FC(f.FCE, f, i, j, 1) = e1;
  f.aE[k] = av;
  f.aW[ke] = av;
}

// (:217-228) the solid-cell rule of the U and V families (their MsCe is
// allocated, so the degenerate-cell rule of :229-243 does not apply): only
// zeros are written, so the loop order does not matter
__global__ void k_cg_solid_uv(Fam f) {
  CELL_LOOP(f)
  const size_t k = I1(f, i, j);
  if (!(f.vofS[k] > 1.0 - kEpsi)) return;
  f.vofS[k] = 1.0;
  f.aW[I0(f, i, j)] = 0.0; f.aE[I0(f, i, j)] = 0.0;
  f.aN[I0(f, i, j)] = 0.0; f.aS[I0(f, i, j)] = 0.0;
  f.aE[I0(f, i - 1, j)] = 0.0; f.aN[I0(f, i, j - 1)] = 0.0;
  f.aW[I0(f, i + 1, j)] = 0.0; f.aS[I0(f, i, j + 1)] = 0.0;
}

// (:262-266) the corner rule's face centres of the P family (its apertures,
// WlLh and normal come from the projection's geometry pipeline)
__global__ void k_cg_corner_fcn(Fam f) {
  CELL_LOOP(f)
  if (j > f.ny - 4) return;
  const double v0 = f.vofS[I1(f, i, j)], v1 = f.vofS[I1(f, i, j + 1)], v2 = f.vofS[I1(f, i, j + 2)];
  if (v0 > -kEpsi && v0 < kEpsi && v1 > 0.6 - kEpsi && v1 < 0.6 + kEpsi && v2 > 0.6 - kEpsi &&
      v2 < 0.6 + kEpsi) {
    FC(f.FCN, f, i, j, 0) = -0.3 * f.dx[I1(f, i, j)];
    FC(f.FCN, f, i, j, 1) = 0.5 * f.dy[I1(f, i, j)];
  }
}

// NewCellFace (:415-497) for one of the U (u = 1) / V (u = 0) families:
// cell centroids, the exchange cells' centroids and CellLinking
__global__ void k_ncf_cent(Fam t, Fam p, int u) {
  CELL_LOOP(t)
  const double tol = 1.0e-24;
  const size_t k = I1(t, i, j);
  const int mo = t.moex[k];
  if (mo != 1 && t.vofS[k] > kEpsi) {
    if (u) {
      C2(t.cent, t, i, j, 0) = FC(p.FCE, p, i, j, 0) - p.dx[k] * 0.5;
      C2(t.cent, t, i, j, 1) = FC(p.FCE, p, i, j, 1);
    } else {
      C2(t.cent, t, i, j, 0) = FC(p.FCN, p, i, j, 0);
      C2(t.cent, t, i, j, 1) = FC(p.FCN, p, i, j, 1) - p.dy[k] * 0.5;
    }
  }
  if (mo != 1) return;
  if (t.vofS[k] < 1.0 - kEpsi) {
    const double nxs = t.nxS[k], nys = t.nyS[k], phs = t.phiS[k];
    const double Nc = t.aN[I0(t, i, j)], Ns = t.aN[I0(t, i, j - 1)];
    const double Ec = t.aE[I0(t, i, j)], Ew = t.aE[I0(t, i - 1, j)];
    double cx = C2(t.cent, t, i, j, 0), cy = C2(t.cent, t, i, j, 1);
    if (Nc * Ns == 0.0) {
      cx = dv(FC(t.FCN, t, i, j, 0) * Nc, Nc + tol) + dv(FC(t.FCN, t, i, j - 1, 0) * Ns, Ns + tol);
    } else {
      cy = dv(FC(t.FCE, t, i, j, 1) * Ec, Ec + tol) + dv(FC(t.FCE, t, i - 1, j, 1) * Ew, Ew + tol);
      cx = dv(-(nys * cy + phs), nxs + tol);
    }
    if (Ec * Ew == 0.0) {
      cy = dv(FC(t.FCE, t, i, j, 1) * Ec, Ec + tol) + dv(FC(t.FCE, t, i - 1, j, 1) * Ew, Ew + tol);
    } else {
      cy = dv(-(nxs * cx + phs), nys + tol);
    }
    C2(t.cent, t, i, j, 0) = cx;
    C2(t.cent, t, i, j, 1) = cy;
  }
  // CellLinking (:702-725); a neighbour outside the grid counts as solid
  const int ii = i + (int)copysign(1.0, t.nxS[k]);
  const int jj = j + (int)copysign(1.0, t.nyS[k]);
  auto vs = [&](int a, int b) {
    return (a >= 1 && a <= t.nx && b >= 1 && b <= t.ny) ? t.vofS[I1(t, a, b)] : 1.0;
  };
  int* ms = t.msce;
  if (vs(ii, j) < vs(i, jj)) {
    ms[k] = ii;
    ms[k + N1(t)] = j;
  } else {
    ms[k] = i;
    ms[k + N1(t)] = jj;
  }
}

// NewCellFace (:498-540): delh and WlLh of the U / V cells
__global__ void k_ncf_delh(Fam t) {
  CELL_LOOP(t)
  const size_t k = I1(t, i, j);
  const double tol = 1.0e-24;
  double d = fabs(C2(t.cent, t, i, j, 0) * t.nxS[k] + C2(t.cent, t, i, j, 1) * t.nyS[k] +
                  t.phiS[k]) + tol;
  if (t.moex[k] == 1) d = 1.0e-20;
  t.delh[k] = d;
  const double a = (t.aE[I0(t, i, j)] - t.aW[I0(t, i, j)]) * t.dx[k];
  const double b = (t.aN[I0(t, i, j)] - t.aS[I0(t, i, j)]) * t.dy[k];
  t.WlLh[k] = sqrt0(a * a + b * b);
}

// EastFaceInterpolationInf (:551-604) for i = 1..nx-1; bdx = BGrid%dx
__global__ void k_ncf_east(Fam t, const double* bdx, int iu) {
  CELL_LOOP(t)
  if (i > t.nx - 1) return;
  const size_t k = I0(t, i, j);
  const double B = bdx[I1(t, i + iu, j)];
  if (t.posnu[k] != -1 && t.posnu[I0(t, i + 1, j)] != -1) {
    const double c0 = C2(t.cent, t, i, j, 0), c1 = C2(t.cent, t, i, j, 1);
    const double e0 = C2(t.cent, t, i + 1, j, 0), e1 = C2(t.cent, t, i + 1, j, 1);
    const double sxe = e0 + B - c0;
    const double sy = e1 - c1;
    double eta = dv(fabs(FC(t.FCE, t, i, j, 0) - c0), sxe);
    if (eta >= 1.0) eta = 0.5;
    const double xf = (1.0 - eta) * c0 + eta * (e0 + B);
    const double yf = (1.0 - eta) * c1 + eta * e1;
    double al, dal;
    if (fabs(sy) > 0.0001 * t.dy[I1(t, i, j)]) {
      const size_t a = I1(t, i, j), b = I1(t, i + 1, j);
      const double nyf = 0.5 * (t.nyS[a] + t.nyS[b]);
      const double ipd = 0.5 * (fabs(xf * t.nxS[a] + yf * t.nyS[a] + t.phiS[a]) +
                                fabs((xf - B) * t.nxS[b] + yf * t.nyS[b] + t.phiS[b]));
      const double f0 = FC(t.FCE, t, i, j, 0), f1 = FC(t.FCE, t, i, j, 1);
      const double fcd = 0.5 * (fabs(f0 * t.nxS[a] + f1 * t.nyS[a] + t.phiS[a]) +
                                fabs((f0 - B) * t.nxS[b] + f1 * t.nyS[b] + t.phiS[b]));
      al = dv(fabs(fcd), fabs(ipd));
      dal = dv(sy * nyf, sxe * fabs(ipd));
      if (fabs(ipd) < 1.0e-5) {
        dal = 0.0;
        al = 1.0;
      }
      if (al >= 2.0) al = 2.0;
    } else {
      dal = 0.0;
      al = 1.0;
    }
    t.SxE[k] = sxe; t.EtaE[k] = eta; t.AlE[k] = al; t.DAlE[k] = dal;
  } else {
    t.AlE[k] = 1.0; t.DAlE[k] = 0.0; t.SxE[k] = B; t.EtaE[k] = 0.5;
  }
}

// (:605-612): columns nx and 0; AlE(0,j) takes AlN(1,j) before this step's
// NorthFaceInterpolationInf
__global__ void k_ncf_east_ghost(Fam t) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > t.ny) return;
  const int nx = t.nx;
  const size_t kn = I0(t, nx, j), km = I0(t, nx - 1, j), k0 = I0(t, 0, j), k1 = I0(t, 1, j);
  t.SxE[kn] = t.SxE[km]; t.EtaE[kn] = t.EtaE[km]; t.DAlE[kn] = t.DAlE[km]; t.AlE[kn] = t.AlE[km];
  t.SxE[k0] = t.SxE[k1]; t.EtaE[k0] = t.EtaE[k1]; t.DAlE[k0] = t.DAlE[k1];
  t.AlE[k0] = t.AlN[k1];
}

// NorthFaceInterpolationInf (:618-690) for j = 1..ny-1; bdy = BGrid%dy
__global__ void k_ncf_north(Fam t, const double* bdy, int iv) {
  CELL_LOOP(t)
  if (j > t.ny - 1) return;
  const size_t k = I0(t, i, j);
  const double B = bdy[I1(t, i, j + iv)];
  if (t.posnu[k] != -1 && t.posnu[I0(t, i, j + 1)] != -1) {
    const double c0 = C2(t.cent, t, i, j, 0), c1 = C2(t.cent, t, i, j, 1);
    const double n0 = C2(t.cent, t, i, j + 1, 0), n1 = C2(t.cent, t, i, j + 1, 1);
    const double syn = n1 + B - c1;
    const double sx = n0 - c0;
    double eta = dv(fabs(FC(t.FCN, t, i, j, 1) - c1), syn);
    if (eta >= 1.0) eta = 0.5;
    const double xf = (1.0 - eta) * c0 + eta * n0;
    const double yf = (1.0 - eta) * c1 + eta * (n1 + B);
    double al, dal;
    if (fabs(sx) >= 0.0001 * t.dx[I1(t, i, j)]) {
      const size_t a = I1(t, i, j), b = I1(t, i, j + 1);
      const double nxf = 0.5 * (t.nxS[a] + t.nxS[b]);
      const double ipd = 0.5 * (fabs(xf * t.nxS[a] + yf * t.nyS[a] + t.phiS[a]) +
                                fabs(xf * t.nxS[b] + (yf - B) * t.nyS[b] + t.phiS[b]));
      const double f0 = FC(t.FCN, t, i, j, 0), f1 = FC(t.FCN, t, i, j, 1);
      const double fcd = 0.5 * (fabs(f0 * t.nxS[a] + f1 * t.nyS[a] + t.phiS[a]) +
                                fabs(f0 * t.nxS[b] + (f1 - B) * t.nyS[b] + t.phiS[b]));
      al = dv(fabs(ipd), fabs(fcd));
      dal = dv(sx * nxf, syn * fabs(ipd));
      if (fabs(ipd) < 1.0e-5) {
        dal = 0.0;
        al = 1.0;
      }
      if (al >= 2.0) al = 2.0;
    } else {
      dal = 0.0;
      al = 1.0;
    }
    t.SyN[k] = syn; t.EtaN[k] = eta; t.AlN[k] = al; t.DAlN[k] = dal;
  } else {
    t.EtaN[k] = 0.5; t.AlN[k] = 1.0; t.DAlN[k] = 0.0; t.SyN[k] = B;
  }
}

// (:691-698): rows ny and 0
__global__ void k_ncf_north_ghost(Fam t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (i > t.nx) return;
  const int ny = t.ny;
  const size_t kn = I0(t, i, ny), km = I0(t, i, ny - 1), k0 = I0(t, i, 0), k1 = I0(t, i, 1);
  t.SyN[kn] = t.SyN[km]; t.EtaN[kn] = t.EtaN[km]; t.DAlN[kn] = t.DAlN[km]; t.AlN[kn] = t.AlN[km];
  t.SyN[k0] = t.SyN[k1]; t.EtaN[k0] = t.EtaN[k1]; t.DAlN[k0] = t.DAlN[k1]; t.AlN[k0] = t.AlN[k1];
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

#define CKC(call)                                                          \
  do {                                                                     \
    if ((call) != cudaSuccess) {                                           \
      rc = SCF_ERR_CUDA;                                                   \
      goto done;                                                           \
    }                                                                      \
  } while (0)

dim3 cells(int nx, int ny) { return dim3((nx + 31) / 32, (ny + 7) / 8); }

// Device work arena kept between calls (allocating and mapping some GB of
// device memory costs more than the whole computation), one per device,
// grown on demand; calls are serialised by arena_lock.
std::mutex arena_lock;
bool arena_get(int device, size_t bytes, char** p) {
  static char* buf[16] = {};
  static size_t cap[16] = {};
  const int d = device & 15;
  if (cap[d] < bytes) {
    if (buf[d]) cudaFree(buf[d]);
    buf[d] = nullptr;
    cap[d] = 0;
    if (cudaMalloc(&buf[d], bytes) != cudaSuccess) {
      (void)cudaGetLastError();
      return false;
    }
    cap[d] = bytes;
  }
  *p = buf[d];
  return true;
}

}  // namespace
}  // namespace scf

using namespace scf;

extern "C" int scf_grid_preprocess(int nx, int ny, const scf_cell_grid grid[3],
                                   const scf_cell_solid solid[3], scf_cell_geom geom[3],
                                   int icorprob, int flags, int device, double* ms) {
  if (nx < 2 || ny < 2 || !grid || !solid || !geom) return SCF_ERR_ARG;
  for (int f = 0; f < 3; ++f) {
    const scf_cell_grid& g = grid[f];
    const scf_cell_solid& s = solid[f];
    if (!g.dx || !g.dy || !g.x || !g.y || !s.vofS || !s.phiS || !s.nxS || !s.nyS)
      return SCF_ERR_ARG;
  }
  const auto t0 = std::chrono::steady_clock::now();
  const bool dev = (flags & SCF_CUTCELL_DEVICE_PTRS) != 0;
  const cudaMemcpyKind in_kind = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind out_kind = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  const size_t n1 = (size_t)nx * ny, n0 = (size_t)(nx + 2) * (ny + 2);
  int rc = SCF_OK;
  bool locked = false;
  cudaStream_t s = nullptr;
  char* arena = nullptr;
  uint8_t *st0 = nullptr, *st1 = nullptr;
  int *counts = nullptr, *flag = nullptr, *flag_host = nullptr;
  Fam F[3];
  const double* raw[3][8] = {};  // device copies: dx, dy, x, y, vofS, phiS, nxS, nyS
  // per family: 8 inputs + vofS/nxS/nyS (n1 doubles each), apertures (4 n0),
  // FCE/FCN (4 n0), FCW/FCS (4 n1), cent (2 n1), WlLh/delh (2 n1),
  // interpolation (8 n0) doubles; posnu (n0), moex (n1), msce (2 n1) ints
  const size_t dbl = 8 * n1 + 3 * n1 + 4 * n0 + 4 * n0 + 4 * n1 + 2 * n1 + 2 * n1 + 8 * n0;
  const size_t ints = n0 + n1 + 2 * n1;
  const size_t per = dbl * 8 + ints * 4 + 256;
  if (cudaSetDevice(device) != cudaSuccess) return SCF_ERR_CUDA;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return SCF_ERR_CUDA;
  // the work arena is kept for the next step (one per device, grown on demand)
  arena_lock.lock();
  locked = true;
  if (!arena_get(device, 3 * per, &arena)) {
    rc = SCF_ERR_NOMEM;
    goto done;
  }
  CKC(cudaMemsetAsync(arena, 0, 3 * per, s));
  for (int f = 0; f < 3; ++f) {
    char* p = arena + f * per;
    auto D = [&](size_t n) {
      double* r = reinterpret_cast<double*>(p);
      p += n * 8;
      return r;
    };
    auto Iv = [&](size_t n) {
      int32_t* r = reinterpret_cast<int32_t*>(p);
      p += n * 4;
      return r;
    };
    Fam& m = F[f];
    m.nx = nx; m.ny = ny; m.is_p = f == 0;
    double* in8[8];
    for (int a = 0; a < 8; ++a) in8[a] = D(n1);
    const double* src[8] = {grid[f].dx, grid[f].dy, grid[f].x, grid[f].y,
                            solid[f].vofS, solid[f].phiS, solid[f].nxS, solid[f].nyS};
    for (int a = 0; a < 8; ++a) {
      CKC(cudaMemcpyAsync(in8[a], src[a], n1 * 8, in_kind, s));
      raw[f][a] = in8[a];
    }
    m.dx = in8[0]; m.dy = in8[1]; m.x = in8[2]; m.y = in8[3]; m.phiS = in8[5];
    m.vofS = D(n1); m.nxS = D(n1); m.nyS = D(n1);
    CKC(cudaMemcpyAsync(m.vofS, in8[4], n1 * 8, cudaMemcpyDeviceToDevice, s));
    CKC(cudaMemcpyAsync(m.nxS, in8[6], n1 * 8, cudaMemcpyDeviceToDevice, s));
    CKC(cudaMemcpyAsync(m.nyS, in8[7], n1 * 8, cudaMemcpyDeviceToDevice, s));
    m.aE = D(n0); m.aW = D(n0); m.aN = D(n0); m.aS = D(n0);
    m.FCE = D(2 * n0); m.FCN = D(2 * n0);
    m.FCW = D(2 * n1); m.FCS = D(2 * n1);
    m.cent = D(2 * n1);
    m.WlLh = D(n1);
    m.delh = D(n1);
    m.SxE = D(n0); m.EtaE = D(n0); m.AlE = D(n0); m.DAlE = D(n0);
    m.SyN = D(n0); m.EtaN = D(n0); m.AlN = D(n0); m.DAlN = D(n0);
    m.posnu = Iv(n0); m.moex = Iv(n1); m.msce = Iv(2 * n1);
    if (f == 0) m.delh = nullptr;
    if (f > 0) {  // in/out arrays start from the caller's values
      const scf_cell_geom& o = geom[f];
      double* io[8] = {m.SxE, m.EtaE, m.AlE, m.DAlE, m.SyN, m.EtaN, m.AlN, m.DAlN};
      double* ci[8] = {o.SxE, o.EtaE, o.AlE, o.DAlE, o.SyN, o.EtaN, o.AlN, o.DAlN};
      for (int a = 0; a < 8; ++a)
        if (ci[a]) CKC(cudaMemcpyAsync(io[a], ci[a], n0 * 8, in_kind, s));
      if (o.msce) CKC(cudaMemcpyAsync(m.msce, o.msce, 2 * n1 * 4, in_kind, s));
    }
  }
  {
    const dim3 g = cells(nx, ny), b(32, 8);
    for (int f = 0; f < 3; ++f) {
      k_cg_edges<<<g, b, 0, s>>>(F[f]);
      k_cg_ghost_cols<<<(ny + 127) / 128, 128, 0, s>>>(F[f]);
      k_cg_ghost_rows<<<(nx + 2 + 127) / 128, 128, 0, s>>>(F[f]);
      k_cg_open<<<g, b, 0, s>>>(F[f]);
      k_cg_average<<<g, b, 0, s>>>(F[f]);
      for (int q = 0; q < 5; ++q) note_launch();
    }
    k_cg_solid_uv<<<g, b, 0, s>>>(F[1]);
    k_cg_solid_uv<<<g, b, 0, s>>>(F[2]);
    note_launch(); note_launch();
    CKC(cudaGetLastError());
    // the P family's apertures, WlLh, rules, corner rule, exchange cells and
    // the three numberings (scf_geom.cu); its face centres are the ones above
    if (cudaMallocAsync(&st0, n0, s) != cudaSuccess || cudaMallocAsync(&st1, n0, s) != cudaSuccess ||
        cudaMallocAsync(&counts, geometry_count_ints(nx) * 4, s) != cudaSuccess ||
        cudaMallocAsync(&flag, 4, s) != cudaSuccess || cudaMallocHost(&flag_host, 4) != cudaSuccess) {
      rc = SCF_ERR_NOMEM;
      goto done;
    }
    GeoIn gi;
    gi.nx = nx; gi.ny = ny; gi.dx = F[0].dx; gi.dy = F[0].dy;
    gi.vofS = raw[0][4]; gi.phiS = raw[0][5]; gi.nxS = raw[0][6]; gi.nyS = raw[0][7];
    gi.vofS_u = raw[1][4];
    gi.vofS_v = raw[2][4];
    GeoOut go;
    go.dx = F[0].dx; go.dy = F[0].dy;
    go.aE = F[0].aE; go.aW = F[0].aW; go.aN = F[0].aN; go.aS = F[0].aS;
    go.WlLh = F[0].WlLh; go.vofS = F[0].vofS; go.nxS = F[0].nxS; go.nyS = F[0].nyS;
    go.vofS_u = F[1].vofS; go.vofS_v = F[2].vofS;
    go.posnu_p = F[0].posnu; go.posnu_u = F[1].posnu; go.posnu_v = F[2].posnu;
    go.moex_u = F[1].moex; go.moex_v = F[2].moex;
    if (geometry_build(gi, go, st0, st1, counts, flag, flag_host, icorprob ? 1 : 0, s) < 0) {
      rc = SCF_ERR_CUDA;
      goto done;
    }
    if (icorprob) {
      k_cg_corner_fcn<<<g, b, 0, s>>>(F[0]);
      note_launch();
    }
    // NewCellFace
    k_ncf_cent<<<g, b, 0, s>>>(F[1], F[0], 1);
    k_ncf_cent<<<g, b, 0, s>>>(F[2], F[0], 0);
    k_ncf_delh<<<g, b, 0, s>>>(F[1]);
    k_ncf_delh<<<g, b, 0, s>>>(F[2]);
    k_ncf_east<<<g, b, 0, s>>>(F[1], F[0].dx, 1);
    k_ncf_east_ghost<<<(ny + 127) / 128, 128, 0, s>>>(F[1]);
    k_ncf_north<<<g, b, 0, s>>>(F[1], F[2].dy, 0);
    k_ncf_north_ghost<<<(nx + 127) / 128, 128, 0, s>>>(F[1]);
    k_ncf_east<<<g, b, 0, s>>>(F[2], F[1].dx, 0);
    k_ncf_east_ghost<<<(ny + 127) / 128, 128, 0, s>>>(F[2]);
    k_ncf_north<<<g, b, 0, s>>>(F[2], F[0].dy, 1);
    k_ncf_north_ghost<<<(nx + 127) / 128, 128, 0, s>>>(F[2]);
    for (int q = 0; q < 12; ++q) note_launch();
    CKC(cudaGetLastError());
  }
  for (int f = 0; f < 3; ++f) {
    const Fam& m = F[f];
    const scf_cell_geom& o = geom[f];
    struct Out {
      void* dst;
      const void* src;
      size_t bytes;
    };
    std::vector<Out> outs = {
        {o.vofS, m.vofS, n1 * 8}, {o.nxS, m.nxS, n1 * 8}, {o.nyS, m.nyS, n1 * 8},
        {o.aE, m.aE, n0 * 8}, {o.aW, m.aW, n0 * 8}, {o.aN, m.aN, n0 * 8}, {o.aS, m.aS, n0 * 8},
        {o.FCE, m.FCE, 2 * n0 * 8}, {o.FCN, m.FCN, 2 * n0 * 8}, {o.cent, m.cent, 2 * n1 * 8},
        {o.WlLh, m.WlLh, n1 * 8}, {o.posnu, m.posnu, n0 * 4}};
    if (f > 0) {
      const std::vector<Out> uv = {
          {o.delh, m.delh, n1 * 8}, {o.moex, m.moex, n1 * 4}, {o.msce, m.msce, 2 * n1 * 4},
          {o.SxE, m.SxE, n0 * 8}, {o.EtaE, m.EtaE, n0 * 8}, {o.AlE, m.AlE, n0 * 8},
          {o.DAlE, m.DAlE, n0 * 8}, {o.SyN, m.SyN, n0 * 8}, {o.EtaN, m.EtaN, n0 * 8},
          {o.AlN, m.AlN, n0 * 8}, {o.DAlN, m.DAlN, n0 * 8}};
      outs.insert(outs.end(), uv.begin(), uv.end());
    }
    for (const Out& q : outs)
      if (q.dst) CKC(cudaMemcpyAsync(q.dst, q.src, q.bytes, out_kind, s));
  }
  CKC(cudaStreamSynchronize(s));
done:
  if (st0) cudaFreeAsync(st0, s);
  if (st1) cudaFreeAsync(st1, s);
  if (counts) cudaFreeAsync(counts, s);
  if (flag) cudaFreeAsync(flag, s);
  if (s) cudaStreamSynchronize(s);
  if (flag_host) cudaFreeHost(flag_host);
  if (s) cudaStreamDestroy(s);
  if (locked) arena_lock.unlock();
  if (ms)
    *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}
