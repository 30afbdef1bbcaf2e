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
// fluxes, which each thread evaluates for its own cell:
//   cell 1:          (t - f1 E1/d1) + phi1 u0 dtv W1/d1
//   cell 2:          (t - f2 E2/d2) + f1 E1/d2
//   cells 3..n-1:    (t (1 - s) + f(i-1) Wi/di) - fi Ei/di
//   cell n:          (t (1 - s) + f(n-1) Wn/dn) - fn En/dn     (Y: - fn/dn)
// The VOF update has the same shape (every face applied to both of its
// cells), after the division of temvf by (1 - vofS); its cell 1 gets the
// inflow through face 0 (X: the wave inlet, Y: vof ve(0) dtv) last.  Face
// fluxes read only the sweep's inputs, never temvf, so each thread
// computes the two fluxes of its cell itself.
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
      l = L.P(1) + L.D(1) / 2.0 * (1.0 - u * dtv / L.D(1)) * (L.P(2) - L.P(1)) / (L.C(2) - L.C(1));
    else if (DIR == SCF_LS_X)
      l = L.P(2) - L.D(2) / 2.0 * (1.0 + u * dtv / L.D(2)) * (L.P(3) - L.P(1)) / (2.0 * L.D(2));
    else
      l = L.P(2) - L.D(2) / 2.0 * (1.0 + u * dtv / L.D(2)) * (L.P(3) - L.P(1)) / (L.C(3) - L.C(1));
    return l * u * dtv;
  }
  if (f == n) {
    if (u > 0.0)
      l = L.P(n) + L.D(n) / 2.0 * (1.0 - u * dtv / L.D(n)) * (L.P(n) - L.P(n - 1)) /
                       (L.C(n) - L.C(n - 1));
    else
      l = L.P(n) - L.D(n - 1) / 2.0 * (1.0 + u * dtv / L.D(n - 1)) * (L.P(n) - L.P(n - 1)) /
                       (L.C(n) - L.C(n - 1));
    return l * u * dtv;
  }
  if (u >= 0.0) l = (L.P(f + 1) + L.P(f - 1)) / 2.0;
  else if (f <= n - 2) l = (L.P(f + 2) + L.P(f)) / 2.0;
  else l = (L.P(f + 1) + L.P(f - 1)) / 2.0;
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
    t = t - face_flux<DIR>(L, 1, dtv) * L.Hi(1) / L.D(1);
    t = t + L.P(1) * L.V(0) * dtv * L.Lo(1) / L.D(1);
  } else if (k == 2) {
    t = t - face_flux<DIR>(L, 2, dtv) * L.Hi(2) / L.D(2);
    t = t + face_flux<DIR>(L, 1, dtv) * L.Hi(1) / L.D(2);
  } else {
    t = t * (1.0 - L.S(k)) + face_flux<DIR>(L, k - 1, dtv) * L.Lo(k) / L.D(k);
    if (k < n || DIR == SCF_LS_X) t = t - face_flux<DIR>(L, k, dtv) * L.Hi(k) / L.D(k);
    else t = t - face_flux<DIR>(L, k, dtv) / L.D(k);
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
  if (tnx <= 1e-20) return 0.5 - diss / dy;
  if (tny <= 1e-20) return 0.5 - diss / dx;
  const double xx = (0.5 * tny * dy - diss) / dx / tnx + 0.5;
  const double yy = (0.5 * tnx * dx - diss) / dy / tny + 0.5;
  const double total = 0.5 * xx * yy;
  double top = 0.0, right = 0.0;
  if (yy > 1.0) {
    const double r = (yy - 1.0) / yy;
    top = r * r;
  }
  if (xx > 1.0) {
    const double r = (xx - 1.0) / xx;
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
  const double dx2 = dx / 2.0, dy2 = dy / 2.0;
  const double d0 = dx2 * nxs - dy2 * nys + phis, d1 = -(dx2 * nxs) - dy2 * nys + phis;
  const double d2 = -(dx2 * nxs) + dy2 * nys + phis, d3 = dx2 * nxs + dy2 * nys + phis;
  int m = 0;
  auto put = [&](double a, double b) {
    px[m] = a;
    py[m] = b;
    ++m;
  };
  if (d0 >= 0.0) put(dx2, -dy2);
  if (d0 * d1 < 0.0) put((dy2 * nys - phis) / nxs, -dy2);
  if (d1 >= 0.0) put(-dx2, -dy2);
  if (d1 * d2 < 0.0) put(-dx2, (dx2 * nxs - phis) / nys);
  if (d2 >= 0.0) put(-dx2, dy2);
  if (d2 * d3 < 0.0) put((-(dy2 * nys) - phis) / nxs, dy2);
  if (d3 >= 0.0) put(dx2, dy2);
  if (d3 * d0 < 0.0) put(dx2, (-(dx2 * nxs) - phis) / nys);
  double vol = 0.0;
  for (int k = 0; k < m; ++k) {
    const int k1 = k + 1 < m ? k + 1 : 0;
    vol = vol + 0.5 * (px[k] * py[k1] - px[k1] * py[k]);
    pd[k] = px[k] * nxl + py[k] * nyl + phil;
  }
  vols = 1.0 - fabs(vol / (dx * dy));
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
      add(px[k] + (px[k1] - px[k]) * w / ws, py[k] + (py[k1] - py[k]) * w / ws);
    }
  }
  if (ml > 0) vol = vol + 0.5 * (lx * fy - fx * ly);
  volf = fabs(vol / (dx * dy));
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
    if (c.vof / (1.0 - c.vofS) >= 1.0 - kVofEps) flux = 1.0 - volss;
    flux = flux / (1.0 - volss + kTolDeno);
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

template <int DIR, bool LS>
__global__ void k_clsvof_sweep(VofIn vin, LsIn lin, double* __restrict__ temvf,
                               double* __restrict__ temls) {
  const int nx = vin.nx, ny = vin.ny;
  const long long total = (long long)nx * ny;
  const double dtv = vin.dtv;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i0 = (int)(idx % nx), j0 = (int)(idx / nx);
    VLine L;
    L.in = &vin;
    const long long e0 = (long long)(i0 + 1) + (long long)(j0 + 1) * (nx + 2);
    int k;
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
    double t = temvf[idx];
    const double s = L.S(k);
    if (s < 1.0 - kVofEps) t = t / (1.0 - s);
    if (k == 1) {
      t = t - vof_face<DIR>(L, 1, dtv) * L.Hi(1) / L.D(1);
      if (DIR == SCF_LS_X) {
        double fin = 0.0;
        if (vin.y[idx] - vin.dy[idx] / 2.0 < vin.level) fin = L.F(1) * L.V(0) * dtv;
        t = t + fin * L.Lo(1) / L.D(1);
      } else {
        t = t + L.F(1) * L.V(0) * dtv * L.Lo(1) / L.D(1);
      }
    } else {
      t = t * (1.0 - s) + vof_face<DIR>(L, k - 1, dtv) * L.Lo(k) / L.D(k);
      t = t - vof_face<DIR>(L, k, dtv) * L.Hi(k) / L.D(k);
    }
    temvf[idx] = t;
    if (LS) temls[idx] = ls_cell<DIR>(lin, idx, i0, j0, temls[idx]);
  }
}

template <int DIR>
__global__ void k_ls_sweep(LsIn in, double* temls) {
  const int nx = in.nx, ny = in.ny;
  const long long total = (long long)nx * ny;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x)
    temls[idx] = ls_cell<DIR>(in, idx, (int)(idx % nx), (int)(idx / nx), temls[idx]);
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
                     const unsigned g = grid_for(n1);
                     if (dir == SCF_LS_X) {
                       if (ls) k_clsvof_sweep<SCF_LS_X, true><<<g, 256, 0, s>>>(vin, lin, o[0], o[1]);
                       else k_clsvof_sweep<SCF_LS_X, false><<<g, 256, 0, s>>>(vin, lin, o[0], o[1]);
                     } else {
                       if (ls) k_clsvof_sweep<SCF_LS_Y, true><<<g, 256, 0, s>>>(vin, lin, o[0], o[1]);
                       else k_clsvof_sweep<SCF_LS_Y, false><<<g, 256, 0, s>>>(vin, lin, o[0], o[1]);
                     }
                   });
}
