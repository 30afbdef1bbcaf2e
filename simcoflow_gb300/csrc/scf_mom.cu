// scf_mom.cu -- implicit solves of the momentum predictor (include/scf_mom.h):
// per velocity component, the operator and right-hand side of SetMatrix /
// SetVectors (src/PredictorUV_mod.f90:622-845), an FP64 BiCGStab solve with
// a diagonal preconditioner, the scatter of DeltaGetValues (:847-885), the
// pressure-gradient update (:517-522, :540-545), the Dp boundary copies
// (:552-562) and the open-top copy of PredictorVelocityBoundaryCondition
// (:563, :2199-2213).
//
// The assembly uses explicitly rounded operations in the reference's order
// (operator, right-hand side and Dp are bit-identical to a CPU restatement);
// the Krylov vector kernels use FMA freely.  Solver arrays use the padded
// level layout of scf_internal.cuh (cell (ix,iy) at base[iy*pitch+ix], zero
// ghost ring), the operator as five per-cell coefficients (it is not
// symmetric): P, W, E, S, N, zero where a neighbour has no unknown.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/scf_mom.h"
#include "scf_internal.cuh"
#include "scf_mgpre.cuh"

namespace scf {
namespace {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
// IEEE division, correctly rounded, on the integer pipe
__device__ __forceinline__ double dvd(double a, double b) { return div_rn(a, b); }

constexpr int TX = 64, TY = 32, NTM = 256;  // Krylov tiles: 64 x 32 cells, 256 threads

struct MomIn {  // device copies of scf_mom_in's arrays
  const double *dx, *dy, *vof, *vofS, *WlLh, *delh, *etaE, *etaN;
  const double *difEW, *edEW, *difNS, *edNS, *flux, *gradp, *u, *v;
  const int32_t* posnu;
  double dt, beta_vis, nua, nuw, nuref, rey, fr;
};

struct MomOp {  // padded solver arrays
  int nx, ny, pitch;
  double *P, *W, *E, *S, *N, *di, *b;
};

struct MomScalars {
  double rho, rho1, alpha, omega, bnorm2, rr, rtol2, ts, tt;
  int iter, maxit, done, status, bad;
  unsigned tickets[4];
};

__device__ __forceinline__ int tl() { return threadIdx.y * blockDim.x + threadIdx.x; }

// sum over the block (any size up to 1024, a multiple of 32); valid in thread 0
__device__ double bsum(double v) {
  __shared__ double w[32];
  __syncthreads();
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int t = tl(), nw = (blockDim.x * blockDim.y) >> 5;
  if ((t & 31) == 0) w[t >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (t == 0)
    for (int k = 0; k < nw; ++k) s += w[k];
  return s;
}

// two sums over the grid, combined by the last block in block order
__device__ bool gsum2(double a, double b, double* part, unsigned* ticket, double* ta,
                      double* tb) {
  __shared__ bool last;
  const int t = tl(), nt = blockDim.x * blockDim.y;
  const unsigned nb = gridDim.x * gridDim.y, bid = blockIdx.y * gridDim.x + blockIdx.x;
  const double sa = bsum(a), sb = bsum(b);
  if (t == 0) {
    part[2 * bid] = sa;
    part[2 * bid + 1] = sb;
    __threadfence();
    last = atomicAdd(ticket, 1u) == nb - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double xa = 0.0, xb = 0.0;
  for (unsigned k = t; k < nb; k += nt) {
    xa += __ldcg(&part[2 * k]);
    xb += __ldcg(&part[2 * k + 1]);
  }
  xa = bsum(xa);
  xb = bsum(xb);
  if (t == 0) {
    *ta = xa;
    *tb = xb;
    *ticket = 0u;
  }
  return true;
}

// x / d where d is 1.0 in most cells (an open cell's 1 - vofS): IEEE
// division by one is exact, so the FP64 division (slow on GB300's FP64
// pipe) is skipped there without changing a bit
__device__ __forceinline__ double div_open(double x, double d, bool one) {
  return one ? x : dvd(x, d);
}
// approximate 1/x for the Jacobi preconditioner (x > 0): an FP32 seed refined
// by two Newton-Raphson steps r <- r (2 - x r) (22 -> 44 -> ~53 correct bits)
__device__ __forceinline__ double rcp_newton(double x) {
  double r = (double)__frcp_rn((float)x);
  r = r * fma(-x, r, 2.0);
  return r * fma(-x, r, 2.0);
}

#define MF1(a, i, j) (a)[(size_t)((i)-1) + (size_t)((j)-1) * (size_t)nx]
#define MF0(a, i, j) (a)[(size_t)(i) + (size_t)(j) * (size_t)(nx + 2)]
#define MFE(a, i, j) (a)[(size_t)((i)-1) + (size_t)((j)-1) * (size_t)(nx + 1)]
#define MFN(a, i, j) (a)[(size_t)((i)-1) + (size_t)((j)-1) * (size_t)nx]

// SetMatrix + SetVectors for one cell per thread; also the Krylov start
// x = 0, r = r^ = b, p = v = 0 and ||b||^2.  Dp is the Fortran (0:nx+1,
// 0:ny+1) array, written for the assembled cells only.
__global__ void __launch_bounds__(256, 3)
k_mom_assemble(MomIn in, int iu, int iv, MomOp M, double* Dp, double* x,
                               double* r, double* rh, double* p0, double* v0, MomScalars* sc,
                               double* part) {
  pdl_wait();
  const int nx = M.nx, ny = M.ny;
  const int ix = blockIdx.x * 32 + threadIdx.x;
  double acc = 0.0;
  bool bad = false;
  const double ob = sub(1.0, in.beta_vis);
  const double ifr2 = dvd(1.0, mul(in.fr, in.fr));  // 1/Fr**2, the same for every cell
  if (ix < nx) {
    for (int iy = blockIdx.y * 8 + threadIdx.y; iy < ny; iy += gridDim.y * 8) {
      const int i = ix + 1, j = iy + 1;
      const size_t g = (size_t)iy * M.pitch + ix;
      double cP = 0.0, cW = 0.0, cE = 0.0, cS = 0.0, cN = 0.0, rhs = 0.0, dinv = 0.0;
      if (i <= nx - iu && j <= ny - iv && MF0(in.posnu, i, j) != -1) {
        const double VofAF = sub(1.0, MF1(in.vofS, i, j));
        const bool one = __double_as_longlong(VofAF) == 0x3ff0000000000000ll;  // 1.0
        double De = div_open(mul(ob, MFE(in.difEW, i + 1, j)), VofAF, one);
        double Dw = div_open(mul(ob, MFE(in.difEW, i, j)), VofAF, one);
        double Dn = div_open(mul(ob, MFN(in.difNS, i, j + 1)), VofAF, one);
        const double Ds = div_open(mul(ob, MFN(in.difNS, i, j)), VofAF, one);
        const double ee = MF0(in.etaE, i, j), ew = MF0(in.etaE, i - 1, j);
        const double en = MF0(in.etaN, i, j), es = MF0(in.etaN, i, j - 1);
        const double fe = MFE(in.edEW, i + 1, j), fw = MFE(in.edEW, i, j);
        const double fn = MFN(in.edNS, i, j + 1), fs = MFN(in.edNS, i, j);
        const double Fep = div_open(mul(fe, sub(1.0, ee)), VofAF, one);
        const double Fem = div_open(mul(fe, ee), VofAF, one);
        const double Fwp = div_open(mul(fw, ew), VofAF, one);
        const double Fwm = div_open(mul(fw, sub(1.0, ew)), VofAF, one);
        const double Fnp = div_open(mul(fn, sub(1.0, en)), VofAF, one);
        const double Fnm = div_open(mul(fn, en), VofAF, one);
        const double Fsp = div_open(mul(fs, es), VofAF, one);
        const double Fsm = div_open(mul(fs, sub(1.0, es)), VofAF, one);
        if (iu == 1) {
          if (j == ny) Dn = 0.0;
          if (i == nx - iu) De = 0.0;
          if (i == 1) Dw = 0.0;
        } else if (j == ny - iv) {
          Dn = 0.0;
        }
        double aE = De, aW = Dw, aN = Dn, aS = Ds;
        const double cwe1 = aW, cwe2 = aE, csn1 = aS;  // CWE(j,1), CWE(j,2), CSN(i,1)
        const double dxy = mul(MF1(in.dx, i, j), MF1(in.dy, i, j));
        double aP = add(add(add(add(dvd(dxy, in.dt), aE), aW), aN), aS);
        const double wl = MF1(in.WlLh, i, j), dh = MF1(in.delh, i, j);
        // the wall-shear term: without a wall (WlLh = 0, finite vof, finite
        // nonzero delh) it is a signed zero added to the positive sum above,
        // which leaves aP unchanged; otherwise (NaN included) it is evaluated
        const bool nowall = wl == 0.0 && isfinite(MF1(in.vof, i, j)) && isfinite(dh) && dh != 0.0;
        if (!nowall) {
          const double rv = dvd(MF1(in.vof, i, j), sub(1.0, MF1(in.vofS, i, j)));
          const double visc = add(dvd(mul(sub(1.0, rv), in.nua), in.nuref),
                                  dvd(mul(rv, in.nuw), in.nuref));
          aP = add(aP, div_open(dvd(mul(dvd(visc, in.rey), wl), dh), VofAF, one));
        }
        aP = sub(add(sub(add(aP, Fep), Fwp), Fnp), Fsp);
        aE = sub(aE, Fem);
        aW = add(aW, Fwm);
        aN = sub(aN, Fnm);
        aS = add(aS, Fsm);
        MF0(Dp, i, j) = dvd(dxy, sub(sub(sub(sub(aP, aE), aW), aN), aS));
        if (j > 1 && MF0(in.posnu, i, j - 1) != -1) cS = -aS;
        if (i > 1 && MF0(in.posnu, i - 1, j) != -1) cW = -aW;
        cP = aP;
        if (i < nx && MF0(in.posnu, i + 1, j) != -1) cE = -aE;
        if (j < ny && MF0(in.posnu, i, j + 1) != -1) cN = -aN;
        if (isnan(aP) || fabs(aP) > 1.0e20) bad = true;
        // SetVectors: convective flux, gravity (v), boundary terms.  On the
        // top row the reference adds CSN(j,2) (index j, not i): every
        // CSN(.,2) it sets is the zeroed top coefficient and the ones it
        // does not set are undefined, so the term is +0 times the ghost.
        const double diu = (double)iu, dv = (double)iv;
        rhs = sub(0.0, MF1(in.flux, i, j));
        if (iv == 1) rhs = sub(rhs, mul(mul(ifr2, MF1(in.dx, i, j)), MF1(in.dy, i, j)));
        if (i == 1)
          rhs = add(rhs, mul(cwe1, add(mul(diu, MF0(in.u, i - 1, j)), mul(dv, MF0(in.v, i - 1, j)))));
        if (i == nx - iu)
          rhs = add(rhs, mul(cwe2, add(mul(diu, MF0(in.u, i + 1, j)), mul(dv, MF0(in.v, i + 1, j)))));
        if (j == 1)
          rhs = add(rhs, mul(csn1, add(mul(diu, MF0(in.u, i, j - 1)), mul(dv, MF0(in.v, i, j - 1)))));
        if (j == ny - iv)
          rhs = add(rhs, mul(0.0, add(mul(diu, MF0(in.u, i, j + 1)), mul(dv, MF0(in.v, i, j + 1)))));
        dinv = rcp_newton(aP);
      }
      M.P[g] = cP; M.W[g] = cW; M.E[g] = cE; M.S[g] = cS; M.N[g] = cN;
      M.b[g] = rhs;
      M.di[g] = dinv;
      x[g] = 0.0; r[g] = rhs; rh[g] = rhs; p0[g] = 0.0; v0[g] = 0.0;
      acc = fma(rhs, rhs, acc);
    }
  }
  if (bad) sc->bad = 1;
  double tot, dummy;
  if (gsum2(acc, 0.0, part, &sc->tickets[0], &tot, &dummy) && tl() == 0) {
    sc->bnorm2 = tot;
    sc->rho1 = tot;  // (r^, r) of the start
    sc->rho = 1.0; sc->alpha = 1.0; sc->omega = 1.0;
    sc->rr = tot;
    sc->iter = 0;
    sc->status = 0;
    sc->done = (tot == 0.0 || !(tot < INFINITY)) ? 1 : 0;
    if (!(tot < INFINITY)) sc->status = kErrNaN;
  }
}

// w = A (D^-1 q_tile) on the CTA's tile, with q formed on the tile and a
// one-cell halo in shared memory by `form` (so every q is computed once per
// CTA, as by its owner).  Writes y = D^-1 q for the owned cells.
template <class Form>
__device__ __forceinline__ void tile_apply(const MomOp& M, Form form, double* y, double* w,
                                           double (&ys)[TY + 2][TX + 2], double* pa,
                                           double* pb, const double* ra, const double* rb) {
  (void)pa; (void)pb; (void)ra; (void)rb;
  const int nx = M.nx, ny = M.ny, P = M.pitch;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, t = tl();
  for (int e = t; e < (TX + 2) * (TY + 2); e += NTM) {
    const int ex = e % (TX + 2), ey = e / (TX + 2);
    const int gx = x0 - 1 + ex, gy = y0 - 1 + ey;
    double yv = 0.0;
    if (gx >= 0 && gx < nx && gy >= 0 && gy < ny) {
      const size_t g = (size_t)gy * P + gx;
      const double q = form(g, ex >= 1 && ex <= TX && ey >= 1 && ey <= TY);
      yv = M.di[g] * q;
    }
    ys[ey][ex] = yv;
  }
  __syncthreads();
  for (int e = t; e < TX * TY; e += NTM) {
    const int ex = e % TX, ey = e / TX, gx = x0 + ex, gy = y0 + ey;
    if (gx < nx && gy < ny) {
      const size_t g = (size_t)gy * P + gx;
      const int lx = ex + 1, ly = ey + 1;
      const double yc = ys[ly][lx];
      double s = M.P[g] * yc;
      s = fma(M.W[g], ys[ly][lx - 1], s);
      s = fma(M.E[g], ys[ly][lx + 1], s);
      s = fma(M.S[g], ys[ly - 1][lx], s);
      s = fma(M.N[g], ys[ly + 1][lx], s);
      y[g] = yc;
      w[g] = s;
    }
  }
}

// BiCGStab step 1: p = r + beta (p_old - omega v_old), y = D^-1 p, v = A y,
// alpha = rho1 / (r^, v)
__global__ void __launch_bounds__(NTM)
k_mom_pv(MomOp M, const double* r, const double* rh, const double* pold, double* pnew,
         const double* vold, double* vnew, double* y, MomScalars* sc, double* part) {
  pdl_wait();
  if (sc->done) return;
  __shared__ double ys[TY + 2][TX + 2];
  const double beta = (sc->rho1 / sc->rho) * (sc->alpha / sc->omega), om = sc->omega;
  auto form = [&](size_t g, bool own) {
    const double pv = fma(beta, fma(-om, vold[g], pold[g]), r[g]);
    if (own) pnew[g] = pv;
    return pv;
  };
  tile_apply(M, form, y, vnew, ys, nullptr, nullptr, nullptr, nullptr);
  __syncthreads();
  double acc = 0.0;
  const int nx = M.nx, ny = M.ny, P = M.pitch, x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  for (int e = tl(); e < TX * TY; e += NTM) {
    const int gx = x0 + e % TX, gy = y0 + e / TX;
    if (gx < nx && gy < ny) {
      const size_t g = (size_t)gy * P + gx;
      acc = fma(rh[g], vnew[g], acc);
    }
  }
  double tot, dummy;
  if (gsum2(acc, 0.0, part, &sc->tickets[1], &tot, &dummy) && tl() == 0) {
    sc->rho = sc->rho1;
    sc->alpha = sc->rho1 / tot;
    if (!isfinite(sc->alpha)) {
      sc->status = kErrNaN;
      sc->done = 1;
    }
  }
}

// BiCGStab step 2: s = r - alpha v, z = D^-1 s, t = A z, omega = (t,s)/(t,t)
__global__ void __launch_bounds__(NTM)
k_mom_st(MomOp M, const double* r, const double* v, double* s, double* z, double* tv,
         MomScalars* sc, double* part) {
  pdl_wait();
  if (sc->done) return;
  __shared__ double ys[TY + 2][TX + 2];
  const double alpha = sc->alpha;
  auto form = [&](size_t g, bool own) {
    const double sv = fma(-alpha, v[g], r[g]);
    if (own) s[g] = sv;
    return sv;
  };
  tile_apply(M, form, z, tv, ys, nullptr, nullptr, nullptr, nullptr);
  __syncthreads();
  double a1 = 0.0, a2 = 0.0;
  const int nx = M.nx, ny = M.ny, P = M.pitch, x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  for (int e = tl(); e < TX * TY; e += NTM) {
    const int gx = x0 + e % TX, gy = y0 + e / TX;
    if (gx < nx && gy < ny) {
      const size_t g = (size_t)gy * P + gx;
      a1 = fma(tv[g], s[g], a1);
      a2 = fma(tv[g], tv[g], a2);
    }
  }
  double ts, tt;
  if (gsum2(a1, a2, part, &sc->tickets[2], &ts, &tt) && tl() == 0) {
    sc->ts = ts;
    sc->tt = tt;
    sc->omega = tt > 0.0 ? ts / tt : 0.0;
  }
}

// BiCGStab step 3: x += alpha y + omega z, r = s - omega t, rho1 = (r^, r),
// convergence on ||r||
__global__ void __launch_bounds__(NTM)
k_mom_xr(MomOp M, double* x, double* r, const double* rh, const double* y, const double* z,
         const double* s, const double* tv, MomScalars* sc, double* part) {
  pdl_wait();
  if (sc->done) return;
  const double alpha = sc->alpha, om = sc->omega;
  double a1 = 0.0, a2 = 0.0;
  const int nx = M.nx, ny = M.ny, P = M.pitch, x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  for (int e = tl(); e < TX * TY; e += NTM) {
    const int gx = x0 + e % TX, gy = y0 + e / TX;
    if (gx < nx && gy < ny) {
      const size_t g = (size_t)gy * P + gx;
      x[g] = fma(om, z[g], fma(alpha, y[g], x[g]));
      const double rv = fma(-om, tv[g], s[g]);
      r[g] = rv;
      a1 = fma(rh[g], rv, a1);
      a2 = fma(rv, rv, a2);
    }
  }
  double rho1, rr;
  if (gsum2(a1, a2, part, &sc->tickets[3], &rho1, &rr) && tl() == 0) {
    sc->rho1 = rho1;
    sc->rr = rr;
    sc->iter += 1;
    if (!isfinite(rr)) {
      sc->status = kErrNaN;
      sc->done = 1;
    } else if (rr <= sc->rtol2 * sc->bnorm2) {
      sc->done = 1;
    } else if (sc->iter >= sc->maxit || sc->omega == 0.0 || rho1 == 0.0) {
      sc->status = kErrNotConverged;
      sc->done = 1;
    }
  }
}

// BiCGStab with a multigrid preconditioner on the right (the projection's
// FP64 V-cycle on the operator's symmetric part, scf_mgpre.cuh): the same
// recurrences as k_mom_pv / k_mom_st / k_mom_xr, with y = M^-1 p and
// z = M^-1 s coming from V-cycles between these kernels instead of the
// diagonal scaling inside them.  One thread per cell, grid-stride rows.
__device__ __forceinline__ double apply5(const MomOp& M, const double* y, size_t g) {
  double v = M.P[g] * y[g];
  v = fma(M.W[g], y[g - 1], v);
  v = fma(M.E[g], y[g + 1], v);
  v = fma(M.S[g], y[g - M.pitch], v);
  return fma(M.N[g], y[g + M.pitch], v);
}

// p = r + beta (p_old - omega v_old)
__global__ void k_momg_p(MomOp M, const double* r, const double* pold, const double* vold,
                         double* pnew, const MomScalars* sc) {
  pdl_wait();
  if (sc->done) return;
  const double beta = (sc->rho1 / sc->rho) * (sc->alpha / sc->omega), om = sc->omega;
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix >= M.nx) return;
  for (int iy = blockIdx.y * 8 + threadIdx.y; iy < M.ny; iy += gridDim.y * 8) {
    const size_t g = (size_t)iy * M.pitch + ix;
    pnew[g] = fma(beta, fma(-om, vold[g], pold[g]), r[g]);
  }
}

// v = A y, alpha = rho1 / (r^, v)
__global__ void k_momg_av(MomOp M, const double* y, double* v, const double* rh, MomScalars* sc,
                          double* part) {
  pdl_wait();
  if (sc->done) return;
  double acc = 0.0;
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix < M.nx)
    for (int iy = blockIdx.y * 8 + threadIdx.y; iy < M.ny; iy += gridDim.y * 8) {
      const size_t g = (size_t)iy * M.pitch + ix;
      const double vv = apply5(M, y, g);
      v[g] = vv;
      acc = fma(rh[g], vv, acc);
    }
  double tot, dummy;
  if (gsum2(acc, 0.0, part, &sc->tickets[1], &tot, &dummy) && tl() == 0) {
    sc->rho = sc->rho1;
    sc->alpha = sc->rho1 / tot;
    if (!isfinite(sc->alpha)) {
      sc->status = kErrNaN;
      sc->done = 1;
    }
  }
}

// s = r - alpha v
__global__ void k_momg_s(MomOp M, const double* r, const double* v, double* s,
                         const MomScalars* sc) {
  pdl_wait();
  if (sc->done) return;
  const double alpha = sc->alpha;
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix >= M.nx) return;
  for (int iy = blockIdx.y * 8 + threadIdx.y; iy < M.ny; iy += gridDim.y * 8) {
    const size_t g = (size_t)iy * M.pitch + ix;
    s[g] = fma(-alpha, v[g], r[g]);
  }
}

// t = A z, omega = (t, s) / (t, t)
__global__ void k_momg_at(MomOp M, const double* z, double* t, const double* s, MomScalars* sc,
                          double* part) {
  pdl_wait();
  if (sc->done) return;
  double a1 = 0.0, a2 = 0.0;
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix < M.nx)
    for (int iy = blockIdx.y * 8 + threadIdx.y; iy < M.ny; iy += gridDim.y * 8) {
      const size_t g = (size_t)iy * M.pitch + ix;
      const double tv = apply5(M, z, g);
      t[g] = tv;
      a1 = fma(tv, s[g], a1);
      a2 = fma(tv, tv, a2);
    }
  double ts, tt;
  if (gsum2(a1, a2, part, &sc->tickets[2], &ts, &tt) && tl() == 0) {
    sc->ts = ts;
    sc->tt = tt;
    sc->omega = tt > 0.0 ? ts / tt : 0.0;
  }
}

// DeltaGetValues + the gradient update of the component's cells
__global__ void k_mom_pred(MomIn in, int iu, int iv, int nx, int ny, int pitch, const double* x,
                           double* pred) {
  pdl_wait();
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix >= nx - iu) return;
  for (int iy = blockIdx.y * 8 + threadIdx.y; iy < ny - iv; iy += gridDim.y * 8) {
    const int i = ix + 1, j = iy + 1;
    const double xv = MF0(in.posnu, i, j) != -1 ? x[(size_t)iy * pitch + ix] : 0.0;
    MF0(pred, i, j) =
        add(xv, dvd(dvd(mul(in.dt, MF1(in.gradp, i, j)), MF1(in.dx, i, j)), MF1(in.dy, i, j)));
  }
}

// Dp boundary copies in the reference's order, then (v) the open top of
// Pred; one CTA, a barrier between dependent copies
__global__ void k_mom_edges(int iu, int nx, int ny, double* Dp, double* pred) {
  pdl_wait();
  const int t = threadIdx.x, nt = blockDim.x;
  auto col = [&](int dst, int src) {
    for (int j = t; j <= ny + 1; j += nt) MF0(Dp, dst, j) = MF0(Dp, src, j);
    __syncthreads();
  };
  auto row = [&](int dst, int src) {
    for (int i = t; i <= nx + 1; i += nt) MF0(Dp, i, dst) = MF0(Dp, i, src);
    __syncthreads();
  };
  if (iu == 1) {
    col(0, 1); col(nx, nx - 1); col(nx + 1, nx);
    row(0, 1); row(ny + 1, ny);
  } else {
    col(0, 1); col(nx + 1, nx);
    row(0, 1); row(ny, ny - 1); row(ny + 1, ny);
    for (int i = 1 + t; i <= nx; i += nt) MF0(pred, i, ny) = MF0(pred, i, ny - 1);
  }
}

#undef MF1
#undef MF0
#undef MFE
#undef MFN

}  // namespace
}  // namespace scf

using namespace scf;

struct scf_mom {
  int nx = 0, ny = 0, pitch = 0, device = 0;
  bool devptrs = false, own_stream = false;
  cudaStream_t stream = nullptr;
  std::vector<void*> allocs;
  MomOp op{};
  double *x = nullptr, *r = nullptr, *rh = nullptr, *p[2] = {nullptr, nullptr},
         *v[2] = {nullptr, nullptr}, *y = nullptr, *s = nullptr, *z = nullptr, *t = nullptr;
  double* part = nullptr;
  MomScalars *sc = nullptr, *sc_host = nullptr;
  // host mode: device staging of every input and of pred / Dp
  std::vector<double*> st;
  int32_t* st_posnu = nullptr;
  double *st_pred = nullptr, *st_Dp = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  bool solved = false;
  scf_proj* mg = nullptr;  // SCF_MOM_MG: multigrid preconditioner (a projection handle)
};

namespace {

#define MCK(call)                                                                     \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      fprintf(stderr, "scf_mom: %s failed: %s (%s:%d)\n", #call, cudaGetErrorString(e_), \
              __FILE__, __LINE__);                                                    \
      return e_ == cudaErrorMemoryAllocation ? SCF_ERR_NOMEM : SCF_ERR_CUDA;          \
    }                                                                                 \
  } while (0)

int malloc_zero(scf_mom* h, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? SCF_ERR_NOMEM : SCF_ERR_CUDA;
  h->allocs.push_back(*p);
  return cudaMemsetAsync(*p, 0, bytes ? bytes : 16, h->stream) == cudaSuccess ? SCF_OK
                                                                             : SCF_ERR_CUDA;
}
// padded array: rows -2 .. ny (base at row 2), zero
int padded(scf_mom* h, double** base) {
  void* p = nullptr;
  const int rc = malloc_zero(h, &p, sizeof(double) * (size_t)(h->ny + 3) * h->pitch);
  if (rc) return rc;
  *base = reinterpret_cast<double*>(p) + 2 * (size_t)h->pitch;
  return SCF_OK;
}

void free_all(scf_mom* h) {
  if (h->mg) scf_proj_destroy(h->mg);
  h->mg = nullptr;
  for (void* p : h->allocs) cudaFree(p);
  h->allocs.clear();
  if (h->sc_host) cudaFreeHost(h->sc_host);
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
}

dim3 row_grid(int nx, int ny) {
  const int gx = (nx + 31) / 32, gy0 = (ny + 7) / 8, cap = (152 * 16 + gx - 1) / gx;
  return dim3(gx, gy0 < cap ? gy0 : (cap < 1 ? 1 : cap));
}

}  // namespace

extern "C" {

int scf_mom_create(scf_mom** out, int nx, int ny, int flags, int device) {
  if (!out || nx < 2 || ny < 2 || nx > 65536 || ny > 65536) return SCF_ERR_ARG;
  *out = nullptr;
  scf_mom* h = new (std::nothrow) scf_mom();
  if (!h) return SCF_ERR_NOMEM;
  h->nx = nx; h->ny = ny; h->device = device;
  h->devptrs = (flags & SCF_FLAG_DEVICE_PTRS) != 0;
  h->pitch = round_up(nx + 2, 32);
  auto fail = [&](int rc) { free_all(h); delete h; return rc; };
  if (cudaSetDevice(device) != cudaSuccess) return fail(SCF_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(SCF_ERR_CUDA);
  h->own_stream = true;
  int rc;
  double** arrs[] = {&h->op.P, &h->op.W, &h->op.E, &h->op.S, &h->op.N, &h->op.di, &h->op.b,
                     &h->x, &h->r, &h->rh, &h->p[0], &h->p[1], &h->v[0], &h->v[1], &h->y,
                     &h->s, &h->z, &h->t};
  for (double** a : arrs)
    if ((rc = padded(h, a))) return fail(rc);
  h->op.nx = nx; h->op.ny = ny; h->op.pitch = h->pitch;
  const dim3 tg((nx + TX - 1) / TX, (ny + TY - 1) / TY), rg = row_grid(nx, ny);
  const size_t nblk = std::max((size_t)tg.x * tg.y, (size_t)rg.x * rg.y);
  if ((rc = malloc_zero(h, (void**)&h->part, sizeof(double) * (2 * nblk + 64)))) return fail(rc);
  if ((rc = malloc_zero(h, (void**)&h->sc, sizeof(MomScalars)))) return fail(rc);
  if (cudaMallocHost((void**)&h->sc_host, sizeof(MomScalars)) != cudaSuccess)
    return fail(SCF_ERR_NOMEM);
  memset(h->sc_host, 0, sizeof(MomScalars));
  if (!h->devptrs) {
    const size_t n1 = (size_t)nx * ny, n0 = (size_t)(nx + 2) * (ny + 2),
                 ne = (size_t)(nx + 1) * ny, nn = (size_t)nx * (ny + 1);
    const size_t sizes[] = {n1, n1, n1, n1, n1, n1, n0, n0, ne, ne, nn, nn, n1, n1, n0, n0};
    for (size_t sz : sizes) {
      void* p = nullptr;
      if ((rc = malloc_zero(h, &p, sz * sizeof(double)))) return fail(rc);
      h->st.push_back(reinterpret_cast<double*>(p));
    }
    if ((rc = malloc_zero(h, (void**)&h->st_posnu, n0 * sizeof(int32_t)))) return fail(rc);
    if ((rc = malloc_zero(h, (void**)&h->st_pred, n0 * sizeof(double)))) return fail(rc);
    if ((rc = malloc_zero(h, (void**)&h->st_Dp, n0 * sizeof(double)))) return fail(rc);
  }
  if (cudaEventCreate(&h->ev[0]) != cudaSuccess || cudaEventCreate(&h->ev[1]) != cudaSuccess)
    return fail(SCF_ERR_CUDA);
  if ((flags & SCF_MOM_MG) && (rc = mgpre_create(&h->mg, nx, ny, device))) return fail(rc);
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return fail(SCF_ERR_CUDA);
  *out = h;
  return SCF_OK;
}

void scf_mom_destroy(scf_mom* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_all(h);
  delete h;
}

int scf_mom_set_stream(scf_mom* h, void* stream) {
  if (!h) return SCF_ERR_ARG;
  MCK(cudaSetDevice(h->device));
  MCK(cudaStreamSynchronize(h->stream));
  if (h->own_stream) cudaStreamDestroy(h->stream);
  if (stream) {
    h->stream = (cudaStream_t)stream;
    h->own_stream = false;
  } else {
    MCK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->own_stream = true;
  }
  return SCF_OK;
}

int scf_mom_solve(scf_mom* h, int comp, const scf_mom_in* in, double* pred, double* Dp,
                  double rtol, int maxit, scf_stats* stt) {
  if (!h || !in || !pred || !Dp || (comp != 0 && comp != 1) || !(rtol >= 0.0) || maxit < 0)
    return SCF_ERR_ARG;
  const double* req[] = {in->dx, in->dy, in->vof, in->vofS, in->WlLh, in->delh, in->etaE,
                         in->etaN, in->difEW, in->edEW, in->difNS, in->edNS, in->flux,
                         in->gradp, in->u, in->v};
  for (const double* a : req)
    if (!a) return SCF_ERR_ARG;
  if (!in->posnu) return SCF_ERR_ARG;
  MCK(cudaSetDevice(h->device));
  const long long l0 = g_launches;
  const int nx = h->nx, ny = h->ny, iu = comp == 0 ? 1 : 0, iv = 1 - iu;
  const size_t n0 = (size_t)(nx + 2) * (ny + 2);
  cudaStream_t s = h->stream;
  MCK(cudaEventRecord(h->ev[0], s));
  MomIn d{};
  double *dpred = pred, *dDp = Dp;
  const double* src[16] = {in->dx, in->dy, in->vof, in->vofS, in->WlLh, in->delh, in->etaE,
                           in->etaN, in->difEW, in->edEW, in->difNS, in->edNS, in->flux,
                           in->gradp, in->u, in->v};
  const double* dev[16];
  if (h->devptrs) {
    for (int k = 0; k < 16; ++k) dev[k] = src[k];
    d.posnu = in->posnu;
  } else {
    const size_t n1 = (size_t)nx * ny, ne = (size_t)(nx + 1) * ny, nn = (size_t)nx * (ny + 1);
    const size_t sizes[16] = {n1, n1, n1, n1, n1, n1, n0, n0, ne, ne, nn, nn, n1, n1, n0, n0};
    for (int k = 0; k < 16; ++k) {
      MCK(cudaMemcpyAsync(h->st[k], src[k], sizes[k] * 8, cudaMemcpyHostToDevice, s));
      dev[k] = h->st[k];
    }
    MCK(cudaMemcpyAsync(h->st_posnu, in->posnu, n0 * 4, cudaMemcpyHostToDevice, s));
    MCK(cudaMemcpyAsync(h->st_pred, pred, n0 * 8, cudaMemcpyHostToDevice, s));
    MCK(cudaMemcpyAsync(h->st_Dp, Dp, n0 * 8, cudaMemcpyHostToDevice, s));
    d.posnu = h->st_posnu;
    dpred = h->st_pred;
    dDp = h->st_Dp;
  }
  d.dx = dev[0]; d.dy = dev[1]; d.vof = dev[2]; d.vofS = dev[3]; d.WlLh = dev[4];
  d.delh = dev[5]; d.etaE = dev[6]; d.etaN = dev[7]; d.difEW = dev[8]; d.edEW = dev[9];
  d.difNS = dev[10]; d.edNS = dev[11]; d.flux = dev[12]; d.gradp = dev[13]; d.u = dev[14];
  d.v = dev[15];
  d.dt = in->dt; d.beta_vis = in->beta_vis; d.nua = in->nua; d.nuw = in->nuw;
  d.nuref = in->nuref; d.rey = in->rey; d.fr = in->fr;
  // scalars: clear, then the solve's limits
  MomScalars init{};
  init.rtol2 = rtol * rtol;
  init.maxit = maxit;
  *h->sc_host = init;
  MCK(cudaMemcpyAsync(h->sc, h->sc_host, sizeof(MomScalars), cudaMemcpyHostToDevice, s));
  const dim3 rg = row_grid(nx, ny), blk(32, 8);
  launch_k(k_mom_assemble, rg, blk, 0, s, d, iu, iv, h->op, dDp, h->x, h->r, h->rh, h->p[0],
           h->v[0], h->sc, h->part);
  MCK(cudaGetLastError());
  const dim3 tg((nx + TX - 1) / TX, (ny + TY - 1) / TY);
  int it = 0, cur = 0;
  // host-polled: chunks of iterations (finished kernels return at once)
  MCK(cudaMemcpyAsync(h->sc_host, h->sc, sizeof(MomScalars), cudaMemcpyDeviceToHost, s));
  MCK(cudaStreamSynchronize(s));
  // the start was written with maxit from init; keep the host copy's limits
  if (h->mg) {  // the multigrid on this operator's symmetric part
    const int rc = mgpre_setup(h->mg, h->op.P, h->op.W, h->op.E, h->op.S, h->op.N, s);
    if (rc) return rc;
  }
  while (!h->sc_host->done && it < maxit) {
    for (int c = 0; c < 4 && it < maxit; ++c, ++it) {
      const int nxt = cur ^ 1;
      if (h->mg) {
        launch_k(k_momg_p, rg, blk, 0, s, h->op, (const double*)h->r, (const double*)h->p[cur],
                 (const double*)h->v[cur], h->p[nxt], (const MomScalars*)h->sc);
        int rc = mgpre_apply(h->mg, h->p[nxt], h->y, s);
        if (rc) return rc;
        launch_k(k_momg_av, rg, blk, 0, s, h->op, (const double*)h->y, h->v[nxt],
                 (const double*)h->rh, h->sc, h->part);
        launch_k(k_momg_s, rg, blk, 0, s, h->op, (const double*)h->r, (const double*)h->v[nxt],
                 h->s, (const MomScalars*)h->sc);
        if ((rc = mgpre_apply(h->mg, h->s, h->z, s))) return rc;
        launch_k(k_momg_at, rg, blk, 0, s, h->op, (const double*)h->z, h->t, (const double*)h->s,
                 h->sc, h->part);
      } else {
        launch_k(k_mom_pv, tg, dim3(NTM), 0, s, h->op, (const double*)h->r,
                 (const double*)h->rh, (const double*)h->p[cur], h->p[nxt],
                 (const double*)h->v[cur], h->v[nxt], h->y, h->sc, h->part);
        launch_k(k_mom_st, tg, dim3(NTM), 0, s, h->op, (const double*)h->r,
                 (const double*)h->v[nxt], h->s, h->z, h->t, h->sc, h->part);
      }
      launch_k(k_mom_xr, tg, dim3(NTM), 0, s, h->op, h->x, h->r, (const double*)h->rh,
               (const double*)h->y, (const double*)h->z, (const double*)h->s,
               (const double*)h->t, h->sc, h->part);
      cur = nxt;
    }
    MCK(cudaGetLastError());
    MCK(cudaMemcpyAsync(h->sc_host, h->sc, sizeof(MomScalars), cudaMemcpyDeviceToHost, s));
    MCK(cudaStreamSynchronize(s));
  }
  launch_k(k_mom_pred, row_grid(nx, ny), blk, 0, s, d, iu, iv, nx, ny, h->pitch,
           (const double*)h->x, dpred);
  launch_k(k_mom_edges, dim3(1), dim3(1024), 0, s, iu, nx, ny, dDp, dpred);
  MCK(cudaGetLastError());
  if (!h->devptrs) {
    MCK(cudaMemcpyAsync(pred, h->st_pred, n0 * 8, cudaMemcpyDeviceToHost, s));
    MCK(cudaMemcpyAsync(Dp, h->st_Dp, n0 * 8, cudaMemcpyDeviceToHost, s));
  }
  MCK(cudaMemcpyAsync(h->sc_host, h->sc, sizeof(MomScalars), cudaMemcpyDeviceToHost, s));
  MCK(cudaEventRecord(h->ev[1], s));
  MCK(cudaStreamSynchronize(s));
  h->solved = true;
  const MomScalars& S = *h->sc_host;
  int status = S.status;
  if (S.bad) status = SCF_ERR_NAN;
  if (!S.done && status == 0 && S.bnorm2 > 0.0) status = SCF_ERR_NOT_CONVERGED;
  if (stt) {
    memset(stt, 0, sizeof(*stt));
    stt->iters = S.iter;
    stt->status = status;
    stt->levels = 1;
    stt->bnorm = sqrt(S.bnorm2);
    stt->relres = S.bnorm2 > 0.0 ? sqrt(S.rr / S.bnorm2) : 0.0;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]);
    stt->ms_total = ms;
    stt->launches = (int)(g_launches - l0);
  }
  return status == kOk ? SCF_OK : status;
}

int scf_mom_get_system(scf_mom* h, double* matr, double* rhm) {
  if (!h || (!matr && !rhm)) return SCF_ERR_ARG;
  if (!h->solved) return SCF_ERR_STATE;
  MCK(cudaSetDevice(h->device));
  const int nx = h->nx, ny = h->ny, P = h->pitch;
  std::vector<double> buf((size_t)(ny + 3) * P);
  auto fetch = [&](const double* base, double* dst, size_t stride_f) -> int {
    MCK(cudaMemcpy(buf.data(), base - 2 * (size_t)P, buf.size() * 8, cudaMemcpyDeviceToHost));
    const double* b0 = buf.data() + 2 * (size_t)P;
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) dst[(size_t)i + (size_t)j * nx + stride_f] = b0[(size_t)j * P + i];
    return SCF_OK;
  };
  MCK(cudaStreamSynchronize(h->stream));
  int rc = SCF_OK;
  const size_t plane = (size_t)nx * ny;
  if (matr) {
    const double* order[5] = {h->op.S, h->op.W, h->op.P, h->op.E, h->op.N};
    for (int f = 0; f < 5 && rc == SCF_OK; ++f) rc = fetch(order[f], matr, f * plane);
  }
  if (rhm && rc == SCF_OK) rc = fetch(h->op.b, rhm, 0);
  return rc;
}

}  // extern "C"
