// scf_kernels.cu -- CUDA kernels (sm_103a) of the FP64 projection path:
// operator assembly, multigrid setup and V-cycle, PCG vector kernels with
// fused FP64 reductions, and the velocity correction.
//
// Arithmetic in the assembly, the multigrid kernels and the correction uses
// explicitly rounded operations (__dmul_rn/__dadd_rn/...) in the reference's
// operation order, so that no multiply-add is fused and results match a
// CPU restatement bit for bit.  The PCG vector updates use FMA freely.
#include <type_traits>

#include "scf_internal.cuh"

namespace scf {
namespace {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
// IEEE division, correctly rounded, on the integer pipe
__device__ __forceinline__ double dvd(double a, double b) { return div_rn(a, b); }

__device__ __forceinline__ int tid2() { return threadIdx.y * blockDim.x + threadIdx.x; }
__device__ __forceinline__ bool block00() {
  return blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0;
}

// Sum over a 256-thread block; the result is valid in thread 0.
__device__ double block_sum(double v) {
  __shared__ double sm[kThreads / 32];
  __syncthreads();
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int t = tid2();
  if ((t & 31) == 0) sm[t >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (t == 0)
    for (int w = 0; w < kThreads / 32; ++w) s += sm[w];
  return s;
}
__device__ double block_max(double v) {
  __shared__ double sm[kThreads / 32];
  __syncthreads();
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  int t = tid2();
  if ((t & 31) == 0) sm[t >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (t == 0)
    for (int w = 0; w < kThreads / 32; ++w) s = fmax(s, sm[w]);
  return s;
}

// Deterministic grid reduction: each block stores its partial, the last
// block to arrive combines all partials in block order.  Returns true in all
// threads of the last block; *total is valid in its thread 0.  The ticket is
// reset by the last block, so the kernel can be relaunched (graph replay).
template <bool kMax>
__device__ bool grid_reduce(double v, double* part, unsigned* ticket, double* total) {
  __shared__ bool last;
  const int t = tid2();
  const unsigned nb = gridDim.x * gridDim.y;
  const unsigned bid = blockIdx.y * gridDim.x + blockIdx.x;
  double s = kMax ? block_max(v) : block_sum(v);
  if (t == 0) {
    part[bid] = s;
    __threadfence();
    unsigned tk = atomicAdd(ticket, 1u);
    last = (tk == nb - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double acc = 0.0;
  for (unsigned k = t; k < nb; k += kThreads) {
    double pv = __ldcg(&part[k]);
    acc = kMax ? fmax(acc, pv) : acc + pv;
  }
  double tot = kMax ? block_max(acc) : block_sum(acc);
  if (t == 0) {
    *total = tot;
    *ticket = 0u;
  }
  return true;
}

// Two sums at once, same scheme (two partial slots per block).
__device__ bool grid_reduce2(double a, double b, double* part, unsigned* ticket, double* ta,
                             double* tb) {
  __shared__ bool last;
  const int t = tid2();
  const unsigned nb = gridDim.x * gridDim.y;
  const unsigned bid = blockIdx.y * gridDim.x + blockIdx.x;
  const double sa = block_sum(a);
  const double sb = block_sum(b);
  if (t == 0) {
    part[2 * bid] = sa;
    part[2 * bid + 1] = sb;
    __threadfence();
    last = (atomicAdd(ticket, 1u) == nb - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double xa = 0.0, xb = 0.0;
  for (unsigned k = t; k < nb; k += kThreads) {
    xa += __ldcg(&part[2 * k]);
    xb += __ldcg(&part[2 * k + 1]);
  }
  xa = block_sum(xa);
  xb = block_sum(xb);
  if (t == 0) {
    *ta = xa;
    *tb = xb;
    *ticket = 0u;
  }
  return true;
}

// ---------------------------------------------------------------------------
// Assembly: ComputePossionMatrixCoefficient + SetPoissonMatrix
// (src/ProjectionP_Mod.f90:395-580, :137-273).
// ---------------------------------------------------------------------------

// 1 = wet, 2 = dry, 0 = neither (NaN input); src/ProjectionP_Mod.f90:409-410, :493-494.
// The comparisons run on the integer pipe (an FP64 compare issues on GB300's
// slow FP64 pipe): for a non-NaN double x and a constant c > 0, x >= c
// exactly when the bit patterns compare so as signed 64-bit integers
// (negative x, -0 included, have negative patterns), and x < 0 exactly when
// the pattern is negative and not that of -0.  NaN operands make every
// comparison false, as in IEEE arithmetic.
__device__ __forceinline__ bool bits_nan(long long b) {
  return (b & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
}
__device__ __forceinline__ int cell_class(double vof, double phi, double vofS) {
  constexpr long long kHalfBits = 0x3fe0000000000000ll;  // 0.5
  constexpr long long kEpsiBits = 0x3f50624dd2f1a9fcll;  // 1.0e-3 (kEpsi)
  const long long v = __double_as_longlong(vof), p = __double_as_longlong(phi),
                  e = __double_as_longlong(vofS);
  const bool vn = bits_nan(v), pn = bits_nan(p), en = bits_nan(e);
  const bool v_ge = !vn && v >= kHalfBits, v_lt = !vn && v < kHalfBits;
  const bool e_lt = !en && e < kEpsiBits, e_ge = !en && e >= kEpsiBits;
  const bool p_neg = p < 0 && p != (long long)0x8000000000000000ull;
  const bool p_lt = !pn && p_neg, p_ge = !pn && !p_neg;
  if ((v_ge && e_lt) || (p_lt && e_ge)) return 1;
  if ((v_lt && e_lt) || (p_ge && e_ge)) return 2;
  return 0;
}

// Weighted density of the face between a cell of class cs and its neighbour
// of class cn (BetaW on wet cells, BetaD on dry cells).  Returns false where
// the reference leaves the coefficient unset.
__device__ __forceinline__ bool face_beta(int cs, int cn, double phis, double phin, double bP,
                                          double bM, double* B) {
  const double tol = 1.0e-24;
  if (cs == 1) {
    if (cn == 2) {
      double l = dvd(fabs(phis), add(add(fabs(phis), fabs(phin)), tol));
      *B = add(mul(l, bM), mul(sub(1.0, l), bP));
      return true;
    }
    if (cn == 1) { *B = bM; return true; }
    return false;
  }
  if (cs == 2) {
    if (cn == 1) {
      double l = dvd(fabs(phis), add(add(fabs(phis), fabs(phin)), tol));
      *B = add(mul(l, bP), mul(sub(1.0, l), bM));
      return true;
    }
    if (cn == 2) { *B = bP; return true; }
  }
  return false;
}
// face on the domain boundary: wet cells use BetaM, dry cells BetaP
__device__ __forceinline__ bool boundary_beta(int cs, double bP, double bM, double* B) {
  if (cs == 1) { *B = bM; return true; }
  if (cs == 2) { *B = bP; return true; }
  return false;
}
// PoCoef = Dp*len/dist*BetaP*BetaM/B, evaluated left to right
__device__ __forceinline__ double pocoef(double Dp, double len, double dist, double bP,
                                         double bM, double B) {
  return dvd(mul(mul(dvd(mul(Dp, len), dist), bP), bM), B);
}

// Inputs of one face's PoCoef, and whether the reference sets the face.
struct FaceIn {
  bool ok;
  double Dp, len, dist, B;
};
__device__ __forceinline__ bool same_bits(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b);
}
__device__ __forceinline__ bool same_face(const FaceIn& a, const FaceIn& b) {
  return a.ok == b.ok && (!a.ok || (same_bits(a.Dp, b.Dp) && same_bits(a.len, b.len) &&
                                    same_bits(a.dist, b.dist) && same_bits(a.B, b.B)));
}
__device__ __forceinline__ double face_pocoef(const FaceIn& f, double bP, double bM) {
  return f.ok ? pocoef(f.Dp, f.len, f.dist, bP, bM, f.B) : 0.0;
}
__device__ __forceinline__ double shfl_up_d(double v, int lane_delta) {
  return __shfl_up_sync(0xffffffffu, v, lane_delta);
}

// Operator assembly, one thread per cell column and a run of consecutive
// rows.  Every cell evaluates PoCoef on its four faces in the reference's
// order, but a face whose inputs (Dp, face length, node distance, density
// factor) equal bit for bit those of the same face seen from the other cell
// -- the east face of the west neighbour (one lane down the warp), the north
// face of the row below (this thread's previous row) -- takes that value
// instead of repeating the two IEEE FP64 divisions: the same function of the
// same bits.  Away from the interface every face qualifies, which halves the
// divisions on GB300's slow FP64 pipe.
__global__ void __launch_bounds__(kThreads, 4) k_assemble(FortranIn in, LevelView L, Scalars* sc) {
  pdl_wait();
  const int nx = in.nx, ny = in.ny;
  const int ix = blockIdx.x * kBX + threadIdx.x;
  const int lane = threadIdx.x;  // blockDim.x == 32: a warp is 32 consecutive columns
  const bool in_x = ix < nx;
  const int nthr_y = gridDim.y * kBY;
  const int chunk = (ny + nthr_y - 1) / nthr_y;
  const int r0 = (blockIdx.y * kBY + threadIdx.y) * chunk;
  const int r1 = r0 + chunk < ny ? r0 + chunk : ny;
  const double bP = in.betaP, bM = in.betaM;
  FaceIn prevN = {false, 0.0, 1.0, 1.0, 1.0};
  double prevNpc = 0.0;
  // the row range is the same for the whole warp: it stays converged for the shuffles
  for (int iy = r0; iy < r1; ++iy) {
    const int i = ix + 1, j = iy + 1;
    const size_t k1 = in_x ? fo1(nx, i, j) : 0, k0 = in_x ? fo0(nx, i, j) : 0;
    const size_t kl = (size_t)iy * L.pitch + ix;
    const bool act = in_x && in.posnu_p[k0] != -1;
    const double phis = act ? in.phi[k1] : 0.0;
    const int cs = act ? cell_class(in.vof[k1], phis, in.vofS[k1]) : 0;
    const double dxP = act ? in.dx[k1] : 1.0, dyP = act ? in.dy[k1] : 1.0;
    FaceIn f[4];  // S, W, E, N
#pragma unroll
    for (int q = 0; q < 4; ++q) f[q] = {false, 0.0, 1.0, 1.0, 1.0};
    if (act) {
      double B;
      if (j > 1) {
        const size_t kn = fo1(nx, i, j - 1);
        if (face_beta(cs, cell_class(in.vof[kn], in.phi[kn], in.vofS[kn]), phis, in.phi[kn], bP, bM, &B))
          f[0] = {true, in.DpV[fo0(nx, i, j - 1)], dxP, in.dyV[kn], B};
      } else if (boundary_beta(cs, bP, bM, &B)) {
        f[0] = {true, in.DpV[k0], dxP, in.dyV[k1], B};
      }
      if (i > 1) {
        const size_t kn = fo1(nx, i - 1, j);
        if (face_beta(cs, cell_class(in.vof[kn], in.phi[kn], in.vofS[kn]), phis, in.phi[kn], bP, bM, &B))
          f[1] = {true, in.DpU[fo0(nx, i - 1, j)], dyP, in.dxU[kn], B};
      } else if (boundary_beta(cs, bP, bM, &B)) {
        f[1] = {true, in.DpU[k0], dyP, in.dxU[k1], B};
      }
      if (i < nx) {
        const size_t kn = fo1(nx, i + 1, j);
        if (face_beta(cs, cell_class(in.vof[kn], in.phi[kn], in.vofS[kn]), phis, in.phi[kn], bP, bM, &B))
          f[2] = {true, in.DpU[k0], dyP, in.dxU[k1], B};
      } else if (boundary_beta(cs, bP, bM, &B)) {
        f[2] = {true, in.DpU[k0], dyP, in.dxU[k1], B};
      }
      if (j < ny) {
        const size_t kn = fo1(nx, i, j + 1);
        if (face_beta(cs, cell_class(in.vof[kn], in.phi[kn], in.vofS[kn]), phis, in.phi[kn], bP, bM, &B))
          f[3] = {true, in.DpV[k0], dxP, in.dyV[k1], B};
      } else if (boundary_beta(cs, bP, bM, &B)) {
        f[3] = {true, in.DpV[k0], dxP, in.dyV[k1], B};
      }
    }
    double pc[4];
    pc[2] = face_pocoef(f[2], bP, bM);
    pc[3] = face_pocoef(f[3], bP, bM);
    // west face: the east face of the lane below (all lanes shuffle)
    FaceIn wl;
    wl.ok = __shfl_up_sync(0xffffffffu, (int)f[2].ok, 1) != 0;
    wl.Dp = shfl_up_d(f[2].Dp, 1);
    wl.len = shfl_up_d(f[2].len, 1);
    wl.dist = shfl_up_d(f[2].dist, 1);
    wl.B = shfl_up_d(f[2].B, 1);
    const double pcl = shfl_up_d(pc[2], 1);
    pc[1] = (lane > 0 && same_face(f[1], wl)) ? pcl : face_pocoef(f[1], bP, bM);
    // south face: this thread's north face of the previous row
    pc[0] = (iy > r0 && same_face(f[0], prevN)) ? prevNpc : face_pocoef(f[0], bP, bM);
    prevN = f[3];
    prevNpc = pc[3];
    if (!in_x) continue;
    if (ix == 0) L.arow[iy] = 0;  // raised by k_excess where the row's entries differ
    if (!act) {
      L.cE[kl] = 0.0; L.cN[kl] = 0.0; L.dg[kl] = -1.0;
      L.wW[kl] = 0.0; L.wS[kl] = 0.0;
      continue;
    }
    const double aS = in.aS[k0], aW = in.aW[k0], aE = in.aE[k0], aN = in.aN[k0];
    const double tS = mul(pc[0], aS), tW = mul(pc[1], aW), tE = mul(pc[2], aE), tN = mul(pc[3], aN);
    double d = add(add(add(tS, tW), tE), tN);
    if (in.sb == 1 && j == 1) d = sub(d, tS);
    if (in.wb == 1 && i == 1) d = sub(d, tW);
    if (in.eb == 1 && i == nx) d = sub(d, tE);
    if (in.nb == 1 && j == ny) d = sub(d, tN);
    d = add(d, mul(copysign(1.0, d), 1.0e-24));
    if (!isfinite(d) || cs == 0) sc->anan = 1;
    L.dg[kl] = d;
    L.cE[kl] = (i < nx && in.posnu_p[fo0(nx, i + 1, j)] != -1) ? tE : 0.0;
    L.cN[kl] = (j < ny && in.posnu_p[fo0(nx, i, j + 1)] != -1) ? tN : 0.0;
    // the row's own west / south entries (src/ProjectionP_Mod.f90:176-195)
    L.wW[kl] = (i > 1 && in.posnu_p[fo0(nx, i - 1, j)] != -1) ? tW : 0.0;
    L.wS[kl] = (j > 1 && in.posnu_p[fo0(nx, i, j - 1)] != -1) ? tS : 0.0;
  }
}

// diagonal excess dg - (cE + cW + cN + cS), clamped at zero, and the
// inverse diagonal (0 where the cell has no unknown; skipped when di is null:
// the mixed-precision hierarchy builds its own FP32 inverse diagonals)
// also clears the per-level largest-coupling words (zero_bits, nzero) that
// the mixed setup's k_max_coupling raises after this kernel
//
// On the fine level (L.wW set) it also compares every row's own west / south
// entries with the neighbours' east / north ones, raises arow for the rows
// where one differs, and counts those faces and their largest relative
// difference into the solve's scalars.
__global__ void k_excess(LevelView L, double* di, unsigned* zero_bits, int nzero, Scalars* sc) {
  pdl_wait();
  if (zero_bits && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.y == 0 && threadIdx.x < nzero)
    zero_bits[threadIdx.x] = 0u;
  const int ix = blockIdx.x * kBX + threadIdx.x;
  int nasym = 0;
  float rmax = 0.0f;
  if (ix < L.nx) {
    for (int iy = blockIdx.y * kBY + threadIdx.y; iy < L.ny; iy += gridDim.y * kBY) {
      const size_t k = (size_t)iy * L.pitch + ix;
      const double d = L.dg[k];
      if (di) di[k] = d > 0.0 ? 1.0 / d : 0.0;
      if (d < 0.0) { L.ex[k] = 0.0; continue; }
      const double cw = L.cE[k - 1], cs = L.cN[k - L.pitch];
      double s = add(add(add(L.cE[k], cw), L.cN[k]), cs);
      double e = sub(d, s);
      L.ex[k] = e > 0.0 ? e : 0.0;
      if (L.wW) {
        const double ww = L.wW[k], ws = L.wS[k];
        const bool dw = ww != cw, ds = ws != cs;
        if (dw || ds) {
          L.arow[iy] = 1;
          nasym += (int)dw + (int)ds;
          if (dw) rmax = fmaxf(rmax, (float)(fabs(ww - cw) / fmax(fabs(ww), fabs(cw))));
          if (ds) rmax = fmaxf(rmax, (float)(fabs(ws - cs) / fmax(fabs(ws), fabs(cs))));
        }
      }
    }
  }
  if (L.wW && sc) {
    for (int o = 16; o > 0; o >>= 1) {
      nasym += __shfl_down_sync(0xffffffffu, nasym, o);
      rmax = fmaxf(rmax, __shfl_down_sync(0xffffffffu, rmax, o));
    }
    if (threadIdx.x == 0 && nasym > 0) {
      atomicAdd(&sc->asym_faces, nasym);
      atomicMax(&sc->asym_max_bits, __float_as_uint(rmax));
    }
  }
}

// Galerkin coarse operator for piecewise-constant 2x2 aggregation (and the
// coarse inverse diagonal)
__global__ void k_coarsen(LevelView F, LevelView C, double* di) {
  pdl_wait();
  const int I = blockIdx.x * kBX + threadIdx.x;
  if (I >= C.nx) return;
  const int nxf = F.nx, nyf = F.ny, pf = F.pitch;
  for (int J = blockIdx.y * kBY + threadIdx.y; J < C.ny; J += gridDim.y * kBY) {
    double ce = 0.0, cn = 0.0, ex = 0.0;
    int active = 0;
    for (int dj = 0; dj < 2; ++dj)
      for (int di = 0; di < 2; ++di) {
        int ix = 2 * I + di, iy = 2 * J + dj;
        if (ix >= nxf || iy >= nyf) continue;
        size_t k = (size_t)iy * pf + ix;
        if (F.dg[k] >= 0.0) active = 1;
        ex = add(ex, F.ex[k]);
        if (di == 1) ce = add(ce, F.cE[k]);
        if (dj == 1) cn = add(cn, F.cN[k]);
      }
    // couplings of the west and south coarse neighbours, same sums
    double cw = 0.0, cs = 0.0;
    if (I > 0)
      for (int dj = 0; dj < 2; ++dj) {
        int ix = 2 * I - 1, iy = 2 * J + dj;
        if (iy < nyf) cw = add(cw, F.cE[(size_t)iy * pf + ix]);
      }
    if (J > 0)
      for (int di = 0; di < 2; ++di) {
        int ix = 2 * I + di, iy = 2 * J - 1;
        if (ix < nxf) cs = add(cs, F.cN[(size_t)iy * pf + ix]);
      }
    const size_t kc = (size_t)J * C.pitch + I;
    C.cE[kc] = ce;
    C.cN[kc] = cn;
    C.ex[kc] = active ? ex : 0.0;
    double d = -1.0;
    if (active) {
      d = add(add(add(add(ce, cw), cn), cs), ex);
      if (!(d > 0.0)) d = -1.0;
    }
    C.dg[kc] = d;
    if (di) di[kc] = d > 0.0 ? 1.0 / d : 0.0;
  }
}

// Dense inverse of the coarsest operator (at most kMaxCoarse unknowns).  The
// operator is SPD with lexicographic numbering, so its bandwidth is at most
// the level's width: A = L D L^T is factored within the band (right-looking,
// no pivoting; one reciprocal per step, taken by the thread that finishes the
// next pivot), then each thread solves L D L^T x = e_c for one column c of
// the inverse.  kCoarseCtas CTAs split the columns; each factors the small
// matrix itself (n dependent steps), which is cheaper than a second launch
// to share the factor.
constexpr int kCoarseCtas = 8;
__global__ void __launch_bounds__(kMaxCoarse) k_coarse_setup(LevelView C, double* Ainv, int* cmap,
                                                             int* nc_out) {
  pdl_wait();
  constexpr int M = kMaxCoarse;
  __shared__ double A[M * M];  // row-major, stride M; L below the diagonal, D on it
  __shared__ double col[M], dinv[M];
  __shared__ int map[M], wsum[M / 32], band;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int ncell = C.nx * C.ny;
  // numbering of the cells that take part (dg >= 0), in lexicographic order
  const int ix = t % C.nx, iy = t / C.nx;
  const size_t kk = (size_t)iy * C.pitch + ix;
  const bool act = t < ncell && C.dg[kk] >= 0.0;
  const unsigned bal = __ballot_sync(0xffffffffu, act);
  if (lane == 0) wsum[w] = __popc(bal);
  if (t == 0) band = 0;
  for (int e = t; e < M * M; e += M) A[e] = 0.0;
  __syncthreads();
  int off = 0, n = 0;
  for (int k = 0; k < M / 32; ++k) {
    off += k < w ? wsum[k] : 0;
    n += wsum[k];
  }
  const int r = act ? off + __popc(bal & ((1u << lane) - 1)) : -1;
  map[t] = r;
  __syncthreads();
  if (act) {
    A[r * M + r] = C.dg[kk];
    int b = 0;
    if (ix + 1 < C.nx && map[t + 1] >= 0) {
      const int c = map[t + 1];
      A[r * M + c] = -C.cE[kk];
      A[c * M + r] = -C.cE[kk];
      b = c - r;
    }
    if (iy + 1 < C.ny && map[t + C.nx] >= 0) {
      const int c = map[t + C.nx];
      A[r * M + c] = -C.cN[kk];
      A[c * M + r] = -C.cN[kk];
      b = max(b, c - r);
    }
    atomicMax(&band, b);
  }
  __syncthreads();
  const int bw = band;
  if (t == 0 && n > 0) dinv[0] = 1.0 / A[0];
  __syncthreads();
  // step k: L[i][k] = A[i][k] / d_k, then A[i][j] -= L[i][k] A[j][k] for
  // k < j <= i <= k + bw (the trailing band triangle)
  for (int k = 0; k < n; ++k) {
    const int last = min(n - 1, k + bw);
    if (t > 0 && k + t <= last) {
      const int i = k + t;
      col[i] = A[i * M + k];
      A[i * M + k] = col[i] * dinv[k];
    }
    __syncthreads();
    const int m = last - k;  // trailing rows
    if (m == 0 && t == 0 && k + 1 < n) dinv[k + 1] = 1.0 / A[(k + 1) * M + k + 1];  // bw 0
    for (int e = t; e < m * m; e += M) {
      const int i = k + 1 + e / m, j = k + 1 + e % m;
      if (j <= i) {
        const double a = A[i * M + j] - A[i * M + k] * col[j];
        A[i * M + j] = a;
        if (e == 0) dinv[k + 1] = 1.0 / a;  // the next pivot is final
      }
    }
    __syncthreads();
  }
  // column c of the inverse: L y = e_c, z = D^-1 y, L^T x = z
  const int c = blockIdx.x + t * (int)gridDim.x;
  if (c < n) {
    double xv[M];
    for (int i = 0; i < n; ++i) {
      double y = i == c ? 1.0 : 0.0;
      if (i > c)
        for (int j = max(c, i - bw); j < i; ++j) y -= A[i * M + j] * xv[j];
      xv[i] = y;
    }
    for (int i = n - 1; i >= 0; --i) {
      double x = xv[i] * dinv[i];
      for (int j = i + 1; j <= min(n - 1, i + bw); ++j) x -= A[j * M + i] * xv[j];
      xv[i] = x;
      Ainv[(size_t)i * n + c] = x;
    }
  }
  if (blockIdx.x == 0) {
    for (int k = t; k < ncell; k += M) cmap[k] = map[k];
    if (t == 0) *nc_out = n;
  }
}

// ---------------------------------------------------------------------------
// Right-hand side: SetPoissonVectors (src/ProjectionP_Mod.f90:306-337).
// Also starts the PCG: r = b, x = 0, scalars reset.
// ---------------------------------------------------------------------------
__device__ void rhs_finish(double acc, bool bad, Scalars* sc, double* part, double rtol,
                           int maxit);

__global__ void k_rhs(FortranIn in, const double* us, const double* vs, double vb, int pitch,
                      double* bvec, double* r, float* r32, double* x, Scalars* sc, double* part,
                      double rtol, int maxit) {
  pdl_wait();
  const int nx = in.nx, ny = in.ny;
  const int ix = blockIdx.x * kBX + threadIdx.x;
  double acc = 0.0;
  bool bad = false;
  if (ix < nx) {
    for (int iy = blockIdx.y * kBY + threadIdx.y; iy < ny; iy += gridDim.y * kBY) {
      const int i = ix + 1, j = iy + 1;
      const size_t k1 = fo1(nx, i, j), k0 = fo0(nx, i, j);
      const size_t kl = (size_t)iy * pitch + ix;
      double bv = 0.0;
      if (in.posnu_p[k0] != -1) {
        const double dx = in.dx[k1], dy = in.dy[k1];
        double tx = mul(sub(mul(us[k0], in.aE[k0]), mul(us[fo0(nx, i - 1, j)], in.aW[k0])), dy);
        double ty = mul(sub(mul(vs[k0], in.aN[k0]), mul(vs[fo0(nx, i, j - 1)], in.aS[k0])), dx);
        bv = add(sub(-tx, ty), mul(mul(vb, in.nyS[k1]), in.WlLh[k1]));
        if (!isfinite(bv)) bad = true;
      }
      bvec[kl] = bv;
      r[kl] = bv;
      if (r32) r32[kl] = (float)bv;
      x[kl] = 0.0;
      acc = fma(bv, bv, acc);
    }
  }
  rhs_finish(acc, bad, sc, part, rtol, maxit);
}

// PCG start from a given right-hand side bF (Fortran (nx,ny) order; zero on
// cells without an unknown): the same state as k_rhs leaves
__global__ void k_rhs_given(int nx, int ny, const double* bF, LevelView L, double* bvec,
                            double* r, float* r32, double* x, Scalars* sc, double* part,
                            double rtol, int maxit) {
  pdl_wait();
  const int ix = blockIdx.x * kBX + threadIdx.x;
  double acc = 0.0;
  bool bad = false;
  if (ix < nx) {
    for (int iy = blockIdx.y * kBY + threadIdx.y; iy < ny; iy += gridDim.y * kBY) {
      const size_t kl = (size_t)iy * L.pitch + ix;
      const double bv = L.dg[kl] > 0.0 ? bF[(size_t)iy * nx + ix] : 0.0;
      if (!isfinite(bv)) bad = true;
      bvec[kl] = bv;
      r[kl] = bv;
      if (r32) r32[kl] = (float)bv;
      x[kl] = 0.0;
      acc = fma(bv, bv, acc);
    }
  }
  rhs_finish(acc, bad, sc, part, rtol, maxit);
}

// last step of the right-hand side kernels: ||b||^2 and the PCG scalars
__device__ void rhs_finish(double acc, bool bad, Scalars* sc, double* part, double rtol,
                           int maxit) {
  if (bad) sc->nan = 1;
  double tot;
  if (grid_reduce<false>(acc, part, &sc->tickets[T_RHS], &tot) && tid2() == 0) {
    sc->bnorm2 = tot;
    sc->rr = tot;
    sc->rr_prev = tot;
    sc->rtol2 = rtol * rtol * tot;
    sc->rz = 0.0; sc->pq = 0.0; sc->alpha = 0.0; sc->beta = 0.0;
    sc->iter = 0;
    sc->maxit = maxit;
    sc->status = kOk;
    sc->done = 0;
    if (!(tot > 0.0)) sc->done = 1;  // b = 0: x = 0 is the solution
    if (!isfinite(tot) || sc->nan) { sc->status = kErrNaN; sc->done = 1; }
    sc->pad[0] = 0;  // guard counter of the graph loop
  }
}

// ---------------------------------------------------------------------------
// PCG vector update.
// ---------------------------------------------------------------------------

// x += alpha p, r -= alpha q, reduce r.r (and, for the flexible PCG, the
// cross term r_new.z of the next beta, with z the preconditioned residual of
// this iteration, in FP32 per thread); the last block advances the
// iteration count, tests convergence and, inside a graph loop, clears the
// loop condition.  Block (0,0) also counts body executions and stops the
// loop after maxit+2 of them whatever else happens.
template <class PT>
__global__ void k_update_xr(LevelView L, double* __restrict__ x, const PT* __restrict__ p,
                            double* __restrict__ r, float* __restrict__ r32,
                            const float* __restrict__ z32, const double* __restrict__ q,
                            Scalars* sc, double* part, unsigned long long cond) {
  pdl_wait();
  if (cond && block00()) {
    int g = atomicAdd(&sc->pad[0], 1);
    if (g + 1 >= sc->maxit + 2) cudaGraphSetConditional(cond, 0u);
  }
  if (sc->done) {
    if (cond && block00()) cudaGraphSetConditional(cond, 0u);
    return;
  }
  const int ix0 = 2 * (blockIdx.x * kBX + threadIdx.x);
  const double alpha = sc->alpha;
  double acc = 0.0;
  float crs = 0.0f;
  if (ix0 < L.nx) {
    for (int iy = blockIdx.y * kBY + threadIdx.y; iy < L.ny; iy += gridDim.y * kBY) {
      const size_t k = (size_t)iy * L.pitch + ix0;
      double2 xv = *reinterpret_cast<double2*>(x + k);
      double2 rv = *reinterpret_cast<double2*>(r + k);
      double2 pv;
      if constexpr (std::is_same<PT, float>::value) {
        const float2 pf = *reinterpret_cast<const float2*>(p + k);
        pv = make_double2(f2d_exact(pf.x), f2d_exact(pf.y));
      } else {
        pv = *reinterpret_cast<const double2*>(p + k);
      }
      const double2 qv = *reinterpret_cast<const double2*>(q + k);
      xv.x = fma(alpha, pv.x, xv.x);
      rv.x = fma(-alpha, qv.x, rv.x);
      acc = fma(rv.x, rv.x, acc);
      if (ix0 + 1 < L.nx) {
        xv.y = fma(alpha, pv.y, xv.y);
        rv.y = fma(-alpha, qv.y, rv.y);
        acc = fma(rv.y, rv.y, acc);
        *reinterpret_cast<double2*>(x + k) = xv;
        *reinterpret_cast<double2*>(r + k) = rv;
        if (r32) {
          const float2 rf = make_float2(d2f_rn(rv.x), d2f_rn(rv.y));
          *reinterpret_cast<float2*>(r32 + k) = rf;
          if (z32) {
            const float2 zf = *reinterpret_cast<const float2*>(z32 + k);
            crs = fmaf(rf.x, zf.x, crs);
            crs = fmaf(rf.y, zf.y, crs);
          }
        }
      } else {
        x[k] = xv.x;
        r[k] = rv.x;
        if (r32) {
          const float rf = d2f_rn(rv.x);
          r32[k] = rf;
          if (z32) crs = fmaf(rf, z32[k], crs);
        }
      }
    }
  }
  double tot, cross;
  if (grid_reduce2(acc, (double)crs, part, &sc->tickets[T_RR], &tot, &cross) && tid2() == 0) {
    sc->rz_cross = cross;
    sc->rr_prev = sc->rr;
    sc->rr = tot;
    sc->iter += 1;
    if (!isfinite(tot) || !isfinite(sc->alpha)) {
      sc->status = kErrNaN;
      sc->done = 1;
    } else if (tot <= sc->rtol2) {
      sc->done = 1;
    } else if (sc->iter >= sc->maxit) {
      sc->status = kErrNotConverged;
      sc->done = 1;
    }
    if (sc->done && cond) cudaGraphSetConditional(cond, 0u);
  }
}

// ---------------------------------------------------------------------------
// Solution scatter, FP64 residual check and velocity correction:
// DeltaPressureGetValues / DeltaPressureBoundaryCondition
// (src/ProjectionP_Mod.f90:356-393, :582-595) and UpdatePUV
// (src/ComputePUV_Mod.f90:59-169).
// ---------------------------------------------------------------------------

// Pressure-gradient correction of one face between cells s (self) and n
// (east or north neighbour): returns false when the reference leaves the
// face alone.  G = (Pp_n - Pp_s)*BetaM*BetaP/BetaW*Dp/dist, every operation
// rounded as in the reference.
__device__ __forceinline__ bool face_grad(int cs, int cn, double phis, double phin, double pps,
                                          double ppn, double bP, double bM, double Dp,
                                          double dist, double* G) {
  const double tol = 1.0e-24;
  const double t = mul(mul(sub(ppn, pps), bM), bP);
  double q;
  if (cs == 1) {
    if (cn == 2) {
      double l = dvd(fabs(phis), add(add(fabs(phis), fabs(phin)), tol));
      q = dvd(t, add(mul(l, bM), mul(sub(1.0, l), bP)));
    } else if (cn == 1) {
      q = dvd(t, bM);
    } else {
      return false;
    }
  } else if (cs == 2) {
    if (cn == 1) {
      double l = dvd(fabs(phis), add(add(fabs(phis), fabs(phin)), tol));
      q = dvd(t, add(mul(l, bP), mul(sub(1.0, l), bM)));
    } else if (cn == 2) {
      q = dvd(t, bP);
    } else {
      return false;
    }
  } else {
    return false;
  }
  *G = dvd(mul(q, Dp), dist);
  return true;
}

__global__ void __launch_bounds__(kThreads, 4)
k_final_solution(FortranIn in, LevelView L, const double* __restrict__ x,
                                 const double* __restrict__ bvec, const double* __restrict__ us,
                                 const double* __restrict__ vs, double* Pp, double* p, double* u,
                                 double* v, int correct, Scalars* sc, double* part) {
  pdl_wait();
  const int nx = in.nx, ny = in.ny;
  const int ix = blockIdx.x * kBX + threadIdx.x;
  const int P = L.pitch;
  double acc = 0.0;
  if (ix < nx) {
    for (int iy = blockIdx.y * kBY + threadIdx.y; iy < ny; iy += gridDim.y * kBY) {
      const int i = ix + 1, j = iy + 1;
      const size_t k1 = fo1(nx, i, j), k0 = fo0(nx, i, j);
      const size_t kl = (size_t)iy * P + ix;
      const bool act = in.posnu_p[k0] != -1;
      const double ppc = act ? x[kl] : 0.0;
      if (Pp) {
        Pp[k0] = ppc;
        if (i == 1) Pp[fo0(nx, 0, j)] = (double)in.wb * ppc;
        if (i == nx) Pp[fo0(nx, nx + 1, j)] = (double)in.eb * ppc;
        if (j == 1) Pp[fo0(nx, i, 0)] = (double)in.sb * ppc;
        if (j == ny) Pp[fo0(nx, i, ny + 1)] = (double)in.nb * ppc;
        if (i == 1 && j == 1) {
          Pp[fo0(nx, 0, 0)] = 0.0; Pp[fo0(nx, nx + 1, 0)] = 0.0;
          Pp[fo0(nx, 0, ny + 1)] = 0.0; Pp[fo0(nx, nx + 1, ny + 1)] = 0.0;
        }
      }
      if (act) {
        const bool own = L.arow && L.arow[iy];  // the row's own west / south entries
        const double cw = own ? L.wW[kl] : L.cE[kl - 1], cs = own ? L.wS[kl] : L.cN[kl - P];
        double ax = pos_part(L.dg[kl]) * x[kl] - L.cE[kl] * x[kl + 1] - cw * x[kl - 1] -
                    L.cN[kl] * x[kl + P] - cs * x[kl - P];
        double rr = bvec[kl] - ax;
        acc = fma(rr, rr, acc);
      }
      if (!correct) continue;
      const double bP = in.betaP, bM = in.betaM;
      const double phis = in.phi[k1];
      const int cs = cell_class(in.vof[k1], phis, in.vofS[k1]);
      if (i <= nx - 1 && in.posnu_u[k0] != -1 && in.moex_u[k1] != 1) {
        const size_t kn = fo1(nx, i + 1, j);
        const double ppn = in.posnu_p[fo0(nx, i + 1, j)] != -1 ? x[kl + 1] : 0.0;
        double G;
        if (face_grad(cs, cell_class(in.vof[kn], in.phi[kn], in.vofS[kn]), phis, in.phi[kn], ppc,
                      ppn, bP, bM, in.DpU[k0], in.dxU[k1], &G))
          u[k0] = sub(us[k0], G);
      }
      if (j <= ny - 1 && in.posnu_v[k0] != -1 && in.moex_v[k1] != 1) {
        const size_t kn = fo1(nx, i, j + 1);
        const double ppn = in.posnu_p[fo0(nx, i, j + 1)] != -1 ? x[kl + P] : 0.0;
        double G;
        if (face_grad(cs, cell_class(in.vof[kn], in.phi[kn], in.vofS[kn]), phis, in.phi[kn], ppc,
                      ppn, bP, bM, in.DpV[k0], in.dyV[k1], &G))
          v[k0] = sub(vs[k0], G);
      }
      if (act) p[k0] = ppc;
    }
  }
  double tot;
  if (grid_reduce<false>(acc, part, &sc->tickets[T_RES], &tot) && tid2() == 0)
    sc->res_true2 = tot;
}

// top-row continuity (src/ComputePUV_Mod.f90:177-182) and mass residual (:184-216)
__global__ void k_final_mres(FortranIn in, double vb, double* u, double* v, double* mres,
                             Scalars* sc, double* part) {
  pdl_wait();
  const int nx = in.nx, ny = in.ny;
  const int ix = blockIdx.x * kBX + threadIdx.x;
  double acc = 0.0;
  if (ix < nx) {
    for (int iy = blockIdx.y * kBY + threadIdx.y; iy < ny; iy += gridDim.y * kBY) {
      const int i = ix + 1, j = iy + 1;
      const size_t k1 = fo1(nx, i, j), k0 = fo0(nx, i, j);
      const double dx = in.dx[k1], dy = in.dy[k1];
      const double aE = in.aE[k0], aW = in.aW[k0], aN = in.aN[k0], aS = in.aS[k0];
      const double ue = u[k0], uw = u[fo0(nx, i - 1, j)], vsb = v[fo0(nx, i, j - 1)];
      double vn = v[k0];
      if (j == ny) {
        vn = dvd(dvd(add(mul(add(-mul(ue, aE), mul(uw, aW)), dy), mul(mul(vsb, aS), dx)), dx), aN);
        v[k0] = vn;
      }
      double m = sub(add(mul(sub(mul(ue, aE), mul(uw, aW)), dy), mul(sub(mul(vn, aN), mul(vsb, aS)), dx)),
                     mul(mul(vb, in.nyS[k1]), in.WlLh[k1]));
      if (in.vofS[k1] > 1.0 - kEpsi) m = 0.0;
      mres[k1] = m;
      if (in.posnu_p[k0] != -1) acc = fmax(acc, fabs(m));
    }
  }
  double tot;
  if (grid_reduce<true>(acc, part, &sc->tickets[T_MRES], &tot) && tid2() == 0) sc->mres_max = tot;
}

// VariablesInternalCellCondition (src/ComputePUV_Mod.f90:227-245)
__global__ void k_final_zero(FortranIn in, double* p, double* u, double* v) {
  pdl_wait();
  const int nx = in.nx, ny = in.ny;
  const int ix = blockIdx.x * kBX + threadIdx.x;
  if (ix >= nx) return;
  for (int iy = blockIdx.y * kBY + threadIdx.y; iy < ny; iy += gridDim.y * kBY) {
    const int i = ix + 1, j = iy + 1;
    const size_t k1 = fo1(nx, i, j), k0 = fo0(nx, i, j);
    if (in.vofS[k1] > 1.0 - kEpsi) p[k0] = 0.0;
    if (in.vofS_u[k1] >= 1.0 - kEpsi) u[k0] = 0.0;
    if (in.vofS_v[k1] >= 1.0 - kEpsi) v[k0] = 0.0;
  }
}

// The reference's dense copy matr(Isize,Jsize,5) of the assembled rows
// (src/ProjectionP_Mod.f90:176-230): S, W, diagonal, E, N entries of each
// row, negated couplings off the diagonal, 0 where the row has no entry and
// on cells without an unknown.
__global__ void k_matr_out(FortranIn in, LevelView L, double* __restrict__ matr) {
  pdl_wait();
  const int nx = in.nx, ny = in.ny;
  const int ix = blockIdx.x * kBX + threadIdx.x;
  if (ix >= nx) return;
  const size_t n1 = (size_t)nx * ny;
  for (int iy = blockIdx.y * kBY + threadIdx.y; iy < ny; iy += gridDim.y * kBY) {
    const int i = ix + 1, j = iy + 1;
    const size_t k1 = fo1(nx, i, j), kl = (size_t)iy * L.pitch + ix;
    double m[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (in.posnu_p[fo0(nx, i, j)] != -1) {
      if (j > 1 && in.posnu_p[fo0(nx, i, j - 1)] != -1) m[0] = -L.wS[kl];
      if (i > 1 && in.posnu_p[fo0(nx, i - 1, j)] != -1) m[1] = -L.wW[kl];
      m[2] = L.dg[kl];
      if (i < nx && in.posnu_p[fo0(nx, i + 1, j)] != -1) m[3] = -L.cE[kl];
      if (j < ny && in.posnu_p[fo0(nx, i, j + 1)] != -1) m[4] = -L.cN[kl];
    }
#pragma unroll
    for (int f = 0; f < 5; ++f) matr[k1 + f * n1] = m[f];
  }
}

// the assembly's division on arrays (diagnostics)
__global__ void k_divide(const double* a, const double* b, double* q, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x)
    q[k] = dvd(a[k], b[k]);
}

// the library's integer-pipe square root on an array (diagnostics)
__global__ void k_sqrt(const double* a, double* q, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x)
    q[k] = sqrt_rn(a[k]);
}

__global__ void k_to_fortran(LevelView L, const double* src, double* dst) {
  pdl_wait();
  const int ix = blockIdx.x * kBX + threadIdx.x;
  if (ix >= L.nx) return;
  for (int iy = blockIdx.y * kBY + threadIdx.y; iy < L.ny; iy += gridDim.y * kBY)
    dst[(size_t)ix + (size_t)iy * L.nx] = src[(size_t)iy * L.pitch + ix];
}
__global__ void k_to_fortran_f(LevelView L, const float* src, double* dst) {
  pdl_wait();
  const int ix = blockIdx.x * kBX + threadIdx.x;
  if (ix >= L.nx) return;
  for (int iy = blockIdx.y * kBY + threadIdx.y; iy < L.ny; iy += gridDim.y * kBY)
    dst[(size_t)ix + (size_t)iy * L.nx] = (double)src[(size_t)iy * L.pitch + ix];
}
__global__ void k_from_fortran_f(LevelView L, const double* src, float* dst) {
  pdl_wait();
  const int ix = blockIdx.x * kBX + threadIdx.x;
  if (ix >= L.nx) return;
  for (int iy = blockIdx.y * kBY + threadIdx.y; iy < L.ny; iy += gridDim.y * kBY)
    dst[(size_t)iy * L.pitch + ix] = (float)src[(size_t)ix + (size_t)iy * L.nx];
}
__global__ void k_from_fortran(LevelView L, const double* src, double* dst) {
  pdl_wait();
  const int ix = blockIdx.x * kBX + threadIdx.x;
  if (ix >= L.nx) return;
  for (int iy = blockIdx.y * kBY + threadIdx.y; iy < L.ny; iy += gridDim.y * kBY)
    dst[(size_t)iy * L.pitch + ix] = src[(size_t)ix + (size_t)iy * L.nx];
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static const dim3 kBlock(kBX, kBY);

void launch_assemble(const FortranIn& in, LevelView L0, Scalars* sc, cudaStream_t s) {
  launch_k(k_assemble, grid_for(in.nx, in.ny, 1), kBlock, 0, s, in, L0, sc);
}
void launch_matr_out(const FortranIn& in, LevelView L0, double* matr, cudaStream_t s) {
  launch_k(k_matr_out, grid_for(in.nx, in.ny, 1), kBlock, 0, s, in, L0, matr);
}
void launch_divide(const double* a, const double* b, double* q, long long n, cudaStream_t s) {
  launch_k(k_divide, dim3(152 * 8), dim3(256), 0, s, a, b, q, n);
}
void launch_sqrt(const double* a, double* q, long long n, cudaStream_t s) {
  launch_k(k_sqrt, dim3(152 * 8), dim3(256), 0, s, a, q, n);
}
void launch_excess(LevelView L, double* di, unsigned* zero_bits, int nzero, Scalars* sc,
                   cudaStream_t s) {
  launch_k(k_excess, grid_for(L.nx, L.ny, 1), kBlock, 0, s, L, di, zero_bits, nzero, sc);
}
void launch_coarsen(LevelView F, LevelView C, double* di, cudaStream_t s) {
  launch_k(k_coarsen, grid_for(C.nx, C.ny, 1), kBlock, 0, s, F, C, di);
}
void launch_coarse_setup(LevelView C, double* Ainv, int* cmap, int* nc, cudaStream_t s) {
  launch_k(k_coarse_setup, dim3(kCoarseCtas), dim3(kMaxCoarse), 0, s, C, Ainv, cmap, nc);
}
void launch_rhs(const FortranIn& in, const double* ustar, const double* vstar, double vb,
                LevelView L0, double* bvec, double* r, float* r32, double* x, Scalars* sc,
                double* part, double rtol, int maxit, cudaStream_t s) {
  launch_k(k_rhs, grid_for(in.nx, in.ny, 1), kBlock, 0, s, in, ustar, vstar, vb, L0.pitch, bvec,
           r, r32, x, sc, part, rtol, maxit);
}
void launch_rhs_given(int nx, int ny, const double* bF, LevelView L0, double* bvec, double* r,
                      float* r32, double* x, Scalars* sc, double* part, double rtol, int maxit,
                      cudaStream_t s) {
  launch_k(k_rhs_given, grid_for(nx, ny, 1), kBlock, 0, s, nx, ny, bF, L0, bvec, r, r32, x, sc,
           part, rtol, maxit);
}
// Grid of the x/r update: one wave of resident CTAs (grid-stride rows), so
// that every thread walks nearly the same number of rows and no partly
// filled second wave follows.
template <class PT>
dim3 xr_grid(int nx, int ny) {
  static int per[16];  // resident CTAs per SM, per device (0 = unknown)
  int dev = 0;
  cudaGetDevice(&dev);
  int& c = per[dev & 15];
  if (c == 0) {
    int sms = 0, n = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_update_xr<PT>, kThreads, 0);
    c = sms * n > 0 ? sms * n : 1;
  }
  const dim3 g = grid_for(nx, ny);
  const int gy = c / (int)g.x > 1 ? c / (int)g.x : 1;
  return dim3(g.x, gy < (int)g.y ? gy : g.y);
}

void launch_update_xr(LevelView L0, double* x, const double* p, double* r, float* r32,
                      const float* z32, const double* q, Scalars* sc, double* part,
                      unsigned long long cond, cudaStream_t s) {
  launch_k(k_update_xr<double>, xr_grid<double>(L0.nx, L0.ny), kBlock, 0, s, L0, x, p, r, r32,
           z32, q, sc, part, cond);
}
void launch_update_xr(LevelView L0, double* x, const float* p, double* r, float* r32,
                      const float* z32, const double* q, Scalars* sc, double* part,
                      unsigned long long cond, cudaStream_t s) {
  launch_k(k_update_xr<float>, xr_grid<float>(L0.nx, L0.ny), kBlock, 0, s, L0, x, p, r, r32,
           z32, q, sc, part, cond);
}
void launch_final_solution(const FortranIn& in, LevelView L0, const double* x,
                           const double* bvec, const double* ustar, const double* vstar,
                           double* Pp, double* p, double* u, double* v, int correct,
                           Scalars* sc, double* part, cudaStream_t s) {
  launch_k(k_final_solution, grid_for(in.nx, in.ny, 1), kBlock, 0, s, in, L0, x, bvec, ustar, vstar, Pp,
                                                                 p, u, v, correct, sc, part);
}
void launch_final_mres(const FortranIn& in, double vb, double* u, double* v, double* mres,
                       Scalars* sc, double* part, cudaStream_t s) {
  launch_k(k_final_mres, grid_for(in.nx, in.ny, 1), kBlock, 0, s, in, vb, u, v, mres, sc, part);
}
void launch_final_zero(const FortranIn& in, double* p, double* u, double* v, cudaStream_t s) {
  launch_k(k_final_zero, grid_for(in.nx, in.ny, 1), kBlock, 0, s, in, p, u, v);
}
void launch_to_fortran(LevelView L, const double* src, double* dst, cudaStream_t s) {
  launch_k(k_to_fortran, grid_for(L.nx, L.ny, 1), kBlock, 0, s, L, src, dst);
}
void launch_to_fortran_f(LevelView L, const float* src, double* dst, cudaStream_t s) {
  launch_k(k_to_fortran_f, grid_for(L.nx, L.ny, 1), kBlock, 0, s, L, src, dst);
}
void launch_from_fortran_f(LevelView L, const double* src, float* dst, cudaStream_t s) {
  launch_k(k_from_fortran_f, grid_for(L.nx, L.ny, 1), kBlock, 0, s, L, src, dst);
}
void launch_from_fortran(LevelView L, const double* src, double* dst, cudaStream_t s) {
  launch_k(k_from_fortran, grid_for(L.nx, L.ny, 1), kBlock, 0, s, L, src, dst);
}

}  // namespace scf
