// scf_line.cu -- alternating zebra line relaxation for the multigrid V-cycle,
// used on anisotropic operators (stretched grids), where the point red-black
// smoother stalls.
//
// One pass relaxes every grid line of one parity in one direction exactly:
// each line is a tridiagonal system (the couplings along the line), its
// right-hand side holds b plus the couplings to the two neighbouring lines
// of the other parity.  Lines run along x in the level's own layout; lines
// along y run the same kernel on a transposed copy of the level (operator
// transposed at setup, x and b transposed inside the V-cycle by tiled
// shared-memory transposes), so every line kernel reads contiguous rows.
// The residual restriction and the prolongation work on the transposed
// copy, and the restriction writes both layouts of the coarse right-hand
// side, so a level costs two transposes of x per V-cycle.
//
// A line is solved by one CTA.  Thread t owns M consecutive cells; the last
// of them is an interface cell, the first M-1 are interior.  Each thread
// eliminates its interior cells (Thomas algorithm with three right-hand
// sides: the data, a unit value on the left interface, a unit value on its
// own interface), which leaves one equation per thread that couples only
// the interfaces of threads t-1, t, t+1 -- the Schur complement, again a
// symmetric diagonally dominant tridiagonal system.  That system is solved
// by the same splitting one level up (each warp's last lane is the warp's
// interface; cyclic reduction by warp shuffles inside each warp, then over
// the warps' interfaces), and every thread then recovers its interior cells
// from its two interface values.  The
// interfaces of an M-matrix keep every pivot positive, so no pivoting is
// needed.
#include <type_traits>

#include "scf_mg.cuh"

namespace scf {
namespace {

template <class CT, class T>
__device__ __forceinline__ T lcoef(const CT* p, size_t k, float cs);
template <>
__device__ __forceinline__ double lcoef<double, double>(const double* p, size_t k, float) {
  return p[k];
}
template <>
__device__ __forceinline__ float lcoef<__nv_bfloat16, float>(const __nv_bfloat16* p, size_t k,
                                                               float cs) {
  return __bfloat162float(p[k]) * cs;
}

// M consecutive values from an aligned row position as T (16-byte vector
// loads; a chunk never extends past the row's padded pitch).  The words of
// each vector are unpacked by value, so nothing goes through local memory.
__device__ __forceinline__ void unpack(const uint4& u, float* e) {
  e[0] = __uint_as_float(u.x); e[1] = __uint_as_float(u.y);
  e[2] = __uint_as_float(u.z); e[3] = __uint_as_float(u.w);
}
__device__ __forceinline__ void unpack(const uint4& u, double* e) {
  e[0] = __hiloint2double((int)u.y, (int)u.x);
  e[1] = __hiloint2double((int)u.w, (int)u.z);
}
__device__ __forceinline__ float bf_lo(unsigned w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf_hi(unsigned w) { return __uint_as_float(w & 0xffff0000u); }
__device__ __forceinline__ uint4 pack(const float* e) {
  return make_uint4(__float_as_uint(e[0]), __float_as_uint(e[1]), __float_as_uint(e[2]),
                    __float_as_uint(e[3]));
}
__device__ __forceinline__ uint4 pack(const double* e) {
  return make_uint4((unsigned)__double2loint(e[0]), (unsigned)__double2hiint(e[0]),
                    (unsigned)__double2loint(e[1]), (unsigned)__double2hiint(e[1]));
}

template <class T, int M>
__device__ __forceinline__ void vload(const T* p, T (&o)[M]) {
  static_assert((M * sizeof(T)) % 16 == 0, "chunk must be whole 16-byte vectors");
  constexpr int PER = 16 / sizeof(T);
#pragma unroll
  for (int v = 0; v < M / PER; ++v) unpack(__ldg(reinterpret_cast<const uint4*>(p) + v), o + v * PER);
}
template <int M>
__device__ __forceinline__ void cvload(const double* p, double (&o)[M], float) {
  vload<double, M>(p, o);
}
// BF16 couplings: 8 per vector, widened to FP32 and scaled
template <int M>
__device__ __forceinline__ void cvload(const __nv_bfloat16* p, float (&o)[M], float cs) {
  static_assert((M * 2) % 16 == 0, "chunk must be whole 16-byte vectors");
#pragma unroll
  for (int v = 0; v < M / 8; ++v) {
    const uint4 u = __ldg(reinterpret_cast<const uint4*>(p) + v);
    float* e = o + v * 8;
    e[0] = bf_lo(u.x) * cs; e[1] = bf_hi(u.x) * cs;
    e[2] = bf_lo(u.y) * cs; e[3] = bf_hi(u.y) * cs;
    e[4] = bf_lo(u.z) * cs; e[5] = bf_hi(u.z) * cs;
    e[6] = bf_lo(u.w) * cs; e[7] = bf_hi(u.w) * cs;
  }
}
template <class T, int M>
__device__ __forceinline__ void vstore(T* p, const T (&o)[M]) {
  constexpr int PER = 16 / sizeof(T);
#pragma unroll
  for (int v = 0; v < M / PER; ++v) reinterpret_cast<uint4*>(p)[v] = pack(o + v * PER);
}

// Reciprocal for the eliminations (a smoother needs no correctly rounded
// quotient).  FP32: the PTX approximate reciprocal (one special-function
// instruction, relative error about 2^-23).  FP64: that FP32 value as a seed,
// refined by two Newton-Raphson steps r <- r (2 - x r), each of which
// doubles the correct bits (22 -> 44 -> full precision); far cheaper than an
// IEEE FP64 division on GB300's FP64 pipe.  x is a positive pivot of an
// M-matrix elimination, well inside FP32's normal range.
__device__ __forceinline__ float lrcp(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ double lrcp(double x) {
  double r = (double)lrcp((float)x);
  r = r * fma(-x, r, 2.0);
  r = r * fma(-x, r, 2.0);
  return r;
}

constexpr int kWarpSlots = 16;  // per-warp values exchanged in k_line (13 used)

// Relax the lines (rows) iy = 2*blockIdx.x + colour of level L.
// ZERO: the iterate is zero on entry (the first pass of a V-cycle level):
// the neighbouring rows are not read, and they are written as zero.
// RZ (colour 0 only, the last pass of the V-cycle on the finest level):
// also reduce r.z over the whole level -- this CTA's row and the row above
// it, whose iterate is final -- and set the PCG beta, as k_dot_rz_t would.
template <class T, class CT, int M, bool ZERO, bool RZ>
__global__ void __launch_bounds__(512, 1)
k_line(MgView<T, CT, T> L, int colour, Scalars* sc, int flexible, double* part) {
  pdl_wait();
  if (sc && sc->done) return;
  extern __shared__ __align__(16) unsigned char line_smem[];
  const int nth = blockDim.x, t = threadIdx.x;
  const int iy = 2 * blockIdx.x + colour;
  if (iy >= L.ny) return;
  const int P = L.pitch, nx = L.nx;
  const size_t g0 = (size_t)iy * P;
  const float cs = L.csp ? __ldg(L.csp) : 1.0f;

  T a[M], d[M], c[M], r[M];
  unsigned actm = 0;  // bit k: cell k has an unknown
  const int ix0 = t * M;
  if (ix0 < nx) {
    // the chunk ends at or before round_up(nx, M) <= pitch: whole vectors
    // stay inside the row (padding cells are zero and count as inactive)
    const size_t g = g0 + ix0;
    T dv[M], ce[M], bv[M];
    vload<T, M>(L.dg + g, dv);
    cvload<M>(L.cE + g, ce, cs);
    vload<T, M>(L.b + g, bv);
    const T aw0 = lcoef<CT, T>(L.cE, g - 1, cs);
    T xn[M], xs[M], cn[M], cs_[M];
    if (!ZERO) {
      vload<T, M>(L.x + g + P, xn);
      vload<T, M>(L.x + g - P, xs);
      cvload<M>(L.cN + g, cn, cs);
      cvload<M>(L.cN + g - P, cs_, cs);
    }
#pragma unroll
    for (int k = 0; k < M; ++k) {
      const bool act = dv[k] > T(0) && ix0 + k < nx;
      T rv = bv[k];
      if (!ZERO) rv = fma(cs_[k], xs[k], fma(cn[k], xn[k], rv));
      const T aw = k == 0 ? aw0 : ce[k - 1];
      actm |= act ? (1u << k) : 0u;
      a[k] = act ? -aw : T(0);
      c[k] = act ? -ce[k] : T(0);
      d[k] = act ? dv[k] : T(1);
      r[k] = act ? rv : T(0);
    }
  } else {
#pragma unroll
    for (int k = 0; k < M; ++k) {
      a[k] = T(0);
      c[k] = T(0);
      d[k] = T(1);
      r[k] = T(0);
    }
  }

  // interior cells 0..M-2: forward elimination with three right-hand sides
  // (data; -a[0] on cell 0 for the left interface; -c[M-2] on cell M-2 for
  // the own interface), then back substitution.  Afterwards
  //   x_k = D_k + S_k * I_{t-1} + T_k * I_t   (k < M-1).
  T cp[M], D[M], S[M], Tr[M];
  {
    T inv = lrcp(d[0]);
    cp[0] = (M == 2) ? T(0) : c[0] * inv;
    D[0] = r[0] * inv;
    S[0] = -a[0] * inv;
    Tr[0] = (M == 2) ? -c[0] * inv : T(0);
#pragma unroll
    for (int k = 1; k < M - 1; ++k) {
      const T den = fma(-a[k], cp[k - 1], d[k]);
      inv = lrcp(den);
      cp[k] = (k == M - 2) ? T(0) : c[k] * inv;
      D[k] = fma(-a[k], D[k - 1], r[k]) * inv;
      S[k] = -a[k] * S[k - 1] * inv;
      Tr[k] = fma(-a[k], Tr[k - 1], (k == M - 2) ? -c[k] : T(0)) * inv;
    }
#pragma unroll
    for (int k = M - 3; k >= 0; --k) {
      D[k] = fma(-cp[k], D[k + 1], D[k]);
      S[k] = fma(-cp[k], S[k + 1], S[k]);
      Tr[k] = fma(-cp[k], Tr[k + 1], Tr[k]);
    }
  }
  // Interface system: one equation per thread,
  //   ea I_{t-1} + eb I_t + ec I_{t+1} = ed,
  // solved in two stages without block-wide reduction steps.  (1) In each
  // warp, lanes 0..30 are interior unknowns and lane 31's interface J_w is
  // the warp's own interface: cyclic reduction over the lanes (shuffles,
  // five steps) gives I_l = P_l + Q_l J_{w-1} + R_l J_w.  (2) Substituting
  // that into lane 31's equation leaves one tridiagonal equation per warp in
  // the J's; every warp forms all of them from shared memory (after the
  // kernel's one block barrier) and reduces them by shuffles itself.
  const int lane = t & 31, warp = t >> 5, nw = nth >> 5;
  T* wsm = reinterpret_cast<T*>(line_smem);  // [nw][kWarpSlots]
  const T aI = a[M - 1], dI = d[M - 1], cI = c[M - 1], rI = r[M - 1];
  // first-cell responses of thread t+1 (lane 31: the next warp's, later)
  const T Dn = __shfl_down_sync(0xffffffffu, D[0], 1);
  const T Sn = __shfl_down_sync(0xffffffffu, S[0], 1);
  const T Tn = __shfl_down_sync(0xffffffffu, Tr[0], 1);
  const T ea = aI * S[M - 2];
  const T ebp = fma(aI, Tr[M - 2], dI), edp = fma(-aI, D[M - 2], rI);
  T pa_ = T(0), pb = T(1), pc = T(0), pd = T(0), pe = T(0), pf = T(0);
  if (lane < 31) {
    const T eb = fma(cI, Sn, ebp), ec = cI * Tn, ed = fma(-cI, Dn, edp);
    pa_ = lane == 0 ? T(0) : ea;
    pb = eb;
    pc = lane == 30 ? T(0) : ec;
    pd = ed;
    pe = lane == 0 ? -ea : T(0);   // coefficient of J_{w-1}
    pf = lane == 30 ? -ec : T(0);  // coefficient of J_w
  }
#pragma unroll
  for (int sh = 1; sh < 32; sh <<= 1) {
    // lanes without a partner at distance sh have the matching coupling
    // already zero, so the partner values (their own, from the shuffle)
    // are multiplied by zero
    const T am = __shfl_up_sync(0xffffffffu, pa_, sh), bm = __shfl_up_sync(0xffffffffu, pb, sh);
    const T cm = __shfl_up_sync(0xffffffffu, pc, sh), dm = __shfl_up_sync(0xffffffffu, pd, sh);
    const T em = __shfl_up_sync(0xffffffffu, pe, sh), fm = __shfl_up_sync(0xffffffffu, pf, sh);
    const T ap = __shfl_down_sync(0xffffffffu, pa_, sh), bp = __shfl_down_sync(0xffffffffu, pb, sh);
    const T cp2 = __shfl_down_sync(0xffffffffu, pc, sh), dp = __shfl_down_sync(0xffffffffu, pd, sh);
    const T ep = __shfl_down_sync(0xffffffffu, pe, sh), fp = __shfl_down_sync(0xffffffffu, pf, sh);
    const T k1 = pa_ * lrcp(bm), k2 = pc * lrcp(bp);
    pa_ = -am * k1;
    pc = -cp2 * k2;
    pb = fma(-ap, k2, fma(-cm, k1, pb));
    pd = fma(-dp, k2, fma(-dm, k1, pd));
    pe = fma(-ep, k2, fma(-em, k1, pe));
    pf = fma(-fp, k2, fma(-fm, k1, pf));
  }
  const T ib = lrcp(pb);
  const T Pl = pd * ib, Ql = pe * ib, Rl = pf * ib;
  const T P30 = __shfl_up_sync(0xffffffffu, Pl, 1), Q30 = __shfl_up_sync(0xffffffffu, Ql, 1),
          R30 = __shfl_up_sync(0xffffffffu, Rl, 1);
  T* ws = wsm + warp * kWarpSlots;
  if (lane == 0) {
    ws[0] = D[0]; ws[1] = S[0]; ws[2] = Tr[0];
    ws[3] = Pl; ws[4] = Ql; ws[5] = Rl;
  } else if (lane == 31) {
    ws[6] = ea; ws[7] = ebp; ws[8] = cI; ws[9] = edp;
    ws[10] = P30; ws[11] = Q30; ws[12] = R30;
  }
  __syncthreads();
  // the warps' interface equations (lane k: warp k), reduced in every warp
  T ja = T(0), jb = T(1), jc = T(0), jd = T(0);
  if (lane < nw) {
    const T* wk = wsm + lane * kWarpSlots;
    const bool nx_ = lane + 1 < nw;
    const T* wn = wk + kWarpSlots;
    const T D0n = nx_ ? wn[0] : T(0), S0n = nx_ ? wn[1] : T(0), T0n = nx_ ? wn[2] : T(0);
    const T P0n = nx_ ? wn[3] : T(0), Q0n = nx_ ? wn[4] : T(0), R0n = nx_ ? wn[5] : T(0);
    const T eak = wk[6], cIk = wk[8];
    const T ebk = fma(cIk, S0n, wk[7]), eck = cIk * T0n, edk = fma(-cIk, D0n, wk[9]);
    ja = eak * wk[11];
    jb = fma(eck, Q0n, fma(eak, wk[12], ebk));
    jc = eck * R0n;
    jd = fma(-eck, P0n, fma(-eak, wk[10], edk));
  }
  for (int sh = 1; sh < nw; sh <<= 1) {
    const T am = __shfl_up_sync(0xffffffffu, ja, sh), bm = __shfl_up_sync(0xffffffffu, jb, sh);
    const T cm = __shfl_up_sync(0xffffffffu, jc, sh), dm = __shfl_up_sync(0xffffffffu, jd, sh);
    const T ap = __shfl_down_sync(0xffffffffu, ja, sh), bp = __shfl_down_sync(0xffffffffu, jb, sh);
    const T cp2 = __shfl_down_sync(0xffffffffu, jc, sh), dp = __shfl_down_sync(0xffffffffu, jd, sh);
    const T k1 = ja * lrcp(bm), k2 = jc * lrcp(bp);
    ja = -am * k1;
    jc = -cp2 * k2;
    jb = fma(-ap, k2, fma(-cm, k1, jb));
    jd = fma(-dp, k2, fma(-dm, k1, jd));
  }
  const T J = jd * lrcp(jb);
  const T Jw = __shfl_sync(0xffffffffu, J, warp);
  const T Jm = warp > 0 ? __shfl_sync(0xffffffffu, J, warp > 0 ? warp - 1 : 0) : T(0);
  const T It = lane == 31 ? Jw : fma(Ql, Jm, fma(Rl, Jw, Pl));
  const T Iup = __shfl_up_sync(0xffffffffu, It, 1);
  const T Il = lane == 0 ? Jm : Iup;
  if (!RZ && ix0 >= nx) return;
  T acc = T(0);
  if (ix0 < nx) {
    T xo[M];
#pragma unroll
    for (int k = 0; k < M; ++k) {
      const T v = (k == M - 1) ? It : fma(S[k], Il, fma(Tr[k], It, D[k]));
      xo[k] = (actm >> k) & 1u ? v : T(0);
    }
    if (ix0 + M <= nx) {
      vstore<T, M>(L.x + g0 + ix0, xo);
    } else {  // the ghost columns past nx keep their zeros
      for (int k = 0; k < nx - ix0; ++k) L.x[g0 + ix0 + k] = xo[k];
    }
    if (ZERO && iy + 1 < L.ny) {
      T z[M];
#pragma unroll
      for (int k = 0; k < M; ++k) z[k] = T(0);
      vstore<T, M>(L.x + g0 + P + ix0, z);
    }
    if (RZ) {  // b and x past nx are zero padding
      T bv[M];
      vload<T, M>(L.b + g0 + ix0, bv);
#pragma unroll
      for (int k = 0; k < M; ++k) acc = fma(bv[k], xo[k], acc);
      if (iy + 1 < L.ny) {
        T xu[M];
        vload<T, M>(L.b + g0 + P + ix0, bv);
        vload<T, M>(L.x + g0 + P + ix0, xu);
#pragma unroll
        for (int k = 0; k < M; ++k) acc = fma(bv[k], xu[k], acc);
      }
    }
  }
  if (RZ) {  // per-thread FP32 sums, combined in FP64 in a fixed order
    __shared__ double red[16];
    __shared__ bool lastblk;
    double v = (double)acc;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (t == 0) {
      double sb = 0.0;
      for (int w = 0; w < nw; ++w) sb += red[w];
      part[blockIdx.x] = sb;
      __threadfence();
      lastblk = atomicAdd(&sc->tickets[T_RZ], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!lastblk) return;
    __threadfence();
    double xs = 0.0;
    for (unsigned k = t; k < gridDim.x; k += nth) xs += __ldcg(&part[k]);
    for (int o = 16; o > 0; o >>= 1) xs += __shfl_down_sync(0xffffffffu, xs, o);
    if (lane == 0) red[warp] = xs;
    __syncthreads();
    if (t == 0) {
      double tot = 0.0;
      for (int w = 0; w < nw; ++w) tot += red[w];
      set_beta(sc, tot, flexible);
      sc->tickets[T_RZ] = 0u;
    }
  }
}

// ---------------------------------------------------------------------------
// Factored line relaxation (FP64 levels).  The line matrices do not change
// between V-cycles, so everything that depends on them alone -- the interior
// pivots, the responses S, T of every interior cell to its two interfaces,
// the interface equations and every multiplier of the cyclic reduction -- is
// computed once per assembly by k_line_factor.  A relaxation pass
// (k_line_solve) is then a forward and a backward substitution, one
// cyclic-reduction sweep of the right-hand side and the recovery: no
// division, five FP64 operations per cell instead of about forty, which
// matters on GB300's slow FP64 pipe.
// Per cell (interior cells of each thread's chunk): INV (1/pivot, 0 where
// the cell has no unknown), GA (sub-diagonal times INV), CP (super-diagonal
// multiplier), S, TR (responses).  Per thread: aI, cI, 1/B of the reduced
// equation (0 where the interface has no unknown), then k1, k2 per
// reduction step.
constexpr int kLineSlots = kLineThreadSlots;  // 3 + 2 x (up to 10 reduction steps)

template <class T, class CT, int M>
__global__ void __launch_bounds__(512, 1)
k_line_factor(MgView<T, CT, T> L, LineFactors<T> F) {
  pdl_wait();
  extern __shared__ __align__(16) unsigned char lf_smem[];
  const int nth = blockDim.x, t = threadIdx.x;
  T* rS0 = reinterpret_cast<T*>(lf_smem);
  T* rT0 = rS0 + nth;
  T* pa = rT0 + nth;  // two buffers of A, B, C
  const int iy = blockIdx.x;
  if (iy >= L.ny) return;
  const int P = L.pitch, nx = L.nx;
  const size_t g0 = (size_t)iy * P;
  const float cs = L.csp ? __ldg(L.csp) : 1.0f;
  T a[M], d[M], c[M];
  unsigned actm = 0;
  const int ix0 = t * M;
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const int ix = ix0 + k;
    T dv = T(-1), aw = T(0), ce = T(0);
    if (ix < nx) {
      const size_t g = g0 + ix;
      dv = L.dg[g];
      aw = lcoef<CT, T>(L.cE, g - 1, cs);
      ce = lcoef<CT, T>(L.cE, g, cs);
    }
    const bool act = dv > T(0);
    actm |= act ? (1u << k) : 0u;
    a[k] = act ? -aw : T(0);
    c[k] = act ? -ce : T(0);
    d[k] = act ? dv : T(1);
  }
  T cp[M], iv[M], S[M], Tr[M];
  {
    T inv = lrcp(d[0]);
    iv[0] = inv;
    cp[0] = (M == 2) ? T(0) : c[0] * inv;
    S[0] = -a[0] * inv;
    Tr[0] = (M == 2) ? -c[0] * inv : T(0);
#pragma unroll
    for (int k = 1; k < M - 1; ++k) {
      inv = lrcp(fma(-a[k], cp[k - 1], d[k]));
      iv[k] = inv;
      cp[k] = (k == M - 2) ? T(0) : c[k] * inv;
      S[k] = -a[k] * S[k - 1] * inv;
      Tr[k] = fma(-a[k], Tr[k - 1], (k == M - 2) ? -c[k] : T(0)) * inv;
    }
#pragma unroll
    for (int k = M - 3; k >= 0; --k) {
      S[k] = fma(-cp[k], S[k + 1], S[k]);
      Tr[k] = fma(-cp[k], Tr[k + 1], Tr[k]);
    }
  }
  if (ix0 < nx) {
#pragma unroll
    for (int k = 0; k < M - 1; ++k) {
      const size_t g = g0 + ix0 + k;
      const bool act = (actm >> k) & 1u;
      F.inv[g] = act ? iv[k] : T(0);
      F.ga[g] = act ? a[k] * iv[k] : T(0);
      F.cp[g] = cp[k];
      F.S[g] = S[k];
      F.tr[g] = Tr[k];
    }
  }
  rS0[t] = S[0];
  rT0[t] = Tr[0];
  __syncthreads();
  const bool last = t == nth - 1;
  const T aI = a[M - 1], dI = d[M - 1], cI = c[M - 1];
  const T Sn = last ? T(0) : rS0[t + 1], Tn = last ? T(0) : rT0[t + 1];
  T* th = F.thr + ((size_t)iy * F.nth + t) * kLineSlots;
  th[0] = aI;
  th[1] = cI;
  pa[t] = aI * S[M - 2];
  pa[nth + t] = fma(cI, Sn, fma(aI, Tr[M - 2], dI));
  pa[2 * nth + t] = cI * Tn;
  __syncthreads();
  int cur = 0, step = 0;
  for (int sdist = 1; sdist < nth; sdist <<= 1, ++step) {
    const T* A_ = pa + cur * 3 * nth;
    const T* B_ = A_ + nth;
    const T* C_ = B_ + nth;
    T na = T(0), nb = B_[t], nc = T(0), k1 = T(0), k2 = T(0);
    if (t - sdist >= 0) {
      k1 = A_[t] * lrcp(B_[t - sdist]);
      na = -A_[t - sdist] * k1;
      nb = fma(-C_[t - sdist], k1, nb);
    }
    if (t + sdist < nth) {
      k2 = C_[t] * lrcp(B_[t + sdist]);
      nc = -C_[t + sdist] * k2;
      nb = fma(-A_[t + sdist], k2, nb);
    }
    th[3 + 2 * step] = k1;
    th[4 + 2 * step] = k2;
    T* W = pa + (cur ^ 1) * 3 * nth;
    W[t] = na;
    W[nth + t] = nb;
    W[2 * nth + t] = nc;
    cur ^= 1;
    __syncthreads();
  }
  const bool actI = (actm >> (M - 1)) & 1u;
  th[2] = actI ? lrcp(pa[cur * 3 * nth + nth + t]) : T(0);
}

// One relaxation pass with the factors of k_line_factor (lines iy = 2*blockIdx.x + colour)
template <class T, class CT, int M, bool ZERO>
__global__ void __launch_bounds__(512, 1)
k_line_solve(MgView<T, CT, T> L, LineFactors<T> F, int colour, const Scalars* sc) {
  pdl_wait();
  if (sc && sc->done) return;
  extern __shared__ __align__(16) unsigned char ls_smem[];
  const int nth = blockDim.x, t = threadIdx.x;
  T* rD0 = reinterpret_cast<T*>(ls_smem);
  T* pd = rD0 + nth;  // two buffers of the reduced right-hand side
  const int iy = 2 * blockIdx.x + colour;
  if (iy >= L.ny) return;
  const int P = L.pitch, nx = L.nx;
  const size_t g0 = (size_t)iy * P;
  const float cs = L.csp ? __ldg(L.csp) : 1.0f;
  const int ix0 = t * M;
  const bool has = ix0 < nx;  // chunks past the row are identity rows
  T r[M], D[M];
  if (has) {
    const size_t g = g0 + ix0;
    vload<T, M>(L.b + g, r);
    if (!ZERO) {
      T xn[M], xs[M], cn[M], cs_[M];
      vload<T, M>(L.x + g + P, xn);
      vload<T, M>(L.x + g - P, xs);
      cvload<M>(L.cN + g, cn, cs);
      cvload<M>(L.cN + g - P, cs_, cs);
#pragma unroll
      for (int k = 0; k < M; ++k) r[k] = fma(cs_[k], xs[k], fma(cn[k], xn[k], r[k]));
    }
    T iv[M], ga[M], cp[M];
    vload<T, M>(F.inv + g, iv);
    vload<T, M>(F.ga + g, ga);
    vload<T, M>(F.cp + g, cp);
    D[0] = r[0] * iv[0];
#pragma unroll
    for (int k = 1; k < M - 1; ++k) D[k] = fma(-ga[k], D[k - 1], r[k] * iv[k]);
#pragma unroll
    for (int k = M - 3; k >= 0; --k) D[k] = fma(-cp[k], D[k + 1], D[k]);
  } else {
#pragma unroll
    for (int k = 0; k < M; ++k) { r[k] = T(0); D[k] = T(0); }
  }
  rD0[t] = D[0];
  const T* th = F.thr + ((size_t)iy * F.nth + t) * kLineSlots;
  const T aI = th[0], cI = th[1], invB = th[2];
  __syncthreads();
  const T Dn = t == nth - 1 ? T(0) : rD0[t + 1];
  pd[t] = fma(-cI, Dn, fma(-aI, D[M - 2], r[M - 1]));
  __syncthreads();
  int cur = 0, step = 0;
  for (int sdist = 1; sdist < nth; sdist <<= 1, ++step) {
    const T* Dc = pd + cur * nth;
    T v = Dc[t];
    if (t - sdist >= 0) v = fma(-th[3 + 2 * step], Dc[t - sdist], v);
    if (t + sdist < nth) v = fma(-th[4 + 2 * step], Dc[t + sdist], v);
    pd[(cur ^ 1) * nth + t] = v;
    cur ^= 1;
    __syncthreads();
  }
  const T It = pd[cur * nth + t] * invB;
  rD0[t] = It;  // rD0's reads all happened before the reduction's first barrier
  __syncthreads();
  const T Il = t > 0 ? rD0[t - 1] : T(0);
  if (!has) return;
  const size_t g = g0 + ix0;
  T S[M], Tr[M], xo[M];
  vload<T, M>(F.S + g, S);
  vload<T, M>(F.tr + g, Tr);
#pragma unroll
  for (int k = 0; k < M - 1; ++k) xo[k] = fma(S[k], Il, fma(Tr[k], It, D[k]));
  xo[M - 1] = It;
  if (ix0 + M <= nx) {
    vstore<T, M>(L.x + g, xo);
  } else {
    for (int k = 0; k < nx - ix0; ++k) L.x[g + k] = xo[k];
  }
  if (ZERO && iy + 1 < L.ny) {
    T z[M];
#pragma unroll
    for (int k = 0; k < M; ++k) z[k] = T(0);
    vstore<T, M>(L.x + g + P, z);
  }
}

// dst (ny rows of pitch pd) = transpose of src (nx-by-ny, pitch ps); only
// interior cells are written, the ghost ring of dst keeps its zeros
template <class E>
__global__ void __launch_bounds__(256)
k_transpose(const E* __restrict__ src, int nx, int ny, int ps, E* __restrict__ dst, int pd,
            const Scalars* sc) {
  pdl_wait();
  if (sc && sc->done) return;
  __shared__ E tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int ix = bx + threadIdx.x, iy = by + j;
    if (ix < nx && iy < ny) tile[j][threadIdx.x] = src[(size_t)iy * ps + ix];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int ox = by + threadIdx.x, oy = bx + j;
    if (ox < ny && oy < nx) dst[(size_t)oy * pd + ox] = tile[threadIdx.x][j];
  }
}

// Transpose of FP32 levels, 64 x 64 cells per CTA with 16-byte vector
// loads and stores (4 cells).  A row of the padded layout starts on a
// 128-byte boundary and its pitch is a multiple of 32 cells, so a vector
// that starts at a multiple of its width stays inside its row; cells past
// nx (padding and the next row's ghost) hold zeros, are read as such and
// written back as zeros.
template <class E>
__global__ void __launch_bounds__(256)
k_transpose_v(const E* __restrict__ src, int nx, int ny, int ps, E* __restrict__ dst, int pd,
              const Scalars* sc) {
  pdl_wait();
  if (sc && sc->done) return;
  constexpr int V = 16 / sizeof(E), TS = 64, VR = TS / V;  // vectors per tile row
  __shared__ E tile[TS][TS + 1];
  const int bx = blockIdx.x * TS, by = blockIdx.y * TS;
  const int t = threadIdx.y * 32 + threadIdx.x;
  for (int e = t; e < TS * VR; e += 256) {
    const int r = e / VR, c = (e % VR) * V;
    const int ix = bx + c, iy = by + r;
    E v[V];
    if (iy < ny && ix < nx) {
      const uint4 u = __ldg(reinterpret_cast<const uint4*>(src + (size_t)iy * ps + ix));
      unpack(u, v);
    } else {
#pragma unroll
      for (int m = 0; m < V; ++m) v[m] = E(0);
    }
#pragma unroll
    for (int m = 0; m < V; ++m) tile[r][c + m] = v[m];
  }
  __syncthreads();
  for (int e = t; e < TS * VR; e += 256) {
    const int o = e / VR, c = (e % VR) * V;  // dst row bx + o, dst cells by + c ..
    const int oy = bx + o, ox = by + c;
    if (oy >= nx || ox >= ny) continue;
    E v[V];
#pragma unroll
    for (int m = 0; m < V; ++m) v[m] = tile[c + m][o];
    *reinterpret_cast<uint4*>(dst + (size_t)oy * pd + ox) = pack(v);
  }
}

// Residual of a level summed 2x2 onto the right-hand side of the coarser
// level, computed on the level's transposed copy Lt (where the last
// relaxation of the pre-smoothing left the iterate) and written to the
// coarse level in both layouts (C natural, Ct transposed), so neither needs
// a transpose.  Lt cell (i, j) is natural cell (j, i); Ct cell (a, b) is C
// cell (b, a).  Terms are summed in natural order (cells by natural row,
// then column; couplings east, west, north, south): the result does not
// depend on the layout the residual is computed in.
template <class T, class CT>
__global__ void __launch_bounds__(256)
k_resid_restrict_lt(MgView<T, CT, T> Lt, MgView<T, CT, T> C, MgView<T, CT, T> Ct,
                    const Scalars* sc) {
  pdl_wait();
  if (sc && sc->done) return;
  // one coarse cell per thread (a CTA: 32 x 8 coarse cells), so the FP64
  // residual chains of different cells run side by side
  __shared__ T tile[8][33];
  const int a0 = blockIdx.x * 32, b0 = blockIdx.y * 8;
  const float cs = Lt.csp ? __ldg(Lt.csp) : 1.0f;
  const int P = Lt.pitch;
  {
    const int bb = threadIdx.y;
    const int a = a0 + threadIdx.x, b = b0 + bb;
    T s = T(0);
    if (a < Ct.nx && b < Ct.ny) {
#pragma unroll
      for (int dj = 0; dj < 2; ++dj)
#pragma unroll
        for (int dq = 0; dq < 2; ++dq) {
          const int gx = 2 * a + dj, gy = 2 * b + dq;  // natural (2b + dq, 2a + dj)
          if (gx >= Lt.nx || gy >= Lt.ny) continue;
          const size_t g = (size_t)gy * P + gx;
          const T dgv = Lt.dg[g];
          if (dgv < T(0)) continue;
          T rr = fma(-dgv, Lt.x[g], Lt.b[g]);
          rr = fma(lcoef<CT, T>(Lt.cN, g, cs), Lt.x[g + P], rr);
          rr = fma(lcoef<CT, T>(Lt.cN, g - P, cs), Lt.x[g - P], rr);
          rr = fma(lcoef<CT, T>(Lt.cE, g, cs), Lt.x[g + 1], rr);
          rr = fma(lcoef<CT, T>(Lt.cE, g - 1, cs), Lt.x[g - 1], rr);
          s += rr;
        }
      Ct.b[(size_t)b * Ct.pitch + a] = s;
    }
    tile[bb][threadIdx.x] = s;
  }
  __syncthreads();
  {
    const int t = threadIdx.y * 32 + threadIdx.x;
    const int bb = t % 8, aa = t / 8;
    const int ix = b0 + bb, iy = a0 + aa;  // C cell (ix, iy) = Ct cell (iy, ix)
    if (ix < C.nx && iy < C.ny) C.b[(size_t)iy * C.pitch + ix] = tile[bb][aa];
  }
}

// The same restriction for FP32/BF16 levels with vector loads: a thread
// owns two coarse cells (a0, a0 + 1) of coarse row b, i.e. four fine cells
// (16 bytes of FP32, 8 bytes of BF16) in each of the fine rows 2b, 2b + 1;
// a CTA owns 64 x 8 coarse cells.  Same terms in the same order as
// k_resid_restrict_lt.
__device__ __forceinline__ void bf4(const __nv_bfloat16* p, float cs, float (&o)[4]) {
  const uint2 u = __ldg(reinterpret_cast<const uint2*>(p));
  o[0] = bf_lo(u.x) * cs; o[1] = bf_hi(u.x) * cs;
  o[2] = bf_lo(u.y) * cs; o[3] = bf_hi(u.y) * cs;
}
__device__ __forceinline__ void f4(const float* p, float (&o)[4]) {
  unpack(__ldg(reinterpret_cast<const uint4*>(p)), o);
}
__global__ void __launch_bounds__(256)
k_resid_restrict_lt4(MgView<float, __nv_bfloat16, float> Lt, MgView<float, __nv_bfloat16, float> C,
                     MgView<float, __nv_bfloat16, float> Ct, const Scalars* sc) {
  pdl_wait();
  if (sc && sc->done) return;
  __shared__ float tile[8][65];
  const int a0 = blockIdx.x * 64 + 2 * threadIdx.x, b = blockIdx.y * 8 + threadIdx.y;
  const float cs = Lt.csp ? __ldg(Lt.csp) : 1.0f;
  const int P = Lt.pitch, nx = Lt.nx, ny = Lt.ny;
  float s0 = 0.0f, s1 = 0.0f;
  if (a0 < Ct.nx && b < Ct.ny) {
    const int c0 = 2 * a0;
    float rr[2][4];  // [fine row 2b + dq][fine column c0 + m]
#pragma unroll
    for (int dq = 0; dq < 2; ++dq) {
      const int gy = 2 * b + dq;
#pragma unroll
      for (int m = 0; m < 4; ++m) rr[dq][m] = 0.0f;
      if (gy >= ny) continue;
      const size_t g = (size_t)gy * P + c0;
      float xv[4], xu[4], xd[4], bv[4], dv[4], ce[4], cn[4], cs_[4];
      f4(Lt.x + g, xv);
      f4(Lt.x + g + P, xu);
      f4(Lt.x + g - P, xd);
      f4(Lt.b + g, bv);
      f4(Lt.dg + g, dv);
      bf4(Lt.cE + g, cs, ce);
      bf4(Lt.cN + g, cs, cn);
      bf4(Lt.cN + g - P, cs, cs_);
      const float xw = Lt.x[g - 1];
      const float cw = __bfloat162float(Lt.cE[g - 1]) * cs;
      const float xe = c0 + 3 < nx ? Lt.x[g + 4] : 0.0f;
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        float r = fmaf(-dv[m], xv[m], bv[m]);
        r = fmaf(cn[m], xu[m], r);
        r = fmaf(cs_[m], xd[m], r);
        r = fmaf(ce[m], m < 3 ? xv[m + 1] : xe, r);
        r = fmaf(m > 0 ? ce[m - 1] : cw, m > 0 ? xv[m - 1] : xw, r);
        // cells past nx and cells without an unknown add nothing
        rr[dq][m] = (c0 + m < nx && dv[m] >= 0.0f) ? r : 0.0f;
      }
    }
    // natural order: fine column (natural row) outer, fine row inner
    s0 = rr[0][0]; s0 += rr[1][0]; s0 += rr[0][1]; s0 += rr[1][1];
    s1 = rr[0][2]; s1 += rr[1][2]; s1 += rr[0][3]; s1 += rr[1][3];
    float* o = Ct.b + (size_t)b * Ct.pitch + a0;
    if (a0 + 1 < Ct.nx) *reinterpret_cast<float2*>(o) = make_float2(s0, s1);
    else o[0] = s0;
  }
  tile[threadIdx.y][2 * threadIdx.x] = s0;
  tile[threadIdx.y][2 * threadIdx.x + 1] = s1;
  __syncthreads();
  const int t = threadIdx.y * 32 + threadIdx.x;
  for (int e = t; e < 64 * 8; e += 256) {
    const int bl = e % 8, al = e / 8;
    const int ix = blockIdx.y * 8 + bl, iy = blockIdx.x * 64 + al;  // C cell = Ct cell (iy, ix)
    if (ix < C.nx && iy < C.ny) C.b[(size_t)iy * C.pitch + ix] = tile[bl][al];
  }
}

// x += omega * x_coarse(parent) on cells with an unknown, applied to the
// transposed copy Lt of a level (where the post-smoothing starts): Lt cell
// (i, j) is natural cell (j, i), whose parent is coarse cell (j/2, i/2) of
// the natural coarse level (nxc x nyc, pitch pc).  A 32 x 16 block of coarse
// values is staged in shared memory for the CTA's 64 x 32 fine cells.
template <class T, class CT>
__global__ void __launch_bounds__(256)
k_prolong_lt(MgView<T, CT, T> Lt, const T* __restrict__ xc, int pc, int nxc, int nyc, T omega,
             const Scalars* sc) {
  pdl_wait();
  if (sc && sc->done) return;
  // CTA: 64 x 32 fine cells, 16-byte vectors along the rows
  constexpr int V = 16 / sizeof(T), TPR = 64 / V, RPP = 256 / TPR;
  __shared__ T ct[32][17];
  const int x0 = blockIdx.x * 64, y0 = blockIdx.y * 32;
  const int t = threadIdx.y * 32 + threadIdx.x;
  for (int e = t; e < 32 * 16; e += 256) {
    const int cx = e % 16, cy = e / 16;  // coarse natural (y0/2 + cx, x0/2 + cy)
    const int ix = (y0 >> 1) + cx, iy = (x0 >> 1) + cy;
    ct[cy][cx] = (ix < nxc && iy < nyc) ? xc[(size_t)iy * pc + ix] : T(0);
  }
  __syncthreads();
  const int li = (t % TPR) * V, i = x0 + li;
  if (i >= Lt.nx) return;
  for (int jj = t / TPR; jj < 32; jj += RPP) {
    const int j = y0 + jj;
    if (j >= Lt.ny) break;
    // a vector reaching past nx covers padding, whose inverse diagonal is 0
    const size_t g = (size_t)j * Lt.pitch + i;
    T dv[V], xv[V];
    unpack(__ldg(reinterpret_cast<const uint4*>(Lt.di + g)), dv);
    unpack(*reinterpret_cast<const uint4*>(Lt.x + g), xv);
#pragma unroll
    for (int m = 0; m < V; ++m)
      if (dv[m] > T(0)) xv[m] = fma(omega, ct[(li + m) >> 1][jj >> 1], xv[m]);
    *reinterpret_cast<uint4*>(Lt.x + g) = pack(xv);
  }
}

// largest aspect ratio max(dx/dy, dy/dx) over the cells, as float bits
__global__ void k_aspect(const double* __restrict__ dx, const double* __restrict__ dy, size_t n,
                         unsigned* out_bits) {
  float m = 0.0f;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const double a = dx[k], b = dy[k];
    if (a > 0.0 && b > 0.0) m = fmaxf(m, (float)fmax(a / b, b / a));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out_bits, __float_as_uint(m));
}

// The coarse end of a line-smoothed V-cycle in one CTA: every level of at
// most kTailMaxCells cells, down to the dense coarsest solve and back up,
// with x, b, the couplings and the diagonal of all those levels in shared
// memory (each level padded by a zero ghost ring).  Each line is solved by
// one thread with the Thomas algorithm (short lines: a serial solve per line
// is cheaper than the partitioned one).  Same passes, in the same order, as
// the per-level kernels.
template <class T, class CT>
__global__ void __launch_bounds__(1024) k_line_tail(TailDesc<T, CT> d, Scalars* sc) {
  pdl_wait();
  if (sc->done) return;
  extern __shared__ __align__(16) unsigned char ltail_smem[];
  T* sm = reinterpret_cast<T*>(ltail_smem);
  double* bd = reinterpret_cast<double*>(ltail_smem + d.bd_off);
  const int t = threadIdx.x, NTT = blockDim.x;
  for (int i = t; i < d.total; i += NTT) sm[i] = T(0);
  __syncthreads();
  auto W = [&](int l) { return d.lv[l].nx + 2; };
  auto WH = [&](int l) { return (d.lv[l].nx + 2) * (d.lv[l].ny + 2); };
  auto X = [&](int l) { return sm + d.off[l]; };
  auto B = [&](int l) { return sm + d.off[l] + WH(l); };
  auto E = [&](int l) { return sm + d.off[l] + 2 * WH(l); };
  auto N = [&](int l) { return sm + d.off[l] + 3 * WH(l); };
  auto G = [&](int l) { return sm + d.off[l] + 4 * WH(l); };
  T* CP = sm + d.off[d.n];  // line-solve scratch, the size of the first tail level
  T* DP = CP + WH(0);
  for (int l = 0; l < d.n; ++l) {
    const MgView<T, CT, T>& L = d.lv[l];
    const float cs = L.csp ? __ldg(L.csp) : 1.0f;
    for (int k = t; k < L.nx * L.ny; k += NTT) {
      const int ix = k % L.nx, iy = k / L.nx;
      const size_t g = (size_t)iy * L.pitch + ix;
      const int si = (iy + 1) * W(l) + ix + 1;
      E(l)[si] = lcoef<CT, T>(L.cE, g, cs);
      N(l)[si] = lcoef<CT, T>(L.cN, g, cs);
      G(l)[si] = L.dg[g];
      if (l == 0) B(0)[si] = L.b[g];
    }
  }
  __syncthreads();
  // lines of one parity: dir 0 rows, dir 1 columns; thread q solves line q
  auto pass = [&](int l, int dir, int colour) {
    const int nx = d.lv[l].nx, ny = d.lv[l].ny, w = W(l);
    const int nlines = dir == 0 ? ny : nx, len = dir == 0 ? nx : ny;
    const int step = dir == 0 ? 1 : w;  // cell stride along the line
    const int cross = dir == 0 ? w : 1;  // stride to the neighbouring line
    const T* Ax = dir == 0 ? E(l) : N(l);  // in-line couplings
    const T* Cx = dir == 0 ? N(l) : E(l);  // cross couplings
    const T* b = B(l);
    const T* g = G(l);
    T* x = X(l);
    if constexpr (std::is_same<T, float>::value) if (len <= 64) {
      // FP32: one warp per line, M = 1 or 2 consecutive cells per lane.  A
      // lane with two cells eliminates its first (x0 = D + S I_{l-1} +
      // T I_l in the interfaces I, each lane's last cell), the interface
      // equations are reduced by cyclic reduction over the lanes (shuffles,
      // five steps) and the first cells recovered.  Reciprocals are the
      // correctly rounded ones: with the approximate reciprocal the
      // reduction costs the coarse correction enough accuracy for an extra
      // PCG iteration.
      const int lane = t & 31, nwarp = NTT >> 5;
      const int M = len <= 32 ? 1 : 2;
      for (int q = colour + 2 * (t >> 5); q < nlines; q += 2 * nwarp) {
        const int s0 = (dir == 0 ? (q + 1) * w + 1 : w + q + 1);
        T av[2], cv[2], dv[2], rv[2], gv[2];
#pragma unroll
        for (int m = 0; m < 2; ++m) {
          const int k = lane * M + m;
          av[m] = T(0); cv[m] = T(0); dv[m] = T(1); rv[m] = T(0); gv[m] = T(0);
          if (m < M && k < len) {
            const int si = s0 + k * step;
            gv[m] = g[si];
            if (gv[m] > T(0)) {
              av[m] = k > 0 ? -Ax[si - step] : T(0);
              cv[m] = k + 1 < len ? -Ax[si] : T(0);
              dv[m] = gv[m];
              T r = fma(Cx[si], x[si + cross], b[si]);
              rv[m] = fma(Cx[si - cross], x[si - cross], r);
            }
          }
        }
        // the lane's interface cell is its last; with two cells the first
        // is eliminated towards the interfaces on both sides
        T D = T(0), S = T(0), Tr = T(0), a, dd, c, r;
        if (M == 2) {
          const T inv0 = __frcp_rn(dv[0]);
          D = rv[0] * inv0;
          S = -av[0] * inv0;
          Tr = -cv[0] * inv0;
          const T Dn = __shfl_down_sync(0xffffffffu, D, 1);
          const T Sn = __shfl_down_sync(0xffffffffu, S, 1);
          const T Tn = __shfl_down_sync(0xffffffffu, Tr, 1);
          const bool last = lane == 31;
          a = av[1] * S;
          dd = fma(av[1], Tr, dv[1]);
          r = fma(-av[1], D, rv[1]);
          if (!last) {
            dd = fma(cv[1], Sn, dd);
            r = fma(-cv[1], Dn, r);
          }
          c = last ? T(0) : cv[1] * Tn;
        } else {
          a = av[0]; dd = dv[0]; c = cv[0]; r = rv[0];
        }
        if (lane == 0) a = T(0);
        if (lane == 31) c = T(0);
        for (int sh = 1; sh < 32; sh <<= 1) {
          const T am = __shfl_up_sync(0xffffffffu, a, sh), bm = __shfl_up_sync(0xffffffffu, dd, sh);
          const T cm = __shfl_up_sync(0xffffffffu, c, sh), rm = __shfl_up_sync(0xffffffffu, r, sh);
          const T ap = __shfl_down_sync(0xffffffffu, a, sh), bp = __shfl_down_sync(0xffffffffu, dd, sh);
          const T cp = __shfl_down_sync(0xffffffffu, c, sh), rp = __shfl_down_sync(0xffffffffu, r, sh);
          const T k1 = a * __frcp_rn(bm), k2 = c * __frcp_rn(bp);
          a = -am * k1;
          c = -cp * k2;
          dd = fma(-ap, k2, fma(-cm, k1, dd));
          r = fma(-rp, k2, fma(-rm, k1, r));
        }
        const T I = r * __frcp_rn(dd);
        const T Im = __shfl_up_sync(0xffffffffu, I, 1);
        const int kl = lane * M + M - 1;  // the interface cell
        if (kl < len) x[s0 + kl * step] = gv[M - 1] > T(0) ? I : T(0);
        if (M == 2 && lane * 2 < len) {
          const T x0 = fma(S, lane > 0 ? Im : T(0), fma(Tr, I, D));
          x[s0 + lane * 2 * step] = gv[0] > T(0) ? x0 : T(0);
        }
      }
      __syncthreads();
      return;
    }
    if (std::is_same<T, double>::value && len <= 32) {
      // FP64: one warp per line, one cell per lane, cyclic reduction by
      // shuffles -- log2 len steps instead of 2 len dependent elimination
      // steps, which the FP64 pipe's latency makes long.
      const int lane = t & 31, nwarp = NTT >> 5;
      for (int q = colour + 2 * (t >> 5); q < nlines; q += 2 * nwarp) {
        const int si = (dir == 0 ? (q + 1) * w + 1 : w + q + 1) + lane * step;
        T a = T(0), c = T(0), dd = T(1), r = T(0);
        const bool in = lane < len;
        const T gv = in ? g[si] : T(0);
        if (gv > T(0)) {
          a = -Ax[si - step];
          c = -Ax[si];
          dd = gv;
          r = fma(Cx[si], x[si + cross], b[si]);
          r = fma(Cx[si - cross], x[si - cross], r);
        }
        if (lane == 0) a = T(0);        // the ghost before the line start
        if (lane >= len - 1) c = T(0);  // and after its end
        for (int sh = 1; sh < len; sh <<= 1) {
          const T am = __shfl_up_sync(0xffffffffu, a, sh), bm = __shfl_up_sync(0xffffffffu, dd, sh);
          const T cm = __shfl_up_sync(0xffffffffu, c, sh), rm = __shfl_up_sync(0xffffffffu, r, sh);
          const T ap = __shfl_down_sync(0xffffffffu, a, sh), bp = __shfl_down_sync(0xffffffffu, dd, sh);
          const T cp = __shfl_down_sync(0xffffffffu, c, sh), rp = __shfl_down_sync(0xffffffffu, r, sh);
          const T k1 = a * lrcp(bm), k2 = c * lrcp(bp);
          a = -am * k1;
          c = -cp * k2;
          dd = fma(-ap, k2, fma(-cm, k1, dd));
          r = fma(-rp, k2, fma(-rm, k1, r));
        }
        if (in) x[si] = gv > T(0) ? r * lrcp(dd) : T(0);
      }
      __syncthreads();
      return;
    }
    for (int q = colour + 2 * t; q < nlines; q += 2 * NTT) {
      int si = (dir == 0 ? (q + 1) * w + 1 : w + q + 1);
      T cpp = T(0), dpp = T(0);
      for (int k = 0; k < len; ++k, si += step) {
        T a = T(0), c = T(0), dd = T(1), r = T(0);
        const T gv = g[si];
        if (gv > T(0)) {
          a = -Ax[si - step];
          c = -Ax[si];
          dd = gv;
          r = fma(Cx[si], x[si + cross], b[si]);
          r = fma(Cx[si - cross], x[si - cross], r);
        }
        const T inv = lrcp(fma(-a, cpp, dd));
        cpp = c * inv;
        dpp = fma(-a, dpp, r) * inv;
        CP[si] = cpp;
        DP[si] = dpp;
      }
      T xn = T(0);
      for (int k = len - 1; k >= 0; --k) {
        si -= step;
        xn = fma(-CP[si], xn, DP[si]);
        x[si] = g[si] > T(0) ? xn : T(0);
      }
    }
    __syncthreads();
  };
  // a step (x-lines, then y-lines) counts as two sweeps
  auto steps = [&](int l, bool post) {
    return ((l >= d.cfrom ? (post ? d.cpost : d.cpre) : (post ? d.npost : d.npre)) + 1) / 2;
  };
  const int n = d.n;
  for (int l = 0; l < n - 1; ++l) {
    const int ns_pre = steps(l, false);
    for (int it = 0; it < ns_pre; ++it) {
      pass(l, 0, 0); pass(l, 0, 1); pass(l, 1, 0); pass(l, 1, 1);
    }
    // residual summed 2x2 onto level l+1
    const MgView<T, CT, T>& L = d.lv[l];
    const MgView<T, CT, T>& C = d.lv[l + 1];
    const T* x = X(l);
    const T* b = B(l);
    T* bc = B(l + 1);
    const int w = W(l), wc = W(l + 1);
    for (int k = t; k < C.nx * C.ny; k += NTT) {
      const int I = k % C.nx, J = k / C.nx;
      T s = T(0);
      for (int dj = 0; dj < 2; ++dj)
        for (int dq = 0; dq < 2; ++dq) {
          const int gx = 2 * I + dq, gy = 2 * J + dj;
          if (gx >= L.nx || gy >= L.ny) continue;
          const int si = (gy + 1) * w + gx + 1;
          const T dgv = G(l)[si];
          if (dgv < T(0)) continue;
          T r = fma(-dgv, x[si], b[si]);
          r = fma(E(l)[si], x[si + 1], r);
          r = fma(E(l)[si - 1], x[si - 1], r);
          r = fma(N(l)[si], x[si + w], r);
          r = fma(N(l)[si - w], x[si - w], r);
          s += r;
        }
      bc[(J + 1) * wc + I + 1] = s;
    }
    __syncthreads();
  }
  {  // dense FP64 solve on the coarsest level
    const MgView<T, CT, T>& C = d.lv[n - 1];
    const int ncell = C.nx * C.ny, nn = *d.nc, w = W(n - 1);
    const T* b = B(n - 1);
    T* x = X(n - 1);
    for (int k = t; k < ncell; k += NTT) {
      const int r = d.cmap[k];
      if (r >= 0) bd[r] = (double)b[(k / C.nx + 1) * w + (k % C.nx) + 1];
    }
    __syncthreads();
    for (int k = t; k < ncell; k += NTT) {
      const int r = d.cmap[k];
      double y = 0.0;
      if (r >= 0)
        for (int c = 0; c < nn; ++c) y = fma(d.Ainv[r * nn + c], bd[c], y);
      x[(k / C.nx + 1) * w + (k % C.nx) + 1] = (T)y;
    }
    __syncthreads();
  }
  for (int l = n - 2; l >= 0; --l) {
    const MgView<T, CT, T>& L = d.lv[l];
    T* x = X(l);
    const T* xc = X(l + 1);
    const int w = W(l), wc = W(l + 1);
    for (int k = t; k < L.nx * L.ny; k += NTT) {
      const int ix = k % L.nx, iy = k / L.nx;
      const int si = (iy + 1) * w + ix + 1;
      if (G(l)[si] > T(0)) x[si] = fma(d.omega, xc[((iy >> 1) + 1) * wc + (ix >> 1) + 1], x[si]);
    }
    __syncthreads();
    const int ns_post = steps(l, true);
    for (int it = 0; it < ns_post; ++it) {
      pass(l, 1, 1); pass(l, 1, 0); pass(l, 0, 1); pass(l, 0, 0);
    }
  }
  {  // x of the first tail level back to global memory
    const MgView<T, CT, T>& L = d.lv[0];
    const T* x = X(0);
    for (int k = t; k < L.nx * L.ny; k += NTT) {
      const int ix = k % L.nx, iy = k / L.nx;
      L.x[(size_t)iy * L.pitch + ix] = x[(iy + 1) * W(0) + ix + 1];
    }
  }
}

}  // namespace

template <class T, class CT>
int line_tail_prepare(TailDesc<T, CT>& d) {
  if (d.n < 1 || d.n + 1 > kTailMaxLevels) return -1;
  int off = 0;
  for (int l = 0; l < d.n; ++l) {
    d.off[l] = off;
    off += 5 * (d.lv[l].nx + 2) * (d.lv[l].ny + 2);
  }
  d.off[d.n] = off;  // scratch
  off += 2 * (d.lv[0].nx + 2) * (d.lv[0].ny + 2);
  d.total = off;
  size_t bytes = (size_t)off * sizeof(T);
  bytes = (bytes + 15) / 16 * 16;
  d.bd_off = (int)bytes;
  bytes += kMaxCoarse * sizeof(double);
  d.smem = (int)bytes;
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
      bytes > (size_t)optin)
    return -1;
  if (allow_max_smem(k_line_tail<T, CT>) != cudaSuccess) {
    (void)cudaGetLastError();
    return -1;
  }
  return 0;
}

template <class T, class CT>
void launch_line_tail(const TailDesc<T, CT>& d, Scalars* sc, cudaStream_t s) {
  launch_k(k_line_tail<T, CT>, dim3(1), dim3(1024), (size_t)d.smem, s, d, sc);
}

template int line_tail_prepare<double, double>(TailDesc<double, double>&);
template int line_tail_prepare<float, __nv_bfloat16>(TailDesc<float, __nv_bfloat16>&);
template void launch_line_tail<double, double>(const TailDesc<double, double>&, Scalars*,
                                               cudaStream_t);
template void launch_line_tail<float, __nv_bfloat16>(const TailDesc<float, __nv_bfloat16>&,
                                                     Scalars*, cudaStream_t);

int line_threads(int len, int* chunk) {
  int m = len <= 4096 ? 8 : len <= 8192 ? 16 : len <= kLineMaxLen ? 32 : 0;
  if (!m) return 0;
  int th = (len + m - 1) / m;
  th = (th + 31) / 32 * 32;
  if (chunk) *chunk = m;
  return th;
}

template <class T, class CT>
void launch_line(const MgView<T, CT, T>& L, int colour, bool zero, Scalars* sc, cudaStream_t s,
                 bool rz, int flexible, double* part) {
  int m = 0;
  const int th = line_threads(L.nx, &m);
  const dim3 g((L.ny - colour + 1) / 2);
  const size_t smem = (size_t)(th / 32) * kWarpSlots * sizeof(T);
  if (g.x == 0) return;
#define SCF_LINE(MM)                                                                           \
  do {                                                                                         \
    if (zero) {                                                                                \
      auto k = k_line<T, CT, MM, true, false>;                                                 \
      allow_max_smem(k);                                                                       \
      launch_k(k, g, dim3(th), smem, s, L, colour, sc, flexible, part);                        \
    } else if (rz) {                                                                           \
      auto k = k_line<T, CT, MM, false, true>;                                                 \
      allow_max_smem(k);                                                                       \
      launch_k(k, g, dim3(th), smem, s, L, colour, sc, flexible, part);                        \
    } else {                                                                                   \
      auto k = k_line<T, CT, MM, false, false>;                                                \
      allow_max_smem(k);                                                                       \
      launch_k(k, g, dim3(th), smem, s, L, colour, sc, flexible, part);                        \
    }                                                                                          \
  } while (0)
  if (m == 8) SCF_LINE(8);
  else if (m == 16) SCF_LINE(16);
  else SCF_LINE(32);
#undef SCF_LINE
}

template <class T, class CT>
void launch_line_factor(const MgView<T, CT, T>& L, const LineFactors<T>& F, cudaStream_t s) {
  int m = 0;
  const int th = line_threads(L.nx, &m);
  const size_t smem = (size_t)8 * th * sizeof(T);
#define SCF_LF(MM)                                                            \
  do {                                                                        \
    auto k = k_line_factor<T, CT, MM>;                                        \
    allow_max_smem(k);                                                        \
    launch_k(k, dim3(L.ny), dim3(th), smem, s, L, F);                         \
  } while (0)
  if (m == 8) SCF_LF(8);
  else if (m == 16) SCF_LF(16);
  else SCF_LF(32);
#undef SCF_LF
}

template <class T, class CT>
void launch_line_solve(const MgView<T, CT, T>& L, const LineFactors<T>& F, int colour, bool zero,
                       const Scalars* sc, cudaStream_t s) {
  int m = 0;
  const int th = line_threads(L.nx, &m);
  const dim3 g((L.ny - colour + 1) / 2);
  const size_t smem = (size_t)3 * th * sizeof(T);
  if (g.x == 0) return;
#define SCF_LS(MM)                                                             \
  do {                                                                         \
    if (zero) {                                                                \
      auto k = k_line_solve<T, CT, MM, true>;                                  \
      allow_max_smem(k);                                                       \
      launch_k(k, g, dim3(th), smem, s, L, F, colour, sc);                     \
    } else {                                                                   \
      auto k = k_line_solve<T, CT, MM, false>;                                 \
      allow_max_smem(k);                                                       \
      launch_k(k, g, dim3(th), smem, s, L, F, colour, sc);                     \
    }                                                                          \
  } while (0)
  if (m == 8) SCF_LS(8);
  else if (m == 16) SCF_LS(16);
  else SCF_LS(32);
#undef SCF_LS
}

template <class E>
void launch_transpose(const E* src, int nx, int ny, int ps, E* dst, int pd, const Scalars* sc,
                      cudaStream_t s) {
  // FP32: 64 x 64 tiles with vector accesses.  FP64 keeps 32 x 32 scalar
  // tiles: a 64 x 64 FP64 tile (33 KB of static shared memory) made the
  // driver hold a shared-memory-heavy L1 split across the PDL-overlapped
  // line relaxations that follow, whose L1 hit rate it cut (4096^2 stretched
  // FP64 projection 90 -> 130 ms, with unchanged kernel times in isolation).
  if constexpr (sizeof(E) == 4) {
    const dim3 g((nx + 63) / 64, (ny + 63) / 64);
    launch_k(k_transpose_v<E>, g, dim3(32, 8), 0, s, src, nx, ny, ps, dst, pd, sc);
  } else {
    const dim3 g((nx + 31) / 32, (ny + 31) / 32);
    launch_k(k_transpose<E>, g, dim3(32, 8), 0, s, src, nx, ny, ps, dst, pd, sc);
  }
}

template <class T, class CT>
void launch_resid_restrict_lt(const MgView<T, CT, T>& Lt, const MgView<T, CT, T>& C,
                              const MgView<T, CT, T>& Ct, const Scalars* sc, cudaStream_t s) {
  if constexpr (std::is_same<T, float>::value) {
    const dim3 g((Ct.nx + 63) / 64, (Ct.ny + 7) / 8);
    launch_k(k_resid_restrict_lt4, g, dim3(32, 8), 0, s, Lt, C, Ct, sc);
  } else {
    const dim3 g((Ct.nx + 31) / 32, (Ct.ny + 7) / 8);
    launch_k(k_resid_restrict_lt<T, CT>, g, dim3(32, 8), 0, s, Lt, C, Ct, sc);
  }
}

template <class T, class CT>
void launch_prolong_lt(const MgView<T, CT, T>& Lt, const MgView<T, CT, T>& C, double omega,
                       const Scalars* sc, cudaStream_t s) {
  const dim3 g((Lt.nx + 63) / 64, (Lt.ny + 31) / 32);
  launch_k(k_prolong_lt<T, CT>, g, dim3(32, 8), 0, s, Lt, (const T*)C.x, C.pitch, C.nx, C.ny,
           (T)omega, sc);
}

void launch_aspect(const double* dx, const double* dy, size_t n, unsigned* out_bits,
                   cudaStream_t s) {
  k_aspect<<<304, 256, 0, s>>>(dx, dy, n, out_bits);
  note_launch();
}

template void launch_line<double, double>(const MgView<double, double, double>&, int, bool,
                                          Scalars*, cudaStream_t, bool, int, double*);
template void launch_line<float, __nv_bfloat16>(const MgView<float, __nv_bfloat16, float>&, int,
                                                bool, Scalars*, cudaStream_t, bool, int, double*);
template void launch_line_factor<double, double>(const MgView<double, double, double>&,
                                                const LineFactors<double>&, cudaStream_t);
template void launch_line_solve<double, double>(const MgView<double, double, double>&,
                                               const LineFactors<double>&, int, bool,
                                               const Scalars*, cudaStream_t);
template void launch_transpose<double>(const double*, int, int, int, double*, int,
                                       const Scalars*, cudaStream_t);
template void launch_transpose<float>(const float*, int, int, int, float*, int, const Scalars*,
                                      cudaStream_t);
template void launch_transpose<__nv_bfloat16>(const __nv_bfloat16*, int, int, int,
                                              __nv_bfloat16*, int, const Scalars*, cudaStream_t);
template void launch_resid_restrict_lt<double, double>(const MgView<double, double, double>&,
                                                       const MgView<double, double, double>&,
                                                       const MgView<double, double, double>&,
                                                       const Scalars*, cudaStream_t);
template void launch_resid_restrict_lt<float, __nv_bfloat16>(
    const MgView<float, __nv_bfloat16, float>&, const MgView<float, __nv_bfloat16, float>&,
    const MgView<float, __nv_bfloat16, float>&, const Scalars*, cudaStream_t);
template void launch_prolong_lt<double, double>(const MgView<double, double, double>&,
                                                const MgView<double, double, double>&, double,
                                                const Scalars*, cudaStream_t);
template void launch_prolong_lt<float, __nv_bfloat16>(const MgView<float, __nv_bfloat16, float>&,
                                                      const MgView<float, __nv_bfloat16, float>&,
                                                      double, const Scalars*, cudaStream_t);

}  // namespace scf
