// scf_mg.cu -- multigrid V-cycle kernels, templated on precision:
//   <double, double, double>  plain FP64 preconditioner
//   <float, bf16, float>      mixed: FP32 state, BF16 couplings (the fine level
//                             reads the FP32 copy of the PCG residual)
// and the PCG direction update, templated on the type of z.
//
// Every smoothing pass is a temporally blocked red-black Gauss-Seidel sweep:
// one CTA owns a 64x32 tile, loads x with a halo into shared memory, updates
// the first colour on the tile plus a ring, syncs, updates the second colour
// on the tile (plus a ring when the residual follows), and writes the tile
// back once.  Ring cells are recomputed from the same inputs as the
// neighbouring CTA computes them, so the result equals the two half sweeps
// of a global red-black iteration.  Optional fusions:
//   ZERO      the iterate starts at zero (no x read)
//   PROLONG   x += omega * x_coarse(parent) while loading (cells with an unknown)
//   RESTRICT  after the sweep, the residual of the tile is summed 2x2 onto
//             the coarse right-hand side (needs a 3-cell halo)
//   RZ        r.z (and r.z_old for the flexible PCG) reduced over the grid,
//             then the PCG beta
#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "scf_mg.cuh"

namespace scf {
namespace {

constexpr int SX = 64, SY = 32, NT = 256;
// the second tile shape of the plain-load sweep (an autotuner candidate):
// twice the CTAs of the default tile on a level, for small grids
constexpr int SX2 = 32, SY2 = 32;

template <class CT, class T>
__device__ __forceinline__ T cload(const CT* p, size_t k, float cs);
template <>
__device__ __forceinline__ double cload<double, double>(const double* p, size_t k, float) {
  return p[k];
}
template <>
__device__ __forceinline__ float cload<__nv_bfloat16, float>(const __nv_bfloat16* p, size_t k,
                                                               float cs) {
  return __bfloat162float(p[k]) * cs;
}

__device__ __forceinline__ int tlin() { return threadIdx.y * blockDim.x + threadIdx.x; }

__device__ double block_sum256(double v) {
  __shared__ double sm[NT / 32];
  __syncthreads();
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int t = tlin();
  if ((t & 31) == 0) sm[t >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (t == 0)
    for (int w = 0; w < NT / 32; ++w) s += sm[w];
  return s;
}

// two sums over the grid, last-block combine in block order (deterministic)
__device__ bool grid_sum2(double a, double b, double* part, unsigned* ticket, double* ta,
                          double* tb) {
  __shared__ bool last;
  const int t = tlin();
  const unsigned nb = gridDim.x * gridDim.y;
  const unsigned bid = blockIdx.y * gridDim.x + blockIdx.x;
  const double sa = block_sum256(a);
  const double sb = block_sum256(b);
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
  for (unsigned k = t; k < nb; k += NT) {
    xa += __ldcg(&part[2 * k]);
    xb += __ldcg(&part[2 * k + 1]);
  }
  xa = block_sum256(xa);
  xb = block_sum256(xb);
  if (t == 0) {
    *ta = xa;
    *tb = xb;
    *ticket = 0u;
  }
  return true;
}


template <class T, class CT, class BT, int FIRST, bool ZERO, bool PROLONG, bool RESTRICT, bool RZ,
          int ITER, int TX, int TY>
__global__ void __launch_bounds__(NT)
k_sweep(MgView<T, CT, BT> L, MgView<T, CT, T> C, T omega, int flexible, Scalars* sc,
        double* part) {
  pdl_wait();
  if (sc->done) return;
  // x halo: one ring per colour phase (ITER red-black iterations), plus one
  // for the residual of the restriction
  constexpr int H = 2 * ITER + (RESTRICT ? 1 : 0);
  constexpr int WX = TX + 2 * H, WY = TY + 2 * H;
  __shared__ T xs[WY][WX];
  const int nx = L.nx, ny = L.ny, P = L.pitch;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int t = tlin();
  const float cs = L.csp ? __ldg(L.csp) : 1.0f;

  // phase 0: x with halo; outside the grid the value is zero
  for (int e = t; e < WX * WY; e += NT) {
    const int ex = e % WX, ey = e / WX;
    const int gx = x0 - H + ex, gy = y0 - H + ey;
    T v = T(0);
    if (gx >= 0 && gx < nx && gy >= 0 && gy < ny) {
      const size_t g = (size_t)gy * P + gx;
      if (!ZERO) v = L.xin[g];
      if (PROLONG) {
        if (L.di[g] > T(0)) v = fma(omega, C.x[(size_t)(gy >> 1) * C.pitch + (gx >> 1)], v);
      }
    }
    xs[ey][ex] = v;
  }
  __syncthreads();

  auto relax = [&](int gx, int gy) {
    const size_t g = (size_t)gy * P + gx;
    const int lx = gx - x0 + H, ly = gy - y0 + H;
    T s = (T)L.b[g];
    s = fma(cload<CT, T>(L.cE, g, cs), xs[ly][lx + 1], s);
    s = fma(cload<CT, T>(L.cE, g - 1, cs), xs[ly][lx - 1], s);
    s = fma(cload<CT, T>(L.cN, g, cs), xs[ly + 1][lx], s);
    s = fma(cload<CT, T>(L.cN, g - P, cs), xs[ly - 1][lx], s);
    xs[ly][lx] = s * L.di[g];
  };

  // colour phases q = 0 .. 2*ITER-1 (FIRST colour on even q): phase q
  // updates its colour on the tile plus a ring of width H-1-q, from values
  // that phase q-1 (or the load) left valid one ring further out
#pragma unroll
  for (int q = 0; q < 2 * ITER; ++q) {
    const int colour = (q & 1) ? 1 - FIRST : FIRST;
    const int R = H - 1 - q;
    const int CW = (TX + 2 * R) / 2, RH = TY + 2 * R;
    for (int e = t; e < CW * RH; e += NT) {
      const int k = e % CW, ey = e / CW;
      const int gy = y0 - R + ey;
      const int gx = x0 - R + ((x0 - R + gy + colour) & 1) + 2 * k;
      if (gx >= 0 && gx < nx && gy >= 0 && gy < ny) relax(gx, gy);
    }
    __syncthreads();
  }

  // phase 3: write the tile; optional r.z (accumulated in T per thread, then
  // combined in FP64)
  T a1 = T(0);
  for (int e = t; e < TX * TY; e += NT) {
    const int ex = e % TX, ey = e / TX;
    const int gx = x0 + ex, gy = y0 + ey;
    if (gx < nx && gy < ny) {
      const size_t g = (size_t)gy * P + gx;
      const T v = xs[ey + H][ex + H];
      L.x[g] = v;
      if (RZ) a1 = fma((T)L.b[g], v, a1);
    }
  }

  if (RESTRICT) {
    // residual of each tile cell, summed 2x2 onto the coarse level
    const int I0 = x0 >> 1, J0 = y0 >> 1;
    for (int e = t; e < (TX / 2) * (TY / 2); e += NT) {
      const int ci = e % (TX / 2), cj = e / (TX / 2);
      const int I = I0 + ci, J = J0 + cj;
      if (I >= C.nx || J >= C.ny) continue;
      T s = T(0);
      for (int dj = 0; dj < 2; ++dj)
        for (int dq = 0; dq < 2; ++dq) {
          const int gx = 2 * I + dq, gy = 2 * J + dj;
          if (gx >= nx || gy >= ny) continue;
          const size_t g = (size_t)gy * P + gx;
          const int lx = gx - x0 + H, ly = gy - y0 + H;
          const T d = L.dg[g];
          if (d < T(0)) continue;
          T r = fma(-d, xs[ly][lx], (T)L.b[g]);
          r = fma(cload<CT, T>(L.cE, g, cs), xs[ly][lx + 1], r);
          r = fma(cload<CT, T>(L.cE, g - 1, cs), xs[ly][lx - 1], r);
          r = fma(cload<CT, T>(L.cN, g, cs), xs[ly + 1][lx], r);
          r = fma(cload<CT, T>(L.cN, g - P, cs), xs[ly - 1][lx], r);
          s += r;
        }
      C.b[(size_t)J * C.pitch + I] = s;
    }
  }

  if (RZ) {
    double tot1, tot2;
    if (grid_sum2((double)a1, 0.0, part, &sc->tickets[T_RZ], &tot1, &tot2) && t == 0)
      set_beta(sc, tot1, flexible);
  }
}

// ---------------------------------------------------------------------------
// TMA-staged sweep (FP32/BF16 levels).  The same fused red-black iterations
// as k_sweep, in the same arithmetic order, but every operand of the tile's
// window -- x, b, the inverse diagonal and both BF16 couplings over 80 x 42
// cells around the 64 x 32 tile -- arrives by one bulk tensor copy per array
// (cp.async.bulk.tensor, completion counted in bytes on an mbarrier), so the
// whole window is in flight at once and the colour phases read shared
// memory only.  Cells outside the grid arrive as zeros (the ghost values).
// The wait on the mbarrier is bounded: past the limit the kernel records a
// timeout, waits (bounded again) for its copies to land, and returns.

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
// One bounded poll: the thread may be suspended inside try_wait until the
// phase completes, but for at most kPollNs nanoseconds (the suspend-time
// hint), so kMbarSpins polls take at most about a second.
constexpr unsigned kPollNs = 1024;
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "n"(kPollNs)
      : "memory");
  return ok != 0;
}
// 2-D tile of the tensor map at `map` (generic address of global memory)
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

constexpr int kBoxCells = kSweepBoxX * kSweepBoxY;
constexpr int kBoxF32 = kBoxCells * 4, kBoxBF16 = kBoxCells * 2;  // bytes per window copy
constexpr int r128(int b) { return (b + 127) / 128 * 128; }
// window regions at 128-byte aligned offsets from a 128-byte aligned base
constexpr int kOffB = r128(kBoxF32), kOffD = 2 * r128(kBoxF32), kOffE = 3 * r128(kBoxF32);
constexpr int kOffN = kOffE + r128(kBoxBF16), kOffBar = kOffN + r128(kBoxBF16);
constexpr int kTmaSmem = 128 + kOffBar + 16;  // + slack to align the base
constexpr int kMbarSpins = 1 << 20;
// Fault injection for tests (scf_diag_tma_timeout): the CTA with this linear
// index, in launches that reduce nothing across the grid, arms its barrier
// without issuing its copies -- nothing is in flight, so its bounded wait
// runs out -- and every wait polls at most g_tma_spins times.
__device__ int g_tma_skip_cta = -1;
__device__ int g_tma_spins = kMbarSpins;

template <int FIRST, bool ZERO, bool PROLONG, bool RESTRICT, bool RZ, int ITER>
__global__ void __launch_bounds__(NT)
k_sweep_tma(MgView<float, __nv_bfloat16, float> L, MgView<float, __nv_bfloat16, float> C,
            float omega, int flexible, Scalars* sc, double* part, const CUtensorMap* maps,
            int xin) {
  pdl_wait();
  if (sc->done) return;
  constexpr int H = 2 * ITER + (RESTRICT ? 1 : 0);  // halo of the colour phases (<= 5)
  constexpr int OX = 8, OY = 5;                     // window origin relative to the tile
  extern __shared__ __align__(128) unsigned char tsm_raw[];
  unsigned char* tsm = tsm_raw + ((128u - (smem_addr(tsm_raw) & 127u)) & 127u);
  float* xw = reinterpret_cast<float*>(tsm);  // [kSweepBoxY][kSweepBoxX]
  float* bw = reinterpret_cast<float*>(tsm + kOffB);
  float* dw = reinterpret_cast<float*>(tsm + kOffD);
  __nv_bfloat16* ew = reinterpret_cast<__nv_bfloat16*>(tsm + kOffE);
  __nv_bfloat16* nw = reinterpret_cast<__nv_bfloat16*>(tsm + kOffN);
  uint64_t* bar = reinterpret_cast<uint64_t*>(tsm + kOffBar);
  const int nx = L.nx, ny = L.ny;
  const int x0 = blockIdx.x * SX, y0 = blockIdx.y * SY;
  const int wx0 = x0 - OX, wy0 = y0 - OY;  // window origin (x: a multiple of 8)
  const int t = tlin();
  const float cs = L.csp ? __ldg(L.csp) : 1.0f;
  const int spins = g_tma_spins;
  const bool skip = !RZ && (int)(blockIdx.y * gridDim.x + blockIdx.x) == g_tma_skip_cta;
  if (t == 0) {
    mbar_init(bar, 1);
    mbar_init_fence();
  }
  __syncthreads();
  if (t == 0) {
    mbar_expect_tx(bar, (ZERO ? 0u : (unsigned)kBoxF32) + 2u * kBoxF32 + 2u * kBoxBF16);
    if (!skip) {
      if (!ZERO) tma_load_2d(xw, maps + xin, wx0, wy0, bar);
      tma_load_2d(bw, maps + 2, wx0, wy0, bar);
      tma_load_2d(dw, maps + 3, wx0, wy0, bar);
      tma_load_2d(ew, maps + 4, wx0, wy0, bar);
      tma_load_2d(nw, maps + 5, wx0, wy0, bar);
    }
  }
  if (ZERO)
    for (int e = t; e < kBoxCells; e += NT) xw[e] = 0.0f;
  // PROLONG: the coarse values of the tile plus its H-cell ring, read while
  // the window is in flight
  constexpr int PW = SX + 2 * H, PH = SY + 2 * H, KP = PROLONG ? (PW * PH + NT - 1) / NT : 1;
  float cx[KP];
  if (PROLONG) {
#pragma unroll
    for (int k = 0; k < KP; ++k) {
      const int e = t + k * NT;
      const int gx = x0 - H + e % PW, gy = y0 - H + e / PW;
      cx[k] = (e < PW * PH && gx >= 0 && gx < nx && gy >= 0 && gy < ny)
                  ? C.x[(size_t)(gy >> 1) * C.pitch + (gx >> 1)]
                  : 0.0f;
    }
  }
  bool ok = false;
  for (int it = 0; it < spins && !ok; ++it) ok = mbar_try_wait(bar, 0);
  // one decision for the whole block (the barrier also orders the window's
  // shared-memory contents before the phases below)
  if (!__syncthreads_and(ok)) {  // record, let the copies land (bounded), leave
    if (t == 0) {
      sc->status = kErrTimeout;
      sc->done = 1;
    }
    for (int it = 0; it < spins && !mbar_try_wait(bar, 0); ++it) {
    }
    return;
  }
  auto W = [&](int gx, int gy) { return (gy - wy0) * kSweepBoxX + (gx - wx0); };
  if (PROLONG) {
#pragma unroll
    for (int k = 0; k < KP; ++k) {
      const int e = t + k * NT;
      const int gx = x0 - H + e % PW, gy = y0 - H + e / PW;
      if (e < PW * PH && gx >= 0 && gx < nx && gy >= 0 && gy < ny) {
        const int w = W(gx, gy);
        if (dw[w] > 0.0f) xw[w] = fmaf(omega, cx[k], xw[w]);
      }
    }
    __syncthreads();
  }
  auto relax = [&](int gx, int gy) {
    const int w = W(gx, gy);
    float s = bw[w];
    s = fmaf(__bfloat162float(ew[w]) * cs, xw[w + 1], s);
    s = fmaf(__bfloat162float(ew[w - 1]) * cs, xw[w - 1], s);
    s = fmaf(__bfloat162float(nw[w]) * cs, xw[w + kSweepBoxX], s);
    s = fmaf(__bfloat162float(nw[w - kSweepBoxX]) * cs, xw[w - kSweepBoxX], s);
    xw[w] = s * dw[w];
  };
#pragma unroll
  for (int q = 0; q < 2 * ITER; ++q) {
    const int colour = (q & 1) ? 1 - FIRST : FIRST;
    const int R = H - 1 - q;
    const int CW = (SX + 2 * R) / 2, RH = SY + 2 * R;
    for (int e = t; e < CW * RH; e += NT) {
      const int k = e % CW, ey = e / CW;
      const int gy = y0 - R + ey;
      const int gx = x0 - R + ((x0 - R + gy + colour) & 1) + 2 * k;
      if (gx >= 0 && gx < nx && gy >= 0 && gy < ny) relax(gx, gy);
    }
    __syncthreads();
  }
  const int P = L.pitch;
  float a1 = 0.0f;
  for (int e = t; e < SX * SY; e += NT) {
    const int gx = x0 + e % SX, gy = y0 + e / SX;
    if (gx < nx && gy < ny) {
      const int w = W(gx, gy);
      const float v = xw[w];
      L.x[(size_t)gy * P + gx] = v;
      if (RZ) a1 = fmaf(bw[w], v, a1);
    }
  }
  if (RESTRICT) {
    const int I0 = x0 >> 1, J0 = y0 >> 1;
    for (int e = t; e < (SX / 2) * (SY / 2); e += NT) {
      const int I = I0 + e % (SX / 2), J = J0 + e / (SX / 2);
      if (I >= C.nx || J >= C.ny) continue;
      float s = 0.0f;
      for (int dj = 0; dj < 2; ++dj)
        for (int dq = 0; dq < 2; ++dq) {
          const int gx = 2 * I + dq, gy = 2 * J + dj;
          if (gx >= nx || gy >= ny) continue;
          const float d = L.dg[(size_t)gy * P + gx];
          if (d < 0.0f) continue;
          const int w = W(gx, gy);
          float r = fmaf(-d, xw[w], bw[w]);
          r = fmaf(__bfloat162float(ew[w]) * cs, xw[w + 1], r);
          r = fmaf(__bfloat162float(ew[w - 1]) * cs, xw[w - 1], r);
          r = fmaf(__bfloat162float(nw[w]) * cs, xw[w + kSweepBoxX], r);
          r = fmaf(__bfloat162float(nw[w - kSweepBoxX]) * cs, xw[w - kSweepBoxX], r);
          s += r;
        }
      C.b[(size_t)J * C.pitch + I] = s;
    }
  }
  if (RZ) {
    double tot1, tot2;
    if (grid_sum2((double)a1, 0.0, part, &sc->tickets[T_RZ], &tot1, &tot2) && t == 0)
      set_beta(sc, tot1, flexible);
  }
}

template <class T, class CT, class BT>
__global__ void k_coarse_solve_t(MgView<T, CT, BT> C, const double* Ainv, const int* cmap,
                                 const int* ncp, Scalars* sc) {
  pdl_wait();
  if (sc->done) return;
  __shared__ double bd[kMaxCoarse];
  const int t = threadIdx.x;
  const int ncell = C.nx * C.ny, nn = *ncp;
  for (int k = t; k < ncell; k += blockDim.x) {
    const int r = cmap[k];
    if (r >= 0) bd[r] = (double)C.b[(size_t)(k / C.nx) * C.pitch + (k % C.nx)];
  }
  __syncthreads();
  for (int k = t; k < ncell; k += blockDim.x) {
    const int r = cmap[k];
    double y = 0.0;
    if (r >= 0)
      for (int c = 0; c < nn; ++c) y = fma(Ainv[r * nn + c], bd[c], y);
    C.x[(size_t)(k / C.nx) * C.pitch + (k % C.nx)] = (T)y;
  }
}

// r.z (and r.z_old) when the V-cycle does not end with a sweep
template <class T, class BT>
__global__ void k_dot_rz_t(int nx, int ny, int pitch, const BT* r, const T* z, int flexible,
                           Scalars* sc, double* part) {
  pdl_wait();
  if (sc->done) return;
  // each thread accumulates its column strip in T (FP32 for the mixed
  // preconditioner, whose z is FP32 anyway), the grid combines in FP64
  T acc = T(0);
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix < nx)
    for (int iy = blockIdx.y * 8 + threadIdx.y; iy < ny; iy += gridDim.y * 8) {
      const size_t k = (size_t)iy * pitch + ix;
      acc = fma((T)r[k], z[k], acc);
    }
  const double a1 = (double)acc, a2 = 0.0;
  double t1, t2;
  if (grid_sum2(a1, a2, part, &sc->tickets[T_RZ], &t1, &t2) && tlin() == 0)
    set_beta(sc, t1, flexible);
}

__device__ __forceinline__ double conv_z(float z) { return f2d_exact(z); }
__device__ __forceinline__ double conv_z(double z) { return z; }

// p_new = z + beta p_old (= z on the first iteration), q = A p_new, p.q and
// alpha = r.z / p.q, with an FP64 direction (the FP64 preconditioner).
// Register-blocked stencil: a warp covers 32 consecutive columns, of which
// it updates the inner 30 (the first and last lane only form p_new for their
// neighbours, so every lane runs the same code), and each thread walks
// `rows` rows of its column, keeping p_new of the rows above and below in
// registers, taking east/west values from the adjacent lanes and loading the
// next row one step ahead.  No shared memory and no block barrier before the
// arithmetic, so the FP64 pipe stays fed: five FP64 operations per cell (the
// product with the diagonal and four FMAs) are the kernel's bound on GB300's
// FP64 pipe.
__global__ void __launch_bounds__(NT)
k_pupdate_spmv_t(LevelView L, const double* __restrict__ z, const double* __restrict__ pold,
                 double* __restrict__ pnew, double* __restrict__ q, Scalars* sc, double* part,
                 int rows) {
  pdl_wait();
  if (sc->done) return;
  const int nx = L.nx, ny = L.ny, P = L.pitch;
  const int lane = threadIdx.x;  // blockDim (32, 8): a warp is 32 consecutive columns
  const int cx = blockIdx.x * 30 - 1 + lane;
  const bool col = cx >= 0 && cx < nx;          // a column of the grid
  const bool upd = col && lane > 0 && lane < 31;  // updated by this lane
  const int r0 = (blockIdx.y * 8 + threadIdx.y) * rows;
  const int r1 = r0 + rows < ny ? r0 + rows : ny;
  const bool first = sc->iter == 0;
  const double beta = sc->beta;
  // raw inputs of p_new at row y of this column (zeros outside the grid)
  struct Raw { double z, p; };
  auto load = [&](int y) -> Raw {
    Raw r{0.0, 0.0};
    if (col && y >= 0 && y < ny) {
      const size_t g = (size_t)y * P + cx;
      r.z = z[g];
      if (!first) r.p = pold[g];
    }
    return r;
  };
  auto form = [&](const Raw& r) -> double { return fma(beta, r.p, r.z); };
  double acc = 0.0;
  if (r0 < r1) {  // uniform across the warp (one threadIdx.y per warp)
    double pm = form(load(r0 - 1));
    double pc = form(load(r0));
    double cNd = col ? L.cN[(size_t)(r0 - 1) * P + cx] : 0.0;
    Raw nxt = load(r0 + 1);
    for (int iy = r0; iy < r1; ++iy) {
      const size_t k = (size_t)iy * P + cx;
      double dg = 0.0, cE = 0.0, cN = 0.0;
      if (col) { dg = L.dg[k]; cE = L.cE[k]; cN = L.cN[k]; }
      const double pp = form(nxt);
      nxt = load(iy + 2);  // one row ahead
      const double pl = __shfl_up_sync(0xffffffffu, pc, 1);
      const double pr = __shfl_down_sync(0xffffffffu, pc, 1);
      double cW = __shfl_up_sync(0xffffffffu, cE, 1), cS = cNd;
      // rows whose own west / south entries differ from the neighbours'
      // east / north ones take them from wW / wS (the row flag is the same
      // for the whole warp)
      if (L.arow && L.arow[iy] && col) {
        cW = L.wW[k];
        cS = L.wS[k];
      }
      double qv = pos_part(dg) * pc;
      qv = fma(-cE, pr, qv);
      qv = fma(-cW, pl, qv);
      qv = fma(-cN, pp, qv);
      qv = fma(-cS, pm, qv);
      if (upd) {
        q[k] = qv;
        pnew[k] = pc;
        acc = fma(pc, qv, acc);
      }
      pm = pc;
      pc = pp;
      cNd = cN;
    }
  }
  double tot, dummy;
  if (grid_sum2(acc, 0.0, part, &sc->tickets[T_PQ], &tot, &dummy) && tlin() == 0) {
    sc->pq = tot;
    sc->alpha = sc->rz / tot;
  }
}

// The same with an FP32 direction (the FP32 preconditioner, whose z carries
// FP32 accuracy anyway): p_new = z + beta p_old and the products of p.q in
// FP32 (Kahan's compensated sum per thread, FP64 across threads; p.q only
// sets the step length alpha).  q = A p keeps FP64 accuracy without the
// FP64 pipe: the operator comes as float pairs (hi + lo within 2^-48 of the
// FP64 entries, split once per setup) and the five products with the FP32
// direction are summed in float-float arithmetic (exact products by FMA,
// Knuth's TwoSum), so q = hi + lo is within about 2^-46 of the sum of the
// magnitudes of its terms -- against 2^-53 for the FP64 sum, far below what
// the recursive residual r -= alpha q notices at the solver's tolerances --
// for one FP64 addition per cell.  Free of the FP64 bound, the kernel is
// bound by memory latency, so it is one thread per cell over a grid-stride
// row loop: each thread has all its loads (the direction of the cell and its
// four neighbours, which mostly hit L1 / L2, and the operator) in flight at
// once.  Cells outside the grid count as zeros.
// (64 registers: four CTAs per SM, so the grid's eight per SM run in two full
// waves; at 72 registers, three per SM, the kernel took 213 against 175 us at 4096^2)
__global__ void __launch_bounds__(NT, 4)
k_pupdate_spmv_ff(LevelView L, const float* __restrict__ z, const float* __restrict__ pold,
                  float* __restrict__ pnew, double* __restrict__ q, Scalars* sc, double* part) {
  pdl_wait();
  if (sc->done) return;
  const int nx = L.nx, ny = L.ny, P = L.pitch;
  const bool first = sc->iter == 0;
  const float beta = first ? 0.0f : (float)sc->beta;
  const float* __restrict__ po = first ? z : pold;  // beta = 0: any finite array
  const float2* __restrict__ fD = L.fD;
  const float2* __restrict__ fE = L.fE;
  const float2* __restrict__ fN = L.fN;
  const int* __restrict__ arow = L.arow;
  const int ix = blockIdx.x * 32 + threadIdx.x;
  const int S = gridDim.y * 8;
  const float2 f0 = make_float2(0.0f, 0.0f);
  // everything a cell reads, fetched one row step ahead of its use
  struct In {
    float z[5], p[5];  // centre, west, east, south, north
    float2 d, e, w, n, s;
    int flag;
  };
  auto fetch = [&](int iy, In& v) {
    const size_t k = (size_t)iy * P + ix;
    const bool in[5] = {true, ix > 0, ix + 1 < nx, iy > 0, iy + 1 < ny};
    const ptrdiff_t off[5] = {0, -1, 1, -(ptrdiff_t)P, (ptrdiff_t)P};
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      v.z[j] = in[j] ? z[k + off[j]] : 0.0f;
      v.p[j] = in[j] ? po[k + off[j]] : 0.0f;
    }
    v.d = fD[k];
    v.e = fE[k];
    v.n = fN[k];
    v.w = in[1] ? fE[k - 1] : f0;
    v.s = in[3] ? fN[k - P] : f0;
    v.flag = arow[iy];
  };
  float accf = 0.0f, accc = 0.0f;
  int iy = blockIdx.y * 8 + threadIdx.y;
  if (ix < nx && iy < ny) {
    In cur;
    fetch(iy, cur);
    for (; iy < ny; iy += S) {
      In nxt;
      const bool more = iy + S < ny;
      if (more) fetch(iy + S, nxt);
      const size_t k = (size_t)iy * P + ix;
      float pv[5];
#pragma unroll
      for (int j = 0; j < 5; ++j) pv[j] = fmaf(beta, cur.p[j], cur.z[j]);
      float2 cW = cur.w, cS = cur.s;
      // rows whose own west / south entries differ from the neighbours'
      // east / north ones take them from wW / wS
      if (cur.flag) {
        cW = split_ff(L.wW[k]);
        cS = split_ff(L.wS[k]);
      }
      const float pc = pv[0];
      float sh = __fmul_rn(cur.d.x, pc);
      float sl = __fmaf_rn(cur.d.y, pc, __fmaf_rn(cur.d.x, pc, -sh));
      ff_sub_prod(cur.e, pv[2], sh, sl);
      ff_sub_prod(cW, pv[1], sh, sl);
      ff_sub_prod(cur.n, pv[4], sh, sl);
      ff_sub_prod(cS, pv[3], sh, sl);
      q[k] = f2d_exact(sh) + f2d_exact(sl);
      pnew[k] = pc;
      // compensated FP32 sum of the FP32 products
      const float y = fmaf(pc, __fadd_rn(sh, sl), -accc);
      const float t = accf + y;
      accc = (t - accf) - y;
      accf = t;
      if (more) cur = nxt;
    }
  }
  const double acc = f2d_exact(accf) - f2d_exact(accc);
  double tot, dummy;
  if (grid_sum2(acc, 0.0, part, &sc->tickets[T_PQ], &tot, &dummy) && tlin() == 0) {
    sc->pq = tot;
    sc->alpha = sc->rz / tot;
  }
}

// inverse diagonal of an FP64 level (0 where the cell has no unknown)
__global__ void k_inv_diag(int nx, int ny, int pitch, const double* dg, double* di) {
  pdl_wait();
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix >= nx) return;
  for (int iy = blockIdx.y * 8 + threadIdx.y; iy < ny; iy += gridDim.y * 8) {
    const size_t k = (size_t)iy * pitch + ix;
    const double d = dg[k];
    di[k] = d > 0.0 ? 1.0 / d : 0.0;
  }
}

// largest coupling of a level, as the bits of a non-negative float
__global__ void k_max_coupling(LevelView F, unsigned* out_bits) {
  pdl_wait();
  float m = 0.0f;
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix < F.nx)
    for (int iy = blockIdx.y * 8 + threadIdx.y; iy < F.ny; iy += gridDim.y * 8) {
      const size_t k = (size_t)iy * F.pitch + ix;
      m = fmaxf(m, (float)fabs(F.cE[k]));
      m = fmaxf(m, (float)fabs(F.cN[k]));
    }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  __shared__ float wm[8];
  const int t = threadIdx.y * 32 + threadIdx.x;
  if ((t & 31) == 0) wm[t >> 5] = m;
  __syncthreads();
  if (t == 0) {
    float b = wm[0];
    for (int w = 1; w < 8; ++w) b = fmaxf(b, wm[w]);
    atomicMax(out_bits, __float_as_uint(b));  // one atomic per block
  }
}

// Mixed level from the FP64 level: BF16 couplings divided by a power-of-two
// scale near the level's largest coupling, FP32 diagonal rebuilt from the
// rounded couplings plus the FP64 excess (so the level stays a diagonally
// dominant M-matrix), FP32 inverse diagonal.
__global__ void k_to_mixed(LevelView F, MgView<float, __nv_bfloat16, float> M,
                           const unsigned* max_bits, float* cscale_out) {
  pdl_wait();
  const float mx = __uint_as_float(*max_bits);
  int ex = 0;
  frexpf(mx > 0.0f ? mx : 1.0f, &ex);
  const float cs = ldexpf(1.0f, ex);  // power of two >= the largest coupling
  const float inv = 1.0f / cs;
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) *cscale_out = cs;
  const int ix = blockIdx.x * 32 + threadIdx.x;
  if (ix >= F.nx) return;
  const int P = F.pitch;
  auto rb = [&](double c) { return __float2bfloat16_rn((float)c * inv); };
  for (int iy = blockIdx.y * 8 + threadIdx.y; iy < F.ny; iy += gridDim.y * 8) {
    const size_t k = (size_t)iy * P + ix;
    const __nv_bfloat16 e16 = rb(F.cE[k]), n16 = rb(F.cN[k]);
    const_cast<__nv_bfloat16*>(M.cE)[k] = e16;
    const_cast<__nv_bfloat16*>(M.cN)[k] = n16;
    float d = -1.0f, di = 0.0f;
    if (F.dg[k] > 0.0) {
      const float sum = (__bfloat162float(e16) + __bfloat162float(rb(F.cE[k - 1])) +
                         __bfloat162float(n16) + __bfloat162float(rb(F.cN[k - P]))) * cs;
      d = sum + (float)F.ex[k];
      if (d > 0.0f) di = 1.0f / d;
      else d = -1.0f;
    }
    const_cast<float*>(M.dg)[k] = d;
    const_cast<float*>(M.di)[k] = di;
    if (F.fD) {  // the fine level's float pairs
      F.fE[k] = split_ff(F.cE[k]);
      F.fN[k] = split_ff(F.cN[k]);
      F.fD[k] = split_ff(pos_part(F.dg[k]));
    }
  }
}

// The coarse end of the V-cycle in one CTA: every level of at most
// kTailMaxCells cells, down to the dense coarsest solve and back up, with x
// and b of all those levels in shared memory (each level padded by a zero
// ghost ring); FP32 tails stage the operators there too, FP64 tails read
// them through L1.  Replaces four kernel
// launches per level, which on such small grids cost launch latency only.
// The arithmetic is that of k_sweep / k_coarse_solve_t, cell for cell.
template <class T, class CT>
__global__ void __launch_bounds__(1024) k_tail(TailDesc<T, CT> d, Scalars* sc) {
  pdl_wait();
  if (sc->done) return;
  // FP32 tails also stage the operators (couplings scaled to FP32, inverse
  // diagonal, diagonal) so that no phase after the first touches global memory
  constexpr bool STAGE = std::is_same<T, float>::value;
  extern __shared__ __align__(16) unsigned char tail_smem[];
  T* sm = reinterpret_cast<T*>(tail_smem);
  double* bd = reinterpret_cast<double*>(tail_smem + d.bd_off);
  const int t = threadIdx.x, NTT = blockDim.x;
  for (int i = t; i < d.total; i += NTT) sm[i] = T(0);
  __syncthreads();
  auto W = [&](int l) { return d.lv[l].nx + 2; };
  auto WH = [&](int l) { return (d.lv[l].nx + 2) * (d.lv[l].ny + 2); };
  auto xs = [&](int l) { return sm + d.off[l]; };
  auto bs = [&](int l) { return sm + d.off[l] + WH(l); };
  auto dis = [&](int l) { return sm + d.off[l] + 2 * WH(l); };
  auto dgs = [&](int l) { return sm + d.off[l] + 3 * WH(l); };
  auto ces = [&](int l) { return sm + d.off[l] + 4 * WH(l); };
  auto cns = [&](int l) { return sm + d.off[l] + 5 * WH(l); };
  {  // right-hand side of the first tail level (restricted by the previous kernel)
    const MgView<T, CT, T>& L = d.lv[0];
    T* b = bs(0);
    for (int k = t; k < L.nx * L.ny; k += NTT) {
      const int ix = k % L.nx, iy = k / L.nx;
      b[(iy + 1) * W(0) + ix + 1] = L.b[(size_t)iy * L.pitch + ix];
    }
  }
  if (STAGE) {
    for (int l = 0; l < d.n; ++l) {
      const MgView<T, CT, T>& L = d.lv[l];
      const float cs = L.csp ? __ldg(L.csp) : 1.0f;
      for (int k = t; k < L.nx * L.ny; k += NTT) {
        const int ix = k % L.nx, iy = k / L.nx;
        const size_t g = (size_t)iy * L.pitch + ix;
        const int si = (iy + 1) * W(l) + ix + 1;
        dis(l)[si] = L.di[g];
        dgs(l)[si] = L.dg[g];
        ces(l)[si] = cload<CT, T>(L.cE, g, cs);
        cns(l)[si] = cload<CT, T>(L.cN, g, cs);
      }
    }
  }
  __syncthreads();
  // operator access: staged copies or the global arrays
  auto opE = [&](int l, int si, size_t g, float cs) {
    return STAGE ? ces(l)[si] : cload<CT, T>(d.lv[l].cE, g, cs);
  };
  auto opN = [&](int l, int si, size_t g, float cs) {
    return STAGE ? cns(l)[si] : cload<CT, T>(d.lv[l].cN, g, cs);
  };
  auto opDi = [&](int l, int si, size_t g) { return STAGE ? dis(l)[si] : d.lv[l].di[g]; };
  auto opDg = [&](int l, int si, size_t g) { return STAGE ? dgs(l)[si] : d.lv[l].dg[g]; };
  auto relax = [&](int l, int colour) {
    const MgView<T, CT, T>& L = d.lv[l];
    const float cs = (!STAGE && L.csp) ? __ldg(L.csp) : 1.0f;
    T* x = xs(l);
    const T* b = bs(l);
    const int w = W(l), P = L.pitch;
    for (int k = t; k < L.nx * L.ny; k += NTT) {
      const int ix = k % L.nx, iy = k / L.nx;
      if (((ix + iy) & 1) != colour) continue;
      const size_t g = (size_t)iy * P + ix;
      const int si = (iy + 1) * w + ix + 1;
      T s = b[si];
      s = fma(opE(l, si, g, cs), x[si + 1], s);
      s = fma(opE(l, si - 1, g - 1, cs), x[si - 1], s);
      s = fma(opN(l, si, g, cs), x[si + w], s);
      s = fma(opN(l, si - w, g - P, cs), x[si - w], s);
      x[si] = s * opDi(l, si, g);
    }
    __syncthreads();
  };
  const int n = d.n;
  for (int l = 0; l < n - 1; ++l) {
    const int np = l >= d.cfrom ? d.cpre : d.npre;  // the coarse schedule from cfrom down
    for (int it = 0; it < np; ++it) { relax(l, 0); relax(l, 1); }
    // residual summed 2x2 onto level l+1
    const MgView<T, CT, T>& L = d.lv[l];
    const MgView<T, CT, T>& C = d.lv[l + 1];
    const float cs = (!STAGE && L.csp) ? __ldg(L.csp) : 1.0f;
    const T* x = xs(l);
    const T* b = bs(l);
    T* bc = bs(l + 1);
    const int w = W(l), wc = W(l + 1), P = L.pitch;
    for (int k = t; k < C.nx * C.ny; k += NTT) {
      const int I = k % C.nx, J = k / C.nx;
      T s = T(0);
      for (int dj = 0; dj < 2; ++dj)
        for (int dq = 0; dq < 2; ++dq) {
          const int gx = 2 * I + dq, gy = 2 * J + dj;
          if (gx >= L.nx || gy >= L.ny) continue;
          const size_t g = (size_t)gy * P + gx;
          const int si = (gy + 1) * w + gx + 1;
          const T dgv = opDg(l, si, g);
          if (dgv < T(0)) continue;
          T r = fma(-dgv, x[si], b[si]);
          r = fma(opE(l, si, g, cs), x[si + 1], r);
          r = fma(opE(l, si - 1, g - 1, cs), x[si - 1], r);
          r = fma(opN(l, si, g, cs), x[si + w], r);
          r = fma(opN(l, si - w, g - P, cs), x[si - w], r);
          s += r;
        }
      bc[(J + 1) * wc + I + 1] = s;
    }
    __syncthreads();
  }
  {  // dense FP64 solve on the coarsest level
    const MgView<T, CT, T>& C = d.lv[n - 1];
    const int ncell = C.nx * C.ny, nn = *d.nc, w = W(n - 1);
    const T* b = bs(n - 1);
    T* x = xs(n - 1);
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
    T* x = xs(l);
    const T* xc = xs(l + 1);
    const int w = W(l), wc = W(l + 1);
    for (int k = t; k < L.nx * L.ny; k += NTT) {
      const int ix = k % L.nx, iy = k / L.nx;
      const int si = (iy + 1) * w + ix + 1;
      if (opDi(l, si, (size_t)iy * L.pitch + ix) > T(0))
        x[si] = fma(d.omega, xc[((iy >> 1) + 1) * wc + (ix >> 1) + 1], x[si]);
    }
    __syncthreads();
    const int nq = l >= d.cfrom ? d.cpost : d.npost;
    for (int it = 0; it < nq; ++it) { relax(l, 1); relax(l, 0); }
  }
  {  // x of the first tail level back to global memory
    const MgView<T, CT, T>& L = d.lv[0];
    const T* x = xs(0);
    for (int k = t; k < L.nx * L.ny; k += NTT) {
      const int ix = k % L.nx, iy = k / L.nx;
      L.x[(size_t)iy * L.pitch + ix] = x[(iy + 1) * W(0) + ix + 1];
    }
  }
}

}  // namespace

template <class T, class CT>
int tail_prepare(TailDesc<T, CT>& d) {
  // x and b per level; FP32 tails also stage di, dg, cE, cN
  const int arrays = std::is_same<T, float>::value ? 6 : 2;
  int off = 0;
  for (int l = 0; l < d.n; ++l) {
    d.off[l] = off;
    off += arrays * (d.lv[l].nx + 2) * (d.lv[l].ny + 2);
  }
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
  if (allow_max_smem(k_tail<T, CT>) != cudaSuccess) {
    (void)cudaGetLastError();
    return -1;
  }
  return 0;
}

template <class T, class CT>
void launch_tail(const TailDesc<T, CT>& d, Scalars* sc, cudaStream_t s) {
  launch_k(k_tail<T, CT>, dim3(1), dim3(1024), (size_t)d.smem, s, d, sc);
}

template int tail_prepare<double, double>(TailDesc<double, double>&);
template int tail_prepare<float, __nv_bfloat16>(TailDesc<float, __nv_bfloat16>&);
template void launch_tail<double, double>(const TailDesc<double, double>&, Scalars*,
                                          cudaStream_t);
template void launch_tail<float, __nv_bfloat16>(const TailDesc<float, __nv_bfloat16>&, Scalars*,
                                                cudaStream_t);

bool pdl_enabled() {
  static const bool on = getenv("SCF_NO_PDL") == nullptr;
  return on;
}

thread_local long long g_launches = 0;

static dim3 tiles(int nx, int ny, int tx = SX, int ty = SY) {
  return dim3((nx + tx - 1) / tx, (ny + ty - 1) / ty);
}
static dim3 small_grid(int nx, int ny) {
  int gy = (ny + 7) / 8;
  return dim3((nx + 31) / 32, gy < 1024 ? gy : 1024);
}
// grid-stride reductions: about 16 blocks of 256 threads per SM
static dim3 reduce_grid(int nx, int ny) {
  const int gx = (nx + 31) / 32;
  int gy = (ny + 7) / 8;
  const int cap = 2432 / gx > 1 ? 2432 / gx : 1;
  return dim3(gx, gy < cap ? gy : cap);
}

template <class T, class CT, class BT>
void launch_sweep(const MgView<T, CT, BT>& L, const MgView<T, CT, T>& C, int first, bool zero,
                  bool prolong, bool restrict_, bool rz, double omega, int flexible, Scalars* sc,
                  double* part, cudaStream_t s, int iters, int tile) {
  const T om = (T)omega;
#define SCF_SWEEP(F, Z, PR, RS, R)                                                              \
  do {                                                                                          \
    if (tile == 1) {                                                                            \
      const dim3 g = tiles(L.nx, L.ny, SX2, SY2);                                               \
      if (iters == 2)                                                                           \
        launch_k(k_sweep<T, CT, BT, F, Z, PR, RS, R, 2, SX2, SY2>, g, dim3(NT), 0, s, L, C, om, \
                 flexible, sc, part);                                                           \
      else                                                                                      \
        launch_k(k_sweep<T, CT, BT, F, Z, PR, RS, R, 1, SX2, SY2>, g, dim3(NT), 0, s, L, C, om, \
                 flexible, sc, part);                                                           \
    } else {                                                                                    \
      const dim3 g = tiles(L.nx, L.ny);                                                         \
      if (iters == 2)                                                                           \
        launch_k(k_sweep<T, CT, BT, F, Z, PR, RS, R, 2, SX, SY>, g, dim3(NT), 0, s, L, C, om,   \
                 flexible, sc, part);                                                           \
      else                                                                                      \
        launch_k(k_sweep<T, CT, BT, F, Z, PR, RS, R, 1, SX, SY>, g, dim3(NT), 0, s, L, C, om,   \
                 flexible, sc, part);                                                           \
    }                                                                                           \
  } while (0)
  // the combinations the V-cycle uses (pre: red first; post: black first)
  if (first == 0 && zero && !prolong && !restrict_ && !rz) SCF_SWEEP(0, true, false, false, false);
  else if (first == 0 && zero && !prolong && restrict_ && !rz) SCF_SWEEP(0, true, false, true, false);
  else if (first == 0 && !zero && !prolong && restrict_ && !rz) SCF_SWEEP(0, false, false, true, false);
  else if (first == 0 && !zero && !prolong && !restrict_ && !rz) SCF_SWEEP(0, false, false, false, false);
  else if (first == 1 && !zero && prolong && !restrict_ && !rz) SCF_SWEEP(1, false, true, false, false);
  else if (first == 1 && !zero && prolong && !restrict_ && rz) SCF_SWEEP(1, false, true, false, true);
  else if (first == 1 && !zero && !prolong && !restrict_ && !rz) SCF_SWEEP(1, false, false, false, false);
  else if (first == 1 && !zero && !prolong && !restrict_ && rz) SCF_SWEEP(1, false, false, false, true);
#undef SCF_SWEEP
}

template <class T, class CT, class BT>
void launch_coarse_solve_t(const MgView<T, CT, BT>& C, const double* Ainv, const int* cmap,
                           const int* nc, Scalars* sc, cudaStream_t s) {
  launch_k(k_coarse_solve_t<T, CT, BT>, dim3(1), dim3(64), 0, s, C, Ainv, cmap, nc, sc);
}

template <class T, class BT>
void launch_dot_rz_t(int nx, int ny, int pitch, const BT* r, const T* z, int flexible,
                     Scalars* sc, double* part, cudaStream_t s) {
  launch_k(k_dot_rz_t<T, BT>, reduce_grid(nx, ny), dim3(32, 8), 0, s, nx, ny, pitch, r, z,
           flexible, sc, part);
}

// Grid of the FP64-direction update + SpMV: 30-column bands times strips of
// 8 warps, each warp `rows` rows long, with `rows` chosen so that the grid is
// at most one wave of resident CTAs (a second, partly filled wave would
// double the kernel's time for a fraction of the work).
dim3 pupdate_grid(int nx, int ny, int* rows) {
  static int cap[16];  // resident CTAs per device (0 = unknown)
  int dev = 0;
  cudaGetDevice(&dev);
  int& c = cap[dev & 15];
  if (c == 0) {
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pupdate_spmv_t, 256, 0);
    c = sms * per > 0 ? sms * per : 1;
  }
  const int bands = (nx + 29) / 30;
  const int strips = c / bands > 1 ? c / bands : 1;
  int r = (ny + 8 * strips - 1) / (8 * strips);
  if (r < 4) r = 4;
  *rows = r;
  return dim3(bands, (ny + 8 * r - 1) / (8 * r));
}

template <>
void launch_pupdate_spmv_t<double>(LevelView L0, const double* z, const double* pold,
                                   double* pnew, double* q, Scalars* sc, double* part,
                                   cudaStream_t s) {
  int rows = 0;
  const dim3 g = pupdate_grid(L0.nx, L0.ny, &rows);
  launch_k(k_pupdate_spmv_t, g, dim3(32, 8), 0, s, L0, z, pold, pnew, q, sc, part, rows);
}
// FP32-direction grid: 32-column bands times row strips, about eight CTAs
// per SM in all (measured best on the 2048^2 and 4096^2 levels: fewer leave
// memory latency exposed, more make the last-block reduction longer), and at
// least eight rows per thread (small grids, many of which run side by side in
// a batch, would otherwise launch a block per eight rows)
dim3 pupdate_ff_grid(int nx, int ny) {
  static int sms[16];
  int dev = 0;
  cudaGetDevice(&dev);
  int& n = sms[dev & 15];
  if (n == 0) {
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  const int gx = (nx + 31) / 32;
  int gy = 8 * n / gx > 1 ? 8 * n / gx : 1;
  const int gmax = (ny + 63) / 64;
  if (gy > gmax) gy = gmax;
  return dim3(gx, gy);
}
template <>
void launch_pupdate_spmv_t<float>(LevelView L0, const float* z, const float* pold, float* pnew,
                                  double* q, Scalars* sc, double* part, cudaStream_t s) {
  launch_k(k_pupdate_spmv_ff, pupdate_ff_grid(L0.nx, L0.ny), dim3(32, 8), 0, s, L0, z, pold,
           pnew, q, sc, part);
}

void launch_inv_diag(const LevelView& L, double* di, cudaStream_t s) {
  launch_k(k_inv_diag, small_grid(L.nx, L.ny), dim3(32, 8), 0, s, L.nx, L.ny, L.pitch, (const double*)L.dg, di);
}

void launch_max_coupling(const LevelView& L, unsigned* out_bits, cudaStream_t s) {
  cudaMemsetAsync(out_bits, 0, sizeof(unsigned), s);
  launch_k(k_max_coupling, small_grid(L.nx, L.ny), dim3(32, 8), 0, s, L, out_bits);
}

void launch_to_mixed(const LevelView& F, const MgView<float, __nv_bfloat16, float>& M,
                     const unsigned* max_bits, float* cscale_out, cudaStream_t s) {
  launch_k(k_to_mixed, small_grid(F.nx, F.ny), dim3(32, 8), 0, s, F, M, max_bits, cscale_out);
}

int set_tma_fault(int cta, int spins) {
  if (cudaMemcpyToSymbol(g_tma_skip_cta, &cta, sizeof(int)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_tma_spins, &spins, sizeof(int)) != cudaSuccess)
    return -1;
  return 0;
}

void launch_sweep_tma(const MgView<float, __nv_bfloat16, float>& L,
                      const MgView<float, __nv_bfloat16, float>& C, const CUtensorMap* maps,
                      int xin, int first, bool zero, bool prolong, bool restrict_, bool rz,
                      double omega, int flexible, Scalars* sc, double* part, cudaStream_t s,
                      int iters) {
  const dim3 g = tiles(L.nx, L.ny);
  const float om = (float)omega;
#define SCF_TSWEEP(F, Z, PR, RS, R)                                                        \
  do {                                                                                     \
    if (iters == 2) {                                                                      \
      auto k = k_sweep_tma<F, Z, PR, RS, R, 2>;                                            \
      allow_max_smem(k);                                                                   \
      launch_k(k, g, dim3(NT), (size_t)kTmaSmem, s, L, C, om, flexible, sc, part, maps, xin); \
    } else {                                                                               \
      auto k = k_sweep_tma<F, Z, PR, RS, R, 1>;                                            \
      allow_max_smem(k);                                                                   \
      launch_k(k, g, dim3(NT), (size_t)kTmaSmem, s, L, C, om, flexible, sc, part, maps, xin); \
    }                                                                                      \
  } while (0)
  if (first == 0 && zero && !prolong && !restrict_ && !rz) SCF_TSWEEP(0, true, false, false, false);
  else if (first == 0 && zero && !prolong && restrict_ && !rz) SCF_TSWEEP(0, true, false, true, false);
  else if (first == 0 && !zero && !prolong && restrict_ && !rz) SCF_TSWEEP(0, false, false, true, false);
  else if (first == 0 && !zero && !prolong && !restrict_ && !rz) SCF_TSWEEP(0, false, false, false, false);
  else if (first == 1 && !zero && prolong && !restrict_ && !rz) SCF_TSWEEP(1, false, true, false, false);
  else if (first == 1 && !zero && prolong && !restrict_ && rz) SCF_TSWEEP(1, false, true, false, true);
  else if (first == 1 && !zero && !prolong && !restrict_ && !rz) SCF_TSWEEP(1, false, false, false, false);
  else if (first == 1 && !zero && !prolong && !restrict_ && rz) SCF_TSWEEP(1, false, false, false, true);
#undef SCF_TSWEEP
}

namespace {
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (EncodeTiledFn) nullptr;
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}
bool encode2d(CUtensorMap* m, const void* base, CUtensorMapDataType dt, int esize, int nx, int ny,
              int pitch) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  // base 16-byte aligned, row stride a multiple of 16 bytes; the box rows are
  // 80 x 4 and 80 x 2 bytes, multiples of 16
  if ((reinterpret_cast<uintptr_t>(base) & 15) || ((size_t)pitch * esize) % 16) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)nx, (cuuint64_t)ny};
  const cuuint64_t strides[1] = {(cuuint64_t)pitch * esize};
  const cuuint32_t box[2] = {(cuuint32_t)kSweepBoxX, (cuuint32_t)kSweepBoxY};
  const cuuint32_t es[2] = {1, 1};
  return fn(m, dt, 2, const_cast<void*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}
}  // namespace

bool make_sweep_maps(const MgView<float, __nv_bfloat16, float>& L, float* const xbuf[2],
                     const float* b, CUtensorMap* m) {
  const int nx = L.nx, ny = L.ny, P = L.pitch;
  return encode2d(&m[0], xbuf[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, nx, ny, P) &&
         encode2d(&m[1], xbuf[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, nx, ny, P) &&
         encode2d(&m[2], b, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, nx, ny, P) &&
         encode2d(&m[3], L.di, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, nx, ny, P) &&
         encode2d(&m[4], L.cE, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, nx, ny, P) &&
         encode2d(&m[5], L.cN, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, nx, ny, P);
}

#define SCF_INST(T, CT, BT)                                                                   \
  template void launch_sweep<T, CT, BT>(const MgView<T, CT, BT>&, const MgView<T, CT, T>&, int, \
                                        bool, bool, bool, bool, double, int, Scalars*, double*, \
                                        cudaStream_t, int, int);                                \
  template void launch_coarse_solve_t<T, CT, BT>(const MgView<T, CT, BT>&, const double*,      \
                                                 const int*, const int*, Scalars*, cudaStream_t);
SCF_INST(double, double, double)
SCF_INST(float, __nv_bfloat16, float)
#undef SCF_INST
template void launch_dot_rz_t<double, double>(int, int, int, const double*, const double*, int,
                                              Scalars*, double*, cudaStream_t);
template void launch_dot_rz_t<float, float>(int, int, int, const float*, const float*, int,
                                            Scalars*, double*, cudaStream_t);

}  // namespace scf
