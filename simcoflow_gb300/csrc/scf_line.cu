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
//
// A line is solved by one CTA.  Thread t owns M consecutive cells; the last
// of them is an interface cell, the first M-1 are interior.  Each thread
// eliminates its interior cells (Thomas algorithm with three right-hand
// sides: the data, a unit value on the left interface, a unit value on its
// own interface), which leaves one equation per thread that couples only
// the interfaces of threads t-1, t, t+1 -- the Schur complement, again a
// symmetric diagonally dominant tridiagonal system.  That system is solved
// by parallel cyclic reduction in shared memory, and every thread then
// recovers its interior cells from its two interface values.  The
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

// Relax the lines (rows) iy = 2*blockIdx.x + colour of level L.
// ZERO: the iterate is zero on entry (the first pass of a V-cycle level):
// the neighbouring rows are not read, and they are written as zero.
template <class T, class CT, int M, bool ZERO>
__global__ void __launch_bounds__(512, 1)
k_line(MgView<T, CT, T> L, int colour, const Scalars* sc) {
  pdl_wait();
  if (sc && sc->done) return;
  extern __shared__ __align__(16) unsigned char line_smem[];
  const int nth = blockDim.x, t = threadIdx.x;
  T* rD0 = reinterpret_cast<T*>(line_smem);  // responses of each thread's first interior cell
  T* rS0 = rD0 + nth;
  T* rT0 = rS0 + nth;
  T* pa = rT0 + nth;  // two PCR buffers of 4 arrays each
  const int iy = 2 * blockIdx.x + colour;
  if (iy >= L.ny) return;
  const int P = L.pitch, nx = L.nx;
  const size_t g0 = (size_t)iy * P;
  const float cs = L.csp ? __ldg(L.csp) : 1.0f;

  T a[M], d[M], c[M], r[M];
  unsigned actm = 0;  // bit k: cell k has an unknown
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const int ix = t * M + k;
    T dv = T(-1), aw = T(0), ce = T(0), rv = T(0);
    if (ix < nx) {
      const size_t g = g0 + ix;
      dv = L.dg[g];
      if (dv > T(0)) {
        aw = lcoef<CT, T>(L.cE, g - 1, cs);
        ce = lcoef<CT, T>(L.cE, g, cs);
        rv = L.b[g];
        if (!ZERO) {
          rv = fma(lcoef<CT, T>(L.cN, g, cs), L.x[g + P], rv);
          rv = fma(lcoef<CT, T>(L.cN, g - P, cs), L.x[g - P], rv);
        }
      }
    }
    const bool act = dv > T(0);
    actm |= act ? (1u << k) : 0u;
    a[k] = act ? -aw : T(0);
    c[k] = act ? -ce : T(0);
    d[k] = act ? dv : T(1);
    r[k] = act ? rv : T(0);
  }

  // interior cells 0..M-2: forward elimination with three right-hand sides
  // (data; -a[0] on cell 0 for the left interface; -c[M-2] on cell M-2 for
  // the own interface), then back substitution.  Afterwards
  //   x_k = D_k + S_k * I_{t-1} + T_k * I_t   (k < M-1).
  T cp[M], D[M], S[M], Tr[M];
  {
    T inv = T(1) / d[0];
    cp[0] = (M == 2) ? T(0) : c[0] * inv;
    D[0] = r[0] * inv;
    S[0] = -a[0] * inv;
    Tr[0] = (M == 2) ? -c[0] * inv : T(0);
#pragma unroll
    for (int k = 1; k < M - 1; ++k) {
      const T den = fma(-a[k], cp[k - 1], d[k]);
      inv = T(1) / den;
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
  rD0[t] = D[0];
  rS0[t] = S[0];
  rT0[t] = Tr[0];
  __syncthreads();
  // interface equation of thread t: couples I_{t-1}, I_t, I_{t+1}
  const T aI = a[M - 1], dI = d[M - 1], cI = c[M - 1], rI = r[M - 1];
  const bool last = t == nth - 1;
  const T Dn = last ? T(0) : rD0[t + 1], Sn = last ? T(0) : rS0[t + 1],
          Tn = last ? T(0) : rT0[t + 1];
  T ea = aI * S[M - 2];
  T eb = fma(cI, Sn, fma(aI, Tr[M - 2], dI));
  T ec = cI * Tn;
  T ed = fma(-cI, Dn, fma(-aI, D[M - 2], rI));
  // parallel cyclic reduction over the nth interface equations
  T* buf[2] = {pa, pa + 4 * nth};
  int cur = 0;
  buf[0][t] = ea;
  buf[0][nth + t] = eb;
  buf[0][2 * nth + t] = ec;
  buf[0][3 * nth + t] = ed;
  __syncthreads();
  for (int s = 1; s < nth; s <<= 1) {
    const T* A_ = buf[cur];
    const T* B_ = A_ + nth;
    const T* C_ = B_ + nth;
    const T* D_ = C_ + nth;
    T na = T(0), nb = B_[t], nc = T(0), nd = D_[t];
    if (t - s >= 0) {
      const T k1 = A_[t] / B_[t - s];
      na = -A_[t - s] * k1;
      nb = fma(-C_[t - s], k1, nb);
      nd = fma(-D_[t - s], k1, nd);
    }
    if (t + s < nth) {
      const T k2 = C_[t] / B_[t + s];
      nc = -C_[t + s] * k2;
      nb = fma(-A_[t + s], k2, nb);
      nd = fma(-D_[t + s], k2, nd);
    }
    T* W = buf[cur ^ 1];
    W[t] = na;
    W[nth + t] = nb;
    W[2 * nth + t] = nc;
    W[3 * nth + t] = nd;
    cur ^= 1;
    __syncthreads();
  }
  const T It = buf[cur][3 * nth + t] / buf[cur][nth + t];
  rD0[t] = It;  // rD0 is no longer read by anyone after the first barrier above
  __syncthreads();
  const T Il = t > 0 ? rD0[t - 1] : T(0);
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const int ix = t * M + k;
    if (ix >= nx) break;
    const T v = (k == M - 1) ? It : fma(S[k], Il, fma(Tr[k], It, D[k]));
    L.x[g0 + ix] = (actm >> k) & 1u ? v : T(0);
    if (ZERO && iy + 1 < L.ny) L.x[g0 + P + ix] = T(0);
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

// residual of level L summed 2x2 onto the right-hand side of level C
template <class T, class CT>
__global__ void __launch_bounds__(256)
k_resid_restrict_l(MgView<T, CT, T> L, MgView<T, CT, T> C, const Scalars* sc) {
  pdl_wait();
  if (sc && sc->done) return;
  const int I = blockIdx.x * 32 + threadIdx.x, J = blockIdx.y * 8 + threadIdx.y;
  if (I >= C.nx || J >= C.ny) return;
  const float cs = L.csp ? __ldg(L.csp) : 1.0f;
  const int P = L.pitch;
  T s = T(0);
#pragma unroll
  for (int dj = 0; dj < 2; ++dj)
#pragma unroll
    for (int dq = 0; dq < 2; ++dq) {
      const int gx = 2 * I + dq, gy = 2 * J + dj;
      if (gx >= L.nx || gy >= L.ny) continue;
      const size_t g = (size_t)gy * P + gx;
      const T dgv = L.dg[g];
      if (dgv < T(0)) continue;
      T rr = fma(-dgv, L.x[g], L.b[g]);
      rr = fma(lcoef<CT, T>(L.cE, g, cs), L.x[g + 1], rr);
      rr = fma(lcoef<CT, T>(L.cE, g - 1, cs), L.x[g - 1], rr);
      rr = fma(lcoef<CT, T>(L.cN, g, cs), L.x[g + P], rr);
      rr = fma(lcoef<CT, T>(L.cN, g - P, cs), L.x[g - P], rr);
      s += rr;
    }
  C.b[(size_t)J * C.pitch + I] = s;
}

// x += omega * x_coarse(parent) on cells with an unknown
template <class T, class CT>
__global__ void __launch_bounds__(256)
k_prolong_l(MgView<T, CT, T> L, const T* __restrict__ xc, int pc, T omega, const Scalars* sc) {
  pdl_wait();
  if (sc && sc->done) return;
  const int ix = blockIdx.x * 32 + threadIdx.x, iy = blockIdx.y * 8 + threadIdx.y;
  if (ix >= L.nx || iy >= L.ny) return;
  const size_t g = (size_t)iy * L.pitch + ix;
  if (L.di[g] > T(0)) L.x[g] = fma(omega, xc[(size_t)(iy >> 1) * pc + (ix >> 1)], L.x[g]);
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

}  // namespace

int line_threads(int len, int* chunk) {
  int m = len <= 4096 ? 8 : len <= 8192 ? 16 : len <= kLineMaxLen ? 32 : 0;
  if (!m) return 0;
  int th = (len + m - 1) / m;
  th = (th + 31) / 32 * 32;
  if (chunk) *chunk = m;
  return th;
}

template <class T, class CT>
void launch_line(const MgView<T, CT, T>& L, int colour, bool zero, const Scalars* sc,
                 cudaStream_t s) {
  int m = 0;
  const int th = line_threads(L.nx, &m);
  const dim3 g((L.ny - colour + 1) / 2);
  const size_t smem = (size_t)11 * th * sizeof(T);
  if (g.x == 0) return;
#define SCF_LINE(MM)                                                                           \
  do {                                                                                         \
    if (zero) {                                                                                \
      auto k = k_line<T, CT, MM, true>;                                                        \
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);         \
      launch_k(k, g, dim3(th), smem, s, L, colour, sc);                                        \
    } else {                                                                                   \
      auto k = k_line<T, CT, MM, false>;                                                       \
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);         \
      launch_k(k, g, dim3(th), smem, s, L, colour, sc);                                        \
    }                                                                                          \
  } while (0)
  if (m == 8) SCF_LINE(8);
  else if (m == 16) SCF_LINE(16);
  else SCF_LINE(32);
#undef SCF_LINE
}

template <class E>
void launch_transpose(const E* src, int nx, int ny, int ps, E* dst, int pd, const Scalars* sc,
                      cudaStream_t s) {
  const dim3 g((nx + 31) / 32, (ny + 31) / 32);
  launch_k(k_transpose<E>, g, dim3(32, 8), 0, s, src, nx, ny, ps, dst, pd, sc);
}

template <class T, class CT>
void launch_resid_restrict_l(const MgView<T, CT, T>& L, const MgView<T, CT, T>& C,
                             const Scalars* sc, cudaStream_t s) {
  const dim3 g((C.nx + 31) / 32, (C.ny + 7) / 8);
  launch_k(k_resid_restrict_l<T, CT>, g, dim3(32, 8), 0, s, L, C, sc);
}

template <class T, class CT>
void launch_prolong_l(const MgView<T, CT, T>& L, const T* xc, int pc, double omega,
                      const Scalars* sc, cudaStream_t s) {
  const dim3 g((L.nx + 31) / 32, (L.ny + 7) / 8);
  launch_k(k_prolong_l<T, CT>, g, dim3(32, 8), 0, s, L, xc, pc, (T)omega, sc);
}

void launch_aspect(const double* dx, const double* dy, size_t n, unsigned* out_bits,
                   cudaStream_t s) {
  k_aspect<<<304, 256, 0, s>>>(dx, dy, n, out_bits);
}

template void launch_line<double, double>(const MgView<double, double, double>&, int, bool,
                                          const Scalars*, cudaStream_t);
template void launch_line<float, __nv_bfloat16>(const MgView<float, __nv_bfloat16, float>&, int,
                                                bool, const Scalars*, cudaStream_t);
template void launch_transpose<double>(const double*, int, int, int, double*, int,
                                       const Scalars*, cudaStream_t);
template void launch_transpose<float>(const float*, int, int, int, float*, int, const Scalars*,
                                      cudaStream_t);
template void launch_transpose<__nv_bfloat16>(const __nv_bfloat16*, int, int, int,
                                              __nv_bfloat16*, int, const Scalars*, cudaStream_t);
template void launch_resid_restrict_l<double, double>(const MgView<double, double, double>&,
                                                      const MgView<double, double, double>&,
                                                      const Scalars*, cudaStream_t);
template void launch_resid_restrict_l<float, __nv_bfloat16>(
    const MgView<float, __nv_bfloat16, float>&, const MgView<float, __nv_bfloat16, float>&,
    const Scalars*, cudaStream_t);
template void launch_prolong_l<double, double>(const MgView<double, double, double>&,
                                               const double*, int, double, const Scalars*,
                                               cudaStream_t);
template void launch_prolong_l<float, __nv_bfloat16>(const MgView<float, __nv_bfloat16, float>&,
                                                     const float*, int, double, const Scalars*,
                                                     cudaStream_t);

}  // namespace scf
