// scf_internal.cuh -- data layout and kernel interfaces shared by the CUDA
// translation units of libscf_proj.so.
//
// Padded level layout (all multigrid levels and PCG vectors):
//   element (ix,iy), 0-based interior cell, at base[iy*pitch + ix];
//   ix in [-1,nx] and iy in [-1,ny] are valid addresses (one ghost ring);
//   pitch = round_up(nx+2, 32), so every row starts 256-byte aligned for
//   FP64 and the ghost ix=-1 of row iy is the last padding column of row iy-1.
//   Ghosts and padding are zeroed once at allocation and never written, so
//   stencils read them without branches (their couplings are zero too).
// Cells without an unknown (Posnu = -1) carry dg = -1 and zero couplings.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace scf {

constexpr double kEpsi = 1.0e-3;  // src/StateVariables.f90:26
constexpr int kBX = 32;           // threads per block in x (2 cells each)
constexpr int kBY = 8;            // threads per block in y
constexpr int kThreads = kBX * kBY;
constexpr int kMaxCoarse = 64;    // largest coarsest level (dense inverse)

struct LevelView {
  int nx, ny, pitch;
  double* cE;  // coupling to east neighbour (>= 0)
  double* cN;  // coupling to north neighbour (>= 0)
  double* dg;  // diagonal, -1 for cells without an unknown
  double* ex;  // diagonal excess dg - sum of couplings, clamped at 0
  double* x;   // iterate / correction
  double* b;   // right-hand side
  // Fine level only (null on coarser levels).  The reference writes each
  // row's west and south entries from the row's own cell (PoCoef(i,j,2) *
  // WEdge_Area(i,j), PoCoef(i,j,1) * SEdge_Area(i,j)), not from the
  // neighbour's east / north entry; the two differ in rounding where the
  // density weight of an interface face is formed from either side, and by
  // more where the face apertures of the two cells were not averaged (the
  // first and last rows and columns).  wW / wS hold the row's own entries
  // (magnitudes, 0 where the row has none) and arow[iy] != 0 marks the rows
  // where some cell's entry differs from its neighbour's cE / cN.  The FP64
  // operator of the PCG (q = A p, the true residual) uses them; the
  // multigrid preconditioner uses the symmetric cE / cN.
  double* wW;
  double* wS;
  int* arow;
  // Fine level of a mixed-precision handle only (null otherwise): cE, cN and
  // max(dg, 0) each split into two floats, (hi, lo) with hi = fl32(c) and
  // lo = fl32(c - hi), so hi + lo carries c to a relative 2^-48.  The PCG's
  // q = A p with an FP32 direction p is summed from them on the FP32 pipe.
  float2* fE;
  float2* fN;
  float2* fD;
};

// Fortran-layout inputs of the assembly, right-hand side and correction.
struct FortranIn {
  int nx, ny;
  const double *dx, *dy, *dxU, *dyV;                 // (nx,ny)
  const double *vof, *phi, *vofS, *nyS, *WlLh;       // (nx,ny)
  const double *aE, *aW, *aN, *aS;                   // (nx+2,ny+2)
  const int32_t *posnu_p, *posnu_u, *posnu_v;        // (nx+2,ny+2)
  const int32_t *moex_u, *moex_v;                    // (nx,ny)
  const double *vofS_u, *vofS_v;                     // (nx,ny)
  const double *DpU, *DpV;                           // (nx+2,ny+2)
  double betaP, betaM;
  int wb, eb, sb, nb;
};

// Device-resident scalars of one PCG solve.
struct Scalars {
  double bnorm2, rr, rz, pq, alpha, beta, rtol2, res_true2, mres_max, rr_prev;
  double rz_cross;  // r_{k+1}.z_k of the flexible PCG, reduced by the x/r update
  int iter, maxit, done, status, nan;
  int pad[2];  // pad[0]: guard counter of the graph loop
  int anan;    // NaN or Inf met by the operator setup (kept until the next assembly)
  unsigned tickets[8];  // last-block counters, one per reduction site
  // set by the assembly: faces whose two rows' entries differ, and the
  // largest relative difference (float bits); kept until the next assembly
  int asym_faces;
  unsigned asym_max_bits;
};

enum Ticket { T_RHS = 0, T_RZ, T_PQ, T_RR, T_RES, T_MRES, T_DOT };

// PCG beta: plain beta = r_k.z_k / r_{k-1}.z_{k-1}; flexible (Polak-Ribiere)
// beta = (r_k.z_k - r_k.z_{k-1}) / r_{k-1}.z_{k-1}, where the cross term
// r_k.z_{k-1} was reduced by the previous iteration's x/r update
__device__ __forceinline__ void set_beta(Scalars* sc, double rz_new, int flexible) {
  if (sc->iter == 0) sc->beta = 0.0;
  else sc->beta = (flexible ? (rz_new - sc->rz_cross) : rz_new) / sc->rz;
  sc->rz = rz_new;
}

// status codes written by the device (mirror scf_proj.h)
constexpr int kOk = 0, kErrNaN = -3, kErrNotConverged = -4, kErrTimeout = -6;

__host__ __device__ inline size_t fo1(int nx, int i, int j) {  // (1:nx,1:ny)
  return (size_t)(i - 1) + (size_t)(j - 1) * (size_t)nx;
}
__host__ __device__ inline size_t fo0(int nx, int i, int j) {  // (0:nx+1,0:ny+1)
  return (size_t)i + (size_t)j * (size_t)(nx + 2);
}

inline int round_up(int a, int b) { return (a + b - 1) / b * b; }

// Programmatic dependent launch.  Kernels are launched with
// cudaLaunchAttributeProgrammaticStreamSerialization, so a kernel's CTAs may
// be scheduled while its predecessor in the stream (or graph) drains; every
// kernel first waits here for the predecessor's completion and memory
// flush, then signals that its own successor may start scheduling.  For a
// kernel launched without the attribute both calls are no-ops.
__device__ __forceinline__ void pdl_wait() {
  cudaGridDependencySynchronize();
  cudaTriggerProgrammaticLaunchCompletion();
}

// Format conversions and selections done on the integer pipe.  On GB300 a
// float <-> double conversion and an FP64 max issue on the FP64 pipe (about
// two per SM and clock, like an FP64 FMA); the kernels that are bound by that
// pipe use these bit-level equivalents instead.  Both conversions follow the
// IEEE-754 binary32/binary64 encodings; the rare operands outside the normal
// range (zero excepted) take the hardware conversion.

// The rare operands take the hardware conversion (or division) through an
// out-of-line call: the compiler then branches around it instead of
// predicating an FP64-pipe instruction into every use.
static __device__ __noinline__ double f2d_rare(float f) { return (double)f; }
static __device__ __noinline__ float d2f_rare(double d) { return (float)d; }
static __device__ __noinline__ double div_rare(double a, double b) { return __ddiv_rn(a, b); }

// exact widening float -> double
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if (e - 1u < 254u) {  // normal: rebias the exponent, widen the fraction
    const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u >> 3) & 0xfffffu);
    return __hiloint2double((int)hi, (int)(u << 29));
  }
  if ((u << 1) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);  // +-0
  return f2d_rare(f);  // subnormal, infinity, NaN
}

// double -> float, round to nearest even
__device__ __forceinline__ float d2f_rn(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned e = (hi >> 20) & 0x7ffu;
  // binary32 normal range before rounding: biased exponent 897 .. 1150
  if (e - 897u < 254u) {
    const unsigned sign = hi & 0x80000000u;
    const unsigned frac = ((hi & 0xfffffu) << 3) | (lo >> 29);  // top 23 fraction bits
    const unsigned rest = lo & 0x1fffffffu;                     // 29 bits dropped
    unsigned f = sign | ((e - 896u) << 23) | frac;
    // ties to even; a carry out of the fraction steps the exponent (up to inf)
    if (rest > 0x10000000u || (rest == 0x10000000u && (frac & 1u))) f += 1u;
    return __uint_as_float(f);
  }
  if (((hi << 1) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);  // +-0
  return d2f_rare(d);  // below or above the binary32 normal range, infinity, NaN
}

// c as hi + lo: hi = fl32(c), lo = fl32(c - hi) (the difference is exact in
// FP64), together within a relative 2^-48 of c (for lo in the binary32
// normal range)
__device__ __forceinline__ float2 split_ff(double c) {
  const float hi = d2f_rn(c);
  return make_float2(hi, d2f_rn(c - f2d_exact(hi)));
}

// (sh, sl) += -(a.x + a.y) * x in float-float arithmetic on the FP32 pipe:
// the product a.x * x exactly as s + e (an FMA gives the rounding error), s
// added to sh by Knuth's TwoSum (the rounding error of the sum recovered
// exactly), the errors and the small product a.y * x collected in sl.  Every
// operation is an explicit round-to-nearest intrinsic, so the compiler
// neither fuses nor reorders the error terms away.
__device__ __forceinline__ void ff_sub_prod(float2 a, float x, float& sh, float& sl) {
  const float s = __fmul_rn(-a.x, x);
  const float e = __fmaf_rn(-a.x, x, -s);
  const float t = __fadd_rn(sh, s);
  const float bv = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bv)), __fsub_rn(s, bv));
  sh = t;
  sl = __fmaf_rn(-a.y, x, __fadd_rn(sl, __fadd_rn(err, e)));
}

// max(v, 0) for a v that is not NaN, by the sign bit (-0 gives +0)
__device__ __forceinline__ double pos_part(double v) {
  return __double2hiint(v) < 0 ? 0.0 : v;
}

// Correctly rounded FP64 quotient a / b (IEEE round to nearest even), on the
// integer pipe: an FP64 division costs about ten instructions on GB300's slow
// FP64 pipe, this one a few dozen integer instructions and one FP32
// reciprocal approximation.  Method: Newton-Raphson iteration
// y <- y (2 - m y) for the reciprocal of b's significand m in [1, 2) in
// 64-bit fixed point (2^63 = 1), seeded by the FP32 reciprocal approximation
// of m truncated to 24 bits (relative error near 2^-22; the steps square it,
// and every truncation keeps y at or below 1/m); the 53-bit quotient of the
// significands from one high product; then the exact remainder corrects the
// last digit and gives the round-to-nearest-even bit, the closing step of long
// division (Knuth, TAOCP vol. 2, 4.3.1).  An exact midpoint cannot occur for
// a quotient of two 53-bit significands.  A power-of-two divisor gives the
// exact quotient by exponent arithmetic alone.  Zero, subnormal, infinite or
// NaN operands and results outside the normal range take the IEEE division.
__device__ __forceinline__ double div_rn(double a, double b) {
  using u64 = unsigned long long;
  const u64 ua = (u64)__double_as_longlong(a), ub = (u64)__double_as_longlong(b);
  const int ea = (int)((ua >> 52) & 0x7ff), eb = (int)((ub >> 52) & 0x7ff);
  const u64 ma = (ua & 0xfffffffffffffull) | (1ull << 52);
  const u64 mb = (ub & 0xfffffffffffffull) | (1ull << 52);
  const bool ge = ma >= mb;                 // quotient of the significands in [1, 2)
  const int E = ea - eb + 1022 + (int)ge;   // biased exponent of the result
  if ((unsigned)(ea - 1) >= 2046u || (unsigned)(eb - 1) >= 2046u || (unsigned)(E - 1) >= 2045u)
    return div_rare(a, b);
  // b a power of two (uniform grid spacings, unit densities): the quotient is
  // a's significand under the exponent E, exact
  if ((ub & 0xfffffffffffffull) == 0ull)
    return __longlong_as_double(
        (long long)(((ua ^ ub) & (1ull << 63)) | ((u64)E << 52) | (ua & 0xfffffffffffffull)));
  float y0;
  asm("rcp.approx.ftz.f32 %0, %1;"
      : "=f"(y0)
      : "f"(__uint_as_float(0x3f800000u | (unsigned)((ub >> 29) & 0x7fffffu))));
  const unsigned yb = __float_as_uint(y0);  // in [0.49, 1]: exponent field 125 .. 127
  u64 Y = (u64)(0x800000u | (yb & 0x7fffffu)) << (39 + (int)(yb >> 23) - 126);
  const u64 M = mb << 11;
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const u64 P = __umul64hi(M, Y);       // m y 2^62
    Y = __umul64hi(Y, (1ull << 63) - P) << 2;  // y (2 - m y) 2^63
  }
  u64 Q = __umul64hi(ma << 11, Y) >> (ge ? 10 : 9);  // the true digit string or one below
  u64 R = (ma << (ge ? 52 : 53)) - Q * mb;           // exact remainder, modulo 2^64
  if ((long long)R < 0) { Q -= 1; R += mb; }
  if (R >= mb) { Q += 1; R -= mb; }
  if (R >= mb) { Q += 1; R -= mb; }
  const u64 R2 = R << 1;
  Q += (u64)((R2 > mb) | ((R2 == mb) & (Q & 1ull)));
  // Q in [2^52, 2^53]: adding it to the exponent field carries 2^53 into it
  const u64 bits = ((ua ^ ub) & (1ull << 63)) | (((u64)(E - 1) << 52) + Q);
  return __longlong_as_double((long long)bits);
}

static __device__ __noinline__ double sqrt_rare(double x) { return __dsqrt_rn(x); }

// Correctly rounded FP64 square root (IEEE round to nearest even) on the
// integer pipe, for the same reason as div_rn.  Method: x = M 2^(2k) with M
// in [1, 4); Newton-Raphson iteration y <- y (3 - M y^2) / 2 for 1/sqrt(M)
// in 64-bit fixed point (2^63 = 1), seeded by the FP32 reciprocal square
// root approximation; the 53-bit root q ~ M y 2^52 of N = M 2^104 from one
// high product; then the exact remainder r = N - q^2 moves q to the floor of
// sqrt(N) and gives the rounding bit (round up when r > q: a square root is
// never exactly halfway between two doubles), the integer square root's
// closing step (Knuth, TAOCP vol. 2, 4.6.4; Muller et al., Handbook of
// Floating-Point Arithmetic, ch. 9).  Zero, negative, subnormal, infinite or
// NaN operands take the IEEE square root.
__device__ __forceinline__ double sqrt_rn(double x) {
  using u64 = unsigned long long;
  const u64 ux = (u64)__double_as_longlong(x);
  const int e = (int)(ux >> 52);  // the sign bit included: positive normal is 1 .. 2046
  if ((unsigned)(e - 1) >= 2046u) return sqrt_rare(x);
  const int E = e - 1023, odd = E & 1;
  const u64 m = (ux & 0xfffffffffffffull) | (1ull << 52);
  const u64 Mf = m << (10 + odd);  // M 2^62
  float y0;
  asm("rsqrt.approx.ftz.f32 %0, %1;"
      : "=f"(y0)
      : "f"(__uint_as_float((0x3f800000u + ((unsigned)odd << 23)) |
                            (unsigned)((ux >> 29) & 0x7fffffu))));
  const unsigned yb = __float_as_uint(y0);  // in (0.5, 1]: exponent field 126 or 127
  u64 Y = (u64)(0x800000u | (yb & 0x7fffffu)) << (39 + (int)(yb >> 23) - 126);  // y 2^63
#pragma unroll
  for (int it = 0; it < 3; ++it) {
    const u64 Z = __umul64hi(Mf, __umul64hi(Y, Y));  // M y^2 2^60
    Y = __umul64hi(Y, (3ull << 60) - Z) << 3;        // y (3 - M y^2) / 2 2^63
  }
  u64 q = __umul64hi(Mf, Y) >> 9;  // M y 2^52: the root, to a unit or two
  long long r = (long long)((m << (52 + odd)) - q * q);  // N - q^2 (small: low words suffice)
  if (r < 0) { q -= 1; r += (long long)(2 * q + 1); }
  if (r < 0) { q -= 1; r += (long long)(2 * q + 1); }
  if (r > (long long)(2 * q)) { r -= (long long)(2 * q + 1); q += 1; }
  if (r > (long long)(2 * q)) { r -= (long long)(2 * q + 1); q += 1; }
  q += (u64)(r > (long long)q);
  const int Er = (E >> 1) + 1023;  // floor(E / 2), biased
  return __longlong_as_double((long long)(((u64)(Er - 1) << 52) + q));
}

// PDL is on unless SCF_NO_PDL is set in the environment.
bool pdl_enabled();

// Kernel launches issued by this host thread (direct launches and launches
// recorded into a graph under capture); the solver reports per-call counts.
extern thread_local long long g_launches;
inline void note_launch() { ++g_launches; }

// Allow a kernel the device's whole opt-in dynamic shared memory.  The
// attribute belongs to the function, not to a launch: graphs of several
// handles capture launches of the same kernel with different sizes, so it
// must only ever be raised, never set to one handle's size.
template <typename F>
inline cudaError_t allow_max_smem(F* kernel) {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  // the kernel's own static shared memory counts against the same limit
  cudaFuncAttributes fa;
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(kernel));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(reinterpret_cast<const void*>(kernel),
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             optin - (int)fa.sharedSizeBytes);
  if (e != cudaSuccess) (void)cudaGetLastError();  // the launch reports what matters
  return e;
}

template <typename... KArgs, typename... Args>
inline void launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                     cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, args...);
  note_launch();
}

// launch geometry: 2 cells per thread in x, rows looped with a grid stride
inline dim3 grid_for(int nx, int ny, int cells_per_thread_x = 2) {
  int gx = (nx + kBX * cells_per_thread_x - 1) / (kBX * cells_per_thread_x);
  int gy_full = (ny + kBY - 1) / kBY;
  int cap = (152 * 16 + gx - 1) / gx;
  int gy = gy_full < cap ? gy_full : cap;
  if (gy < 1) gy = 1;
  return dim3(gx, gy);
}

// ---- kernel launchers (scf_kernels.cu) ----
void launch_assemble(const FortranIn& in, LevelView L0, Scalars* sc, cudaStream_t s);
void launch_divide(const double* a, const double* b, double* q, long long n, cudaStream_t s);
void launch_sqrt(const double* a, double* q, long long n, cudaStream_t s);
void launch_matr_out(const FortranIn& in, LevelView L0, double* matr, cudaStream_t s);
void launch_excess(LevelView L, double* di, unsigned* zero_bits, int nzero, Scalars* sc,
                   cudaStream_t s);
void launch_coarsen(LevelView F, LevelView C, double* di, cudaStream_t s);
void launch_coarse_setup(LevelView C, double* Ainv, int* cmap, int* nc, cudaStream_t s);
void launch_rhs(const FortranIn& in, const double* ustar, const double* vstar, double vb,
                LevelView L0, double* bvec, double* r, float* r32, double* x, Scalars* sc,
                double* part, double rtol, int maxit, cudaStream_t s);
void launch_rhs_given(int nx, int ny, const double* bF, LevelView L0, double* bvec, double* r,
                      float* r32, double* x, Scalars* sc, double* part, double rtol, int maxit,
                      cudaStream_t s);
void launch_update_xr(LevelView L0, double* x, const double* p, double* r, float* r32,
                      const float* z32, const double* q, Scalars* sc, double* part,
                      unsigned long long cond, cudaStream_t s);
void launch_update_xr(LevelView L0, double* x, const float* p, double* r, float* r32,
                      const float* z32, const double* q, Scalars* sc, double* part,
                      unsigned long long cond, cudaStream_t s);
void launch_final_solution(const FortranIn& in, LevelView L0, const double* x,
                           const double* bvec, const double* ustar, const double* vstar,
                           double* Pp, double* p, double* u, double* v, int correct,
                           Scalars* sc, double* part, cudaStream_t s);
void launch_final_mres(const FortranIn& in, double vb, double* u, double* v, double* mres,
                       Scalars* sc, double* part, cudaStream_t s);
void launch_final_zero(const FortranIn& in, double* p, double* u, double* v, cudaStream_t s);
void launch_to_fortran(LevelView L, const double* src, double* dst, cudaStream_t s);
void launch_from_fortran(LevelView L, const double* src, double* dst, cudaStream_t s);
void launch_to_fortran_f(LevelView L, const float* src, double* dst, cudaStream_t s);
void launch_from_fortran_f(LevelView L, const double* src, float* dst, cudaStream_t s);

}  // namespace scf
