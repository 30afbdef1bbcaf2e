// scf_mg.cuh -- multigrid level views and launchers shared by scf_mg.cu and
// the host side.
#pragma once
#include <cuda.h>

#include "scf_internal.cuh"

namespace scf {

// One multigrid level as the V-cycle kernels see it.
//   T   state type (x, b of coarse levels, diagonal, inverse diagonal)
//   CT  coupling type (double, or bf16 scaled by *csp)
//   BT  right-hand-side type (double on the fine level of the mixed path,
//       where b is the FP64 PCG residual itself)
template <class T, class CT, class BT>
struct MgView {
  int nx, ny, pitch;
  const CT* cE;
  const CT* cN;
  const T* dg;  // diagonal, negative where the cell has no unknown
  const T* di;  // inverse diagonal, 0 where the cell has no unknown
  T* x;         // iterate written by a sweep
  BT* b;
  const T* xin;  // iterate read by a sweep: the other buffer of the level's pair.
                 // A fused sweep reads its halo from neighbouring tiles, which
                 // other CTAs of the same kernel overwrite, so input and output
                 // must never alias.
  const float* csp;  // device pointer to the BF16 coupling scale (power of two);
                     // null for FP64 levels.  Kept in device memory so that a
                     // captured graph stays valid when the operator is reassembled.
};

// The coarse end of a V-cycle in one CTA (levels of at most kTailMaxCells
// cells, the last of them the coarsest).
constexpr int kTailMaxCells = 1024;
constexpr int kLineTailMaxCells32 = 4096;  // FP32 line tails (lines of at most 64 cells)
constexpr int kTailMaxLevels = 12;
template <class T, class CT>
struct TailDesc {
  int n;  // number of tail levels
  MgView<T, CT, T> lv[kTailMaxLevels];
  int off[kTailMaxLevels];  // shared-memory offset of each level's x (b, then di, dg, cE, cN in FP32)
  int total;                // elements of T in shared memory
  int bd_off, smem;         // byte offset of the coarse gather buffer, total bytes
  int npre, npost;
  // tail levels cfrom and coarser use cpre / cpost sweeps
  int cfrom, cpre, cpost;
  T omega;
  const double* Ainv;
  const int* cmap;
  const int* nc;
};
template <class T, class CT>
int tail_prepare(TailDesc<T, CT>& d);  // fills offsets and sizes; 0 on success
// the same for the line-smoother tail (scf_line.cu): per level x, b, cE, cN,
// dg in shared memory, plus two line-solve scratch arrays of the first level
template <class T, class CT>
int line_tail_prepare(TailDesc<T, CT>& d);
template <class T, class CT>
void launch_line_tail(const TailDesc<T, CT>& d, Scalars* sc, cudaStream_t s);
template <class T, class CT>
void launch_tail(const TailDesc<T, CT>& d, Scalars* sc, cudaStream_t s);

// TMA-staged sweep of FP32/BF16 levels.  Per level, six tensor maps live in
// device memory (64-byte aligned): the two iterate buffers, b, the inverse
// diagonal, cE, cN.  Dims (nx, ny), row stride = pitch, box kSweepBoxX x
// kSweepBoxY; cells outside the grid read as zero.
constexpr int kSweepBoxX = 80, kSweepBoxY = 42;  // 64x32 tile + 8 / 5 cells around
constexpr int kSweepMaps = 6;                    // x0, x1, b, di, cE, cN
// encodes the six maps into host memory; false when the CUDA driver has no tensor
// maps or refuses one
bool make_sweep_maps(const MgView<float, __nv_bfloat16, float>& L, float* const xbuf[2],
                     const float* b, CUtensorMap* maps);
// Fault injection for tests: in the TMA sweeps that reduce nothing across
// the grid, the CTA of linear index `cta` (-1: none) arms its barrier without
// issuing its copies, and every barrier wait polls at most `spins` times
// (default 1 << 20).  Device-wide; returns 0 or -1 (CUDA error).
int set_tma_fault(int cta, int spins);
void launch_sweep_tma(const MgView<float, __nv_bfloat16, float>& L,
                      const MgView<float, __nv_bfloat16, float>& C, const CUtensorMap* maps,
                      int xin, int first, bool zero, bool prolong, bool restrict_, bool rz,
                      double omega, int flexible, Scalars* sc, double* part, cudaStream_t s,
                      int iters);

// One fused launch of `iters` (1 or 2) red-black iterations on level L.
// tile 0: 64 x 32 cells per CTA; 1: 32 x 32 (see SCF_TILE_* in scf_proj.h).
template <class T, class CT, class BT>
void launch_sweep(const MgView<T, CT, BT>& L, const MgView<T, CT, T>& C, int first, bool zero,
                  bool prolong, bool restrict_, bool rz, double omega, int flexible, Scalars* sc,
                  double* part, cudaStream_t s, int iters = 1, int tile = 0);

template <class T, class CT, class BT>
void launch_coarse_solve_t(const MgView<T, CT, BT>& C, const double* Ainv, const int* cmap,
                           const int* nc, Scalars* sc, cudaStream_t s);

template <class T, class BT>
void launch_dot_rz_t(int nx, int ny, int pitch, const BT* r, const T* z, int flexible,
                     Scalars* sc, double* part, cudaStream_t s);

// grids of the direction update + SpMV kernels: FP64 direction (and rows
// per thread), FP32 direction
dim3 pupdate_grid(int nx, int ny, int* rows);
dim3 pupdate_ff_grid(int nx, int ny);
template <class ZT>
void launch_pupdate_spmv_t(LevelView L0, const ZT* z, const ZT* pold, ZT* pnew,
                           double* q, Scalars* sc, double* part, cudaStream_t s);

// Line relaxation (scf_line.cu).  Lines longer than kLineMaxLen cells are
// not supported by the line smoother.
constexpr int kLineMaxLen = 16384;
int line_threads(int len, int* chunk);  // CTA size for a line; 0 if too long
template <class T, class CT>
void launch_line(const MgView<T, CT, T>& L, int colour, bool zero, Scalars* sc, cudaStream_t s,
                 bool rz = false, int flexible = 0, double* part = nullptr);
template <class E>
void launch_transpose(const E* src, int nx, int ny, int ps, E* dst, int pd, const Scalars* sc,
                      cudaStream_t s);
// factored line relaxation (FP64 levels): factors of every line of a level
// (per cell: level-shaped padded arrays; per thread: thr[row][nth][slots])
template <class T>
struct LineFactors {
  T *inv, *ga, *cp, *S, *tr;
  T* thr;
  int nth;  // threads per line
};
constexpr int kLineThreadSlots = 23;  // 3 + 2 x 10 reduction steps
template <class T, class CT>
void launch_line_factor(const MgView<T, CT, T>& L, const LineFactors<T>& F, cudaStream_t s);
template <class T, class CT>
void launch_line_solve(const MgView<T, CT, T>& L, const LineFactors<T>& F, int colour, bool zero,
                       const Scalars* sc, cudaStream_t s);
// residual restriction and prolongation of the line V-cycle, both on the
// transposed copy Lt of a level; the restriction writes the coarse
// right-hand side in both layouts (C, Ct), the prolongation reads the
// natural coarse iterate C.x
template <class T, class CT>
void launch_resid_restrict_lt(const MgView<T, CT, T>& Lt, const MgView<T, CT, T>& C,
                              const MgView<T, CT, T>& Ct, const Scalars* sc, cudaStream_t s);
template <class T, class CT>
void launch_prolong_lt(const MgView<T, CT, T>& Lt, const MgView<T, CT, T>& C, double omega,
                       const Scalars* sc, cudaStream_t s);
void launch_aspect(const double* dx, const double* dy, size_t n, unsigned* out_bits,
                   cudaStream_t s);

void launch_inv_diag(const LevelView& L, double* di, cudaStream_t s);
void launch_max_coupling(const LevelView& L, unsigned* out_bits, cudaStream_t s);
void launch_to_mixed(const LevelView& F, const MgView<float, __nv_bfloat16, float>& M,
                     const unsigned* max_bits, float* cscale_out, cudaStream_t s);

}  // namespace scf
