// scf_mg.cuh -- multigrid level views and launchers shared by scf_mg.cu and
// the host side.
#pragma once
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
  T* x;
  BT* b;
  const float* csp;  // device pointer to the BF16 coupling scale (power of two);
                     // null for FP64 levels.  Kept in device memory so that a
                     // captured graph stays valid when the operator is reassembled.
};

template <class T, class CT, class BT>
void launch_sweep(const MgView<T, CT, BT>& L, const MgView<T, CT, T>& C, int first, bool zero,
                  bool prolong, bool restrict_, bool rz, double omega, const T* zold,
                  int flexible, Scalars* sc, double* part, cudaStream_t s);

template <class T, class CT, class BT>
void launch_coarse_solve_t(const MgView<T, CT, BT>& C, const double* Ainv, const int* cmap,
                           const int* nc, Scalars* sc, cudaStream_t s);

template <class T, class BT>
void launch_dot_rz_t(int nx, int ny, int pitch, const BT* r, const T* z, const T* zold,
                     int flexible, Scalars* sc, double* part, cudaStream_t s);

template <class ZT>
void launch_pupdate_spmv_t(LevelView L0, const ZT* z, const double* pold, double* pnew,
                           double* q, Scalars* sc, double* part, cudaStream_t s);

void launch_inv_diag(const LevelView& L, double* di, cudaStream_t s);
void launch_max_coupling(const LevelView& L, unsigned* out_bits, cudaStream_t s);
void launch_to_mixed(const LevelView& F, const MgView<float, __nv_bfloat16, float>& M,
                     const unsigned* max_bits, float* cscale_out, cudaStream_t s);

}  // namespace scf
