// scf_noalloc.cu -- scf_rhs_norm_noalloc: the right-hand side of the
// pressure equation and its 2-norm, computed without allocating anything.
//
// Who needs this: a caller that cannot call cudaMalloc at the point where it
// needs the right-hand side -- for example a Fortran time loop that owns all
// of its device memory through a fixed arena (OpenACC / CUDA Fortran data
// regions) and forbids hidden allocations, or code that must not trigger the
// device-wide synchronisation that cudaMalloc and cudaFree can imply while
// other streams are busy.  The regular path (scf_proj_create and friends)
// allocates its work space once per handle; this entry point needs no
// handle at all.
//
// The only scratch memory is the file-scope array g_rhs_scratch below:
// per-block partial sums of the norm reduction plus the ticket counter of the
// last-block combine.  It lives in the library's device image, so every GPU
// that loads the library holds it (about 33 KB) until the process exits.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdint>
#include <mutex>

#include "../../include/scf_proj.h"

namespace {

constexpr int kBX = 32, kBY = 8, kThreads = kBX * kBY;
// Grid shape used by the kernel: one thread per cell in x, rows strided so
// that at most kMaxRowBlocks block-rows run; the grid therefore has at most
// ceil(SCF_NOALLOC_MAX_SIDE/32) * kMaxRowBlocks blocks.
constexpr int kMaxRowBlocks = 8;
constexpr int kMaxBlocks = (SCF_NOALLOC_MAX_SIDE + kBX - 1) / kBX * kMaxRowBlocks;
constexpr int kTicketSlot = kMaxBlocks;  // the ticket lives after the partials

// The scratch: kMaxBlocks partial sums + one slot for the ticket counter.
static __device__ __align__(256) double g_rhs_scratch[kMaxBlocks + 32];

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

__device__ double block_sum(double v) {
  __shared__ double sm[kThreads / 32];
  __syncthreads();
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  if ((t & 31) == 0) sm[t >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (t == 0)
    for (int w = 0; w < kThreads / 32; ++w) s += sm[w];
  return s;
}

// SetPoissonVectors (src/ProjectionP_Mod.f90:313-317) per cell, written to
// rhs(1:nx,1:ny) (0 where Posnu = -1), and ||rhs||_2 through the scratch.
__global__ void k_rhs_norm_noalloc(int nx, int ny, const double* __restrict__ us,
                                   const double* __restrict__ vs, const double* __restrict__ aE,
                                   const double* __restrict__ aW, const double* __restrict__ aN,
                                   const double* __restrict__ aS, const double* __restrict__ dxp,
                                   const double* __restrict__ dyp, const double* __restrict__ nyS,
                                   const double* __restrict__ WlLh,
                                   const int32_t* __restrict__ posnu, double vb,
                                   double* __restrict__ rhs, double* __restrict__ bnorm,
                                   double* scratch) {
  const int ix = blockIdx.x * kBX + threadIdx.x;
  const size_t ld0 = (size_t)nx + 2;
  double acc = 0.0;
  if (ix < nx) {
    for (int iy = blockIdx.y * kBY + threadIdx.y; iy < ny; iy += gridDim.y * kBY) {
      const int i = ix + 1, j = iy + 1;
      const size_t k1 = (size_t)ix + (size_t)iy * nx;
      const size_t k0 = (size_t)i + (size_t)j * ld0;
      double b = 0.0;
      if (posnu[k0] != -1) {
        const double tx = mul(sub(mul(us[k0], aE[k0]), mul(us[k0 - 1], aW[k0])), dyp[k1]);
        const double ty = mul(sub(mul(vs[k0], aN[k0]), mul(vs[k0 - ld0], aS[k0])), dxp[k1]);
        b = add(sub(-tx, ty), mul(mul(vb, nyS[k1]), WlLh[k1]));
      }
      rhs[k1] = b;
      acc = fma(b, b, acc);
    }
  }
  // deterministic grid reduction: partials in the scratch, last block combines
  __shared__ bool last;
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  const unsigned nb = gridDim.x * gridDim.y;
  const unsigned bid = blockIdx.y * gridDim.x + blockIdx.x;
  unsigned* ticket = reinterpret_cast<unsigned*>(scratch + kTicketSlot);
  const double s = block_sum(acc);
  if (t == 0) {
    scratch[bid] = s;
    __threadfence();
    last = (atomicAdd(ticket, 1u) == nb - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double tot = 0.0;
  for (unsigned k = t; k < nb; k += kThreads) tot += __ldcg(&scratch[k]);
  tot = block_sum(tot);
  if (t == 0) {
    *bnorm = sqrt(tot);
    *ticket = 0u;
  }
}

// Device address of g_rhs_scratch per device.  Only a successful lookup is
// kept: a failed one (for example a first call made while its stream was
// being captured) leaves the slot empty and the next call tries again.
constexpr int kMaxDevices = 64;
std::atomic<double*> g_scratch_ptr[kMaxDevices];
std::mutex g_scratch_mu;

}  // namespace

extern "C" int scf_rhs_norm_noalloc(int nx, int ny, const double* ustar, const double* vstar,
                                    const double* aE, const double* aW, const double* aN,
                                    const double* aS, const double* dx, const double* dy,
                                    const double* nyS, const double* WlLh,
                                    const int32_t* posnu_p, double vb, double* rhs,
                                    double* bnorm, void* stream) {
  if (nx < 1 || ny < 1) return SCF_ERR_ARG;
  if (nx > SCF_NOALLOC_MAX_SIDE || ny > SCF_NOALLOC_MAX_SIDE) return SCF_ERR_ARG;
  if (!ustar || !vstar || !aE || !aW || !aN || !aS || !dx || !dy || !nyS || !WlLh || !posnu_p ||
      !rhs || !bnorm)
    return SCF_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SCF_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return SCF_ERR_ARG;
  // with the device current, until one lookup succeeds: the host-side name
  // of the array is only a stand-in, the kernel needs its device address
  double* scratch = g_scratch_ptr[dev].load(std::memory_order_acquire);
  if (!scratch) {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    scratch = g_scratch_ptr[dev].load(std::memory_order_relaxed);
    if (!scratch) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_rhs_scratch) != cudaSuccess || !p) return SCF_ERR_CUDA;
      scratch = static_cast<double*>(p);
      g_scratch_ptr[dev].store(scratch, std::memory_order_release);
    }
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the ticket must start at zero (a previous call that was cut short could
  // have left it set); memset does not allocate
  if (cudaMemsetAsync(scratch + kTicketSlot, 0, sizeof(double), s) != cudaSuccess)
    return SCF_ERR_CUDA;
  const int gx = (nx + kBX - 1) / kBX;
  int gy = (ny + kBY - 1) / kBY;
  if (gy > kMaxRowBlocks) gy = kMaxRowBlocks;
  k_rhs_norm_noalloc<<<dim3(gx, gy), dim3(kBX, kBY), 0, s>>>(
      nx, ny, ustar, vstar, aE, aW, aN, aS, dx, dy, nyS, WlLh, posnu_p, vb, rhs, bnorm, scratch);
  if (cudaGetLastError() != cudaSuccess) return SCF_ERR_CUDA;
  return SCF_OK;
}
