// scf_clsvof.cu -- level-set transport of the CLSVOF sweeps (include/scf_clsvof.h):
// the level-set part of X_Sweep (src/Clsvof_Mod.f90:1074-1123) and Y_Sweep
// (:1191-1244).
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
// Compiled with -fmad=false: the operations and their order are the
// reference's, so results are bit-identical to the sequential loops.
#include <chrono>
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

template <int DIR>
__global__ void k_ls_sweep(LsIn in, double* temls) {
  const int nx = in.nx, ny = in.ny;
  const long long total = (long long)nx * ny;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i0 = (int)(idx % nx), j0 = (int)(idx / nx);  // 0-based cell
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
    const int n = L.n;
    const double dtv = in.dtv;
    double t = temls[idx];
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
    temls[idx] = t;
  }
}

}  // namespace
}  // namespace scf

using namespace scf;

extern "C" int scf_ls_sweep(int dir, int nx, int ny, const scf_ls_fields* f, double dtv,
                            double* temls, int flags, int device, double* ms) {
  if ((dir != SCF_LS_X && dir != SCF_LS_Y) || nx < 3 || ny < 3 || !f || !temls)
    return SCF_ERR_ARG;
  const double* arr[12] = {f->phi, f->vofS, f->dx, f->dy, f->x,  f->y,
                           f->aE,  f->aW,   f->aN, f->aS, f->ue, f->ve};
  for (auto a : arr)
    if (!a) return SCF_ERR_ARG;
  const auto t0 = std::chrono::steady_clock::now();
  if (cudaSetDevice(device) != cudaSuccess) return SCF_ERR_CUDA;
  const size_t n1 = (size_t)nx * ny, n0 = (size_t)(nx + 2) * (ny + 2);
  const size_t cnt[12] = {n1, n1, n1, n1, n1, n1, n0, n0, n0, n0, (size_t)(nx + 1) * ny,
                          (size_t)nx * (ny + 1)};
  const bool dev = (flags & SCF_LS_DEVICE_PTRS) != 0;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return SCF_ERR_CUDA;
  void* mem = nullptr;
  int rc = SCF_OK;
  const double* d[12];
  double* dt = temls;
  do {
    if (!dev) {
      size_t tot = n1;
      for (size_t c : cnt) tot += c;
      if (cudaMalloc(&mem, tot * 8) != cudaSuccess) {
        rc = SCF_ERR_NOMEM;
        break;
      }
      double* p = static_cast<double*>(mem);
      for (int a = 0; a < 12 && rc == SCF_OK; ++a) {
        if (cudaMemcpyAsync(p, arr[a], cnt[a] * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
          rc = SCF_ERR_CUDA;
        d[a] = p;
        p += cnt[a];
      }
      dt = p;
      if (rc == SCF_OK &&
          cudaMemcpyAsync(dt, temls, n1 * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
        rc = SCF_ERR_CUDA;
      if (rc) break;
    } else {
      for (int a = 0; a < 12; ++a) d[a] = arr[a];
    }
    const LsIn in{nx, ny, dtv, d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8], d[9],
                  d[10], d[11]};
    const unsigned blocks = (unsigned)((n1 + 255) / 256 < 152 * 8 ? (n1 + 255) / 256 : 152 * 8);
    if (dir == SCF_LS_X) k_ls_sweep<SCF_LS_X><<<blocks, 256, 0, s>>>(in, dt);
    else k_ls_sweep<SCF_LS_Y><<<blocks, 256, 0, s>>>(in, dt);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) {
      rc = SCF_ERR_CUDA;
      break;
    }
    if (!dev && cudaMemcpyAsync(temls, dt, n1 * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess)
      rc = SCF_ERR_CUDA;
  } while (false);
  if (cudaStreamSynchronize(s) != cudaSuccess && rc == SCF_OK) rc = SCF_ERR_CUDA;
  if (mem) cudaFree(mem);
  cudaStreamDestroy(s);
  if (ms)
    *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}
