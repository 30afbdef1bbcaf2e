// scf_geom_gpu.cuh -- device-side cut-cell geometry (scf_geom.cu): inputs
// and outputs in the reference's Fortran layouts, all device pointers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace scf {

struct GeoIn {
  int nx, ny;
  const double *dx, *dy;                 // (1:nx,1:ny) PGrid
  const double *vofS, *phiS, *nxS, *nyS; // (1:nx,1:ny) PCell solid fields
  const double *vofS_u, *vofS_v;         // (1:nx,1:ny) UCell%vofS, VCell%vofS
};

struct GeoOut {
  const double *dx, *dy;                 // the grid again (wall lengths)
  double *aE, *aW, *aN, *aS;             // (0:nx+1,0:ny+1) E/W/N/SEdge_Area
  double *WlLh, *vofS, *nxS, *nyS;       // (1:nx,1:ny)
  double *vofS_u, *vofS_v;               // (1:nx,1:ny)
  int32_t *posnu_p, *posnu_u, *posnu_v;  // (0:nx+1,0:ny+1)
  int32_t *moex_u, *moex_v;              // (1:nx,1:ny)
};

size_t geometry_count_ints(int nx);  // size of the numbering scratch
int geometry_build(const GeoIn& in, const GeoOut& o, uint8_t* st0, uint8_t* st1, int* counts,
                   int* flag, int* flag_host, int icorprob, cudaStream_t s);

}  // namespace scf
