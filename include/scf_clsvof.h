/* scf_clsvof.h -- level-set transport of SIMCOFlow's CLSVOF sweeps on the GPU.
 *
 * Replaces the level-set part of X_Sweep (src/Clsvof_Mod.f90:1074-1123) and
 * of Y_Sweep (:1191-1244): the face fluxes of the level set phi (central
 * averages inside, the one-sided slope formulas on the first and last
 * faces) and their update of temls, which the reference applies in one
 * sequential loop over faces.  Each cell's result here is the value that
 * loop leaves, with the same operations in the same order (IEEE FP64, no
 * FMA contraction), so the output is bit-identical to a literal restatement
 * of those loops.  The VOF part of the sweeps (PLIC face fluxes after
 * Interface_Reconstruct) and Redistance are not part of this library.
 *
 * Arrays are the reference's Fortran arrays (column-major):
 *   (nx,ny)      phi, vofS, dx, dy, x, y, temls   (1:Isize,1:Jsize)
 *   (nx+2,ny+2)  aE, aW, aN, aS                   E/W/N/SEdge_Area (0:Isize+1,0:Jsize+1)
 *   (nx+1,ny)    ue                               ue(0:Isize,1:Jsize)
 *   (nx,ny+1)    ve                               ve(1:Isize,0:Jsize)
 * Host pointers, or device pointers with SCF_LS_DEVICE_PTRS.  nx, ny >= 3
 * (the boundary formulas read three cells).
 */
#ifndef SCF_CLSVOF_H
#define SCF_CLSVOF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SCF_LS_DEVICE_PTRS 1
#define SCF_LS_X 0 /* X_Sweep */
#define SCF_LS_Y 1 /* Y_Sweep */

typedef struct scf_ls_fields {
  const double *phi, *vofS;      /* TCell%phi (phi), PCell%vofS */
  const double *dx, *dy, *x, *y; /* PGrid */
  const double *aE, *aW, *aN, *aS;
  const double *ue, *ve;
} scf_ls_fields;

/* One sweep's level-set update of temls (in/out, (nx,ny)) with time step
 * dtv.  ms, when not NULL, receives the elapsed wall time of the call. */
int scf_ls_sweep(int dir, int nx, int ny, const scf_ls_fields *f, double dtv, double *temls,
                 int flags, int device, double *ms);

#ifdef __cplusplus
}
#endif
#endif
