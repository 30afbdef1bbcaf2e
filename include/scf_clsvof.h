/* scf_clsvof.h -- SIMCOFlow's CLSVOF sweeps on the GPU.
 *
 * Replaces X_Sweep (src/Clsvof_Mod.f90:989-1124) and Y_Sweep (:1126-1245)
 * after their call of Interface_Reconstruct:
 *  - the level-set part (:1074-1123, :1191-1244): face fluxes of phi
 *    (central averages inside, one-sided slope formulas on the first and
 *    last faces) and their update of temls;
 *  - the VOF part (:1004-1069, :1141-1189): the PLIC face fluxes of the
 *    upwind cell (frac for cells without solid, CellGeoCal for cut cells,
 *    the full/empty and solid shortcuts of topflux .. leftflux, :1416-1522),
 *    their update of temvf after its division by (1 - vofS), and the
 *    inflow through the first face (X: the wave inlet, Y: vof ve(0) dtv).
 * The reference applies each in one sequential loop over faces.  Each
 * cell's result here is the value that loop leaves, with the same
 * operations in the same order (IEEE FP64, no FMA contraction), so the
 * output is bit-identical to a literal restatement of those loops.
 * Interface_Reconstruct, which each sweep calls first, is
 * scf_interface_reconstruct below, Redistance scf_redistance, and the
 * whole Coupled_LS_VOF step with a fixed solid scf_clsvof_step.
 *
 * Arrays are the reference's Fortran arrays (column-major):
 *   (nx,ny)      phi, vofS, dx, dy, x, y, temls   (1:Isize,1:Jsize)
 *   (nx+2,ny+2)  aE, aW, aN, aS                   E/W/N/SEdge_Area (0:Isize+1,0:Jsize+1)
 *   (nx+1,ny)    ue                               ue(0:Isize,1:Jsize)
 *   (nx,ny+1)    ve                               ve(1:Isize,0:Jsize)
 *   (nx,ny)      vof, nx, ny, dis, nxs, nys, phiS, temvf
 * Host pointers, or device pointers with SCF_LS_DEVICE_PTRS.  The level-set
 * update needs nx, ny >= 3 (its boundary formulas read three cells).
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

typedef struct scf_vof_fields {
  const double *vof;            /* vfl = PCell%vof */
  const double *nx, *ny, *dis;  /* interface normal and distance of Interface_Reconstruct */
  const double *nxs, *nys;      /* PCell%nxs, PCell%nys */
  const double *phiS;           /* PCell%phiS */
} scf_vof_fields;

/* X_Sweep's wave inlet (src/Clsvof_Mod.f90:1057-1068): cells of column 1
 * whose bottom lies below Depthw + Amp0 sin(kw xwu - omew (NondiT + k dtv)),
 * xwu = x(1,1) - dx(1,1)/2, take in vof(1,j) ue(0,j) dtv through face 0.
 * The sine is evaluated on the host (libm), as by the reference. */
typedef struct scf_vof_wave {
  double amp0, kw, omew, depthw; /* Amp0, kw, omew, Depthw (src/Main.f90:156-166) */
  double nondit;                 /* NondiT */
  int k;                         /* the sub-step k of Coupled_LS_VOF */
} scf_vof_wave;

/* One whole sweep (X_Sweep or Y_Sweep after Interface_Reconstruct): the VOF
 * update of temvf (in/out, (nx,ny)) and, when temls is not NULL, the
 * level-set update of temls, in one kernel.  f->phi is read only with
 * temls.  wave is read by the X sweep only; NULL: no inflow through face 0
 * of X.  nx, ny >= 1 (>= 3 with temls). */
int scf_clsvof_sweep(int dir, int nx, int ny, const scf_ls_fields *f, const scf_vof_fields *v,
                     const scf_vof_wave *wave, double dtv, double *temvf, double *temls,
                     int flags, int device, double *ms);

/* Interface_Reconstruct (src/Clsvof_Mod.f90:1250-1321, UpdateNorVec = 1):
 * the PLIC interface of every cell from the liquid fraction vof, the level
 * set phi and the solid's vofS, nxs, nys, phiS -- the unit normal (nxv,
 * nyv) from Normal_Vector_Irre (:1710-1919) or the one-sided boundary
 * differences, and the line distance dis from distance (:1323-1369) for
 * two-phase cells or DistanceFluidCalculate's Ridders root (:1957-2155) for
 * cells cut by the solid; (0, 1) and the flat-interface distance elsewhere.
 * Bit-identical to the reference's sequential loop, including the values
 * its locals carry from one cell to the next (a boundary cell's missing
 * normal component, a failed bracket's distance).
 * Where the reference pauses for the operator, the library goes on as after
 * the operator's "go"; where it reads outside an array or a value never set
 * it takes a defined one (Vset(1,:) for a direction search whose cosines
 * are all NaN, 0 for a distance carried from before the first cell, an
 * empty liquid polygon when the non-solid polygon has no vertex).  Each such
 * event is counted in *events (may be NULL).  nx, ny >= 3. */
typedef struct scf_ir_fields {
  const double *vof, *vofS, *phi; /* PCell%vof, vofS, phi */
  const double *nxs, *nys, *phiS; /* PCell%nxs, nys, phiS */
  const double *x, *y, *dx, *dy;  /* PGrid */
} scf_ir_fields;

int scf_interface_reconstruct(int nx, int ny, const scf_ir_fields *f, double *nxv, double *nyv,
                              double *dis, int *events, int flags, int device, double *ms);

/* Redistance (src/Clsvof_Mod.f90:1525-1708): phi (in/out, (nx,ny)) rebuilt
 * as the signed distance to the PLIC interface (nx, ny, dis of
 * Interface_Reconstruct) within 4 cells of every interface cell, and
 * +-5 sqrt(dx^2 + dy^2) outside that band.  Bit-identical to the
 * reference's scatter over interface cells: each full or empty cell applies
 * its sources' updates in the reference's order.  *events (may be NULL)
 * counts the reference's two 'pause' checks that fire.  nx, ny >= 1. */
typedef struct scf_rd_fields {
  const double *vof, *vofS, *nxs, *nys, *phiS; /* PCell */
  const double *x, *y, *dx, *dy;              /* PGrid */
  const double *nx, *ny, *dis;                /* Interface_Reconstruct's output */
} scf_rd_fields;

int scf_redistance(int nx, int ny, const scf_rd_fields *f, double *phi, int *events, int flags,
                   int device, double *ms);

/* Coupled_LS_VOF (src/Clsvof_Mod.f90:730-959) with a fixed solid: six
 * sub-steps of dt/6, each an X_Sweep then a Y_Sweep (odd sub-steps) or the
 * reverse (even), every sweep after its Interface_Reconstruct, with the
 * reference's updates of vof and phi after each sweep and Boundary_Condition
 * between them; then Boundary_Condition, Interface_Reconstruct (nx, ny, dis
 * out: PCell%nx, PCell%ny and the distance) and Redistance of phi.
 * ObjectMovement and SolidVolumeFraction, which move the solid between
 * sub-steps, stay with the caller: the solid fields are held as given.
 * vof and phi are in/out.  wave: the X inlet (its k is ignored: each
 * sub-step uses its own), or NULL.  Bit-identical to the reference's loops.
 * *events (may be NULL) counts the reconstructions' and Redistance's
 * events (see above).  nx, ny >= 3. */
typedef struct scf_clsvof_fields {
  const double *vofS, *nxs, *nys, *phiS; /* PCell: the solid */
  const double *x, *y, *dx, *dy;         /* PGrid */
  const double *aE, *aW, *aN, *aS;       /* (nx+2,ny+2) apertures */
  const double *ue, *ve;                 /* the sweeps' face velocities */
} scf_clsvof_fields;

int scf_clsvof_step(int nx, int ny, const scf_clsvof_fields *f, const scf_vof_wave *wave,
                    double dt, double *vof, double *phi, double *nx_out, double *ny_out,
                    double *dis, int *events, int flags, int device, double *ms);

#ifdef __cplusplus
}
#endif
#endif
