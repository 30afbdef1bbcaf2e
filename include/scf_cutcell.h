/* scf_cutcell.h -- the per-time-step cut-cell geometry of SIMCOFlow for all
 * three cell families, computed on the GPU.
 *
 * Replaces, for the P, U and V cells:
 *   Grid_Preprocess   src/Cutcell_Mod.f90:18-32
 *     Cell_Geo_Cal (:34-300, with Edge_Geo_Cal :302-337) of each family,
 *     DefineMomentumExchangeCell (:360-397), NumberExternalCell (:340-358)
 *   NewCellFace       src/Cutcell_Mod.f90:399-549
 *     cell centroids of the U/V cells, CellLinking (:702-725), delh, WlLh,
 *     EastFaceInterpolationInf (:551-616), NorthFaceInterpolationInf (:618-700)
 * i.e. every geometry field that Solver_Mod recomputes each step
 * (src/Solver_Mod.f90:186-187, :303-304) from the solid level-set fields
 * Initial_Clsvof leaves in the cells.  Results are bit-identical to a literal
 * restatement of those routines (IEEE FP64, the reference's operation
 * order, no FMA contraction).
 *
 * Arrays are the reference's Fortran arrays (column-major):
 *   (nx,ny)        (1:Isize,1:Jsize)
 *   (nx+2,ny+2)    (0:Isize+1,0:Jsize+1)
 *   (nx,ny,2)      Cell_Cent, MsCe (1:Isize,1:Jsize,2)
 *   (nx+2,ny+2,2)  FCE, FCN (0:Isize+1,0:Jsize+1,2)
 * Family index: 0 = P (PGrid, PCell), 1 = U, 2 = V.  Host pointers, or
 * device pointers with SCF_CUTCELL_DEVICE_PTRS.
 *
 * Where the reference reads memory it never writes, this library uses:
 * ghost apertures 0 (the reference only writes zeros there, into fresh
 * allocations); Posnu -1 outside the numbering loops (U cells at i = nx, V
 * cells at j = ny); a solid (vofS = 1) neighbour when CellLinking would read
 * vofS outside the grid.  Arrays marked in/out keep their entry values
 * where the reference does not write them this step (MsCe of cells that are
 * not exchange cells; the rows / columns of the interpolation coefficients
 * outside the reference's loops), and AlN's entry values supply AlE(0,j) =
 * AlN(1,j) (:612), as in the reference.
 */
#ifndef SCF_CUTCELL_H
#define SCF_CUTCELL_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SCF_CUTCELL_DEVICE_PTRS 1

typedef struct scf_cell_grid {   /* TYPE(Grid) of one family: (nx,ny) */
  const double *dx, *dy, *x, *y;
} scf_cell_grid;

typedef struct scf_cell_solid {  /* solid level-set fields of one family: (nx,ny) */
  const double *vofS, *phiS, *nxS, *nyS;
} scf_cell_solid;

typedef struct scf_cell_geom {   /* results of one family; NULL: not wanted */
  double *vofS, *nxS, *nyS;          /* (nx,ny) after the solid / corner rules */
  double *aE, *aW, *aN, *aS;         /* (nx+2,ny+2) E/W/N/SEdge_Area */
  double *FCE, *FCN;                 /* (nx+2,ny+2,2) face centres */
  double *cent;                      /* (nx,ny,2) Cell_Cent */
  double *WlLh, *delh;               /* (nx,ny); delh: U and V only */
  int32_t *posnu;                    /* (nx+2,ny+2) */
  int32_t *moex;                     /* (nx,ny) MoExCell: U and V only */
  int32_t *msce;                     /* (nx,ny,2) MsCe, in/out: U and V only */
  double *SxE, *EtaE, *AlE, *DAlE;   /* (nx+2,ny+2) in/out: U and V only */
  double *SyN, *EtaN, *AlN, *DAlN;   /* (nx+2,ny+2) in/out: U and V only */
} scf_cell_geom;

/* Grid_Preprocess + NewCellFace.  grid[3], solid[3]: inputs per family;
 * geom[3]: outputs per family (P's U/V-only members are ignored).  icorprob:
 * the ICorProb corner rule of Cell_Geo_Cal (src/Main.f90:204).  ms, when not
 * NULL, receives the elapsed wall time.  Returns SCF_OK or an SCF_ERR_*
 * code of scf_proj.h. */
int scf_grid_preprocess(int nx, int ny, const scf_cell_grid grid[3],
                        const scf_cell_solid solid[3], scf_cell_geom geom[3], int icorprob,
                        int flags, int device, double *ms);

#ifdef __cplusplus
}
#endif
#endif
