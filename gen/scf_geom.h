/*
 * scf_geom.h -- host-side builder of cut-cell geometry for synthetic
 * projection workloads (library libscf_geom.so).
 *
 * Replaces, for seeded synthetic cases, the CPU geometry pipeline that
 * SIMCOFlow runs before every projection:
 *   Initial_Grid, InitialUVGrid          src/Mesh_Mod.f90:54-175
 *   Initial_Clsvof (level sets, frac)    src/Clsvof_Mod.f90:39-400, 1371-1404
 *   Grid_Preprocess                      src/Cutcell_Mod.f90:18-32
 *     (Cell_Geo_Cal :34-300, Edge_Geo_Cal :302-337,
 *      NumberExternalCell :340-358, DefineMomentumExchangeCell :360-397)
 * All arrays use the reference's Fortran layouts (column-major, i fastest).
 * Any output pointer may be NULL.
 */
#ifndef SCF_GEOM_H
#define SCF_GEOM_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SCF_SOLID_CIRCLE 0
#define SCF_SOLID_BOX 1
#define SCF_SURF_MAXMODES 8

/* One solid body; the solid level set is the minimum of the bodies'
 * signed distances (positive in the fluid). */
typedef struct scf_solid {
    int kind;        /* SCF_SOLID_CIRCLE or SCF_SOLID_BOX */
    double cx, cy;   /* centre */
    double r;        /* circle radius */
    double hw, hh;   /* box half width and half height */
    double angle;    /* box rotation, radians counter-clockwise */
} scf_solid;

/* Free surface y = y0 + sum_m amp[m] sin(k[m] x + phase[m]); the liquid
 * (level set phi < 0) lies below it. */
typedef struct scf_surface {
    double y0;
    int nmodes;
    double amp[SCF_SURF_MAXMODES], k[SCF_SURF_MAXMODES], phase[SCF_SURF_MAXMODES];
} scf_surface;

typedef struct scf_geom_out {
    /* P-grid, (1:nx,1:ny): TYPE(Grid) x,y,dx,dy (src/Mesh_Mod.f90:11-15) */
    double *x, *y, *dx, *dy;
    double *dxU; /* UGrid%dx (1:nx,1:ny) */
    double *dyV; /* VGrid%dy (1:nx,1:ny) */
    /* P cells, (1:nx,1:ny): TYPE(Cell) vof, phi, vofS, phiS, nxS, nyS, WlLh */
    double *vof, *phi, *vofS, *phiS, *nxS, *nyS, *WlLh;
    /* P-cell apertures, (0:nx+1,0:ny+1): E/W/N/SEdge_Area */
    double *aE, *aW, *aN, *aS;
    int32_t *posnu_p;          /* PCell%Posnu (0:nx+1,0:ny+1) */
    int32_t *posnu_u, *posnu_v;/* UCell%Posnu, VCell%Posnu (0:nx+1,0:ny+1) */
    int32_t *moex_u, *moex_v;  /* UCell%MoExCell, VCell%MoExCell (1:nx,1:ny) */
    double *vofS_u, *vofS_v;   /* UCell%vofS, VCell%vofS (1:nx,1:ny) */
    /* the solid fields before Grid_Preprocess, as Initial_Clsvof leaves them
     * (the inputs of scf_proj_set_solid), (1:nx,1:ny) */
    double *vofS_in, *nxS_in, *nyS_in, *vofS_u_in, *vofS_v_in;
} scf_geom_out;

/* Face coordinates of one axis: npts = cells+1 values from s0 to s1,
 * uniform, or (nonuniform=1) with a uniform band [r0,r1] of nrec points and
 * geometric growth outside it, as Initial_Grid with NonUniformMesh=1
 * (src/Mesh_Mod.f90:67-125).  Returns 0 or -1 on bad arguments. */
int scf_geom_axis(int npts, double s0, double s1, int nonuniform, double r0, double r1,
                  int nrec, double *out);

/* Build the full geometry for an nx-by-ny P grid with face coordinates
 * xf[0..nx], yf[0..ny].  icorprob reproduces the ICorProb corner rule of
 * Cell_Geo_Cal (set .TRUE. in src/Main.f90:204).  Returns the number of
 * pressure unknowns (PCell%ExtCell+1), or -1 on bad arguments. */
int scf_geom_build(int nx, int ny, const double *xf, const double *yf, int nsolid,
                   const scf_solid *solids, const scf_surface *surf, int icorprob,
                   const scf_geom_out *out);

#ifdef __cplusplus
}
#endif
#endif
