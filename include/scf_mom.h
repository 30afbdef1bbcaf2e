/*
 * scf_mom.h -- C-ABI of the implicit solves of SIMCOFlow's momentum
 * predictor on one GB300, one velocity component per call.
 *
 * One scf_mom_solve replaces, for the component comp (0: u on the U cells,
 * 1: v on the V cells), the sequence of Predictor_UV
 * (src/PredictorUV_mod.f90:507-563):
 *   SetMatrix          (:622-768)  operator and Dp = dx dy / (aP - sum a)
 *   SetVectors         (:770-845)  right-hand side (convective flux, gravity
 *                                  for v, boundary terms)
 *   SetBasicSolver + HYPRE PCG/BoomerAMG (:507-513, :530-536, :588-620)
 *                                  replaced by FP64 BiCGStab with a diagonal
 *                                  or a multigrid (SCF_MOM_MG) preconditioner
 *                                  to rtol (the operator is not symmetric)
 *   DeltaGetValues     (:847-885)  solution scattered to the cells
 *   Pred += dt GradP / dx / dy     (:517-522, :540-545)
 *   Dp boundary copies (:552-562) and, for v, the open top of
 *   PredictorVelocityBoundaryCondition (:563, :2199-2213).
 * Arrays are Fortran ordered with the reference's bounds; by default host
 * memory (copied in and out on the handle's stream), device memory when the
 * handle was created with SCF_FLAG_DEVICE_PTRS (scf_proj.h).  Status codes
 * are those of scf_proj.h.  Cells with Posnu = -1 keep their input Dp.
 */
#ifndef SCF_MOM_H
#define SCF_MOM_H
#include <stdint.h>

#include "scf_proj.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct scf_mom_in {
  /* the component's grid and cells (UGrid/UCell or VGrid/VCell) */
  const double *dx, *dy;            /* (1:nx,1:ny) TGrid%dx, %dy */
  const int32_t *posnu;             /* (0:nx+1,0:ny+1) TCell%Posnu */
  const double *vof, *vofS;         /* (1:nx,1:ny) TCell%vof, %vofS */
  const double *WlLh, *delh;        /* (1:nx,1:ny) TCell%WlLh, %delh */
  const double *etaE, *etaN;        /* (0:nx+1,0:ny+1) TCell%EtaE, %EtaN */
  /* the component's slices of the predictor's face fluxes */
  const double *difEW, *edEW;       /* (1:nx+1,1:ny) DifFluxEW(:,:,c), EDFluxEW(:,:,c) */
  const double *difNS, *edNS;       /* (1:nx,1:ny+1) DifFluxNS(:,:,c), EDFluxNS(:,:,c) */
  const double *flux;               /* (1:nx,1:ny) FluxDiv(:,:,c) */
  const double *gradp;              /* (1:nx,1:ny) GradP(:,:,c) */
  const double *u, *v;              /* (0:nx+1,0:ny+1) TVar%u, TVar%v (boundary terms) */
  /* dt; BetaVis, nua, nuw (src/StateVariables.f90:26-28); nuref, Rey, Fr
   * (src/StateVariables.f90:12-13, :97-98) */
  double dt, beta_vis, nua, nuw, nuref, rey, fr;
} scf_mom_in;

typedef struct scf_mom scf_mom;

/* Multigrid preconditioner for the BiCGStab solve (creation flag): one FP64
 * V-cycle (red-black Gauss-Seidel, 2 + 2 sweeps, Galerkin aggregation
 * coarsening, coarse correction weighted 1.9, dense coarsest solve) on the
 * symmetric part of the operator per preconditioner application, on the
 * right, in place of the diagonal.
 * The reference preconditions these solves with BoomerAMG
 * (src/PredictorUV_mod.f90:588-620); the diagonal suffices where dx dy / dt
 * dominates the operator (high Reynolds numbers, small time steps), the
 * multigrid where diffusion does. */
#define SCF_MOM_MG 4

/* flags: SCF_FLAG_DEVICE_PTRS, SCF_MOM_MG, or 0 */
int scf_mom_create(scf_mom **h, int nx, int ny, int flags, int device);
void scf_mom_destroy(scf_mom *h);
/* stream for all work of the handle (cudaStream_t; NULL: the handle's own) */
int scf_mom_set_stream(scf_mom *h, void *stream);

/* The implicit step of component comp.  pred ((0:nx+1,0:ny+1), in/out) is
 * Pred%u or Pred%v: the solved cells and the gradient update are written,
 * other entries keep their values; Dp ((0:nx+1,0:ny+1), in/out) is PU%Dp or
 * PV%Dp.  The solve stops at ||b - A x|| <= rtol ||b|| (FP64 recursive
 * residual) or after maxit iterations (SCF_ERR_NOT_CONVERGED).  st may be
 * NULL (iters, status, bnorm, relres, ms_total, launches are filled). */
int scf_mom_solve(scf_mom *h, int comp, const scf_mom_in *in, double *pred, double *Dp,
                  double rtol, int maxit, scf_stats *st);

/* Diagnostics of the last solve: the operator in the reference's matr
 * layout ((1:nx,1:ny,5): S, W, P, E, N; zero where a neighbour has no
 * unknown and for cells without one) and the right-hand side rhm
 * ((1:nx,1:ny)), as host arrays. */
int scf_mom_get_system(scf_mom *h, double *matr, double *rhm);

#ifdef __cplusplus
}
#endif
#endif
