/*
 * scf_proj.h -- C-ABI of the GB300 pressure-projection library
 * (libscf_proj.so, CUDA kernels for sm_103a).
 *
 * Drop-in replacement for the projection step of SIMCOFlow:
 *   PoissonEquationSolver   src/ProjectionP_Mod.f90:26-99
 *   (ComputePossionMatrixCoefficient :395-580, SetBasicSolver :101-135,
 *    SetPoissonMatrix :137-273, SetPoissonVectors :275-354,
 *    HYPRE_ParCSRPCGSetup/Solve :57-58, DeltaPressureGetValues :356-393,
 *    DeltaPressureBoundaryCondition :582-595)
 *   UpdatePUV, projection part   src/ComputePUV_Mod.f90:56-218
 *    (velocity correction :59-152, pressure copy :163-169, top-row
 *     continuity :177-182, mass residual :184-217,
 *     VariablesInternalCellCondition :227-245)
 * The HYPRE IJ / ParCSR-PCG / BoomerAMG calls are replaced by a matrix-free
 * FP64 PCG preconditioned by a geometric multigrid V-cycle on the GPU.
 *
 * Arrays are passed exactly as the Fortran caller holds them: column-major,
 * i fastest, with the bounds given beside each argument:
 *   (nx,ny)     means (1:Isize,1:Jsize)
 *   (nx+2,ny+2) means (0:Isize+1,0:Jsize+1)
 * Pointers are host pointers unless the handle was created with
 * SCF_FLAG_DEVICE_PTRS, in which case every array argument is a device
 * pointer (cudaMalloc'd) on the handle's device.  With device pointers,
 * set_grid / set_geometry keep the pointers (no copy): the arrays must stay
 * alive and unchanged until the next set_* call.
 *
 * Threading: one handle per host thread; calls on one handle are not
 * re-entrant.  All work is ordered on the handle's CUDA stream; every call
 * returns after its results are on the host (host mode) or after its work
 * has been enqueued and completed (device mode).
 * Errors: every function returns SCF_OK (0) or a negative SCF_ERR_* code;
 * nothing aborts, exits or pauses (the reference pauses on NaN,
 * src/ProjectionP_Mod.f90:209-213, :322-325, :383-386).
 */
#ifndef SCF_PROJ_H
#define SCF_PROJ_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SCF_OK 0
#define SCF_ERR_ARG (-1)           /* bad argument or size */
#define SCF_ERR_CUDA (-2)          /* a CUDA call failed */
#define SCF_ERR_NAN (-3)           /* NaN or Inf in the operator, RHS or iterate */
#define SCF_ERR_NOT_CONVERGED (-4) /* maxit reached before rtol */
#define SCF_ERR_STALL (-5)         /* residual stopped decreasing */
#define SCF_ERR_TIMEOUT (-6)       /* a bounded device-side wait ran out */
#define SCF_ERR_STATE (-7)         /* call order: e.g. solve before assemble */
#define SCF_ERR_NOMEM (-8)         /* device allocation failed */
#define SCF_ERR_IO (-9)            /* a file could not be opened or written */

#define SCF_PREC_FP64 0  /* FP64 MG preconditioner inside FP64 PCG */
#define SCF_PREC_MIXED 1 /* FP32 MG with BF16 couplings inside FP64 flexible PCG */

#define SCF_FLAG_DEVICE_PTRS 1 /* array arguments are device pointers */
#define SCF_FLAG_NO_GRAPH 2    /* launch kernels one by one, no CUDA graph */

/* Multigrid smoother.  POINT: red-black Gauss-Seidel.  LINE: alternating
 * zebra line Gauss-Seidel (exact tridiagonal solves along x, then along y),
 * robust on stretched grids; lines of at most 16384 cells.  AUTO: LINE when
 * some cell's aspect ratio max(dx/dy, dy/dx) exceeds 2, else POINT.
 * BoomerAMG, which this replaces (src/ProjectionP_Mod.f90:116-133), adapts
 * to anisotropy through its strength-of-connection coarsening. */
/* Preconditioner of the flexible PCG.  MG: the multigrid V-cycle.  LEARNED
 * (mixed precision only): the U-Net of scf_unet.h, given by
 * scf_proj_set_network, for as long as each of its iterations reduces the
 * residual norm by at least the factor 0.6; from the first iteration that
 * does not, the V-cycle for the rest of the solve (stats.fallbacks = 1).
 * The FP64 residual decides convergence either way. */
#define SCF_PRECOND_MG 0
#define SCF_PRECOND_LEARNED 1

#define SCF_SMOOTH_AUTO 0
#define SCF_SMOOTH_POINT 1
#define SCF_SMOOTH_LINE 2

typedef struct scf_opts {
    int precision;   /* SCF_PREC_FP64 or SCF_PREC_MIXED */
    int flags;       /* SCF_FLAG_* */
    int device;      /* CUDA device ordinal */
    int maxit;       /* outer PCG iterations (reference: 50, :108) */
    double rtol;     /* stop at ||b-Ax||_2 <= rtol ||b||_2 (reference: 1e-20, :111) */
    int npre, npost; /* sweeps before / after the coarse correction: red-black
                        Gauss-Seidel iterations (point smoother); line smoother: a step
                        of x-lines then y-lines counts as two */
    double omega;    /* scale of the coarse-grid correction */
    int coarse_max;  /* coarsest level has at most this many cells (<= 64) */
    int smoother;    /* SCF_SMOOTH_AUTO (default), SCF_SMOOTH_POINT or SCF_SMOOTH_LINE */
    int precond;     /* SCF_PRECOND_MG (default) or SCF_PRECOND_LEARNED */
    int coarse_sweeps; /* sweeps before / after the coarse correction on level
                          coarse_from (0: the finest) and every coarser level (as
                          npre / npost count them); 0 (default): npre / npost there too */
    int coarse_from;
    int reserved[4];
} scf_opts;

typedef struct scf_stats {
    int iters;          /* outer PCG iterations taken */
    int status;         /* SCF_OK or SCF_ERR_NOT_CONVERGED / _NAN / _STALL */
    int levels;         /* multigrid levels */
    int fallbacks;      /* preconditioner fallbacks taken */
    double bnorm;       /* ||b||_2 */
    double relres;      /* recursive ||r||_2/||b||_2 at exit */
    double relres_true; /* FP64 recomputed ||b - A x||_2/||b||_2 */
    double mres_max;    /* max |mres| over cells with Posnu /= -1 (update_puv) */
    double ms_h2d, ms_assemble, ms_solve, ms_correct, ms_d2h, ms_total;
    int smoother;       /* SCF_SMOOTH_POINT or SCF_SMOOTH_LINE: the smoother used */
    int learned_iters;  /* iterations preconditioned by the network (SCF_PRECOND_LEARNED) */
    int launches;       /* kernel launches of this call, graph nodes counted per
                           execution, including those of the assembly before it */
    int asym_faces;     /* faces whose two rows carry different entries (the
                           reference forms a row's W/S entries from the row's
                           own cell, src/ProjectionP_Mod.f90:176-195); the
                           solve applies those rows exactly */
} scf_stats;

typedef struct scf_proj scf_proj;

/* Network of SCF_PRECOND_LEARNED: params is a host array of
 * scf_unet_num_params() floats in the order of scf_unet.h.  The handle keeps
 * its own device copy.  No reference counterpart (the reference
 * preconditions with BoomerAMG, src/ProjectionP_Mod.f90:116-133). */
int scf_proj_set_network(struct scf_proj *h, const float *params, int nparams);

/* Solve A x = b with the assembled operator for an arbitrary right-hand
 * side b ((nx,ny), zero on cells without an unknown), at most maxit
 * iterations (0 <= maxit <= opts.maxit; 0 gives x = 0).  x and, when not
 * null, the final recursive residual r are (nx,ny) outputs.  Returns
 * SCF_ERR_NOT_CONVERGED when maxit ran out before opts.rtol, with x and r
 * written.  This is the same PCG as PoissonEquationSolver's (without the
 * HYPRE vector setup of src/ProjectionP_Mod.f90:275-354); it generates the
 * residual/error pairs that train the learned preconditioner. */
int scf_proj_solve_rhs(struct scf_proj *h, const double *b, double *x, double *r, int maxit,
                       struct scf_stats *st);

/* Change the V-cycle schedule of an existing handle (sweeps before / after
 * the coarse correction, correction scale); rebuilds its graph.  Used by the
 * autotuner. */
int scf_proj_set_opts(struct scf_proj *h, int npre, int npost, double omega);

/* Sweeps (1..8, counted as npre / npost count them: red-black iterations of
 * the point smoother, two per alternating step of the line smoother) before
 * and after the coarse correction on level coarse_from (0: the finest) and
 * every coarser level, 0 for npre / npost there too; rebuilds the graph.
 * The coarse levels are latency-bound, so more smoothing there can cost less
 * than the PCG iterations it saves.  Used by the autotuner. */
int scf_proj_set_coarse_sweeps(struct scf_proj *h, int coarse_from, int sweeps);

/* Sweep tile of the red-black (point) smoother on an existing handle;
 * rebuilds its graph.  SCF_TILE_64X32 (default): 64 x 32 cells per CTA, the
 * larger FP32 levels staged by TMA; SCF_TILE_32X32: 32 x 32 cells per CTA,
 * plain loads on every level (twice the CTAs, for small grids).  Both give
 * the same V-cycle bit for bit (the PCG's r.z, summed per tile, differs in
 * the last bits); the autotuner picks by time.  No effect on
 * the line smoother.  No counterpart in the reference. */
#define SCF_TILE_64X32 0
#define SCF_TILE_32X32 1
int scf_proj_set_tile(struct scf_proj *h, int tile);

/* Batched projections: many independent, assembled handles (device-pointer
 * mode, one device, MG preconditioner, graphs on) solved by ONE graph
 * launch.  Each instance is an independent branch of the graph: operator
 * setup, right-hand side, the PCG loop as a conditional WHILE node, the
 * correction (as scf_proj_update_puv) and its scalars.  The arrays given to
 * scf_batch_set_io are baked into the graph; setting them again rebuilds it.
 * stats: one entry per instance; ms_total is the whole batch.  Returns the
 * first non-OK instance status.  The reference has no batched path: it
 * solves one projection per HYPRE call (src/ProjectionP_Mod.f90:21-99). */
typedef struct scf_batch scf_batch;
int scf_batch_create(scf_batch **b, struct scf_proj *const *handles, int count);
int scf_batch_set_io(scf_batch *b, int i, const double *ustar, const double *vstar, double vb,
                     double *Pp, double *p, double *u, double *v, double *mres);
int scf_batch_run(scf_batch *b, void *stream, struct scf_stats *stats);
int scf_batch_destroy(scf_batch *b);

/* Fill opts with defaults: FP64, host pointers, device 0, maxit 200,
 * rtol 1e-8, 2 pre / 2 post sweeps, omega 1.9, coarse_max 64. */
void scf_opts_default(scf_opts *opts);

/* Create a solver for an nx-by-ny pressure grid (Isize, Jsize).  Allocates
 * all device memory for the operator, the multigrid hierarchy and the PCG
 * vectors once; the handle is reused across time steps (the reference
 * rebuilds its HYPRE objects on every call, src/ProjectionP_Mod.f90:52-69). */
int scf_proj_create(scf_proj **h, int nx, int ny, const scf_opts *opts);
int scf_proj_destroy(scf_proj *h);

/* Use the given cudaStream_t (passed as void*) for all later work. */
int scf_proj_set_stream(scf_proj *h, void *stream);

/* Grid spacings: PGrid%dx, PGrid%dy, UGrid%dx, VGrid%dy, each (nx,ny)
 * (TYPE(Grid), src/Mesh_Mod.f90:11-15). */
int scf_proj_set_grid(scf_proj *h, const double *dx, const double *dy, const double *dxU,
                      const double *dyV);

/* Cut-cell and interface geometry (TYPE(Cell), src/Mesh_Mod.f90:17-41):
 *   vof, phi, vofS, nyS, WlLh         PCell fields, (nx,ny)
 *   aE, aW, aN, aS                    PCell%E/W/N/SEdge_Area, (nx+2,ny+2)
 *   posnu_p                           PCell%Posnu, (nx+2,ny+2)
 *   posnu_u, posnu_v                  UCell%Posnu, VCell%Posnu, (nx+2,ny+2)
 *   moex_u, moex_v                    UCell%MoExCell, VCell%MoExCell, (nx,ny)
 *   vofS_u, vofS_v                    UCell%vofS, VCell%vofS, (nx,ny)
 * Host mode: the six U/V arrays are read only by the velocity correction, so
 * their copies are made by the next scf_proj_poisson_solve / update_puv
 * while its PCG runs; those six host arrays must stay unchanged until that
 * call returns (the others may be reused once this call returns). */
int scf_proj_set_geometry(scf_proj *h, const double *vof, const double *phi,
                          const double *vofS, const double *nyS, const double *WlLh,
                          const double *aE, const double *aW, const double *aN,
                          const double *aS, const int32_t *posnu_p, const int32_t *posnu_u,
                          const int32_t *moex_u, const double *vofS_u,
                          const int32_t *posnu_v, const int32_t *moex_v,
                          const double *vofS_v);

/* Assemble the variable-density cut-cell operator and set up the multigrid
 * hierarchy.  Replaces ComputePossionMatrixCoefficient + SetPoissonMatrix +
 * HYPRE_ParCSRPCGSetup (src/ProjectionP_Mod.f90:50-57).
 *   DpU, DpV   PU%Dp, PV%Dp, (nx+2,ny+2) (src/PredictorUV_mod.f90:700)
 *   betaP, betaM  1/(row/Roref), 1/(roa/Roref) (src/ComputePUV_Mod.f90:42-43)
 *   wb, eb, sb, nb  1 = Neumann, 0 = Dirichlet (the reference passes 1,1,1,0)
 * Asynchronous on the handle's stream: it returns once DpU/DpV are copied
 * (host mode) and leaves the setup running; a NaN, Inf or invalid cell class
 * met by the setup is reported by the next solve as SCF_ERR_NAN. */
int scf_proj_assemble(scf_proj *h, const double *DpU, const double *DpV, double betaP,
                      double betaM, int wb, int eb, int sb, int nb);

/* PoissonEquationSolver: right-hand side from the predicted velocities
 * ustar = Pred%u, vstar = Pred%v (nx+2,ny+2) and the body velocity vb,
 * then the PCG solve, then Pp = Proj%Pp (nx+2,ny+2) with the ghost
 * conditions of DeltaPressureBoundaryCondition.  st may be NULL. */
int scf_proj_poisson_solve(scf_proj *h, const double *ustar, const double *vstar, double vb,
                           double *Pp, scf_stats *st);

/* The projection part of UpdatePUV (src/ComputePUV_Mod.f90:56-218):
 * poisson_solve, then the pressure-gradient correction of the faces,
 * p = Pp on cells with an unknown, top-row continuity, the mass residual
 * and the zeroing of solid cells.
 *   u, v, p  TVar%u, TVar%v, TVar%p (nx+2,ny+2): in = old values (faces that
 *            the reference does not correct keep them), out = new values
 *   mres     TVar%mres (nx,ny), out
 *   Pp       Proj%Pp (nx+2,ny+2), out; may be NULL */
int scf_proj_update_puv(scf_proj *h, const double *ustar, const double *vstar, double vb,
                        double *Pp, double *p, double *u, double *v, double *mres,
                        scf_stats *st);

/* The cut-cell geometry computed on the GPU, in place of
 * scf_proj_set_geometry: what Grid_Preprocess derives every time step from
 * the cells' solid level-set fields (src/Cutcell_Mod.f90:18-397: Cell_Geo_Cal
 * with Edge_Geo_Cal for the pressure cells, the U/V clamps,
 * DefineMomentumExchangeCell, NumberExternalCell), so that only those fields
 * cross to the GPU.  Inputs (same memory kind as the handle's other arrays):
 *   vof, phi        PCell%vof, %phi (nx,ny) from the free-surface step
 *   vofS, phiS,     PCell%VofS, %PhiS, %nxS, %nyS (nx,ny) as Initial_Clsvof
 *   nxS, nyS        leaves them for the body
 *   vofS_u, vofS_v  UCell%VofS, VCell%VofS (nx,ny)
 *   icorprob        the ICorProb corner rule of Cell_Geo_Cal (src/Main.f90:204)
 * The handle keeps the result (apertures, WlLh, VofS after the solid and
 * degenerate-cell rules, nxS/nyS after the corner rule, Posnu of the three
 * families, MoExCell, clamped U/V solid fractions) on the GPU; it is
 * bit-identical to the CPU restatement.  Needs scf_proj_set_grid first. */
int scf_proj_set_solid(scf_proj *h, const double *vof, const double *phi, const double *vofS,
                       const double *phiS, const double *nxS, const double *nyS,
                       const double *vofS_u, const double *vofS_v, int icorprob);

/* The geometry the handle holds (from scf_proj_set_geometry or
 * scf_proj_set_solid) as host arrays in the layouts of scf_proj_set_geometry;
 * nxS is available after scf_proj_set_solid only.  Any pointer may be NULL. */
int scf_proj_get_geometry(scf_proj *h, double *vofS, double *nxS, double *nyS, double *WlLh,
                          double *aE, double *aW, double *aN, double *aS, int32_t *posnu_p,
                          int32_t *posnu_u, int32_t *posnu_v, int32_t *moex_u,
                          int32_t *moex_v, double *vofS_u, double *vofS_v);

/* Diagnostics: the east / north entries and the diagonal of the assembled
 * rows in Fortran (nx,ny) layout (the full rows: scf_proj_get_matrix).
 * cE(i,j) = -A(row(i,j), row(i+1,j)), cN(i,j) = -A(row(i,j), row(i,j+1)),
 * diag(i,j) = A(row(i,j), row(i,j)) (-1 where Posnu = -1); rhs (nx,ny) is
 * the last right-hand side (0 where Posnu = -1).  Any pointer may be NULL;
 * always host pointers. */
int scf_proj_get_operator(scf_proj *h, double *cE, double *cN, double *diag, double *rhs);

/* The assembled matrix as the reference's dense copy matr(Isize,Jsize,5)
 * of SetPoissonMatrix (src/ProjectionP_Mod.f90:176-230, written at :183,
 * :193, :228, :240, :250): per cell the S, W, diagonal, E and N entries of
 * its row, off-diagonals negated, 0 where the row has no entry and on cells
 * with Posnu = -1.  Each row's W and S entries are the row's own
 * (PoCoef(i,j,2)*WEdge_Area(i,j), PoCoef(i,j,1)*SEdge_Area(i,j)), which may
 * differ from the neighbouring row's E / N entry: in the last bits where an
 * interface face's density weight is formed from either side
 * (:415-418 against :493-498), and by more on the first and last rows and
 * columns, whose face apertures the reference does not average
 * (src/Cutcell_Mod.f90:161-204).  The solve applies every row as written.
 * asym_faces (may be NULL) receives the number of faces whose two entries
 * differ, asym_max (may be NULL) the largest relative difference.  matr may
 * be NULL; host pointers always. */
int scf_proj_get_matrix(scf_proj *h, double *matr, int *asym_faces, double *asym_max);

/* Fault injection for tests of the bounded device waits (the reference's
 * only failure mechanism is a pause, src/ProjectionP_Mod.f90:209-213; here
 * a wait that runs out returns SCF_ERR_TIMEOUT).  On `device`, every later
 * TMA-staged sweep (mixed precision, levels of at least 128 x 64 cells) that
 * reduces nothing across the grid lets its CTA of linear index `cta` arm its
 * shared-memory barrier without issuing the copies, so that CTA's wait runs
 * out after `spins` polls of at most about a microsecond each: the solve
 * returns SCF_ERR_TIMEOUT with no copy in flight.  cta = -1 and
 * spins = 1048576 restore normal operation.  Re-assemble (or use a new
 * handle) after an injected timeout.  Device-wide; not for production use. */
int scf_diag_tma_timeout(int device, int cta, int spins);

/* Diagnostics: apply one multigrid V-cycle (the preconditioner) to b and
 * return x, both host arrays in Fortran (nx,ny) layout. */
int scf_proj_vcycle(scf_proj *h, const double *b, double *x);

/* Measurement: launch one kernel of the path `reps` times back to back on
 * the handle's stream, bracketed by CUDA events, and store the average
 * milliseconds per launch.  Overwrites the solver's work vectors (call it
 * between solves, after assemble).  No counterpart in the reference; it
 * exists so that per-kernel bandwidth can be measured live. */
#define SCF_K_SMOOTH 0         /* one red-black half sweep on the fine grid */
#define SCF_K_PUPDATE_SPMV 1   /* p = z + beta p, q = A p, p.q */
#define SCF_K_UPDATE_XR 2      /* x += alpha p, r -= alpha q, r.r */
#define SCF_K_RESID_RESTRICT 3 /* fine residual summed onto the first coarse level */
#define SCF_K_PROLONG 4        /* fine x += omega * coarse x */
#define SCF_K_ASSEMBLE 5       /* operator assembly from the Fortran arrays */
#define SCF_K_VCYCLE 6         /* one whole V-cycle, captured as a CUDA graph */
#define SCF_K_SETUP 7          /* assembly + multigrid hierarchy setup (device work only) */
#define SCF_K_LINE 8           /* one fine-level pass of the line smoother (one parity of the
                                  lines along x, iterate not zero), as the V-cycle runs it */
#define SCF_K_FINE_PRE 9       /* the fine level's first pre-smoothing launch of the point
                                  smoother (zero start, fused iterations, restriction) */
#define SCF_K_FINE_POST 10     /* its last post-smoothing launch (prolongation, fused
                                  iterations, r.z of the PCG) */
int scf_proj_time_kernel(scf_proj *h, int kernel, int reps, double *ms_per_launch);

/* Diagnostics: q[k] = a[k] / b[k] for k < n by the FP64 division that the
 * assembly, the correction, the momentum and the geometry kernels use
 * (integer-pipe arithmetic, correctly rounded to nearest even like IEEE
 * division).  Host arrays; runs on the given device.  No counterpart in the
 * reference; it exists so that tests can compare the division bit for bit
 * with IEEE division on many operands. */
int scf_diag_divide(const double *a, const double *b, double *q, int64_t n, int device);

/* Diagnostics: q[k] = sqrt(a[k]) by the FP64 square root that the CLSVOF
 * kernels use (integer-pipe arithmetic, correctly rounded to nearest even
 * like the IEEE square root).  Host arrays.  No counterpart in the
 * reference; it exists so that tests can compare it bit for bit with the
 * IEEE square root. */
int scf_diag_sqrt(const double *a, double *q, int64_t n, int device);

/* Allocation-free right-hand side.  Computes the right-hand side of the
 * pressure equation exactly as SetPoissonVectors does
 * (src/ProjectionP_Mod.f90:313-317) into rhs (nx,ny) (0 where Posnu = -1)
 * and its 2-norm into *bnorm, without allocating any memory.
 * No counterpart in the reference (SIMCOFlow builds the right-hand side on
 * the CPU inside PoissonEquationSolver).  It is meant for callers that cannot
 * allocate device memory where they need this value: a Fortran host that
 * keeps all of its GPU memory in its own arena and forbids hidden
 * cudaMalloc calls, or a time loop that must not pay the device-wide
 * synchronisation that cudaMalloc and cudaFree can cause.
 *  - Every array argument is a device pointer owned by the caller, in the
 *    layouts of scf_proj_set_grid / scf_proj_set_geometry; ustar and vstar
 *    are (nx+2,ny+2); rhs (nx,ny) and bnorm (one double) are outputs.
 *  - Its only scratch is one fixed array inside the library (about 33 KB,
 *    kept on every GPU that loads the library until the process exits).
 *    nx and ny must not exceed SCF_NOALLOC_MAX_SIDE; larger grids are
 *    rejected with SCF_ERR_ARG before anything runs.
 *  - Asynchronous on `stream` (a cudaStream_t; NULL = default stream): the
 *    outputs are valid once the stream has passed this call.
 *  - The first call on each device looks up the scratch array's device
 *    address (cudaGetSymbolAddress); make that first call on a device before
 *    any stream capture.  Only a lookup that succeeded is kept; after a
 *    failed one (SCF_ERR_CUDA) the next call looks the address up again.
 *  - All calls share the one scratch array, which keeps the last call's
 *    contents: calls that overlap on the GPU (different streams or host
 *    threads) race, so the caller must serialise them. */
#define SCF_NOALLOC_MAX_SIDE 16384
int scf_rhs_norm_noalloc(int nx, int ny, const double *ustar, const double *vstar,
                         const double *aE, const double *aW, const double *aN, const double *aS,
                         const double *dx, const double *dy, const double *nyS,
                         const double *WlLh, const int32_t *posnu_p, double vb, double *rhs,
                         double *bnorm, void *stream);

/* Human-readable text for a status code. */
const char *scf_strerror(int code);

#ifdef __cplusplus
}
#endif
#endif
