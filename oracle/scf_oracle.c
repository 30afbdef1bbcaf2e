/*
 * scf_oracle.c -- CPU restatement of the SIMCOFlow pressure-projection path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA path is
 * checked against.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py load it.  Nothing in the simcoflow_gb300 package
 * links or calls it, and the product path never falls back to it.
 *
 * Parity status: UNPINNED.  The reference (Fortran 90 + HYPRE + MPI) cannot
 * be compiled here (no Fortran compiler, no MPI, no HYPRE) and ships no golden
 * vectors or tests.  The restatement is pinned instead against the
 * reference's own built-in identities (the per-row |A p - b| <= 1e-10 check of
 * src/ProjectionP_Mod.f90:70-93 and the mass residual of
 * src/ComputePUV_Mod.f90:184-216) and against analytic known-answer cases.
 *
 * Every routine follows the reference loop by loop, in the same loop order
 * and with the same floating-point operation order (compile with
 * -ffp-contract=off so that no multiply-add is fused; the reference is built
 * by mpif77 without FMA-generating flags).
 *
 * Array conventions are the reference's (Fortran, column-major, i fastest):
 *   F1(a,i,j)  arrays dimensioned (1:nx,1:ny)
 *   F0(a,i,j)  arrays dimensioned (0:nx+1,0:ny+1)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define F1(a, i, j) (a)[(size_t)((i)-1) + (size_t)((j)-1) * (size_t)nx]
#define F0(a, i, j) (a)[(size_t)(i) + (size_t)(j) * (size_t)(nx + 2)]
#define PC(f, i, j) pocoef[(size_t)((i)-1) + (size_t)((j)-1) * (size_t)nx + (size_t)((f)-1) * (size_t)nx * (size_t)ny]
#define MT(f, i, j) matr[(size_t)((i)-1) + (size_t)((j)-1) * (size_t)nx + (size_t)((f)-1) * (size_t)nx * (size_t)ny]

static const double EPSI = 1.0e-3; /* src/StateVariables.f90:26 */

/* wet / dry predicates, src/ProjectionP_Mod.f90:409-410 and :493-494 */
static inline int is_wet(double vof, double phi, double vofS) {
    return (vof >= 0.5 && vofS < EPSI) || (phi < 0.0 && vofS >= EPSI);
}
static inline int is_dry(double vof, double phi, double vofS) {
    return (vof < 0.5 && vofS < EPSI) || (phi >= 0.0 && vofS >= EPSI);
}

/*
 * ComputePossionMatrixCoefficient, src/ProjectionP_Mod.f90:395-580.
 * pocoef is (nx,ny,4) with faces S=1, W=2, E=3, N=4 (comment at :45).
 * literal=1 keeps the reference's loop-carried BetaW/BetaD variables,
 * including the dry-cell / dry-south branch (:504-508) that assigns BetaW
 * but divides by the BetaD left over from the previous cell; literal=0
 * uses the intended rule (BetaD = BetaP in that branch).
 */
/* One cell of ComputePossionMatrixCoefficient; *pBetaW / *pBetaD carry the
 * loop's BetaW / BetaD from the previously visited cell (literal mode reads
 * them, see below). */
static void pocoef_cell(int nx, int ny, int i, int j, int literal, const double *vof,
                        const double *phi, const double *vofS, const double *dxP,
                        const double *dyP, const double *dxU, const double *dyV,
                        const double *DpU, const double *DpV, double betaP, double betaM,
                        double *pocoef, double *pBetaW, double *pBetaD) {
    const double tol = 1.0e-24;
    double BetaW = *pBetaW, BetaD = *pBetaD, Lamda;
#define WET(ii, jj) is_wet(F1(vof, ii, jj), F1(phi, ii, jj), F1(vofS, ii, jj))
#define DRY(ii, jj) is_dry(F1(vof, ii, jj), F1(phi, ii, jj), F1(vofS, ii, jj))
#define LAM(ii, jj) (fabs(F1(phi, i, j)) / ((fabs(F1(phi, i, j)) + fabs(F1(phi, ii, jj))) + tol))
    if (WET(i, j)) {
        /* south */
        if (j > 1) {
            if (DRY(i, j - 1)) {
                Lamda = LAM(i, j - 1);
                BetaW = Lamda * betaM + (1.0 - Lamda) * betaP;
                PC(1, i, j) = F0(DpV, i, j - 1) * F1(dxP, i, j) / F1(dyV, i, j - 1) * betaP * betaM / BetaW;
            } else if (WET(i, j - 1)) {
                BetaW = betaM;
                PC(1, i, j) = F0(DpV, i, j - 1) * F1(dxP, i, j) / F1(dyV, i, j - 1) * betaP * betaM / BetaW;
            }
        } else {
            BetaW = betaM;
            PC(1, i, j) = F0(DpV, i, j) * F1(dxP, i, j) / F1(dyV, i, j) * betaP * betaM / BetaW;
        }
        /* west */
        if (i > 1) {
            if (DRY(i - 1, j)) {
                Lamda = LAM(i - 1, j);
                BetaW = Lamda * betaM + (1.0 - Lamda) * betaP;
                PC(2, i, j) = F0(DpU, i - 1, j) * F1(dyP, i, j) / F1(dxU, i - 1, j) * betaP * betaM / BetaW;
            } else if (WET(i - 1, j)) {
                BetaW = betaM;
                PC(2, i, j) = F0(DpU, i - 1, j) * F1(dyP, i, j) / F1(dxU, i - 1, j) * betaP * betaM / BetaW;
            }
        } else {
            BetaW = betaM;
            PC(2, i, j) = F0(DpU, i, j) * F1(dyP, i, j) / F1(dxU, i, j) * betaP * betaM / BetaW;
        }
        /* east */
        if (i < nx) {
            if (DRY(i + 1, j)) {
                Lamda = LAM(i + 1, j);
                BetaW = Lamda * betaM + (1.0 - Lamda) * betaP;
                PC(3, i, j) = F0(DpU, i, j) * F1(dyP, i, j) / F1(dxU, i, j) * betaP * betaM / BetaW;
            } else if (WET(i + 1, j)) {
                BetaW = betaM;
                PC(3, i, j) = F0(DpU, i, j) * F1(dyP, i, j) / F1(dxU, i, j) * betaP * betaM / BetaW;
            }
        } else {
            BetaW = betaM;
            PC(3, i, j) = F0(DpU, i, j) * F1(dyP, i, j) / F1(dxU, i, j) * betaP * betaM / BetaW;
        }
        /* north */
        if (j < ny) {
            if (DRY(i, j + 1)) {
                Lamda = LAM(i, j + 1);
                BetaW = Lamda * betaM + (1.0 - Lamda) * betaP;
                PC(4, i, j) = F0(DpV, i, j) * F1(dxP, i, j) / F1(dyV, i, j) * betaP * betaM / BetaW;
            } else if (WET(i, j + 1)) {
                BetaW = betaM;
                PC(4, i, j) = F0(DpV, i, j) * F1(dxP, i, j) / F1(dyV, i, j) * betaP * betaM / BetaW;
            }
        } else {
            BetaW = betaM;
            PC(4, i, j) = F0(DpV, i, j) * F1(dxP, i, j) / F1(dyV, i, j) * betaP * betaM / BetaW;
        }
    } else if (DRY(i, j)) {
        /* south */
        if (j > 1) {
            if (WET(i, j - 1)) {
                Lamda = LAM(i, j - 1);
                BetaD = Lamda * betaP + (1.0 - Lamda) * betaM;
                PC(1, i, j) = F0(DpV, i, j - 1) * F1(dxP, i, j) / F1(dyV, i, j - 1) * betaP * betaM / BetaD;
            } else if (DRY(i, j - 1)) {
                if (literal) BetaW = betaP; /* :506 assigns BetaW, :507 divides by BetaD */
                else BetaD = betaP;
                PC(1, i, j) = F0(DpV, i, j - 1) * F1(dxP, i, j) / F1(dyV, i, j - 1) * betaP * betaM / BetaD;
            }
        } else {
            BetaD = betaP;
            PC(1, i, j) = F0(DpV, i, j) * F1(dxP, i, j) / F1(dyV, i, j) * betaP * betaM / BetaD;
        }
        /* west */
        if (i > 1) {
            if (WET(i - 1, j)) {
                Lamda = LAM(i - 1, j);
                BetaD = Lamda * betaP + (1.0 - Lamda) * betaM;
                PC(2, i, j) = F0(DpU, i - 1, j) * F1(dyP, i, j) / F1(dxU, i - 1, j) * betaP * betaM / BetaD;
            } else if (DRY(i - 1, j)) {
                BetaD = betaP;
                PC(2, i, j) = F0(DpU, i - 1, j) * F1(dyP, i, j) / F1(dxU, i - 1, j) * betaP * betaM / BetaD;
            }
        } else {
            BetaD = betaP;
            PC(2, i, j) = F0(DpU, i, j) * F1(dyP, i, j) / F1(dxU, i, j) * betaP * betaM / BetaD;
        }
        /* east */
        if (i < nx) {
            if (WET(i + 1, j)) {
                Lamda = LAM(i + 1, j);
                BetaD = Lamda * betaP + (1.0 - Lamda) * betaM;
                PC(3, i, j) = F0(DpU, i, j) * F1(dyP, i, j) / F1(dxU, i, j) * betaP * betaM / BetaD;
            } else if (DRY(i + 1, j)) {
                BetaD = betaP;
                PC(3, i, j) = F0(DpU, i, j) * F1(dyP, i, j) / F1(dxU, i, j) * betaP * betaM / BetaD;
            }
        } else {
            BetaD = betaP;
            PC(3, i, j) = F0(DpU, i, j) * F1(dyP, i, j) / F1(dxU, i, j) * betaP * betaM / BetaD;
        }
        /* north */
        if (j < ny) {
            if (WET(i, j + 1)) {
                Lamda = LAM(i, j + 1);
                BetaD = Lamda * betaP + (1.0 - Lamda) * betaM;
                PC(4, i, j) = F0(DpV, i, j) * F1(dxP, i, j) / F1(dyV, i, j) * betaP * betaM / BetaD;
            } else if (DRY(i, j + 1)) {
                BetaD = betaP;
                PC(4, i, j) = F0(DpV, i, j) * F1(dxP, i, j) / F1(dyV, i, j) * betaP * betaM / BetaD;
            }
        } else {
            BetaD = betaP;
            PC(4, i, j) = F0(DpV, i, j) * F1(dxP, i, j) / F1(dyV, i, j) * betaP * betaM / BetaD;
        }
    }
#undef WET
#undef DRY
#undef LAM
    *pBetaW = BetaW;
    *pBetaD = BetaD;
    (void)ny;
}

void oracle_pocoef(int nx, int ny, int literal, const double *vof, const double *phi,
                   const double *vofS, const double *dxP, const double *dyP,
                   const double *dxU, const double *dyV, const double *DpU,
                   const double *DpV, double betaP, double betaM, double *pocoef) {
    const size_t n4 = (size_t)nx * ny * 4;
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n4; ++k) pocoef[k] = 0.0;
    if (literal) {
        /* the reference's loop order (j innermost): the stale BetaD read by
           the dry/dry south face is the one cell (i,j-1) left behind */
        double BetaW = NAN, BetaD = NAN;
        for (int i = 1; i <= nx; ++i)
            for (int j = 1; j <= ny; ++j)
                pocoef_cell(nx, ny, i, j, 1, vof, phi, vofS, dxP, dyP, dxU, dyV, DpU, DpV,
                            betaP, betaM, pocoef, &BetaW, &BetaD);
        return;
    }
    /* the intended rule reads nothing left over from another cell, so the
       cells are independent: memory order (i innermost), all threads */
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j) {
        double BetaW = NAN, BetaD = NAN;
        for (int i = 1; i <= nx; ++i)
            pocoef_cell(nx, ny, i, j, 0, vof, phi, vofS, dxP, dyP, dxU, dyV, DpU, DpV, betaP,
                        betaM, pocoef, &BetaW, &BetaD);
    }
}

/*
 * SetPoissonMatrix, src/ProjectionP_Mod.f90:137-273.
 * Fills matr(nx,ny,5) (S,W,diag,E,N; zero where the reference leaves no
 * entry) and the CSR matrix in the reference's row numbering (Posnu) with
 * the reference's column order within a row (S, W, diag, E, N).
 * rowptr has n_rows+1 entries, cols/vals room for 5*n_rows.
 * Returns the number of rows (ExtCell+1).
 */
/* One row of SetPoissonMatrix into matr (and vals/cols when given). */
static int matrix_row(int nx, int ny, int i, int j, const double *pocoef, const double *aE,
                      const double *aW, const double *aN, const double *aS,
                      const int32_t *posnu, int wb, int eb, int sb, int nbc, double *matr,
                      double *values, int *cc) {
    const double tol = 1.0e-24;
    int nnz = 0;
    if (j > 1 && F0(posnu, i, j - 1) != -1) {
        cc[nnz] = F0(posnu, i, j - 1);
        values[nnz] = -PC(1, i, j) * F0(aS, i, j);
        MT(1, i, j) = values[nnz];
        nnz++;
    }
    if (i > 1 && F0(posnu, i - 1, j) != -1) {
        cc[nnz] = F0(posnu, i - 1, j);
        values[nnz] = -PC(2, i, j) * F0(aW, i, j);
        MT(2, i, j) = values[nnz];
        nnz++;
    }
    cc[nnz] = F0(posnu, i, j);
    double d = PC(1, i, j) * F0(aS, i, j) + PC(2, i, j) * F0(aW, i, j) +
               PC(3, i, j) * F0(aE, i, j) + PC(4, i, j) * F0(aN, i, j);
    if (sb == 1 && j == 1) d = d - PC(1, i, j) * F0(aS, i, j);
    if (wb == 1 && i == 1) d = d - PC(2, i, j) * F0(aW, i, j);
    if (eb == 1 && i == nx) d = d - PC(3, i, j) * F0(aE, i, j);
    if (nbc == 1 && j == ny) d = d - PC(4, i, j) * F0(aN, i, j);
    d = d + copysign(1.0, d) * tol;
    values[nnz] = d;
    MT(3, i, j) = d;
    nnz++;
    if (i < nx && F0(posnu, i + 1, j) != -1) {
        cc[nnz] = F0(posnu, i + 1, j);
        values[nnz] = -PC(3, i, j) * F0(aE, i, j);
        MT(4, i, j) = values[nnz];
        nnz++;
    }
    if (j < ny && F0(posnu, i, j + 1) != -1) {
        cc[nnz] = F0(posnu, i, j + 1);
        values[nnz] = -PC(4, i, j) * F0(aN, i, j);
        MT(5, i, j) = values[nnz];
        nnz++;
    }
    return nnz;
}

int oracle_matrix(int nx, int ny, const double *pocoef, const double *aE, const double *aW,
                  const double *aN, const double *aS, const int32_t *posnu, int wb, int eb,
                  int sb, int nbc, double *matr, int32_t *rowptr, int32_t *cols, double *vals) {
    const size_t n5 = (size_t)nx * ny * 5;
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n5; ++k) matr[k] = 0.0;
    if (!rowptr) {
        /* the dense copy only: rows are independent */
#pragma omp parallel for schedule(static)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                double values[5];
                int cc[5];
                if (F0(posnu, i, j) != -1)
                    matrix_row(nx, ny, i, j, pocoef, aE, aW, aN, aS, posnu, wb, eb, sb, nbc,
                               matr, values, cc);
            }
        int nrows = 0;
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i)
                if (F0(posnu, i, j) != -1) nrows++;
        return nrows;
    }
    /* rows are numbered with j fastest (src/Cutcell_Mod.f90:347-351), which is
       also the visiting order here, so CSR rows are written in order */
    int nnz_total = 0, nrows = 0;
    rowptr[0] = 0;
    for (int i = 1; i <= nx; ++i) {
        for (int j = 1; j <= ny; ++j) {
            int row = F0(posnu, i, j);
            if (row == -1) continue;
            double values[5];
            int cc[5];
            int nnz = matrix_row(nx, ny, i, j, pocoef, aE, aW, aN, aS, posnu, wb, eb, sb, nbc,
                                 matr, values, cc);
            for (int k = 0; k < nnz; ++k) {
                cols[nnz_total + k] = cc[k];
                vals[nnz_total + k] = values[k];
            }
            nnz_total += nnz;
            rowptr[row + 1] = nnz_total;
            nrows++;
        }
    }
    return nrows;
}

/*
 * SetPoissonVectors, src/ProjectionP_Mod.f90:275-354 (formula :313-317).
 * u, v are the predicted velocities (0:nx+1,0:ny+1); rhm is (nx,ny) and is
 * zero where the cell has no row; rhs is in Posnu order.
 */
void oracle_rhs(int nx, int ny, const double *u, const double *v, const double *aE,
                const double *aW, const double *aN, const double *aS, const double *dxP,
                const double *dyP, const double *nyS, const double *WlLh, const int32_t *posnu,
                double vb, double *rhm, double *rhs) {
    /* cells are independent: memory order, all threads */
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j) {
        for (int i = 1; i <= nx; ++i) {
            int ictr = F0(posnu, i, j);
            F1(rhm, i, j) = 0.0;
            if (ictr == -1) continue;
            double dx = F1(dxP, i, j), dy = F1(dyP, i, j);
            double r = -((F0(u, i, j) * F0(aE, i, j) - F0(u, i - 1, j) * F0(aW, i, j)) * dy) -
                       (F0(v, i, j) * F0(aN, i, j) - F0(v, i, j - 1) * F0(aS, i, j)) * dx +
                       vb * F1(nyS, i, j) * F1(WlLh, i, j);
            if (rhs) rhs[ictr] = r;
            F1(rhm, i, j) = r;
        }
    }
}

/*
 * DeltaPressureGetValues + DeltaPressureBoundaryCondition,
 * src/ProjectionP_Mod.f90:356-393 and :582-595.  x is in Posnu order;
 * Pp is (0:nx+1,0:ny+1) and its four corners stay zero as in UpdatePUV
 * (src/ComputePUV_Mod.f90:50).
 */
void oracle_scatter(int nx, int ny, const int32_t *posnu, const double *x, int wb, int eb,
                    int sb, int nbc, double *Pp) {
    const size_t n0 = (size_t)(nx + 2) * (ny + 2);
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n0; ++k) Pp[k] = 0.0;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            int c = F0(posnu, i, j);
            F0(Pp, i, j) = (c != -1) ? x[c] : 0.0;
        }
    for (int i = 1; i <= nx; ++i) {
        F0(Pp, i, 0) = (double)sb * F0(Pp, i, 1);
        F0(Pp, i, ny + 1) = (double)nbc * F0(Pp, i, ny);
    }
    for (int j = 1; j <= ny; ++j) {
        F0(Pp, 0, j) = (double)wb * F0(Pp, 1, j);
        F0(Pp, nx + 1, j) = (double)eb * F0(Pp, nx, j);
    }
}

/*
 * Velocity correction, pressure copy, top-row continuity, mass residual and
 * solid-cell zeroing: UpdatePUV src/ComputePUV_Mod.f90:59-100 (u), :111-152
 * (v), :163-169 (p), :177-182 (top v), :184-217 (mres) and
 * VariablesInternalCellCondition :227-245.
 * u, v, p are TVar fields (0:nx+1,0:ny+1): in = old values, out = new.
 * ustar, vstar are Pred%u, Pred%v; mres is (nx,ny).
 */
void oracle_correct(int nx, int ny, const double *Pp, const double *ustar, const double *vstar,
                    const double *vof, const double *phi, const double *vofS, const double *nyS,
                    const double *WlLh, const double *aE, const double *aW, const double *aN,
                    const double *aS, const int32_t *posnu_p, const int32_t *posnu_u,
                    const int32_t *moex_u, const double *vofS_u, const int32_t *posnu_v,
                    const int32_t *moex_v, const double *vofS_v, const double *dxP,
                    const double *dyP, const double *dxU, const double *dyV, const double *DpU,
                    const double *DpV, double betaP, double betaM, double vb, double *u,
                    double *v, double *p, double *mres) {
    const double tol = 1.0e-24;
#define WET(ii, jj) is_wet(F1(vof, ii, jj), F1(phi, ii, jj), F1(vofS, ii, jj))
#define DRY(ii, jj) is_dry(F1(vof, ii, jj), F1(phi, ii, jj), F1(vofS, ii, jj))
    /* every stage below writes each element from its own loop iteration only
       (reading what earlier stages wrote), so a stage's iterations run in
       memory order on all threads without changing a result */
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j) {
        for (int i = 1; i <= nx - 1; ++i) {
            if (F0(posnu_u, i, j) != -1 && F1(moex_u, i, j) != 1) {
                double BetaW, Lamda, G;
                int set = 0;
                if (WET(i, j)) {
                    if (DRY(i + 1, j)) {
                        Lamda = fabs(F1(phi, i, j)) / ((fabs(F1(phi, i, j)) + fabs(F1(phi, i + 1, j))) + tol);
                        BetaW = Lamda * betaM + (1.0 - Lamda) * betaP;
                        set = 1;
                    } else if (WET(i + 1, j)) {
                        BetaW = betaM;
                        set = 1;
                    }
                } else if (DRY(i, j)) {
                    if (WET(i + 1, j)) {
                        Lamda = fabs(F1(phi, i, j)) / ((fabs(F1(phi, i, j)) + fabs(F1(phi, i + 1, j))) + tol);
                        BetaW = Lamda * betaP + (1.0 - Lamda) * betaM;
                        set = 1;
                    } else if (DRY(i + 1, j)) {
                        BetaW = betaP;
                        set = 1;
                    }
                }
                if (set) {
                    G = (F0(Pp, i + 1, j) - F0(Pp, i, j)) * betaM * betaP / BetaW * F0(DpU, i, j) / F1(dxU, i, j);
                    F0(u, i, j) = F0(ustar, i, j) - G;
                }
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny - 1; ++j) {
        for (int i = 1; i <= nx; ++i) {
            if (F0(posnu_v, i, j) != -1 && F1(moex_v, i, j) != 1) {
                double BetaW, Lamda, G;
                int set = 0;
                if (WET(i, j)) {
                    if (DRY(i, j + 1)) {
                        Lamda = fabs(F1(phi, i, j)) / ((fabs(F1(phi, i, j)) + fabs(F1(phi, i, j + 1))) + tol);
                        BetaW = Lamda * betaM + (1.0 - Lamda) * betaP;
                        set = 1;
                    } else if (WET(i, j + 1)) {
                        BetaW = betaM;
                        set = 1;
                    }
                } else if (DRY(i, j)) {
                    if (WET(i, j + 1)) {
                        Lamda = fabs(F1(phi, i, j)) / ((fabs(F1(phi, i, j)) + fabs(F1(phi, i, j + 1))) + tol);
                        BetaW = Lamda * betaP + (1.0 - Lamda) * betaM;
                        set = 1;
                    } else if (DRY(i, j + 1)) {
                        BetaW = betaP;
                        set = 1;
                    }
                }
                if (set) {
                    G = (F0(Pp, i, j + 1) - F0(Pp, i, j)) * betaM * betaP / BetaW * F0(DpV, i, j) / F1(dyV, i, j);
                    F0(v, i, j) = F0(vstar, i, j) - G;
                }
            }
        }
    }
#undef WET
#undef DRY
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i)
            if (F0(posnu_p, i, j) != -1) F0(p, i, j) = F0(Pp, i, j);
    for (int i = 1; i <= nx; ++i) {
        int j = ny;
        F0(v, i, j) = ((-(F0(u, i, j) * F0(aE, i, j)) + F0(u, i - 1, j) * F0(aW, i, j)) * F1(dyP, i, j) +
                       F0(v, i, j - 1) * F0(aS, i, j) * F1(dxP, i, j)) /
                      F1(dxP, i, j) / F0(aN, i, j);
    }
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j) {
        for (int i = 1; i <= nx; ++i) {
            F1(mres, i, j) = (F0(u, i, j) * F0(aE, i, j) - F0(u, i - 1, j) * F0(aW, i, j)) * F1(dyP, i, j) +
                             (F0(v, i, j) * F0(aN, i, j) - F0(v, i, j - 1) * F0(aS, i, j)) * F1(dxP, i, j) -
                             vb * F1(nyS, i, j) * F1(WlLh, i, j);
            if (F1(vofS, i, j) > 1.0 - EPSI) F1(mres, i, j) = 0.0;
        }
    }
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j) {
        for (int i = 1; i <= nx; ++i) {
            if (F1(vofS, i, j) > 1.0 - EPSI) F0(p, i, j) = 0.0;
            if (F1(vofS_u, i, j) >= 1.0 - EPSI) F0(u, i, j) = 0.0;
            if (F1(vofS_v, i, j) >= 1.0 - EPSI) F0(v, i, j) = 0.0;
        }
    }
}

/* The per-row residual self-check of src/ProjectionP_Mod.f90:70-93:
 * returns max |A Pp - rhm| over rows with Posnu /= -1. */
double oracle_row_residual(int nx, int ny, const double *matr, const double *Pp,
                           const double *rhm, const int32_t *posnu) {
    double worst = 0.0;
    for (int i = 1; i <= nx; ++i)
        for (int j = 1; j <= ny; ++j) {
            double resi = 0.0;
            if (j > 1) resi = resi + MT(1, i, j) * F0(Pp, i, j - 1);
            if (i > 1) resi = resi + MT(2, i, j) * F0(Pp, i - 1, j);
            resi = resi + MT(3, i, j) * F0(Pp, i, j);
            if (i < nx) resi = resi + MT(4, i, j) * F0(Pp, i + 1, j);
            if (j < ny) resi = resi + MT(5, i, j) * F0(Pp, i, j + 1);
            double d = fabs(resi - F1(rhm, i, j));
            if (F0(posnu, i, j) != -1 && d > worst) worst = d;
        }
    return worst;
}

/* ------------------------------------------------------------------------
 * CPU FP64 MG-PCG: the same algorithm as the CUDA path, restated on the CPU.
 * Used as the FP64 oracle solve at sizes the direct solver cannot reach and
 * as the timed CPU baseline.  Symmetric 5-point storage per level:
 *   cE(i,j): coupling of (i,j) and (i+1,j); cN(i,j): of (i,j) and (i,j+1);
 *   dg(i,j): diagonal; a cell without an unknown has dg = -1 and no couplings.
 * The PCG's own operator applies the rows as assembled: the optional cW /
 * cS of oracle_mgpcg are each row's own west / south couplings
 * (-matr(.,.,2), -matr(.,.,1)), which may differ from the neighbour's cE / cN.
 * The fine level is taken from matr: cE = -matr(.,.,4), cN = -matr(.,.,5),
 * dg = matr(.,.,3).  Coarse levels are the Galerkin product P^T A P with
 * piecewise-constant 2x2 aggregation, computed as summed couplings plus the
 * summed diagonal excess (dg - sum of couplings, clamped at 0).
 * V-cycle: x=0; pre-smooth red then black; residual; restrict (sum);
 * recurse; x += omega * P e (not into cells without an unknown); post-smooth
 * black then red.  Coarsest level: dense Cholesky.  With the line smoother a
 * pre-smoothing step is: even rows, odd rows, even columns, odd columns,
 * each line solved exactly; post-smoothing runs the reverse order.
 * Arrays are 0-based, x fastest: a[ix + iy*nx].
 * ------------------------------------------------------------------------ */
typedef struct {
    int nx, ny;
    double *cE, *cN, *dg, *ex;
    double *x, *b, *r;
    /* fine level of the PCG operator only (NULL elsewhere): each row's own
       west / south couplings, -matr(.,.,2) and -matr(.,.,1).  The reference
       forms them from the row's cell (src/ProjectionP_Mod.f90:183,193), so
       they may differ from the neighbour's cE / cN; the V-cycle uses the
       symmetric cE / cN. */
    const double *cW, *cS;
} olevel;

typedef struct {
    int nlev;
    olevel lev[32];
    double omega;
    int npre, npost;
    int cfrom, csweeps; /* csweeps sweeps on levels cfrom and coarser (0: npre / npost) */
    int line;        /* 1: alternating zebra line smoother */
    int nc;          /* coarsest unknowns */
    double *chol;    /* nc x nc lower Cholesky factor */
    int *cmap;       /* coarsest cell -> dense index or -1 */
} omg;

static double *dalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }
static void pzero(double *a, size_t n) {
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n; ++k) a[k] = 0.0;
}
static void pcopy(double *dst, const double *src, size_t n) {
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n; ++k) dst[k] = src[k];
}


static void level_alloc(olevel *L, int nx, int ny) {
    size_t n = (size_t)nx * ny;
    L->nx = nx; L->ny = ny;
    L->cE = dalloc(n); L->cN = dalloc(n); L->dg = dalloc(n); L->ex = dalloc(n);
    L->x = dalloc(n); L->b = dalloc(n); L->r = dalloc(n);
}
static void level_free(olevel *L) {
    free(L->cE); free(L->cN); free(L->dg); free(L->ex); free(L->x); free(L->b); free(L->r);
}

static void compute_excess(olevel *L) {
    int nx = L->nx, ny = L->ny;
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nx; ++ix) {
            size_t k = (size_t)iy * nx + ix;
            if (L->dg[k] < 0.0) { L->ex[k] = 0.0; continue; }
            double s = L->cE[k] + (ix > 0 ? L->cE[k - 1] : 0.0) + L->cN[k] + (iy > 0 ? L->cN[k - nx] : 0.0);
            double e = L->dg[k] - s;
            L->ex[k] = e > 0.0 ? e : 0.0;
        }
}

static void coarsen(const olevel *F, olevel *C) {
    int nxf = F->nx, nyf = F->ny, nxc = (nxf + 1) / 2, nyc = (nyf + 1) / 2;
    level_alloc(C, nxc, nyc);
#pragma omp parallel for schedule(static)
    for (int J = 0; J < nyc; ++J)
        for (int I = 0; I < nxc; ++I) {
            double ce = 0.0, cn = 0.0, ex = 0.0;
            int active = 0;
            for (int dj = 0; dj < 2; ++dj)
                for (int di = 0; di < 2; ++di) {
                    int ix = 2 * I + di, iy = 2 * J + dj;
                    if (ix >= nxf || iy >= nyf) continue;
                    size_t k = (size_t)iy * nxf + ix;
                    if (F->dg[k] >= 0.0) active = 1;
                    ex += F->ex[k];
                    if (di == 1) ce += F->cE[k];
                    if (dj == 1) cn += F->cN[k];
                }
            size_t kc = (size_t)J * nxc + I;
            C->cE[kc] = ce;
            C->cN[kc] = cn;
            C->ex[kc] = active ? ex : 0.0;
            C->dg[kc] = active ? 0.0 : -1.0;
        }
#pragma omp parallel for schedule(static)
    for (int J = 0; J < nyc; ++J)
        for (int I = 0; I < nxc; ++I) {
            size_t kc = (size_t)J * nxc + I;
            if (C->dg[kc] < 0.0) continue;
            double s = C->cE[kc] + (I > 0 ? C->cE[kc - 1] : 0.0) + C->cN[kc] + (J > 0 ? C->cN[kc - nxc] : 0.0);
            C->dg[kc] = s + C->ex[kc];
            if (!(C->dg[kc] > 0.0)) C->dg[kc] = -1.0;
        }
}

static void coarse_factor(omg *M) {
    olevel *L = &M->lev[M->nlev - 1];
    int nx = L->nx, ny = L->ny, n = 0;
    M->cmap = (int *)malloc(sizeof(int) * (size_t)nx * ny);
    for (int k = 0; k < nx * ny; ++k) M->cmap[k] = L->dg[k] >= 0.0 ? n++ : -1;
    M->nc = n;
    M->chol = dalloc((size_t)n * n);
    double *A = M->chol;
    for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nx; ++ix) {
            int k = iy * nx + ix, r = M->cmap[k];
            if (r < 0) continue;
            A[(size_t)r * n + r] = L->dg[k];
            if (ix + 1 < nx && M->cmap[k + 1] >= 0) {
                int c = M->cmap[k + 1];
                A[(size_t)r * n + c] = -L->cE[k]; A[(size_t)c * n + r] = -L->cE[k];
            }
            if (iy + 1 < ny && M->cmap[k + nx] >= 0) {
                int c = M->cmap[k + nx];
                A[(size_t)r * n + c] = -L->cN[k]; A[(size_t)c * n + r] = -L->cN[k];
            }
        }
    /* in-place lower Cholesky */
    for (int j = 0; j < n; ++j) {
        double d = A[(size_t)j * n + j];
        for (int k = 0; k < j; ++k) d -= A[(size_t)j * n + k] * A[(size_t)j * n + k];
        d = d > 0.0 ? sqrt(d) : 1e-300;
        A[(size_t)j * n + j] = d;
        for (int i = j + 1; i < n; ++i) {
            double s = A[(size_t)i * n + j];
            for (int k = 0; k < j; ++k) s -= A[(size_t)i * n + k] * A[(size_t)j * n + k];
            A[(size_t)i * n + j] = s / d;
        }
    }
}

static void coarse_solve(omg *M) {
    olevel *L = &M->lev[M->nlev - 1];
    int n = M->nc, N = L->nx * L->ny;
    double *y = dalloc((size_t)n);
    for (int k = 0; k < N; ++k) if (M->cmap[k] >= 0) y[M->cmap[k]] = L->b[k];
    const double *A = M->chol;
    for (int i = 0; i < n; ++i) {
        double s = y[i];
        for (int k = 0; k < i; ++k) s -= A[(size_t)i * n + k] * y[k];
        y[i] = s / A[(size_t)i * n + i];
    }
    for (int i = n - 1; i >= 0; --i) {
        double s = y[i];
        for (int k = i + 1; k < n; ++k) s -= A[(size_t)k * n + i] * y[k];
        y[i] = s / A[(size_t)i * n + i];
    }
    for (int k = 0; k < N; ++k) L->x[k] = M->cmap[k] >= 0 ? y[M->cmap[k]] : 0.0;
    free(y);
}

/* one red-black half sweep: color 0 updates cells with (ix+iy) even */
static void rbgs_half(olevel *L, int color) {
    int nx = L->nx, ny = L->ny;
    const double *cE = L->cE, *cN = L->cN, *dg = L->dg, *b = L->b;
    double *x = L->x;
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < ny; ++iy) {
        int ix0 = (iy + color) & 1;
        for (int ix = ix0; ix < nx; ix += 2) {
            size_t k = (size_t)iy * nx + ix;
            double s = b[k];
            if (ix + 1 < nx) s = s + cE[k] * x[k + 1];
            if (ix > 0) s = s + cE[k - 1] * x[k - 1];
            if (iy + 1 < ny) s = s + cN[k] * x[k + nx];
            if (iy > 0) s = s + cN[k - nx] * x[k - nx];
            x[k] = dg[k] > 0.0 ? s / dg[k] : 0.0;
        }
    }
}

/* Exact solves of the lines of one parity: dir 0 rows (iy % 2 == color),
 * dir 1 columns (ix % 2 == color).  Each line is the tridiagonal system of
 * its in-line couplings, with the couplings to the neighbouring lines of the
 * other parity on the right-hand side; Thomas algorithm.  Cells without an
 * unknown get x = 0. */
static void line_half(olevel *L, int dir, int color) {
    int nx = L->nx, ny = L->ny;
    const double *cE = L->cE, *cN = L->cN, *dg = L->dg, *b = L->b;
    double *x = L->x;
    int nlines = dir == 0 ? ny : nx, len = dir == 0 ? nx : ny;
    /* lines along y are solved LB at a time (LB lines of one parity, two
       columns apart), interleaved cell by cell, so that a row's cache lines
       serve all of them; each line's arithmetic is that of a lone solve */
    enum { LB = 8 };
    const int per = dir == 0 ? 1 : LB;
    const int nblk = ((nlines - color + 1) / 2 + per - 1) / per;
#pragma omp parallel
    {
        double *cp = dalloc((size_t)len * per), *dp = dalloc((size_t)len * per);
#pragma omp for schedule(static)
        for (int blk = 0; blk < nblk; ++blk) {
            int q0 = color + 2 * per * blk, nq = 0;
            int qs[LB];
            for (int t = 0; t < per && q0 + 2 * t < nlines; ++t) qs[nq++] = q0 + 2 * t;
            /* cell k of line q: index and its in-line / cross couplings */
            for (int k = 0; k < len; ++k) {
                for (int t = 0; t < nq; ++t) {
                    int q = qs[t];
                    int ix = dir == 0 ? k : q, iy = dir == 0 ? q : k;
                    size_t c = (size_t)iy * nx + ix;
                    double a = 0.0, up = 0.0, d = 1.0, r = 0.0;
                    if (dg[c] > 0.0) {
                        d = dg[c];
                        r = b[c];
                        if (dir == 0) {
                            a = ix > 0 ? -cE[c - 1] : 0.0;
                            up = ix + 1 < nx ? -cE[c] : 0.0;
                            if (iy + 1 < ny) r = r + cN[c] * x[c + nx];
                            if (iy > 0) r = r + cN[c - nx] * x[c - nx];
                        } else {
                            a = iy > 0 ? -cN[c - nx] : 0.0;
                            up = iy + 1 < ny ? -cN[c] : 0.0;
                            if (ix + 1 < nx) r = r + cE[c] * x[c + 1];
                            if (ix > 0) r = r + cE[c - 1] * x[c - 1];
                        }
                    }
                    double *cpt = cp + (size_t)t * len, *dpt = dp + (size_t)t * len;
                    double den = k > 0 ? d - a * cpt[k - 1] : d;
                    cpt[k] = up / den;
                    dpt[k] = (k > 0 ? r - a * dpt[k - 1] : r) / den;
                }
            }
            double xn[LB];
            for (int t = 0; t < nq; ++t) xn[t] = 0.0;
            for (int k = len - 1; k >= 0; --k) {
                for (int t = 0; t < nq; ++t) {
                    int q = qs[t];
                    int ix = dir == 0 ? k : q, iy = dir == 0 ? q : k;
                    size_t c = (size_t)iy * nx + ix;
                    const double *cpt = cp + (size_t)t * len, *dpt = dp + (size_t)t * len;
                    xn[t] = dpt[k] - (k + 1 < len ? cpt[k] * xn[t] : 0.0);
                    x[c] = dg[c] > 0.0 ? xn[t] : 0.0;
                }
            }
        }
        free(cp); free(dp);
    }
}

/* one smoothing step of the line smoother; post: the reverse order */
static void line_step(olevel *L, int post) {
    if (!post) { line_half(L, 0, 0); line_half(L, 0, 1); line_half(L, 1, 0); line_half(L, 1, 1); }
    else { line_half(L, 1, 1); line_half(L, 1, 0); line_half(L, 0, 1); line_half(L, 0, 0); }
}

static void residual(olevel *L) {
    int nx = L->nx, ny = L->ny;
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nx; ++ix) {
            size_t k = (size_t)iy * nx + ix;
            if (L->dg[k] < 0.0) { L->r[k] = 0.0; continue; }
            double s = L->b[k] - L->dg[k] * L->x[k];
            if (ix + 1 < nx) s = s + L->cE[k] * L->x[k + 1];
            if (ix > 0) s = s + L->cE[k - 1] * L->x[k - 1];
            if (iy + 1 < ny) s = s + L->cN[k] * L->x[k + nx];
            if (iy > 0) s = s + L->cN[k - nx] * L->x[k - nx];
            L->r[k] = s;
        }
}

static void restrict_sum(const olevel *F, olevel *C) {
    int nxf = F->nx, nyf = F->ny, nxc = C->nx, nyc = C->ny;
#pragma omp parallel for schedule(static)
    for (int J = 0; J < nyc; ++J)
        for (int I = 0; I < nxc; ++I) {
            double s = 0.0;
            for (int dj = 0; dj < 2; ++dj)
                for (int di = 0; di < 2; ++di) {
                    int ix = 2 * I + di, iy = 2 * J + dj;
                    if (ix < nxf && iy < nyf) s = s + F->r[(size_t)iy * nxf + ix];
                }
            C->b[(size_t)J * nxc + I] = s;
        }
}

static void prolong_add(olevel *F, const olevel *C, double omega) {
    int nxf = F->nx, nyf = F->ny, nxc = C->nx;
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < nyf; ++iy)
        for (int ix = 0; ix < nxf; ++ix) {
            size_t k = (size_t)iy * nxf + ix;
            if (F->dg[k] < 0.0) continue;
            F->x[k] = F->x[k] + omega * C->x[(size_t)(iy / 2) * nxc + (ix / 2)];
        }
}

/* the coarse-level schedule of the next MG-PCG or V-cycle call: sweeps on
   level cfrom (0: the finest) and coarser (point smoother: red-black
   iterations; line smoother: a step of x-lines then y-lines counts as two);
   sweeps 0 keeps npre / npost everywhere */
static int g_cfrom = 0, g_csweeps = 0;
void oracle_set_coarse_sweeps(int cfrom, int sweeps) { g_cfrom = cfrom; g_csweeps = sweeps; }

static int sweeps_at(const omg *M, int l, int post) {
    return M->csweeps > 0 && l >= M->cfrom ? M->csweeps : (post ? M->npost : M->npre);
}
static int line_steps(const omg *M, int l, int post) { return (sweeps_at(M, l, post) + 1) / 2; }

static void vcycle(omg *M, int l) {
    olevel *L = &M->lev[l];
    size_t n = (size_t)L->nx * L->ny;
    if (l == M->nlev - 1) { coarse_solve(M); return; }
    pzero(L->x, n);
    if (M->line) {
        /* a line step (x-lines and y-lines) counts as two sweeps */
        for (int s = 0; s < line_steps(M, l, 0); ++s) line_step(L, 0);
    } else {
        for (int s = 0; s < sweeps_at(M, l, 0); ++s) { rbgs_half(L, 0); rbgs_half(L, 1); }
    }
    residual(L);
    restrict_sum(L, &M->lev[l + 1]);
    vcycle(M, l + 1);
    prolong_add(L, &M->lev[l + 1], M->omega);
    if (M->line) {
        for (int s = 0; s < line_steps(M, l, 1); ++s) line_step(L, 1);
    } else {
        for (int s = 0; s < sweeps_at(M, l, 1); ++s) { rbgs_half(L, 1); rbgs_half(L, 0); }
    }
}

static double dot(const double *a, const double *b, size_t n) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (size_t k = 0; k < n; ++k) s += a[k] * b[k];
    return s;
}

static void apply_A(const olevel *L, const double *p, double *q) {
    int nx = L->nx, ny = L->ny;
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nx; ++ix) {
            size_t k = (size_t)iy * nx + ix;
            double s = (L->dg[k] > 0.0 ? L->dg[k] : 0.0) * p[k];
            if (ix + 1 < nx) s = s - L->cE[k] * p[k + 1];
            if (ix > 0) s = s - (L->cW ? L->cW[k] : L->cE[k - 1]) * p[k - 1];
            if (iy + 1 < ny) s = s - L->cN[k] * p[k + nx];
            if (iy > 0) s = s - (L->cS ? L->cS[k] : L->cN[k - nx]) * p[k - nx];
            q[k] = s;
        }
}

/*
 * Solve A x = b by MG-preconditioned CG.  cE, cN, dg, b, x are 0-based
 * (nx*ny, x fastest); x is output (initial guess zero).  Returns iterations;
 * *relres gets the recomputed ||b - A x|| / ||b||.
 * maxit<0 selects a fixed number of V-cycles per application (the HYPRE
 * setting of 10 cycles, src/ProjectionP_Mod.f90:130): ncyc = -maxit/1000,
 * iterations = (-maxit)%1000.
 */
int oracle_mgpcg(int nx, int ny, const double *cE, const double *cN, const double *dg,
                 const double *cW, const double *cS,
                 const double *b, double *x, double rtol, int maxit, int npre, int npost,
                 double omega, int coarse_max, double *relres, int *nlev_out, int smoother) {
    omg M;
    memset(&M, 0, sizeof(M));
    M.omega = omega; M.npre = npre; M.npost = npost; M.line = smoother == 1;
    M.cfrom = g_cfrom; M.csweeps = g_csweeps;
    int ncyc = 1;
    if (maxit < 0) { ncyc = (-maxit) / 1000; maxit = (-maxit) % 1000; if (ncyc < 1) ncyc = 1; }
    size_t n = (size_t)nx * ny;
    level_alloc(&M.lev[0], nx, ny);
    pcopy(M.lev[0].cE, cE, n);
    pcopy(M.lev[0].cN, cN, n);
    pcopy(M.lev[0].dg, dg, n);
    compute_excess(&M.lev[0]);
    M.nlev = 1;
    while (M.lev[M.nlev - 1].nx * M.lev[M.nlev - 1].ny > coarse_max && M.nlev < 32 &&
           (M.lev[M.nlev - 1].nx > 1 || M.lev[M.nlev - 1].ny > 1)) {
        coarsen(&M.lev[M.nlev - 1], &M.lev[M.nlev]);
        M.nlev++;
    }
    coarse_factor(&M);
    if (nlev_out) *nlev_out = M.nlev;
    /* the PCG applies the rows as assembled (the V-cycle never reads these) */
    olevel Fx = M.lev[0];
    Fx.cW = cW;
    Fx.cS = cS;
    olevel *F = &M.lev[0];
    double *r = dalloc(n), *z = dalloc(n), *p = dalloc(n), *q = dalloc(n);
    pzero(x, n);
    pcopy(r, b, n);
    double bnorm = sqrt(dot(b, b, n));
    int it = 0;
    if (bnorm == 0.0) { *relres = 0.0; goto done; }
    double rz = 0.0;
    for (it = 0; it < maxit; ++it) {
        /* z = M^{-1} r (ncyc V-cycles, each on the current residual) */
        pcopy(F->b, r, n);
        vcycle(&M, 0);
        pcopy(z, F->x, n);
        for (int c = 1; c < ncyc; ++c) {
            apply_A(&Fx, z, q);
#pragma omp parallel for schedule(static)
            for (size_t k = 0; k < n; ++k) F->b[k] = r[k] - q[k];
            vcycle(&M, 0);
#pragma omp parallel for schedule(static)
            for (size_t k = 0; k < n; ++k) z[k] += F->x[k];
        }
        double rz_new = dot(r, z, n);
        if (it == 0) pcopy(p, z, n);
        else {
            double beta = rz_new / rz;
#pragma omp parallel for schedule(static)
            for (size_t k = 0; k < n; ++k) p[k] = z[k] + beta * p[k];
        }
        rz = rz_new;
        apply_A(&Fx, p, q);
        double alpha = rz / dot(p, q, n);
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < n; ++k) { x[k] += alpha * p[k]; r[k] -= alpha * q[k]; }
        double rn = sqrt(dot(r, r, n));
        if (rn <= rtol * bnorm) { it++; break; }
    }
    apply_A(&Fx, x, q);
    {
        double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
        for (size_t k = 0; k < n; ++k) { double d = b[k] - q[k]; s += d * d; }
        *relres = sqrt(s) / bnorm;
    }
done:
    free(r); free(z); free(p); free(q);
    for (int l = 0; l < M.nlev; ++l) level_free(&M.lev[l]);
    free(M.chol); free(M.cmap);
    return it;
}

/*
 * The same MG-PCG taking the reference's matr(nx,ny,5) and rhm(nx,ny)
 * directly (Fortran layouts) and returning x in the (nx,ny) interior layout
 * (0 on cells with Posnu = -1); the storage conversions run on all threads.
 * This is the timed CPU baseline's solve: no Python work between assembly
 * and correction.
 */
int oracle_mgpcg_matr(int nx, int ny, const double *matr, const double *rhm,
                      const int32_t *posnu, double *xint, double rtol, int maxit, int npre,
                      int npost, double omega, int coarse_max, double *relres, int *nlev_out,
                      int smoother) {
    const size_t n = (size_t)nx * ny;
    double *cE = dalloc(n), *cN = dalloc(n), *dg = dalloc(n), *cW = dalloc(n), *cS = dalloc(n);
    double *b = dalloc(n), *x = dalloc(n);
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            const size_t k = (size_t)(j - 1) * nx + (i - 1);
            const int act = F0(posnu, i, j) != -1;
            cE[k] = act ? -MT(4, i, j) + 0.0 : 0.0;
            cN[k] = act ? -MT(5, i, j) + 0.0 : 0.0;
            cW[k] = act ? -MT(2, i, j) + 0.0 : 0.0;
            cS[k] = act ? -MT(1, i, j) + 0.0 : 0.0;
            dg[k] = act ? MT(3, i, j) : -1.0;
            b[k] = F1(rhm, i, j);
        }
    int it = oracle_mgpcg(nx, ny, cE, cN, dg, cW, cS, b, x, rtol, maxit, npre, npost, omega,
                          coarse_max, relres, nlev_out, smoother);
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i)
            F1(xint, i, j) = F0(posnu, i, j) != -1 ? x[(size_t)(j - 1) * nx + (i - 1)] : 0.0;
    free(cE); free(cN); free(dg); free(cW); free(cS); free(b); free(x);
    return it;
}

/* DeltaPressureGetValues + DeltaPressureBoundaryCondition from an (nx,ny)
 * interior solution (0 where Posnu = -1) instead of a Posnu-ordered vector */
void oracle_scatter_interior(int nx, int ny, const int32_t *posnu, const double *xint, int wb,
                             int eb, int sb, int nbc, double *Pp) {
    const size_t n0 = (size_t)(nx + 2) * (ny + 2);
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n0; ++k) Pp[k] = 0.0;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i)
            F0(Pp, i, j) = F0(posnu, i, j) != -1 ? F1(xint, i, j) : 0.0;
    for (int i = 1; i <= nx; ++i) {
        F0(Pp, i, 0) = (double)sb * F0(Pp, i, 1);
        F0(Pp, i, ny + 1) = (double)nbc * F0(Pp, i, ny);
    }
    for (int j = 1; j <= ny; ++j) {
        F0(Pp, 0, j) = (double)wb * F0(Pp, 1, j);
        F0(Pp, nx + 1, j) = (double)eb * F0(Pp, nx, j);
    }
}

/* one V-cycle on b (0-based), output x; exposed for bitwise tests */
void oracle_vcycle(int nx, int ny, const double *cE, const double *cN, const double *dg,
                   const double *b, double *x, int npre, int npost, double omega,
                   int coarse_max, int smoother) {
    omg M;
    memset(&M, 0, sizeof(M));
    M.omega = omega; M.npre = npre; M.npost = npost; M.line = smoother == 1;
    M.cfrom = g_cfrom; M.csweeps = g_csweeps;
    size_t n = (size_t)nx * ny;
    level_alloc(&M.lev[0], nx, ny);
    memcpy(M.lev[0].cE, cE, n * sizeof(double));
    memcpy(M.lev[0].cN, cN, n * sizeof(double));
    memcpy(M.lev[0].dg, dg, n * sizeof(double));
    compute_excess(&M.lev[0]);
    M.nlev = 1;
    while (M.lev[M.nlev - 1].nx * M.lev[M.nlev - 1].ny > coarse_max && M.nlev < 32 &&
           (M.lev[M.nlev - 1].nx > 1 || M.lev[M.nlev - 1].ny > 1)) {
        coarsen(&M.lev[M.nlev - 1], &M.lev[M.nlev]);
        M.nlev++;
    }
    coarse_factor(&M);
    memcpy(M.lev[0].b, b, n * sizeof(double));
    vcycle(&M, 0);
    memcpy(x, M.lev[0].x, n * sizeof(double));
    for (int l = 0; l < M.nlev; ++l) level_free(&M.lev[l]);
    free(M.chol); free(M.cmap);
}

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
