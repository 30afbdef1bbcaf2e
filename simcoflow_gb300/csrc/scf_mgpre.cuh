// scf_mgpre.cuh -- the projection's FP64 multigrid V-cycle as a
// preconditioner of another 5-point operator on the same padded layout
// (scf_proj.cu); used by the momentum predictor's implicit solves.
#pragma once
#include <cuda_runtime.h>

struct scf_proj;

namespace scf {
// An FP64 point-smoothed multigrid handle of nx x ny cells on the device
// (device-pointer mode, direct launches).
int mgpre_create(scf_proj** out, int nx, int ny, int device);
// Setup from the operator's entries P (diagonal; <= 0: no unknown), W, E,
// S, N (the off-diagonal entries as they stand in the matrix), device arrays
// in the padded layout (pitch round_up(nx + 2, 32), zero ghosts): the
// multigrid works on the symmetric part, couplings max(0, -(E_i + W_i+1) / 2)
// and max(0, -(N_j + S_j+1) / 2), with Galerkin coarsening below it.
int mgpre_setup(scf_proj* h, const double* P, const double* W, const double* E,
                const double* S, const double* N, cudaStream_t s);
// z = one V-cycle applied to b (padded arrays; z's ghosts stay zero)
int mgpre_apply(scf_proj* h, double* b, double* z, cudaStream_t s);
}  // namespace scf
