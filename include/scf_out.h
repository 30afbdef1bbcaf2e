/* scf_out.h -- result files of SIMCOFlow written from the GPU: the Tecplot
 * files and the ParaView (VTR) file.
 *
 * Replaces Print_Result_Tecplot_PCent / _UCent / _VCent
 * (src/PrintResult.f90:39-168): the same files, byte for byte, with the text
 * of every value ("(f24.14)": one value per line, 24 characters, 14 digits
 * after the decimal point) formatted by a GPU kernel from the fields where
 * they already are, then copied to the host through pinned 16 MiB chunks
 * that a writer thread passes on while the next chunks are still in flight.
 *
 * Number format (Fortran F24.14): right-justified in 24 characters, a minus
 * sign for negative values (negative zero and negative values that round to
 * zero included), a leading "0" before the decimal point, the decimal value
 * of the binary number rounded to 14 fractional digits (ties to even),
 * 24 asterisks where the number does not fit, "NaN", "Infinity" and
 * "-Infinity" right-justified for the special values.
 *
 * Arrays are the reference's Fortran arrays (column-major):
 *   (nx,ny)          (1:Isize,1:Jsize)
 *   (nx+2,ny+2)      (0:Isize+1,0:Jsize+1)
 *   (nx+2,ny+2,2)    Flux_n1(0:Isize+1,0:Jsize+1,2) (src/Solver_Mod.f90:49)
 * as host pointers, or device pointers with SCF_OUT_DEVICE_PTRS.
 * Errors are status codes (scf_proj.h's SCF_ERR_*); no CPU fallback.
 */
#ifndef SCF_OUT_H
#define SCF_OUT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SCF_OUT_DEVICE_PTRS 1

/* Print_Result_Tecplot_PCent's fields (src/PrintResult.f90:39-110) */
typedef struct scf_tecplot_pcell {
  const double *x, *y;              /* PGrid%x, %y (nx,ny) */
  const double *p, *u, *v;          /* TVar%p, %u, %v (nx+2,ny+2) */
  const double *phi, *vof;          /* PCell%phi, %vof (nx,ny) */
  const double *phiS, *vofS;        /* PCell%phiS, %vofS (nx,ny) */
  const double *mres;               /* TVar%mres (nx,ny) */
  const double *flux;               /* Flux_n1 (nx+2,ny+2,2) */
  const double *nxS, *nyS;          /* PCell%nxS, %nyS (nx,ny) */
} scf_tecplot_pcell;

/* Print_Result_Tecplot_UCent / _VCent's fields (src/PrintResult.f90:112-168) */
typedef struct scf_tecplot_vcell {
  const double *x, *y;              /* UGrid (VGrid) %x, %y (nx,ny) */
  const double *vel;                /* TVar%u (TVar%v) (nx+2,ny+2) */
  const double *phi, *vof;          /* UCell (VCell) %phi, %vof (nx,ny) */
  const double *phiS, *vofS;        /* UCell (VCell) %phiS, %vofS (nx,ny) */
} scf_tecplot_vcell;

#define SCF_TECPLOT_PCELL 0 /* Pressure_<iter>.dat */
#define SCF_TECPLOT_UCELL 1 /* Uvelocity_<iter>.dat */
#define SCF_TECPLOT_VCELL 2 /* Vvelocity_<iter>.dat */

/* Bytes of the file of `kind` for an nx-by-ny grid. */
int64_t scf_tecplot_size(int kind, int nx, int ny);

/* The whole file text of `kind` into buf (capacity cap bytes, host memory;
 * *len receives the size).  fields: a scf_tecplot_pcell for
 * SCF_TECPLOT_PCELL, a scf_tecplot_vcell otherwise. */
int scf_tecplot_text(int kind, int nx, int ny, const void *fields, int flags, char *buf,
                     int64_t cap, int64_t *len, int device);

/* Write the file dir/Tecplot/<name>_<iter as %08d>.dat (the reference's
 * file name; the Tecplot/ directory must exist, as in the reference).  ms,
 * when not NULL, receives the elapsed wall time. */
int scf_tecplot_write(int kind, int nx, int ny, const void *fields, int flags, int64_t iter,
                      const char *dir, int device, double *ms);

/* The records only (the file without its three header lines) into the
 * device buffer dev_text (nvars * nx * ny * 25 bytes: 15 variables for
 * SCF_TECPLOT_PCELL, 8 otherwise), enqueued on `stream` (a cudaStream_t;
 * NULL for the legacy default stream); fields are device pointers.  For
 * callers that move the text on themselves (another file system, a network
 * sink); no counterpart in the reference. */
int scf_tecplot_format(int kind, int nx, int ny, const void *fields, char *dev_text,
                       void *stream);

/* Diagnostics: format n doubles (host arrays) as F24.14 into out (24*n
 * bytes, no line ends). */
int scf_format_f24_14(const double *v, int64_t n, char *out, int device);

/* ---- ParaView file: Print_Result_VTK_2D (src/PrintResult.f90:165-190)
 * through VTR_open_file / VTR_write_mesh / VTR_write_var / VTR_close_file
 * (src/VTR_mod.f90:79-379).  The XML records are the module's, byte for
 * byte.  The values are REAL(4) (real(x, kind=4), round to nearest) in
 * list-directed output, whose text the Fortran standard leaves to the
 * compiler; this library writes each value as a blank and 15 characters
 * (the sign or a blank, then the correctly rounded "%.8E" of the exact
 * REAL(4) value: 9 significant digits, which read back to the same REAL(4);
 * "NaN", "Infinity", "-Infinity" right-justified), five values per record. */
typedef struct scf_vtr_fields {
  const double *x, *y;              /* TGrid%x, %y (nx,ny): x(:,1), y(1,:) are written */
  const double *u, *v, *p;          /* TVar%u, %v, %p (nx+2,ny+2): (1:nx,1:ny) written */
  const double *phi, *phiS;         /* TCell%phi, %phiS (nx,ny) */
  const double *vof, *vofS;         /* TCell%vof, %vofS (nx,ny) */
} scf_vtr_fields;

/* Bytes of the file for an nx-by-ny grid. */
int64_t scf_vtr_size(int nx, int ny);

/* The whole file text into buf (host memory, capacity cap; *len receives
 * the size). */
int scf_vtr_text(int nx, int ny, const scf_vtr_fields *fields, int flags, char *buf, int64_t cap,
                 int64_t *len, int device);

/* Write dir/Paraview/FlowField_<iter as %08d>.vtr (the reference's name; the
 * Paraview/ directory must exist).  ms, when not NULL, receives the elapsed
 * wall time. */
int scf_vtr_write(int nx, int ny, const scf_vtr_fields *fields, int flags, int64_t iter,
                  const char *dir, int device, double *ms);

/* Diagnostics: the 15 characters of real(v[k], kind=4) for n doubles (host
 * arrays) into out (15*n bytes, no separators). */
int scf_format_e15_8(const double *v, int64_t n, char *out, int device);

#ifdef __cplusplus
}
#endif
#endif
