/*
 * out_oracle.c -- CPU restatement of SIMCOFlow's Tecplot result files:
 * Print_Result_Tecplot_PCent / _UCent / _VCent (src/PrintResult.f90:39-168).
 *
 * TEST INFRASTRUCTURE ONLY: only tests/, smoke() and the CPU-baseline leg of
 * bench.py load it; the product path never calls it.
 * Parity status: UNPINNED against the reference binary (no Fortran compiler
 * here); the number format is the F edit descriptor of the Fortran standard
 * as gfortran prints it, restated through the C library's correctly rounded
 * "%24.14f" (round to nearest, ties to even, on the exact binary value).
 *
 * Records (one value per record, "(f24.14)", i fastest, as the implied DO
 * loops ((a(i,j),i=1,nx),j=1,ny) write them):
 *   F24.14: 24 characters, right-justified, leading "0" before the point, a
 *   minus sign for negative values (also when they round to zero); 24
 *   asterisks when the number does not fit; "NaN", "Infinity", "-Infinity"
 *   right-justified.
 * Headers: list-directed character output (a leading blank, adjacent
 * character items not separated) and format (1x,'zone i=',i5,',k=',i5,
 * ',f=block').
 * Arrays: (nx,ny) = (1:nx,1:ny); (nx+2,ny+2) = (0:nx+1,0:ny+1); flux =
 * Flux_n1(0:nx+1,0:ny+1,2).
 *
 * Also the ParaView file of Print_Result_VTK_2D (src/PrintResult.f90:165-190)
 * through the VTR module (src/VTR_mod.f90:79-379): XML records "(100A)"
 * exactly as the module writes them, and the values as REAL(4)
 * (real(x, kind=4): round to nearest) in list-directed output.  The text of
 * a list-directed real is processor-dependent (the Fortran standard leaves
 * its layout to the compiler), so this format is defined here, not taken
 * from a compiler: every value is a blank and 15 characters, the sign ('-'
 * or a blank) and the correctly rounded "%.8E" of the exact value (9
 * significant digits, enough to give back the same REAL(4)); "NaN",
 * "Infinity", "-Infinity" right-justified in the 15; five values per record.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

/* F24.14 of x into o[0..23] (no terminator) */
void oracle_f24_14(double x, char *o) {
  char b[64];
  const char *word = NULL;
  if (isnan(x)) word = "NaN";
  else if (isinf(x)) word = x < 0 ? "-Infinity" : "Infinity";
  if (word) {
    const int n = (int)strlen(word);
    memset(o, ' ', 24 - n);
    memcpy(o + 24 - n, word, n);
    return;
  }
  const int n = snprintf(b, sizeof b, "%24.14f", x);
  if (n != 24) {
    memset(o, '*', 24);
    return;
  }
  memcpy(o, b, 24);
}

void oracle_format_many(const double *v, int64_t n, char *out) {
  for (int64_t k = 0; k < n; ++k) oracle_f24_14(v[k], out + 24 * k);
}

#define A1(a, i, j) (a)[(size_t)((i) - 1) + (size_t)((j) - 1) * (size_t)nx]
#define A0(a, i, j) (a)[(size_t)(i) + (size_t)(j) * (size_t)(nx + 2)]

static char *put_header(char *p, const char *vars, int nx, int ny) {
  p += sprintf(p, " title = \"flow\"\n");
  p += sprintf(p, " variables =%s\n", vars);
  char bi[16], bk[16];
  if (nx > 99999) strcpy(bi, "*****"); else sprintf(bi, "%5d", nx);
  if (ny > 99999) strcpy(bk, "*****"); else sprintf(bk, "%5d", ny);
  p += sprintf(p, " zone i=%s,k=%s,f=block\n", bi, bk);
  return p;
}

/* one block of records; kind: 0 = a(i,j) of (nx,ny), 1 = a(i,j) of
 * (0:nx+1,0:ny+1), 2 = 0.5*(a(i-1,j)+a(i,j)), 3 = 0.5*(a(i,j-1)+a(i,j)),
 * 4 = 1 - a(i,j) - b(i,j) */
static char *put_block(char *p, int kind, const double *a, const double *b, int nx, int ny) {
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      char *r = p + ((size_t)(j - 1) * nx + (i - 1)) * 25;
      double v;
      switch (kind) {
        case 0: v = A1(a, i, j); break;
        case 1: v = A0(a, i, j); break;
        case 2: v = 0.5 * (A0(a, i - 1, j) + A0(a, i, j)); break;
        case 3: v = 0.5 * (A0(a, i, j - 1) + A0(a, i, j)); break;
        default: v = 1.0 - A1(a, i, j) - A1(b, i, j); break;
      }
      oracle_f24_14(v, r);
      r[24] = '\n';
    }
  return p + (size_t)nx * ny * 25;
}

/* Print_Result_Tecplot_PCent without the particle files; returns bytes */
int64_t oracle_tecplot_pcell(int nx, int ny, const double *x, const double *y, const double *pr,
                             const double *u, const double *v, const double *phi,
                             const double *vof, const double *phiS, const double *vofS,
                             const double *mres, const double *flux, const double *nxS,
                             const double *nyS, char *buf) {
  char *p = put_header(buf,
                       "\"x\",\"y\",\"p\",\"u\",\"v\",\"phi\",\"vof\",\"phiS\",\"vofS\","
                       "\"vofA\",\"Mres\",\"FluxU\",\"FluxV\",\"nxS\",\"nyS\"",
                       nx, ny);
  const size_t n0 = (size_t)(nx + 2) * (ny + 2);
  p = put_block(p, 0, x, NULL, nx, ny);
  p = put_block(p, 0, y, NULL, nx, ny);
  p = put_block(p, 1, pr, NULL, nx, ny);   /* p(i,j) either branch of :54-58 */
  p = put_block(p, 2, u, NULL, nx, ny);
  p = put_block(p, 3, v, NULL, nx, ny);
  p = put_block(p, 0, phi, NULL, nx, ny);
  p = put_block(p, 0, vof, NULL, nx, ny);
  p = put_block(p, 0, phiS, NULL, nx, ny);
  p = put_block(p, 0, vofS, NULL, nx, ny);
  p = put_block(p, 4, vof, vofS, nx, ny);
  p = put_block(p, 0, mres, NULL, nx, ny);
  p = put_block(p, 1, flux, NULL, nx, ny);
  p = put_block(p, 1, flux + n0, NULL, nx, ny);
  p = put_block(p, 0, nxS, NULL, nx, ny);
  p = put_block(p, 0, nyS, NULL, nx, ny);
  return (int64_t)(p - buf);
}

/* Print_Result_Tecplot_UCent (comp = 0) / _VCent (comp = 1) */
int64_t oracle_tecplot_vcell(int comp, int nx, int ny, const double *x, const double *y,
                             const double *vel, const double *phi, const double *vof,
                             const double *phiS, const double *vofS, char *buf) {
  char *p = put_header(buf,
                       comp == 0 ? "\"x\",\"y\",\"u\",\"phi\",\"vof\",\"phiS\",\"vofS\",\"vofA\""
                                 : "\"x\",\"y\",\"v\",\"phi\",\"vof\",\"phiS\",\"vofS\",\"vofA\"",
                       nx, ny);
  p = put_block(p, 0, x, NULL, nx, ny);
  p = put_block(p, 0, y, NULL, nx, ny);
  p = put_block(p, 1, vel, NULL, nx, ny);
  p = put_block(p, 0, phi, NULL, nx, ny);
  p = put_block(p, 0, vof, NULL, nx, ny);
  p = put_block(p, 0, phiS, NULL, nx, ny);
  p = put_block(p, 0, vofS, NULL, nx, ny);
  p = put_block(p, 4, vof, vofS, nx, ny);
  return (int64_t)(p - buf);
}

/* ------------------------------------------------------------------------
 * ParaView VTR file (src/PrintResult.f90:165-190, src/VTR_mod.f90)
 * ------------------------------------------------------------------------ */

/* the 15 characters of one REAL(4) value */
void oracle_e15_8(double x, char *o) {
  const float f = (float)x;
  const char *word = NULL;
  if (isnan(f)) word = "NaN";
  else if (isinf(f)) word = f < 0 ? "-Infinity" : "Infinity";
  if (word) {
    const int n = (int)strlen(word);
    memset(o, ' ', 15 - n);
    memcpy(o + 15 - n, word, n);
    return;
  }
  char b[32];
  const int n = snprintf(b, sizeof b, "%.8E", (double)f);
  memset(o, ' ', 15);
  memcpy(o + 15 - n, b, n);
}

void oracle_format_e15_8(const double *v, int64_t n, char *out) {
  for (int64_t k = 0; k < n; ++k) oracle_e15_8(v[k], out + 15 * k);
}

/* list-directed record(s) of n values: value k is a blank and its 15
 * characters; a line end after every fifth value and after the last */
static char *put_values(char *p, int64_t n, double (*get)(const void *, int64_t),
                        const void *ctx) {
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < n; ++k) {
    char *o = p + k * 16 + k / 5;  /* after k values and k / 5 line ends */
    o[0] = ' ';
    oracle_e15_8(get(ctx, k), o + 1);
    if (k % 5 == 4 || k == n - 1) o[16] = '\n';
  }
  return p + n * 16 + (n + 4) / 5;
}

struct vtr_ctx {
  int nx, ny;
  const double *a, *b;
};
static double get_x(const void *c, int64_t k) {  /* x(i,1) */
  const struct vtr_ctx *q = c;
  return q->a[k];
}
static double get_y(const void *c, int64_t k) {  /* y(1,j) */
  const struct vtr_ctx *q = c;
  return q->a[(size_t)k * q->nx];
}
static double get_zero(const void *c, int64_t k) {
  (void)c;
  (void)k;
  return 0.0;
}
static double get_11(const void *c, int64_t k) {  /* a(i,j) of (nx,ny) */
  const struct vtr_ctx *q = c;
  return q->a[k];
}
static double get_00(const void *c, int64_t k) {  /* a(i,j) of (0:nx+1,0:ny+1) */
  const struct vtr_ctx *q = c;
  const int64_t i = k % q->nx + 1, j = k / q->nx + 1;
  return q->a[(size_t)i + (size_t)j * (q->nx + 2)];
}
static double get_vel3(const void *c, int64_t k) {  /* (u, v, 0) per point */
  const struct vtr_ctx *q = c;
  const int64_t cell = k / 3, comp = k % 3;
  if (comp == 2) return 0.0;
  const int64_t i = cell % q->nx + 1, j = cell / q->nx + 1;
  return (comp == 0 ? q->a : q->b)[(size_t)i + (size_t)j * (q->nx + 2)];
}

/* integer of "(I6)" after trim(adjustl()) */
static void i6(int v, char *b) {
  if (v < -99999 || v > 999999) strcpy(b, "******");
  else sprintf(b, "%d", v);
}

/* Print_Result_VTK_2D: x, y (nx,ny); u, v, pr (0:nx+1,0:ny+1); phi, phiS,
 * vof, vofS (nx,ny).  Returns the bytes written into buf. */
int64_t oracle_vtr(int nx, int ny, const double *x, const double *y, const double *u,
                   const double *v, const double *pr, const double *phi, const double *phiS,
                   const double *vof, const double *vofS, char *buf) {
  char *p = buf, ni[16], nj[16];
  i6(nx, ni);
  i6(ny, nj);
  struct vtr_ctx c = {nx, ny, NULL, NULL};
  const int64_t n = (int64_t)nx * ny;
  p += sprintf(p, "<VTKFile type=\"RectilinearGrid\" version=\"0.1\" format=\"ascii\">\n");
  p += sprintf(p, " <RectilinearGrid WholeExtent=\"1 %s 1 %s 1 1 \">\n", ni, nj);
  p += sprintf(p, "  <Piece Extent=\"1 %s 1 %s 1 1 \">\n", ni, nj);
  p += sprintf(p, "   <Coordinates>\n");
  const char *axes[3] = {"X", "Y", "Z"};
  for (int a = 0; a < 3; ++a) {
    p += sprintf(p, "    <DataArray type=\"Float32\" Name=\"%s_COORDINATES\" "
                    "NumberOfComponents=\"1\" format=\"ascii\">\n", axes[a]);
    c.a = a == 0 ? x : y;
    p = a == 0 ? put_values(p, nx, get_x, &c)
        : a == 1 ? put_values(p, ny, get_y, &c) : put_values(p, 1, get_zero, &c);
    p += sprintf(p, "    </DataArray>\n");
  }
  p += sprintf(p, "   </Coordinates>\n");
  p += sprintf(p, "   <PointData>\n");
  /* VTR_write_vector_2d (src/VTR_mod.f90:212-262) */
  const char *vnames[3] = {"Velocity", "X_Velocity", "Y_Velocity"};
  for (int a = 0; a < 3; ++a) {
    p += sprintf(p, "        <DataArray type=\"Float32\" Name=\"%s\" NumberOfComponents=\"%d\" "
                    "format=\"ascii\">\n", vnames[a], a == 0 ? 3 : 1);
    c.a = a == 2 ? v : u;
    c.b = v;
    p = a == 0 ? put_values(p, 3 * n, get_vel3, &c) : put_values(p, n, get_00, &c);
    p += sprintf(p, "        </DataArray>\n");
  }
  /* VTR_write_scalar_2d (src/VTR_mod.f90:330-344) */
  const char *snames[5] = {"Pressure", "Levelset", "SolidLvs", "Vof", "SolidVof"};
  const double *sarr[5] = {pr, phi, phiS, vof, vofS};
  for (int a = 0; a < 5; ++a) {
    p += sprintf(p, "         <DataArray type=\"Float32\" Name=\"%s\" NumberOfComponents=\"1\" "
                    "format=\"ascii\">\n", snames[a]);
    c.a = sarr[a];
    p = put_values(p, n, a == 0 ? get_00 : get_11, &c);
    p += sprintf(p, "         </DataArray>\n");
  }
  /* VTR_close_file (src/VTR_mod.f90:363-379) */
  p += sprintf(p, "     </PointData>\n   </Piece>\n  </RectilinearGrid>\n</VTKFile>\n");
  return (int64_t)(p - buf);
}
