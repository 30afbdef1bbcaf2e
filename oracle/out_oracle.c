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
