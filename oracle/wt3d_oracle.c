/*
 * CPU oracle for the wtomo3d forward-modelling hot path.
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker; the product never calls it.
 * See wt3d_oracle.h for what is restated and how parity is pinned.
 */
#include "wt3d_oracle.h"
#include <stdlib.h>
#include <string.h>
#include <math.h>

/* ---------------------------------------------------------------------- */
/* Pattern: srel3d_getsize / srel3d (srgraphs.f:626-734), SPARSE_ADJ2CRS   */
/* (sparse.f:13-49).                                                       */
/* ---------------------------------------------------------------------- */
void ora_srel3d_getsize(int nx, int ny, int nz, long long *numvert, long long *nedge)
{
    long long x = nx, y = ny, z = nz;
    *numvert = 3 * x * y * z;
    *nedge = 120 * x * y * z - 81 * (x * y + x * z + y * z) + 54 * (x + z + y) - 36;
}

/* George-Liu adjacency of the 3-dof 27-point graph without the diagonal,
 * rows in node order, columns ascending (srgraphs.f:665-727). */
static int srel3d(int nx, int ny, int nz, long long *xadj, int *adjncy)
{
    long long nvto = 1, iter = 0, nedger = 0;
    for (int iy = 1; iy <= ny; iy++) {
        int ym = iy - 1 < 1 ? 1 : iy - 1, yp = iy + 1 > ny ? ny : iy + 1;
        for (int ix = 1; ix <= nx; ix++) {
            int xm = ix - 1 < 1 ? 1 : ix - 1, xp = ix + 1 > nx ? nx : ix + 1;
            for (int iz = 1; iz <= nz; iz++) {
                int zm = iz - 1 < 1 ? 1 : iz - 1, zp = iz + 1 > nz ? nz : iz + 1;
                long long ngrid = iz + (long long)(ix - 1) * nz + (long long)(iy - 1) * nx * nz;
                for (int irow = 1; irow <= 3; irow++) {
                    long long nvt = 0;
                    for (int j = ym; j <= yp; j++)
                        for (int i = xm; i <= xp; i++)
                            for (int k = zm; k <= zp; k++) {
                                long long igrid = k + (long long)(i - 1) * nz + (long long)(j - 1) * nx * nz;
                                long long iu = 3 * igrid - 2;
                                for (int c = 1; c <= 3; c++, iu++) {
                                    if (igrid != ngrid || irow != c) {
                                        adjncy[nedger++] = (int)iu;
                                        nvt++;
                                    }
                                }
                            }
                    xadj[iter++] = nvto;
                    nvto += nvt;
                }
            }
        }
    }
    xadj[iter] = nvto;
    return 0;
}

int ora_pattern(int nx, int ny, int nz, int *irptr, int *jcptr)
{
    long long n, nedge;
    ora_srel3d_getsize(nx, ny, nz, &n, &nedge);
    long long nzero = 2 * nedge + n;
    long long *xadj = (long long *)malloc(sizeof(long long) * (n + 1));
    int *adjncy = (int *)malloc(sizeof(int) * (2 * nedge));
    if (!xadj || !adjncy) { free(xadj); free(adjncy); return 1; }
    srel3d(nx, ny, nz, xadj, adjncy);
    if (xadj[n] - 1 != 2 * nedge) { free(xadj); free(adjncy); return 2; }
    /* SPARSE_ADJ2CRS: insert the diagonal before the first larger column;
     * the last row gets it appended (sparse.f:28-48). */
    long long izero = 0;
    irptr[0] = 1;
    for (long long i = 1; i <= n; i++) {
        long long jbeg = xadj[i - 1], jend = xadj[i] - 1;
        int ldiag = 0;
        for (long long j = jbeg; j <= jend; j++) {
            if (!ldiag && adjncy[j - 1] > i) {
                jcptr[izero++] = (int)i;
                ldiag = 1;
            }
            jcptr[izero++] = adjncy[j - 1];
        }
        irptr[i] = (int)(izero + 1);
    }
    jcptr[izero++] = (int)n;
    irptr[n] = (int)(nzero + 1);
    free(xadj); free(adjncy);
    return izero == nzero ? 0 : 3;
}

void ora_spmv_c128(int n, const int *irptr, const int *jcptr, const double complex *a,
                   const double complex *x, double complex *y)
{
    for (int i = 0; i < n; i++) {
        double complex s = 0;
        for (int k = irptr[i] - 1; k < irptr[i + 1] - 1; k++) s += a[k] * x[jcptr[k] - 1];
        y[i] = s;
    }
}

long long ora_point_source(const ora_grid *g, double xloc, double yloc, double zloc,
                           int comp, double complex sterm, double complex *rhs)
{
    /* srcsetup.f:55-57 (REAL arithmetic in the reference) */
    int ixs = (int)(0.5f + (float)(xloc / g->dx)) + 1;
    int iys = (int)(0.5f + (float)(yloc / g->dx)) + 1;
    int izs = (int)(0.5f + (float)(zloc / g->dx)) + 1;
    long long n = 3LL * g->nx * g->ny * g->nz;
    for (long long i = 0; i < n; i++) rhs[i] = 0;
    if (ixs < 1 || ixs > g->nx || iys < 1 || iys > g->ny || izs < 1 || izs > g->nz) return -1;
    long long node = izs + (long long)(ixs - 1) * g->nz + (long long)(iys - 1) * g->nx * g->nz;
    rhs[3 * (node - 1) + comp] = sterm;
    return node;
}

/* ---------------------------------------------------------------------- */
/* Assembly in complex128 and complex64                                    */
/* ---------------------------------------------------------------------- */
#define RT double
#define CT double complex
#define SQRTC csqrt
#define CREALC creal
#define LOGR log
#define FN(x) x##_c128
#include "asm_impl.inc"
#undef RT
#undef CT
#undef SQRTC
#undef CREALC
#undef LOGR
#undef FN

#define RT float
#define CT float complex
#define SQRTC csqrtf
#define CREALC crealf
#define LOGR logf
#define FN(x) x##_c64
#include "asm_impl.inc"
#undef RT
#undef CT
#undef SQRTC
#undef CREALC
#undef LOGR
#undef FN

int ora_assemble_c128(const ora_grid *g, const float *vp, const float *vs, const float *rho,
                      double omega_re, double omega_im, const int *irptr, double complex *a)
{
    return assemble_c128(g, vp, vs, rho, omega_re, omega_im, irptr, a);
}

int ora_assemble_c64(const ora_grid *g, const float *vp, const float *vs, const float *rho,
                     double omega_re, double omega_im, const int *irptr, float complex *a)
{
    return assemble_c64(g, vp, vs, rho, omega_re, omega_im, irptr, a);
}

int ora_node_blocks_c128(const ora_grid *g, const float *vp, const float *vs, const float *rho,
                         double omega_re, double omega_im, int iz, int ix, int iy,
                         double complex *blk, int *active)
{
    return node_blocks_c128(g, vp, vs, rho, omega_re, omega_im, iz, ix, iy, blk, active);
}
