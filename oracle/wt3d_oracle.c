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

/* ---------------------------------------------------------------------- */
/* SRCSETUP with ireg > 0 (srcsetup.f:78-211) over SRCREG (srcreg.f:77-304) */
/* in FP64.  I0 from its power series sum_k ((x/2)^k / k!)^2; the         */
/* reference evaluates it by a rational approximation in REAL.            */
/* ---------------------------------------------------------------------- */
static double ora_i0(double x)
{
    double t = 1.0, s = 1.0, q = 0.25 * x * x;
    for (int k = 1; k < 200; k++) {
        t *= q / ((double)k * (double)k);
        s += t;
        if (t < 1e-17 * s) break;
    }
    return s;
}

static double ora_sinc(int ireg, double x)
{
    const double pi = 3.141592653589793;
    double a, lx, v = (x <= 1e-10) ? 1.0 : sin(pi * x) / (pi * x);
    switch (ireg) {   /* srcreg.f:206-226 */
    case 1: a = 1.24; break;
    case 2: a = 2.94; break;
    case 3: a = 4.53; break;
    case 4: a = 6.31; break;
    case 5: a = 7.91; break;
    case 6: a = 9.42; break;
    case 7: a = 10.95; break;
    case 8: a = 12.53; break;
    case 9: a = 14.09; break;
    default: a = 14.18;
    }
    lx = x / (double)ireg;
    if (lx < 1.0) return v * ora_i0(a * sqrt(1.0 - lx * lx)) / ora_i0(a);
    return 0.0;
}

static double ora_dirac(double h, double x)
{
    if (x < h) return (1.0 - x * x / (2.0 * h * h)) / (2.0 * h);
    if (x < 2.0 * h) return (1.0 + (x * x - 4.0 * x * h) / (4.0 * h * h)) / h;
    return 0.0;
}

int ora_source_weights(const ora_grid *g, double xloc, double yloc, double zloc, int ireg, double sprd,
                       double complex sterm, double complex *swave)
{
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    const double dx = g->dx;
    double fs[17][17][17];   /* (iz, ix, iy), 1-based as srcreg */
    int ixs, iys, izs, half, lenw, ix, iy, iz;
    double xoff, yoff, zoff, xs, ys, zs, amp = 1.0;
    if (ireg <= 0) return 1;
    ixs = (int)(xloc / dx) + 1; iys = (int)(yloc / dx) + 1; izs = (int)(zloc / dx) + 1;
    xoff = xloc - (ixs - 1) * dx; yoff = yloc - (iys - 1) * dx; zoff = zloc - (izs - 1) * dx;
    if (sprd <= 0.5) { half = ireg; lenw = 2 * ireg + 1; }
    else { if (sprd <= 1e-10) return 1; half = (int)(2 * sprd); lenw = (int)(4 * sprd) + 1; }
    if (lenw > 16) return 1;
    xs = half + 1 + xoff / dx; ys = half + 1 + yoff / dx; zs = half + 1 + zoff / dx;
    if (sprd > 0.5) amp = 0.0;
    for (iy = 1; iy <= lenw; iy++)
        for (ix = 1; ix <= lenw; ix++)
            for (iz = 1; iz <= lenw; iz++) {
                double v;
                if (sprd <= 0.5)
                    v = ora_sinc(ireg, fabs(iz - zs)) * ora_sinc(ireg, fabs(iy - ys)) * ora_sinc(ireg, fabs(ix - xs));
                else
                    v = ora_dirac(sprd, fabs(iz - zs)) * ora_dirac(sprd, fabs(iy - ys)) * ora_dirac(sprd, fabs(ix - xs));
                fs[iz][ix][iy] = v;
                if (sprd > 0.5) amp += v;
            }
    {
        int izmins = izs - half, izmaxs = izs + half, ixmins = ixs - half, ixmaxs = ixs + half;
        int iymins = iys - half, iymaxs = iys + half;
        int izmin = izmins, izmax = izmaxs, ixmin = ixmins, ixmax = ixmaxs, iymin = iymins, iymax = iymaxs;
        if (izmin < 1 && !g->fst) izmin = 1;   /* freesurf(1): top; other faces absorbing */
        if (izmax > nz) izmax = nz;
        if (ixmin < 1) ixmin = 1;
        if (ixmax > nx) ixmax = nx;
        if (iymin < 1) iymin = 1;
        if (iymax > ny) iymax = ny;
        for (iz = izmin; iz <= izmax; iz++) {
            int izsrg = iz - izmins + 1, izfs = iz < 1 ? 2 - iz : (iz > nz ? 2 * nz - iz : iz);
            if (izfs < 1 || izfs > nz) continue;
            for (ix = ixmin; ix <= ixmax; ix++) {
                int ixsrg = ix - ixmins + 1;
                for (iy = iymin; iy <= iymax; iy++) {
                    int iysrg = iy - iymins + 1;
                    long long off = (long long)(izfs - 1) + (long long)nz * (ix - 1) + (long long)nz * nx * (iy - 1);
                    double f = fs[izsrg][ixsrg][iysrg] / amp;
                    if (iz == izfs) swave[off] += f * sterm;
                    else swave[off] -= f * sterm;
                }
            }
        }
    }
    return 0;
}

/* ---------------------------------------------------------------------- */
/* Adjoint-state gradient in FP64 by central differences of node blocks.  */
/* The reference has no gradient code on this path; this differentiates   */
/* the restated ASMBLE operator numerically, independently of the GPU's    */
/* analytic per-row derivatives.  For every node g and each of lambda, mu  */
/* and rho (the Lame arrays of modelio.f90:78-92), the array entry at g is */
/* moved by +-h (h = 1e-6 of the node's stiffness or density scale) and    */
/* the blocks of the 27 rows that read node g are recomputed               */
/* (setcoefs3d + fdfd3d, asmble.f90:96-601):                               */
/*     dchi/dp = -Re sum_j lam_j^H (dA/dp) u_j,                            */
/* then mu = Vs^2 rho, lambda = Vp^2 rho - 2 mu give (Vp, Vs, rho).        */
/* ---------------------------------------------------------------------- */
static void row_blocks_c128(const ora_grid *g, const double complex *da, const double complex *mu,
                            const double *ro, double complex om, double pmld, double pmlf, int ipml,
                            int iz, int ix, int iy, double complex blk[27][3][3], int act[27])
{
    coefs_c128 c;
    setcoefs3d_c128(g, da, mu, ro, iz, ix, iy, &c);
    for (int s = 0; s < 27; s++) {
        act[s] = slot_active_c128(g, s, iz, ix, iy);
        if (act[s]) fdfd3d_c128(g, &c, om, g->dx, pmld, pmlf, ipml, s, iz, ix, iy, blk[s]);
    }
}

int ora_gradient_c128(const ora_grid *g, const float *vp, const float *vs, const float *rho,
                      double omega_re, double omega_im, int nrhs, const double complex *U,
                      const double complex *L, double *grad)
{
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    const long long nn = (long long)nx * ny * nz, n = 3 * nn;
    double complex *da = (double complex *)malloc(sizeof(double complex) * nn);
    double complex *mu = (double complex *)malloc(sizeof(double complex) * nn);
    double *ro = (double *)malloc(sizeof(double) * nn);
    if (!da || !mu || !ro) { free(da); free(mu); free(ro); return 1; }
    lame_c128(nn, vp, vs, rho, da, mu, ro);
    double pmld, pmlf; int ipml;
    pml_params_c128(g, &pmld, &pmlf, &ipml);
    const double complex om = omega_re + omega_im * I;
    for (int iy = 1; iy <= ny; iy++)
    for (int ix = 1; ix <= nx; ix++)
    for (int iz = 1; iz <= nz; iz++) {
        const long long off = (iz - 1) + (long long)nz * (ix - 1) + (long long)nz * nx * (iy - 1);
        const double scale_s = fmax(fabs(creal(da[off])), fabs(creal(mu[off])));
        double dl[3];
        for (int p = 0; p < 3; p++) {
            const double h = 1e-6 * (p < 2 ? scale_s : ro[off]);
            double complex acc = 0;
            for (int ry = iy - 1; ry <= iy + 1; ry++)
            for (int rx = ix - 1; rx <= ix + 1; rx++)
            for (int rz = iz - 1; rz <= iz + 1; rz++) {
                if (ry < 1 || ry > ny || rx < 1 || rx > nx || rz < 1 || rz > nz) continue;
                double complex bp[27][3][3], bm[27][3][3];
                int act[27];
                for (int sg = 0; sg < 2; sg++) {
                    const double d = sg == 0 ? h : -h;
                    if (p == 0) da[off] += d; else if (p == 1) mu[off] += d; else ro[off] += d;
                    row_blocks_c128(g, da, mu, ro, om, pmld, pmlf, ipml, rz, rx, ry, sg == 0 ? bp : bm, act);
                    if (p == 0) da[off] -= d; else if (p == 1) mu[off] -= d; else ro[off] -= d;
                }
                const long long row = (rz - 1) + (long long)nz * (rx - 1) + (long long)nz * nx * (ry - 1);
                for (int s = 0; s < 27; s++) {
                    if (!act[s]) continue;
                    const int dy = s / 9 - 1, dxo = (s / 3) % 3 - 1, dz = s % 3 - 1;
                    const long long nb = row + dz + (long long)nz * dxo + (long long)nz * nx * dy;
                    for (int a = 0; a < 3; a++)
                        for (int b = 0; b < 3; b++) {
                            const double complex dB = (bp[s][a][b] - bm[s][a][b]) / (2.0 * h);
                            if (dB == 0) continue;
                            double complex t = 0;
                            for (int j = 0; j < nrhs; j++)
                                t += conj(L[(long long)j * n + 3 * row + a]) * U[(long long)j * n + 3 * nb + b];
                            acc += dB * t;
                        }
                }
            }
            dl[p] = -creal(acc);
        }
        const double P = vp[off], S = vs[off], R = rho[off];
        grad[off] = 2.0 * P * R * dl[0];
        grad[nn + off] = 2.0 * S * R * dl[1] - 4.0 * S * R * dl[0];
        grad[2 * nn + off] = (P * P - 2.0 * S * S) * dl[0] + S * S * dl[1] + dl[2];
    }
    free(da); free(mu); free(ro);
    return 0;
}

/* DISPERSION (dispersion.f:78-114) in FP64, then ASMBLE.  qp, qs hold 1/Q.
 * At omega1 = Re(omega) > eps and omegabase = 2 pi freqbase > 0:
 *   c = c1 * max(1 + (1/Q)/pi * ln(omega1/omegabase), 0.1),
 *   vc = (c, -c (1/Q) / 2),  mu = vcs^2 rho,  lambda = vcp^2 rho - 2 mu. */
int ora_assemble_q_c128(const ora_grid *g, const float *vp, const float *vs, const float *rho, const float *qp,
                        const float *qs, double freqbase, double omega_re, double omega_im, const int *irptr,
                        double complex *a)
{
    const double pi = 3.141592653589793, eps = 10.0 * 1.1920929e-07;
    long long nn = (long long)g->nx * g->ny * g->nz, i;
    double complex *da = (double complex *)malloc(sizeof(double complex) * nn);
    double complex *mu = (double complex *)malloc(sizeof(double complex) * nn);
    double *ro = (double *)malloc(sizeof(double) * nn);
    const double omegabase = freqbase * 2.0 * pi;
    int rc;
    if (!da || !mu || !ro) { free(da); free(mu); free(ro); return 1; }
    lame_c128(nn, vp, vs, rho, da, mu, ro);
    if (omega_re > eps && omegabase > 0.0) {
        const double fac1 = log(omega_re / omegabase);
        for (i = 0; i < nn; i++) {
            double fs = 1.0 + (qs[i] / pi) * fac1, fp = 1.0 + (qp[i] / pi) * fac1, cs, cp;
            double complex vc;
            if (fs < 0.1) fs = 0.1;
            if (fp < 0.1) fp = 0.1;
            cs = vs[i] * fs;
            vc = cs - I * (cs * qs[i] / 2.0);
            mu[i] = vc * vc * (double)rho[i];
            cp = vp[i] * fp;
            vc = cp - I * (cp * qp[i] / 2.0);
            da[i] = vc * vc * (double)rho[i] - 2.0 * mu[i];
        }
    }
    rc = assemble_lame_c128(g, da, mu, ro, omega_re, omega_im, irptr, a);
    free(da); free(mu); free(ro);
    return rc;
}

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

/* ---------------------------------------------------------------------- */
/* HASKGRN (haskgrn.f:31-672): Thomson-Haskell 1-D response at the nodes   */
/* iz = 1..nz to a unit incident P (s_wave = 0) or S plane wave.  FP64.    */
/* Layer tops h1d[0..nl-1] (h1d[0] = 0), layer nl is the half-space;       */
/* vp1disc = vp1d, vs1disc = vs1d.  Kept quirks of the reference: the      */
/* layer-entry refresh tests vp1disc(m) / vs1disc(m) with the loop index m */
/* left over from the previous propagation loop (haskgrn.f:454,466), and   */
/* nodes below the last interface are placed in layer nl-1 (the layer      */
/* search ends with i = nl, haskgrn.f:427-434).                            */
/* ---------------------------------------------------------------------- */
static void hk_layer_cs(double hc, double r1, double r2, double cv, double vp, double vs,
                        double *e1, double *c01, double *s01, double *e2, double *c02, double *s02)
{
    double z01 = hc * r1, z02 = hc * r2, x;
    if (cv > vp) { *e1 = 1; *c01 = cos(z01); *s01 = sin(z01); }
    else { x = exp(z01); *e1 = -1; *c01 = 0.5 * (x + 1. / x); *s01 = 0.5 * (x - 1. / x); }
    if (cv > vs) { *e2 = 1; *c02 = cos(z02); *s02 = sin(z02); }
    else { x = exp(z02); *e2 = -1; *c02 = 0.5 * (x + 1. / x); *s02 = 0.5 * (x - 1. / x); }
}

/* product of the layer matrices of layers 1..top into b (4x2), H53 p.21-23 */
static void hk_propagate(int top, const double *vs, const double *r1, const double *r2, const double *e1,
                         const double *e2, const double *c01, const double *s01, const double *c02,
                         const double *s02, const double *tt, const double *aag, const double *aag1,
                         const double *xh, const double *xh1, double b[4][2])
{
    b[0][0] = 1; b[0][1] = 0; b[1][0] = 0; b[1][1] = 1;
    b[2][0] = 0; b[2][1] = 0; b[3][0] = 0; b[3][1] = 0;
    for (int m = 0; m < top; m++) {
        double pd = s01[m] / r1[m], qd = s02[m] / r2[m];
        double pm = e1[m] * s01[m] * r1[m], qm = e2[m] * s02[m] * r2[m];
        double cp = c01[m], cq = c02[m], tm = tt[m], ag = aag[m], ag1 = aag1[m], x = xh[m], y = xh1[m];
        double a[4][4];
        if (vs[m] != 0.0) {
            a[0][0] = ag * cp - ag1 * cq;  a[0][1] = ag1 * pd + ag * qm;
            a[0][2] = (cq - cp) / tm;      a[0][3] = (pd + qm) / tm;
            a[1][0] = -ag * pm - ag1 * qd; a[1][1] = ag * cq - ag1 * cp;
            a[1][2] = (pm + qd) / tm;      a[1][3] = a[0][2];
            a[2][0] = tm * ag * ag1 * (cp - cq); a[2][1] = tm * (y * pd + x * qm);
            a[2][2] = a[1][1];             a[2][3] = a[0][1];
            a[3][0] = tm * (x * pm + y * qd); a[3][1] = a[2][0];
            a[3][2] = a[1][0];             a[3][3] = a[0][0];
        } else {
            for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) a[i][j] = 0;
            a[0][1] = -pd; a[0][2] = -cp / tm; a[1][1] = cp; a[1][2] = pm / tm;
            a[2][1] = tm * pd; a[2][2] = cp;
        }
        double d[4][2];
        d[0][0] = a[0][0] * b[0][0] - a[0][1] * b[1][0] + a[0][2] * b[2][0] - a[0][3] * b[3][0];
        d[0][1] = a[0][0] * b[0][1] + a[0][1] * b[1][1] + a[0][2] * b[2][1] + a[0][3] * b[3][1];
        d[1][0] = a[1][0] * b[0][0] + a[1][1] * b[1][0] + a[1][2] * b[2][0] + a[1][3] * b[3][0];
        d[1][1] = -a[1][0] * b[0][1] + a[1][1] * b[1][1] - a[1][2] * b[2][1] + a[1][3] * b[3][1];
        d[2][0] = a[2][0] * b[0][0] - a[2][1] * b[1][0] + a[2][2] * b[2][0] - a[2][3] * b[3][0];
        d[2][1] = a[2][0] * b[0][1] + a[2][1] * b[1][1] + a[2][2] * b[2][1] + a[2][3] * b[3][1];
        d[3][0] = a[3][0] * b[0][0] + a[3][1] * b[1][0] + a[3][2] * b[2][0] + a[3][3] * b[3][0];
        d[3][1] = -a[3][0] * b[0][1] + a[3][1] * b[1][1] - a[3][2] * b[2][1] + a[3][3] * b[3][1];
        for (int i = 0; i < 4; i++) { b[i][0] = d[i][0]; b[i][1] = d[i][1]; }
    }
}

int ora_haskgrn(int nl, const double *vp, const double *vs, const double *rh, const double *h1d, double omega,
                double ain, int s_wave, int nz, double dz, double zorig, double complex *ugrn,
                double complex *wgrn)
{
    if (nl < 1 || nl > 64) return 1;
    double r1[64], r2[64], aag[64], aag1[64], tt[64], xh[64], xh1[64], h[64];
    double e1[64], e2[64], c01[64], s01[64], c02[64], s02[64];
    const double cv = (s_wave ? vs[nl - 1] : vp[nl - 1]) / sin(ain);
    const double pic = omega / cv;
    for (int i = 0; i < nl - 1; i++) h[i] = h1d[i + 1] - h1d[i];
    for (int m = 0; m < nl; m++) {
        double cova = cv / vp[m];
        double covb = vs[m] != 0.0 ? cv / vs[m] : 1.0;
        double x = cova * cova - 1.;
        r1[m] = copysign(sqrt(fabs(x)), x);
        x = covb * covb - 1.;
        r2[m] = copysign(sqrt(fabs(x)), x);
        aag[m] = 2. / (covb * covb);
        aag1[m] = aag[m] - 1.;
        if (m < nl - 1) {
            tt[m] = rh[m] * cv * cv;
            xh[m] = aag[m] * aag[m];
            xh1[m] = aag1[m] * aag1[m];
            hk_layer_cs(pic * h[m], r1[m], r2[m], cv, vp[m], vs[m], &e1[m], &c01[m], &s01[m], &e2[m], &c02[m],
                        &s02[m]);
        }
    }
    /* scaled inverse E of the half-space (haskgrn.f:201-211) */
    double x = -aag1[nl - 1] * cv * cv;
    double e11 = 2. * vs[nl - 1] * vs[nl - 1], e13 = -1. / rh[nl - 1];
    double e22 = x / r1[nl - 1], e24 = e13 / r1[nl - 1], e31 = x / r2[nl - 1], e33 = -e13 / r2[nl - 1];
    double e42 = -e11, e44 = e13;
    double b[4][2];
    hk_propagate(nl - 1, vs, r1, r2, e1, e2, c01, s01, c02, s02, tt, aag, aag1, xh, xh1, b);
    double c11 = e11 * b[0][0] + e13 * b[2][0], c12 = e11 * b[0][1] + e13 * b[2][1];
    double c21 = e22 * b[1][0] + e24 * b[3][0], c22 = e22 * b[1][1] + e24 * b[3][1];
    double c31 = e31 * b[0][0] + e33 * b[2][0], c32 = e31 * b[0][1] + e33 * b[2][1];
    double c41 = e42 * b[1][0] + e44 * b[3][0], c42 = e42 * b[1][1] + e44 * b[3][1];
    double scl1 = -1. / (vp[nl - 1] * vp[nl - 1]), scl2 = -1. / (2.0 * vs[nl - 1] * vs[nl - 1]);
    c11 *= scl1; c12 *= scl1; c21 *= scl1; c22 *= scl1;
    c31 *= scl2; c32 *= scl2; c41 *= scl2; c42 *= scl2;
    x = -c11 * c42 + c21 * c32 + c31 * c22 - c41 * c12;
    double y = c11 * c32 + c21 * c42 - c31 * c12 - c41 * c22;
    double ag = x * x + y * y;
    double tm = s_wave ? cv / (vs[nl - 1] * ag) : 2. * cv / (vp[nl - 1] * ag);
    double wr, wi, ur, ui;
    if (!s_wave) {
        wr = tm * (c31 * x - c41 * y); wi = tm * (-c31 * y - c41 * x);
        ur = tm * (c42 * x - c32 * y); ui = tm * (-c42 * y - c32 * x);
    } else {
        wr = tm * (-c11 * x + c21 * y); wi = tm * (c11 * y + c21 * x);
        ur = tm * (-c22 * x + c12 * y); ui = tm * (c22 * y + c12 * x);
    }
    const double qrw = wr, qiw = wi, qru = ur, qiu = ui;
    ugrn[0] = qru + I * qiu;
    wgrn[0] = qrw + I * qiw;
    int ibovo = 1, ifin = 0;
    int mstale = nl;   /* Fortran loop index after "do 7 m = 1, nl-1" */
    for (int iz = 2; iz <= nz; iz++) {
        double dept = dz * (iz - 1) + zorig;
        int i;
        for (i = 2; i <= nl; i++)
            if (dept < h1d[i - 1]) break;
        if (i > nl) i = nl;
        int ibov = i - 1;
        double dloc = dept - h1d[i - 2];
        if (dloc < 0.) return 2;
        if (ibov != ibovo) {
            ibovo = ibov;
            if (ibov > 1) {
                ifin++;
                /* refresh layer ifin with its full thickness, comparing against the stale m */
                hk_layer_cs(pic * h[ifin - 1], r1[ifin - 1], r2[ifin - 1], cv, vp[mstale - 1], vs[mstale - 1],
                            &e1[ifin - 1], &c01[ifin - 1], &s01[ifin - 1], &e2[ifin - 1], &c02[ifin - 1],
                            &s02[ifin - 1]);
            }
        }
        hk_layer_cs(pic * dloc, r1[ibov - 1], r2[ibov - 1], cv, vp[ibov - 1], vs[ibov - 1], &e1[ibov - 1],
                    &c01[ibov - 1], &s01[ibov - 1], &e2[ibov - 1], &c02[ibov - 1], &s02[ibov - 1]);
        hk_propagate(ibov, vs, r1, r2, e1, e2, c01, s01, c02, s02, tt, aag, aag1, xh, xh1, b);
        mstale = ibov + 1;
        ur = b[0][0] * qru - b[0][1] * qiw;
        ui = b[0][0] * qiu + b[0][1] * qrw;
        wr = -b[1][0] * qiu + b[1][1] * qrw;
        wi = b[1][0] * qru + b[1][1] * qiw;
        ugrn[iz - 1] = ur + I * ui;
        wgrn[iz - 1] = wr + I * wi;
    }
    return 0;
}
