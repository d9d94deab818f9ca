/* C driver of the drop-in job protocol, in the order elwave.f90:141-190 calls
 * it: job 1 on the pattern, then per frequency ASMBLE + job 2 (factor) and a
 * job 3 solve, then job -1.  Everything passes by reference with 1-based CSR
 * and complex64 values, as the Fortran BIND(C) interface does.  The second
 * pass gives the same operator under a node permutation, which job 1 no
 * longer recognises as the grid graph (general ordering).
 *
 * Test program (tests/test_gpu_c_driver.py builds and runs it on a GPU):
 * prints one line per solve and "ok" when every check holds; exit status 1
 * otherwise. */
#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "wtomo3d_gpu.h"

static const double PI = 3.14159265358979323846;

static int fail(const char *what)
{
    printf("FAIL: %s (%s)\n", what, wt3d_last_error());
    return 1;
}

/* relative residual ||b - A x|| / ||b|| in double, A 1-based CSR complex64 */
static double relres(int n, const int *ir, const int *jc, const float complex *a, const float complex *b,
                     const float complex *x)
{
    double rr = 0, bb = 0;
    for (int r = 0; r < n; r++) {
        double complex s = b[r];
        for (int k = ir[r] - 1; k < ir[r + 1] - 1; k++) s -= (double complex)a[k] * (double complex)x[jc[k] - 1];
        rr += creal(s) * creal(s) + cimag(s) * cimag(s);
        bb += crealf(b[r]) * crealf(b[r]) + cimagf(b[r]) * cimagf(b[r]);
    }
    return sqrt(rr / bb);
}

int main(void)
{
    const int nx = 10, ny = 9, nz = 11;
    const double dx = 20.0;
    wt3d_grid g = {nx, ny, nz, dx, 3 * dx, 0.0, 1, 1};
    int n = 3 * nx * ny * nz, nn = nx * ny * nz;
    int nnz = (int)wt3d_pattern_nnz(nx, ny, nz);
    int *ir = malloc(sizeof(int) * (n + 1)), *jc = malloc(sizeof(int) * nnz);
    int *irp = malloc(sizeof(int) * (n + 1)), *jcp = malloc(sizeof(int) * nnz);
    int *ir0 = malloc(sizeof(int) * (n + 1)), *jc0 = malloc(sizeof(int) * nnz);
    float *vp = malloc(sizeof(float) * nn), *vs = malloc(sizeof(float) * nn), *rho = malloc(sizeof(float) * nn);
    double complex *a128 = malloc(sizeof(double complex) * nnz);
    float complex *a = malloc(sizeof(float complex) * nnz), *ap = malloc(sizeof(float complex) * nnz);
    float complex *b = malloc(sizeof(float complex) * n), *bp = malloc(sizeof(float complex) * n);
    float complex *x = malloc(sizeof(float complex) * n);
    float complex *x0 = malloc(sizeof(float complex) * 2 * n);   /* grid-pattern solutions per frequency */
    int *q = malloc(sizeof(int) * nn), *iq = malloc(sizeof(int) * nn);
    if (!ir || !jc || !irp || !jcp || !ir0 || !jc0 || !vp || !vs || !rho || !a128 || !a || !ap || !b || !bp || !x ||
        !q || !iq || !x0)
        return fail("host allocation");
    if (wt3d_pattern(nx, ny, nz, 1, ir, jc)) return fail("wt3d_pattern");
    /* two layers, Vs = Vp / 1.73, Gardner density; (nz, nx, ny) order */
    for (int i = 0; i < nn; i++) {
        const int iz = i % nz;
        vp[i] = iz < nz / 2 ? 3000.0f : 4500.0f;
        vs[i] = vp[i] / 1.73f;
        rho[i] = 310.0f * powf(vp[i], 0.25f);
    }
    /* a node permutation (new node -> old node) by a seeded shuffle */
    unsigned long long s = 12345;
    for (int i = 0; i < nn; i++) q[i] = i;
    for (int i = nn - 1; i > 0; i--) {
        s = s * 6364136223846793005ULL + 1442695040888963407ULL;
        const int j = (int)((s >> 33) % (unsigned long long)(i + 1));
        const int t = q[i]; q[i] = q[j]; q[j] = t;
    }
    for (int i = 0; i < nn; i++) iq[q[i]] = i;
    /* permuted pattern: row 3 q'[g] + c of the new matrix is row 3 g + c of the old */
    irp[0] = 1;
    for (int R = 0; R < n; R++) {
        const int r = 3 * q[R / 3] + R % 3;
        int k = irp[R] - 1;
        for (int t = ir[r] - 1; t < ir[r + 1] - 1; t++) {
            const int c = jc[t] - 1;
            jcp[k++] = 3 * iq[c / 3] + c % 3 + 1;
        }
        irp[R + 1] = k + 1;
    }
    int ok = 1;
    for (int pass = 0; pass < 2; pass++) {
        /* (complex.h takes the name I) */
        int *pir = pass ? irp : ir, *pjc = pass ? jcp : jc;
        float complex *pa = pass ? ap : a, *pb = pass ? bp : b;
        memcpy(ir0, pir, sizeof(int) * (n + 1));
        memcpy(jc0, pjc, sizeof(int) * nnz);
        int job = 1, ierr = 0;
        strumpack_serial_finter(&job, &n, &nnz, pir, pjc, pa, pb, x, &ierr);
        if (ierr) return fail("job 1");
        const double freqs[2] = {0.5, 2.0};
        for (int fi = 0; fi < 2; fi++) {
            if (wt3d_assemble(&g, vp, vs, rho, 2 * PI * freqs[fi], 0.0, a128)) return fail("wt3d_assemble");
            for (int k = 0; k < nnz; k++) a[k] = (float complex)a128[k];
            if (pass) {   /* values in the permuted row order */
                for (int R = 0; R < n; R++) {
                    const int r = 3 * q[R / 3] + R % 3;
                    memcpy(ap + irp[R] - 1, a + ir[r] - 1, sizeof(float complex) * (ir[r + 1] - ir[r]));
                }
            }
            /* a vertical point force at the centre node */
            memset(b, 0, sizeof(float complex) * n);
            const int node = nz / 2 + nz * (nx / 2 + nx * (ny / 2));
            b[3 * node + 2] = 1.0f;
            for (int R = 0; R < n; R++) bp[R] = b[3 * q[R / 3] + R % 3];
            job = 2;
            strumpack_serial_finter(&job, &n, &nnz, pir, pjc, pa, pb, x, &ierr);
            if (ierr) return fail("job 2");
            job = 3;
            strumpack_serial_finter(&job, &n, &nnz, pir, pjc, pa, pb, x, &ierr);
            if (ierr) return fail("job 3");
            const double rr = relres(n, pir, pjc, pa, pb, x), rf = wt3d_finter_last_relres();
            /* the two orderings solve the same system: compare in the grid order */
            double dd = 0, xx = 0;
            if (!pass) memcpy(x0 + (size_t)fi * n, x, sizeof(float complex) * n);
            else
                for (int R = 0; R < n; R++) {
                    const float complex e = x[R] - x0[(size_t)fi * n + 3 * q[R / 3] + R % 3];
                    dd += crealf(e) * crealf(e) + cimagf(e) * cimagf(e);
                    xx += crealf(x[R]) * crealf(x[R]) + cimagf(x[R]) * cimagf(x[R]);
                }
            const double diff = pass ? sqrt(dd / xx) : 0.0;
            printf("%s pattern, %.1f Hz: relres of the complex64 solution %.2e, refinement %.2e, vs grid %.2e\n",
                   pass ? "permuted" : "grid", freqs[fi], rr, rf, diff);
            /* complex64 output of an FP64-refined solve: float rounding of x
             * (~2.5e-8 here) times the operator's conditioning */
            if (!(rr <= 1e-4) || !(rf <= 1e-10) || !(diff <= 1e-5)) ok = 0;
        }
        job = -1;
        strumpack_serial_finter(&job, &n, &nnz, pir, pjc, pa, pb, x, &ierr);
        if (ierr) return fail("job -1");
        if (memcmp(ir0, pir, sizeof(int) * (n + 1)) || memcmp(jc0, pjc, sizeof(int) * nnz))
            return fail("irptr/jcptr modified");
    }
    if (!ok) return fail("residual check");
    printf("ok\n");
    return 0;
}
