/*
 * CPU oracle for the wtomo3d forward-modelling hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the tests, the
 * smoke entry point and the CPU-baseline leg of the benchmark load it to
 * compare against the CUDA path.  Nothing in the product links or calls it.
 *
 * It is a plain-C restatement of the reference Fortran, formula for formula
 * and in the same operation order, in two precisions:
 *   _c128 : complex128 throughout (the parity oracle),
 *   _c64  : complex64, as the reference computes (calcwts in FP64 then
 *           rounded to float, calcwts.f:65-71).
 *
 * Parity pinning: the reference ships no golden vectors or known-answer
 * tests; only its self-checks pin results (the closed-form nnz of
 * srgraphs.f:626-636 and the per-row nnz check of asmble.f90:556-564).
 * Both are reproduced and tested.  Value parity against the reference's
 * own binary is unpinned (the Fortran sources cannot be built here: no
 * Fortran compiler, and several sources named by its Makefile are missing).
 *
 * Indexing: grid node g = iz + nz*(ix-1) + nx*nz*(iy-1) (1-based, z fastest,
 * srgraphs.f:689,696), dofs 3g-2..3g = (u,v,w).  Model arrays are (nz,nx,ny)
 * column-major, i.e. element (iz,ix,iy) at offset g-1.
 */
#ifndef WT3D_ORACLE_H
#define WT3D_ORACLE_H

#include <complex.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nx, ny, nz;
    double dx;        /* dx = dy = dz (readini.f90:55-59) */
    double pmld;      /* PML width (m) */
    double pmlr;      /* PML reflection coefficient */
    int fst;          /* free surface on top (freesurf(1)) */
    int usemin;       /* Min-cell free surface (optional:usemin) */
} ora_grid;

/* srel3d_getsize (srgraphs.f:626-636) */
void ora_srel3d_getsize(int nx, int ny, int nz, long long *numvert, long long *nedge);

/* srel3d (srgraphs.f:638-734) then SPARSE_ADJ2CRS (sparse.f:13-49): 1-based CSR
 * with the diagonal inserted.  irptr has n+1 entries, jcptr nnz entries.
 * Returns 0 on success. */
int ora_pattern(int nx, int ny, int nz, int *irptr, int *jcptr);

/* ASMBLE (asmble.f90:1-636) over SETCOEFS3D/CALCWTS/FDFD3D/PFDFD3D/PML3D/FIXED3D/TPFREE.
 * vp, vs, rho: (nz,nx,ny) float arrays (as read by modelio.f90), converted to
 * lambda/mu by modelio.f90:78-92.  omega complex angular frequency.
 * ibg selects the background model arrays (vpb, vsb, rhob) when 1, as
 * SETCOEFS3D(...,ibg) does; they may be NULL when ibg == 0.
 * Returns ierr as the reference accumulates it (0 on success). */
int ora_assemble_c128(const ora_grid *g, const float *vp, const float *vs, const float *rho,
                      double omega_re, double omega_im, const int *irptr,
                      double complex *a);
int ora_assemble_c64(const ora_grid *g, const float *vp, const float *vs, const float *rho,
                     double omega_re, double omega_im, const int *irptr,
                     float complex *a);

/* DISPERSION (dispersion.f:78-114) then ASMBLE, complex128: qp, qs are 1/Q
 * per node, freqbase the reference frequency (Hz) of vp and vs. */
int ora_assemble_q_c128(const ora_grid *g, const float *vp, const float *vs, const float *rho, const float *qp,
                        const float *qs, double freqbase, double omega_re, double omega_im, const int *irptr,
                        double complex *a);

/* One node's 27 3x3 blocks (slot s = 9(dy+1)+3(dx+1)+(dz+1), rows/cols u,v,w),
 * and a mask of the slots present in the pattern.  1-based node indices. */
int ora_node_blocks_c128(const ora_grid *g, const float *vp, const float *vs, const float *rho,
                         double omega_re, double omega_im, int iz, int ix, int iy,
                         double complex *blk /*27*9*/, int *active /*27*/);

/* FP64 adjoint-state gradient by central differences of node blocks.
 * U (forward) and L (adjoint) wavefields: complex128, column-major 3nn x nrhs.
 * grad[3*nn] = (dchi/dVp, dchi/dVs, dchi/drho) per node, with
 * dchi/dm = -Re sum_j L_j^H (dA/dm) U_j for the operator ora_assemble_c128 builds. */
int ora_gradient_c128(const ora_grid *g, const float *vp, const float *vs, const float *rho,
                      double omega_re, double omega_im, int nrhs, const double complex *U,
                      const double complex *L, double *grad);

/* CSR complex128 SpMV y = A x (1-based CSR). */
void ora_spmv_c128(int n, const int *irptr, const int *jcptr, const double complex *a,
                   const double complex *x, double complex *y);

/* srcsetup with ireg = 0 (srcsetup.f:50-73): nearest-node point source.
 * Writes sterm into component comp (0=u,1=v,2=w) of the dof vector rhs(3N).
 * Returns the 1-based node index used. */
long long ora_point_source(const ora_grid *g, double xloc, double yloc, double zloc,
                           int comp, double complex sterm, double complex *rhs);

/* SRCSETUP with ireg > 0 (srcsetup.f:78-211) and SRCREG (srcreg.f:77-304):
 * adds the spread source sterm at (xloc, yloc, zloc) (metres from node 1)
 * into the node field swave[nz*nx*ny] (model order).  Kaiser-windowed sinc
 * of half-width ireg nodes when sprd <= 0.5, normalised discrete Dirac of
 * half-width sprd nodes otherwise; mirrored with a sign change above a free
 * top (g->fst), dropped beyond the other faces.  Returns 0 on success. */
int ora_source_weights(const ora_grid *g, double xloc, double yloc, double zloc, int ireg, double sprd,
                       double complex sterm, double complex *swave);

/* HASKGRN (haskgrn.f:31-672) in FP64: ugrn[nz], wgrn[nz] for a unit incident
 * P (s_wave = 0) or S plane wave with incidence angle ain (radians) at angular
 * frequency omega, nl layers with tops h1d[] (h1d[0] = 0; layer nl = half-space). */
int ora_haskgrn(int nl, const double *vp1d, const double *vs1d, const double *rh1d, const double *h1d,
                double omega, double ain, int s_wave, int nz, double dz, double zorig,
                double complex *ugrn, double complex *wgrn);

#ifdef __cplusplus
}
#endif
#endif
