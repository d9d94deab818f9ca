/*
 * wtomo3d-gb300: GB300-native forward-modelling hot path of wtomo3d.
 *
 * C ABI of libwtomo3d_gpu.so.  Every entry point takes plain pointers and
 * sizes and returns an int status (0 = success) unless stated otherwise.
 * Complex values are interleaved (re, im) pairs: `double _Complex` /
 * `float _Complex` in C, COMPLEX(C_DOUBLE_COMPLEX)/COMPLEX(C_FLOAT_COMPLEX)
 * in Fortran.
 *
 * Grid ordering follows the reference: node g = iz + nz*(ix-1) + nx*nz*(iy-1)
 * (1-based, z fastest; srgraphs.f:689,696), dofs 3g-2..3g = (u, v, w).
 * Model arrays are (nz, nx, ny) column-major float arrays (modelio.f90:104-111
 * layout after MODELIO_H52WT_MODEL).
 */
#ifndef WTOMO3D_GPU_H
#define WTOMO3D_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define WT3D_OK                0
#define WT3D_ERR_ARG           1   /* invalid argument                        */
#define WT3D_ERR_CUDA          2   /* CUDA runtime error                      */
#define WT3D_ERR_NOMEM         3   /* device or host allocation failed        */
#define WT3D_ERR_STATE         4   /* call out of order (no model, no factor) */
#define WT3D_ERR_PATTERN       5   /* CSR pattern malformed                   */
#define WT3D_ERR_NOCONV        6   /* refinement did not reach the tolerance  */
#define WT3D_ERR_NOGPU         7   /* no CUDA device                          */

/* ---- precisions --------------------------------------------------------- */
#define WT3D_PREC_MIXED        0   /* complex64 fronts + FP64 refinement      */
#define WT3D_PREC_FP64         1   /* complex128 fronts (the FP64 GPU oracle)  */

/* Grid and boundary description.  Replaces the INIT_/MODEL_/PML_MODULE
 * globals read by ASMBLE (modules.F90:1-76) and the ini keys of
 * readini.f90:46-86,216.  pmld <= 0 selects the reference default 10*dx;
 * pmlr <= 0 selects 1e-3. */
typedef struct wt3d_grid {
    int    nx, ny, nz;
    double dx;          /* dx = dy = dz (readini.f90:55-59)                 */
    double pmld;        /* PML width in metres                              */
    double pmlr;        /* PML reflection coefficient                       */
    int    fst;         /* free surface on top (model:fst, default true)    */
    int    usemin;      /* Min-cell free surface (optional:usemin)          */
} wt3d_grid;

/* ---- drop-in boundary of the reference ---------------------------------
 * Replaces strumpack_serial_finter (strumpack_finter.c:9-121; Fortran
 * interface interface.f90:295-309).  Same symbol, signature, job protocol and
 * error convention:
 *   job  1 : initialise and analyse the 1-based CSR pattern (values unused)
 *   job  2 : (re)set values and factor
 *   job  3 : solve one right-hand side: sol = A^-1 rhs
 *   job -1 : destroy
 * *ierr = 0 on success, 1 on error (with a message on stdout), as the
 * reference.  irptr/jcptr are read, never modified.  The 27-point, 3-dof grid
 * graph built by srel3d + SPARSE_ADJ2CRS is recognised (the grid is recovered
 * from it and ordered by plane separators); any other pattern is ordered as
 * wt3d_solver_create_csr does.  Factorisation is
 * complex64 with FP64 iterative
 * refinement; the solution is returned in complex64 as the reference does.
 * Not re-entrant (one global instance, like the reference). */
void strumpack_serial_finter(int *job, int *nrows, int *nnz,
                             int *irptr, int *jcptr, float _Complex *a,
                             float _Complex *rhs, float _Complex *sol,
                             int *ierr);

/* Refinement target of job 3 (default relative residual 1e-10 within 20
 * substitution passes).  The reference sets its refinement tolerances once,
 * at job 1 (STRUMPACK_set_rctol / set_actol, strumpack_finter.c:38-39),
 * and a caller cannot change them; this setter serves the same purpose.
 * Job 3 sets *ierr = 1 and prints the residual reached when the target is
 * missed, and still returns that last iterate in sol.  Returns WT3D_ERR_ARG
 * for tol <= 0 or maxit < 0. */
int wt3d_finter_set_refinement(double tol, int maxit);
/* Relative residual ||b - A x|| / ||b|| (FP64, assembled operator) that the
 * last job-3 call reached. */
double wt3d_finter_last_relres(void);

/* ---- pattern and assembly ----------------------------------------------
 * wt3d_pattern replaces srel3d_getsize + srel3d + SPARSE_ADJ2CRS
 * (srgraphs.f:626-734, sparse.f:13-49).  n = 3*nx*ny*nz, nnz =
 * 9(3nx-2)(3ny-2)(3nz-2).  base = 0 or 1.  Host arrays irptr[n+1], jcptr[nnz]. */
long long wt3d_pattern_nnz(int nx, int ny, int nz);
int wt3d_pattern(int nx, int ny, int nz, int base, int *irptr, int *jcptr);

/* wt3d_assemble replaces ASMBLE (asmble.f90:1-636; interface.f90:4-12) with
 * the model set up as modelio.f90:78-92 does.  Host arrays in and out; the
 * work runs on the current CUDA device.  a[nnz] receives complex128 values in
 * the CSR order of wt3d_pattern.  omega = 2*pi*f (+ i/tau) as elwave.f90:151,164. */
int wt3d_assemble(const wt3d_grid *g, const float *vp, const float *vs, const float *rho,
                  double omega_re, double omega_im, double _Complex *a);

/* Device-pointer variant: d_vp/d_vs/d_rho device floats, d_irptr the 0-based
 * row pointer on the device (n+1 ints), d_a device complex128[nnz].
 * stream is a cudaStream_t (NULL = default stream).  Asynchronous. */
int wt3d_assemble_device(const wt3d_grid *g, const float *d_vp, const float *d_vs,
                         const float *d_rho, double omega_re, double omega_im,
                         const int *d_irptr, void *d_a, void *stream);

/* ---- plane-wave sources ------------------------------------------------
 * Layered 1-D medium for the Thomson-Haskell response: nl >= 2 layers, layer
 * nl is the half-space; ztop[0] = 0 and ztop[i] is the depth (m) of the top of
 * layer i+1 (HASKELL_MODULE vp1d/vs1d/rh1d/h1d, modules.F90:204-213). */
typedef struct wt3d_layered1d {
    int nl;
    const double *vp, *vs, *rho, *ztop;
} wt3d_layered1d;

/* HASKGRN (haskgrn.f:31-672): response U(z), W(z) at the nz node depths
 * zorig + dz*(iz-1) to a unit P (s_wave = 0) or S plane wave of incidence
 * angle ain (radians) at angular frequency omega.  Host, FP64. */
int wt3d_haskgrn(const wt3d_layered1d *m, double omega, double ain, int s_wave, int nz, double dz,
                 double zorig, double _Complex *U, double _Complex *W);

/* ---- handle-based solver (re-entrant siblings of the job protocol) ------ */
typedef struct wt3d_solver wt3d_solver;

/* Analyse: nested-dissection ordering and symbolic factorisation of the grid
 * graph on the host; allocates the front storage on the device. */
int wt3d_solver_create(wt3d_solver **h, const wt3d_grid *g, int precision);
int wt3d_solver_destroy(wt3d_solver *h);

/* Analyse any CSR pattern (n rows, nnz >= 1 entries, index base 0 or 1,
 * columns in any order, no duplicates), as STRUMPACK's reordering does for
 * the job-1 pattern (strumpack_finter.c:42-48): an unsymmetric pattern is
 * stored as the pattern of A + A^T (the added entries hold zeros), then
 * ordered by automatic nested dissection (level-structure separators) on the
 * graph of supervariables (runs of consecutive rows with equal column sets),
 * with the same multifrontal symbolic factorisation and device storage as
 * the grid.  The handle takes values with wt3d_set_values_c64 / _c128 in the
 * caller's CSR order and solves with wt3d_solve*, wt3d_apply*; the entry
 * points that need the grid (model, sources, receivers, gradient) return
 * WT3D_ERR_STATE.  A malformed pattern returns WT3D_ERR_PATTERN. */
int wt3d_solver_create_csr(wt3d_solver **h, int n, long long nnz, const int *irptr, const int *jcptr, int base,
                           int precision);

/* Model (host arrays, (nz,nx,ny) floats). */
int wt3d_set_model(wt3d_solver *h, const float *vp, const float *vs, const float *rho);

/* Attenuation (the Q model of DISPERSION, dispersion.f:78-114): qp_inv,
 * qs_inv = 1/Qp, 1/Qs per node ((nz,nx,ny) floats), freqbase the frequency
 * (Hz) at which vp and vs are given (model:freqbase, readini.f90:65, default
 * 20).  Each wt3d_factor then disperses the Lame arrays to Re(omega):
 * c = c1 max(1 + ln(Re omega / 2 pi freqbase)/(pi Q), 0.1), complex velocity
 * (c, -c/(2Q)).  NULL pointers return to the elastic model.  The background
 * of the plane-wave sources stays elastic, as in the reference.  The
 * gradient entry points reject attenuating models. */
int wt3d_set_attenuation(wt3d_solver *h, const float *qp_inv, const float *qs_inv, double freqbase);

/* Assemble A(omega) on the device and factor it (precision from create).
 * omega may be complex: the anti-alias frequency 2 pi f + i/tau of
 * elwave.f90:164 (the mass terms keep only REAL(omega^2), pfdfd3d.f:140-142). */
int wt3d_factor(wt3d_solver *h, double omega_re, double omega_im);

/* Set caller-assembled operator values (complex64, host, in the CSR order of
 * wt3d_pattern, or of the pattern given to wt3d_solver_create_csr);
 * wt3d_factor_values then factors them.  Together the job-2 path of
 * strumpack_serial_finter (strumpack_finter.c:68-92). */
int wt3d_set_values_c64(wt3d_solver *h, const float _Complex *a);
/* The same with complex128 values (no job-protocol counterpart). */
int wt3d_set_values_c128(wt3d_solver *h, const double _Complex *a);
int wt3d_factor_values(wt3d_solver *h);

/* Background model (host floats, (nz,nx,ny)) of the scattered-field sources:
 * the dap/mup/rhop arrays SETCOEFS3D reads with ibg = 1 (setcoefs3d.f:98-101). */
int wt3d_set_background(wt3d_solver *h, const float *vp, const float *vs, const float *rho);

/* Plane-wave scattered-field sources at the last factored omega, replacing
 * haskgrn + plane-wave expansion + hetfldsrc (hetfldsrc.f90:17-1038):
 *   u0_j = [U_j*(z) rx, U_j*(z) ry, W_j*(z)] exp(i omega p_j (x rx + y ry)),
 *   (* = complex conjugate: Haskell's time sign is the reverse of the
 *   operator's, dispersion.f:17-22),
 *   (rx, ry) = -(cos baz_j, sin baz_j), p_j = sin(ain_j) / v_halfspace,
 *   f_j = (A_bg - A) u0_j   (source spectrum 1, srcin = 3).
 * d_F: device complex128, column-major n x nsrc.  d_U0 (optional, may be NULL):
 * device complex128 column-major n x nsrc receiving u0. */
int wt3d_rhs_planewave(wt3d_solver *h, const wt3d_layered1d *m, int nsrc, const double *ain,
                       const double *baz, const int *s_wave, void *d_F, void *d_U0);

/* Solve A X = B for nrhs right-hand sides (host arrays, column k of B at
 * B + k*n, complex128).  Mixed precision refines in FP64 until every column
 * has ||b - A x|| / ||b|| <= tol or maxit refinement steps are done.
 * relres[nrhs] (may be NULL) receives the final relative residuals,
 * *iters (may be NULL) the refinement steps taken.  Returns WT3D_ERR_NOCONV
 * (with X filled) if the tolerance was not reached. */
int wt3d_solve(wt3d_solver *h, int nrhs, const double _Complex *B, double _Complex *X,
               double tol, int maxit, double *relres, int *iters);

/* Conjugate-transpose solve A^H X = B reusing the resident factors. */
int wt3d_solve_adjoint(wt3d_solver *h, int nrhs, const double _Complex *B, double _Complex *X,
                       double tol, int maxit, double *relres, int *iters);

/* Device-pointer solve: d_B, d_X device complex128, column-major n x nrhs.
 *
 * Calls that take caller device buffers (wt3d_*_device, wt3d_rhs_*,
 * wt3d_sample_*, wt3d_gradient_contract, wt3d_misfit_gradient, wt3d_memcpy)
 * first wait for all work already queued on the legacy default stream (where
 * PyTorch runs unless told otherwise), so buffers filled there need no
 * synchronisation; work on other streams must be complete before the call.
 * Each call synchronises before it returns, so its outputs are ready. */
int wt3d_solve_device(wt3d_solver *h, int nrhs, const void *d_B, void *d_X,
                      double tol, int maxit, double *relres, int *iters, int adjoint);

/* y = A x with the assembled complex128 operator (host arrays), for checks. */
int wt3d_apply(wt3d_solver *h, int nrhs, const double _Complex *X, double _Complex *Y);

/* y = A x on device arrays (complex128, column-major n x nrhs).  No
 * reference counterpart (the reference never applies A outside STRUMPACK). */
int wt3d_apply_device(wt3d_solver *h, int nrhs, const void *d_X, void *d_Y);

/* Re-assemble the complex128 operator from the handle's current model
 * (wt3d_set_model) at the last factored omega, keeping the factors.  Later
 * solves refine against the new operator with the old factors as the
 * preconditioner, which converges while the model change is small (model
 * perturbations, line searches).  No reference counterpart. */
int wt3d_update_operator(wt3d_solver *h);

/* ---- adjoint-state gradient --------------------------------------------
 * No counterpart on the reference's path: wtomo3d's gradient lives outside
 * the forward-modelling routines.  The operator differentiated is the one
 * ASMBLE builds (asmble.f90:96-601) from the Lame arrays of
 * modelio.f90:78-92, with respect to the model arrays (Vp, Vs, rho) of the
 * handle's current model at the last factored omega, including the
 * mass-lumping weights (calcwts.f:1-75) and the PML stretch's dependence on
 * the centre node's vp (pml3d.f:201-295).
 *
 * Contraction: grad[0..nn) = dchi/dVp, grad[nn..2nn) = dchi/dVs,
 * grad[2nn..3nn) = dchi/drho at every node (nn = nx*ny*nz, model order), with
 *     dchi/dm = -Re sum_j lam_j^H (dA/dm) u_j .
 * d_U: forward wavefields (the total field for plane waves), d_Lam: adjoint
 * wavefields, both device complex128 column-major n x nrhs; d_grad: device
 * double[3*nn]. */
int wt3d_gradient_contract(wt3d_solver *h, int nrhs, const void *d_U, const void *d_Lam, void *d_grad);

/* Waveform misfit chi = 1/2 sum_j sum_r |u_j(rec_r) - dobs|^2 over the three
 * components of nrec receivers at grid nodes rec_node[] (0-based node
 * indices), and its gradient.  Forward: X = A^-1 F (d_F device n x nsrc),
 * total field u = X + U0 (d_U0 device or NULL).  Adjoint: A^H lam =
 * R^T (R u - dobs) with the resident factors.  dobs, dpred (may be NULL):
 * host complex128 [(j*nrec + r)*3 + c]; grad: host double[3*nn] as above.
 * Both solves refine to tol.  Returns WT3D_ERR_NOCONV (with outputs filled)
 * if a solve did not reach tol. */
int wt3d_misfit_gradient(wt3d_solver *h, int nsrc, const void *d_F, const void *d_U0, int nrec,
                         const long long *rec_node, const double _Complex *dobs, double tol, int maxit,
                         double *chi, double *grad, double _Complex *dpred);

/* ---- sources and receivers between nodes --------------------------------
 * Weights of a point at (x, y, z) metres from node 1 on the grid, as
 * SRCSETUP/SRCREG spread a source or sample a receiver (srcsetup.f:50-211,
 * srcreg.f:77-304): ireg = 0 nearest node; ireg > 0 Kaiser-windowed sinc of
 * half-width ireg nodes (sprd <= 0.5) or the normalised discrete Dirac of
 * half-width sprd nodes (sprd > 0.5); terms beyond a free top (g->fst) are
 * mirrored with a sign change, terms beyond the other faces dropped.  FP64,
 * I0 from std::cyl_bessel_i (the reference: REAL, rational I0; ~1e-7).
 * Writes up to cap (0-based node, weight) pairs; *count = pairs produced. */
int wt3d_source_weights(const wt3d_grid *g, double x, double y, double z, int ireg, double sprd, int cap,
                        long long *node, double *weight, int *count);

/* Point-force right-hand sides on the device: column j of d_F (complex128,
 * column-major n x nsrc) = the source sterm[j] (NULL: 1) spread by the
 * weights above onto component comp[j] (0 u, 1 v, 2 w) at xyz[3j..3j+2]. */
int wt3d_rhs_sources(wt3d_solver *h, int nsrc, const double *xyz, const int *comp, const double _Complex *sterm,
                     int ireg, double sprd, void *d_F);

/* Three-component receiver samples of device wavefields d_U (n x nrhs):
 * out[(j*nrec + r)*3 + c] = sum of weight * u_j(node, c) over receiver r's
 * weights (SRCSETUP with lsetup = .false., srcsetup.f:192-206). */
int wt3d_sample_receivers(wt3d_solver *h, int nrhs, const void *d_U, int nrec, const double *xyz, int ireg,
                          double sprd, double _Complex *out);

/* Hydrophone pressure of device wavefields d_U (n x nrhs), makeuh.f:113-167:
 * p = (lambda + 2 mu / 3) (du/dx + dv/dy + dw/dz) with lambda, mu of the
 * node INT(1.5 + x/dx) (clamped) and each derivative the centred difference
 * of receiver samples at +-dx, divided by (-i omega) and negated as written
 * there.  out[j*nrec + r].  A receiver response (recin, makeuh.f:92-97) is a
 * per-receiver factor the caller applies. */
int wt3d_sample_pressure(wt3d_solver *h, int nrhs, const void *d_U, int nrec, const double *xyz, int ireg,
                         double sprd, double _Complex *out);

/* Number of SMs the persistent tensor-core GEMM of the factorisations leaves
 * idle, process-wide (default 0).  A nonzero reserve lets the substitution
 * passes of another handle run during a factorisation (two handles pipelining
 * frequencies).  No reference counterpart. */
int wt3d_set_sm_reserve(int n);

/* Statistics of the last factorisation. */
typedef struct wt3d_stats {
    long long n, nnz;              /* unknowns, operator nonzeros             */
    long long nfronts;             /* fronts in the elimination tree          */
    long long factor_entries;      /* complex entries stored in the factors   */
    double    factor_flops;        /* real-flop count, sum of 8(p^3/3+p^2 b+p b^2) */
    double    factor_bytes;        /* bytes held by the factors on the device */
    double    device_bytes;        /* total device bytes held by the handle   */
    double    t_analyse_ms, t_assemble_ms, t_factor_ms, t_solve_ms; /* last calls */
    int       perturbed_pivots;    /* pivots replaced by the static threshold */
    int       levels;              /* depth of the elimination tree + 1       */
    int       kernels_factor;      /* kernels launched by the last factor call */
    int       kernels_solve;       /* kernels launched by the last solve call  */
    double    t_gradient_ms;       /* last gradient contraction               */
    double    workspace_bytes;     /* factorisation workspace shared by the
                                      handles of this grid and precision     */
} wt3d_stats;
int wt3d_get_stats(const wt3d_solver *h, wt3d_stats *st);

/* Device buffers owned by the handle for ncols right-hand sides and
 * solutions (complex128, column-major n x ncols), grown on demand and freed
 * with the handle; counted in wt3d_stats.device_bytes.  For callers that keep
 * no device memory of their own (the serving loop).  No reference counterpart. */
int wt3d_batch_buffers(wt3d_solver *h, int ncols, void **d_F, void **d_X);

/* Copy `bytes` between host and device memory in either direction on the
 * handle's stream, returning when done.  No reference counterpart. */
int wt3d_memcpy(wt3d_solver *h, void *dst, const void *src, long long bytes);

/* Free and total device memory of the current device. */
int wt3d_mem_info(double *free_bytes, double *total_bytes);

/* Device memory of a handle for grid g, before creating it (host analysis
 * only, cached per grid): out[0] = bytes a factored handle holds on its own,
 * out[1] = additional bytes once plane-wave sources are built (background
 * operator), out[2] = level-parity update buffers of the factorisation
 * workspace, shared by all handles of the same grid and precision (their
 * factorisations are serialised).  No reference counterpart. */
int wt3d_solver_bytes(const wt3d_grid *g, int precision, double *out);

/* Host-only view of the analysis (nested dissection + symbolic
 * factorisation; no GPU needed).  info[8] = {fronts, factor entries, levels,
 * max pivots, max border, border entries, update buffer 0, update buffer 1};
 * *flops = sum of 8(p^3/3 + p^2 b + p b^2).  leaf_nodes <= 0 selects 64. */
int wt3d_analyse_info(int nx, int ny, int nz, int leaf_nodes, long long *info, double *flops);
/* Export the elimination structure: perm[n] (new dof -> natural dof), per
 * front p, b, first pivot, parent, depth, and the concatenated border dofs
 * (new indices) and their positions in the parent front (rel). */
int wt3d_analyse_export(int nx, int ny, int nz, int leaf_nodes, int *perm, int *fp, int *fb, int *ffirst,
                        int *fparent, int *flevel, int *border, int *rel);
/* The same two for a general CSR pattern (as wt3d_solver_create_csr):
 * leaf_dofs <= 0 selects 192.  info also requires every entry to fall inside
 * its front (the scatter map). */
/* 1 if the library was built with the CUDA toolkit's METIS
 * (libmetis_static.a): the general ordering then also takes METIS's vertex
 * separator (METIS_ComputeVertexSeparator) at every split where it is the
 * smallest; 0 if not. */
int wt3d_general_ordering_uses_metis(void);
int wt3d_analyse_csr_info(int n, long long nnz, const int *irptr, const int *jcptr, int base, int leaf_dofs,
                          long long *info, double *flops);
int wt3d_analyse_csr_export(int n, long long nnz, const int *irptr, const int *jcptr, int base, int leaf_dofs,
                            int *perm, int *fp, int *fb, int *ffirst, int *fparent, int *flevel, int *border,
                            int *rel);

/* Select the CUDA device of the calling thread (one process per GPU). */
int wt3d_set_device(int dev);

/* The CUDA stream (cudaStream_t) the factorisation and operator calls of this
 * handle run on.  Solves and refinement run on a second stream of the
 * handle, created with the greatest priority, so that they are scheduled
 * ahead of other handles' factorisations. */
void *wt3d_get_stream(wt3d_solver *h);

/* Factor the current operator once with an event pair around every launch
 * (no CUDA graph).  out[0..8] = ms in {memset, scatter, extend-add, panel,
 * trsm, SIMT gemm, diagonal solve, tensor-core operand split, tensor-core
 * gemm} launches, out[9] = GEMM real flops (both paths), out[10] = GEMM
 * launches.  out must hold 11 doubles. */
int wt3d_profile_factor(wt3d_solver *h, double *out);

/* One forward + backward substitution pass over m right-hand sides (no CUDA
 * graph, an event pair per launch): out[0..10] as wt3d_profile_factor,
 * out[11] = ms of one FP64 residual over m columns.  out holds 12 doubles. */
int wt3d_profile_solve(wt3d_solver *h, int m, double *out);

/* Per-launch profile of the factor schedule (which = 0; factors the current
 * operator) or of one substitution pass over m <= 32 columns (which = 1):
 * out[4i..4i+3] = launch kind (0 memset, 1 scatter, 2 extend-add, 3 panel,
 * 4 trsm, 5 SIMT GEMM, 6 diagonal solve, 7 tensor-core split, 8 tensor-core
 * GEMM), milliseconds, real flops, operand bytes; at most cap launches are
 * written and *count receives the number of launches. */
int wt3d_profile_launches(wt3d_solver *h, int which, int m, double *out, int cap, int *count);

/* Copy internal device state to the host for checks (what = 0: factor pool,
 * complex entries of the handle's precision; 1: pivot indices). */
int wt3d_debug_fetch(wt3d_solver *h, int what, void *out, long long count);

/* One complex64 GEMM C -= A B on host row-major arrays through the tensor-core
 * kernel (path 1), the SIMT kernel (path 0) or the tall-skinny tensor-core
 * kernel of the substitution passes (path 3, N <= 32; path 4 also gathers B
 * rows K-1-k and scatters C rows M-1-r; path 5 computes C -= A^H B with A
 * given as the K x M block, lda >= M); for checks of the kernels. */
int wt3d_debug_gemm(int path, int M, int N, int K, const void *A, int lda, const void *B, int ldb, void *C,
                    int ldc);

/* Device-resident timing of the GEMM kernels: average ms of `iters`
 * launches of C -= A B (M x K by K x N complex64, device-filled operands);
 * path 1 = tensor-core kernel (operand split excluded), 0 = SIMT kernel,
 * 2 = tall-skinny SIMT kernel, 3 = tall-skinny tensor-core kernel (B
 * expansion excluded; A by TMA when 16-byte aligned with an even stride),
 * 6 = path 3 with A always copied by the loader warps; paths 2, 3 and 6 need
 * N <= 32. */
int wt3d_bench_gemm(int path, int M, int N, int K, int iters, double *ms_out);

/* ---- allocation-free entry point ----------------------------------------
 * No counterpart in the reference.  C -= A B for complex64 device arrays
 * (row-major, leading dimensions in elements; A is M x K, B is K x N, C is
 * M x N) on the tensor cores, like the front updates, without allocating any
 * device memory: the operand split lives in a fixed scratch array inside the
 * library, wt3d_gemm_noalloc_max_floats() floats (64 MiB) held on every GPU
 * that loads the library until the process exits.  For callers that cannot
 * call cudaMalloc (device memory owned by another allocator or budget, or a
 * path that must not pay for allocation and its device synchronisation).
 * Problems needing more than the limit (2 M Kr + 4 N Kr floats, Kr = 2K
 * rounded up to 64) are rejected with WT3D_ERR_ARG.  The first call on a
 * device resolves the scratch address on that device.  All calls share the
 * scratch, so calls that overlap on the GPU race.  Runs on `stream`
 * (cudaStream_t, NULL = default) and returns when the product is complete. */
long long wt3d_gemm_noalloc_max_floats(void);
int wt3d_gemm_noalloc(int M, int N, int K, const void *dA, int lda, const void *dB, int ldb, void *dC, int ldc,
                      void *stream);

/* Factorisation workspaces per grid (1 to 8, default 1).  The level update
 * buffers a factorisation needs while it runs (the F22 Schur blocks of two
 * tree levels) are shared by the handles of a grid, which then factor one at
 * a time.  With n > 1, handles created later get their own workspace while
 * fewer than n exist, so up to n factorisations of one grid run at once, at
 * the cost of one more workspace each (wt3d_solver_bytes out[2]).  Applies to
 * handles created afterwards.  No counterpart in the reference, which holds a
 * single solver instance (strumpack_finter.c:15,19-20). */
int wt3d_set_workspaces_per_grid(int n);

/* Last error message of the calling thread (static storage). */
const char *wt3d_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
