// C ABI of libwtomo3d_gpu: the drop-in strumpack_serial_finter job protocol,
// the handle-based wt3d_* solver, and the FP64 iterative refinement that wraps
// the complex64 multifrontal factorisation.
#include <atomic>
#include "engine.cuh"
#include "wtomo3d_gpu.h"
#include <array>
#include <chrono>
#include <map>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <mutex>

namespace wt3d {

static thread_local std::string g_err;
void set_error(const std::string &msg) { g_err = msg; }

// ---------------------------------------------------------------------------
// FP64 refinement kernels (natural ordering, row-major n x MAXRHS complex128)
// ---------------------------------------------------------------------------
__global__ void k_cm_to_rm(long long n, int m, const double2 *__restrict__ cm, double2 *__restrict__ rm)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int j = 0; j < m; j++) rm[i * MAXRHS + j] = cm[(long long)j * n + i];
}

__global__ void k_rm_to_cm(long long n, int m, const double2 *__restrict__ rm, double2 *__restrict__ cm)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int j = 0; j < m; j++) cm[(long long)j * n + i] = rm[i * MAXRHS + j];
}

__global__ void k_rm_to_cm_neg(long long n, int m, const double2 *__restrict__ rm, double2 *__restrict__ cm)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int j = 0; j < m; j++) {
        const double2 v = rm[i * MAXRHS + j];
        cm[(long long)j * n + i] = make_double2(-v.x, -v.y);
    }
}

// R = B - op(A) X (op = A or A^H), per-column squared norms of R into nr and of B into nb.
// One warp per grid node; lane l holds right-hand sides l, l + 32, ...
// (NH = MAXRHS / 32 of them).  The node's three rows (u, v, w) are contiguous
// in the CSR and share one column list, so each column index and each row of
// X is loaded once for the three rows.
constexpr int NH = MAXRHS / 32;
static_assert(MAXRHS % 32 == 0, "k_residual maps right-hand sides to lanes in groups of 32");
__global__ void __launch_bounds__(256) k_residual(long long n, int m, const int *__restrict__ irptr,
                                                  const int *__restrict__ jcptr, const double2 *__restrict__ a,
                                                  const int *__restrict__ tpos, const double2 *__restrict__ X,
                                                  const double2 *__restrict__ B, double2 *__restrict__ R,
                                                  double *__restrict__ nr, double *__restrict__ nb, int adjoint)
{
    const int lane = threadIdx.x & 31;
    const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const long long nnode = n / 3;
    bool on[NH];
    double sr[NH], sb[NH];
#pragma unroll
    for (int h = 0; h < NH; h++) { on[h] = lane + 32 * h < m; sr[h] = sb[h] = 0; }
    for (long long g = w0; g < nnode; g += nw) {
        const long long r0 = 3 * g;
        const int k0 = irptr[r0];
        const int len = irptr[r0 + 1] - k0;
        double2 acc[3][NH];
#pragma unroll
        for (int q = 0; q < 3; q++)
#pragma unroll
            for (int h = 0; h < NH; h++) acc[q][h] = make_double2(0, 0);
#pragma unroll 3
        for (int t = 0; t < len; t++) {
            const int k = k0 + t;
            const double2 *xr = X + (long long)jcptr[k] * MAXRHS + lane;
            double2 x[NH];
#pragma unroll
            for (int h = 0; h < NH; h++) x[h] = on[h] ? xr[32 * h] : make_double2(0, 0);
#pragma unroll
            for (int q = 0; q < 3; q++) {
                double2 av;
                if (adjoint) { av = a[tpos[k + q * len]]; av.y = -av.y; }
                else av = a[k + q * len];
#pragma unroll
                for (int h = 0; h < NH; h++) {
                    acc[q][h].x = fma(av.x, x[h].x, fma(-av.y, x[h].y, acc[q][h].x));
                    acc[q][h].y = fma(av.x, x[h].y, fma(av.y, x[h].x, acc[q][h].y));
                }
            }
        }
#pragma unroll
        for (int h = 0; h < NH; h++) {
            if (!on[h]) continue;
            const int j = lane + 32 * h;
#pragma unroll
            for (int q = 0; q < 3; q++) {
                // B == nullptr: R = op(A) X (the products of the Krylov solver)
                const double2 b = B ? B[(r0 + q) * MAXRHS + j] : make_double2(0, 0);
                const double2 r = B ? make_double2(b.x - acc[q][h].x, b.y - acc[q][h].y) : acc[q][h];
                R[(r0 + q) * MAXRHS + j] = r;
                sr[h] += r.x * r.x + r.y * r.y;
                sb[h] += b.x * b.x + b.y * b.y;
            }
        }
    }
#pragma unroll
    for (int h = 0; h < NH; h++)
        if (on[h]) { atomicAdd(&nr[lane + 32 * h], sr[h]); atomicAdd(&nb[lane + 32 * h], sb[h]); }
}

// The same residual for a general pattern: one warp per row, rows of any
// length and columns in any order.
__global__ void __launch_bounds__(256) k_residual_rows(long long n, int m, const int *__restrict__ irptr,
                                                       const int *__restrict__ jcptr, const double2 *__restrict__ a,
                                                       const int *__restrict__ tpos, const double2 *__restrict__ X,
                                                       const double2 *__restrict__ B, double2 *__restrict__ R,
                                                       double *__restrict__ nr, double *__restrict__ nb, int adjoint)
{
    const int lane = threadIdx.x & 31;
    const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    bool on[NH];
    double sr[NH], sb[NH];
#pragma unroll
    for (int h = 0; h < NH; h++) { on[h] = lane + 32 * h < m; sr[h] = sb[h] = 0; }
    for (long long r = w0; r < n; r += nw) {
        double2 acc[NH];
#pragma unroll
        for (int h = 0; h < NH; h++) acc[h] = make_double2(0, 0);
        for (int k = irptr[r]; k < irptr[r + 1]; k++) {
            const double2 *xr = X + (long long)jcptr[k] * MAXRHS + lane;
            double2 av;
            if (adjoint) { av = a[tpos[k]]; av.y = -av.y; }
            else av = a[k];
#pragma unroll
            for (int h = 0; h < NH; h++) {
                const double2 x = on[h] ? xr[32 * h] : make_double2(0, 0);
                acc[h].x = fma(av.x, x.x, fma(-av.y, x.y, acc[h].x));
                acc[h].y = fma(av.x, x.y, fma(av.y, x.x, acc[h].y));
            }
        }
#pragma unroll
        for (int h = 0; h < NH; h++) {
            if (!on[h]) continue;
            const int j = lane + 32 * h;
            const double2 b = B ? B[r * MAXRHS + j] : make_double2(0, 0);
            const double2 q = B ? make_double2(b.x - acc[h].x, b.y - acc[h].y) : acc[h];
            R[r * MAXRHS + j] = q;
            sr[h] += q.x * q.x + q.y * q.y;
            sb[h] += b.x * b.x + b.y * b.y;
        }
    }
#pragma unroll
    for (int h = 0; h < NH; h++)
        if (on[h]) { atomicAdd(&nr[lane + 32 * h], sr[h]); atomicAdd(&nb[lane + 32 * h], sb[h]); }
}

// ---- batched Krylov kernels over n x MAXRHS row-major FP64 blocks -------
// Column c of every block is an independent system; reductions go through
// per-block partial sums and a second pass, so they do not depend on
// scheduling.
constexpr int GM_KMAX = 16;      // longest restart of the flexible GMRES (per-call length gmres_restart())
constexpr int GM_BLOCKS = 304;   // 2 blocks per SM for the reductions

// part[b][i][c] = sum over the rows of block b of conj(V_i[row, c]) W[row, c], i < nv.
__global__ void __launch_bounds__(256) k_mdot(long long n, int m, int nv, const double2 *__restrict__ V,
                                              long long vstride, const double2 *__restrict__ W,
                                              double2 *__restrict__ part)
{
    __shared__ double2 red[8][MAXRHS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (int i = 0; i < nv; i++) {
        const double2 *Vi = V + (long long)i * vstride;
        double2 acc[NH];
#pragma unroll
        for (int h = 0; h < NH; h++) acc[h] = make_double2(0, 0);
        for (long long r = w0; r < n; r += nw) {
#pragma unroll
            for (int h = 0; h < NH; h++) {
                const int c = lane + 32 * h;
                if (c >= m) continue;
                const double2 v = Vi[r * MAXRHS + c], w = W[r * MAXRHS + c];
                acc[h].x = fma(v.x, w.x, fma(v.y, w.y, acc[h].x));
                acc[h].y = fma(v.x, w.y, fma(-v.y, w.x, acc[h].y));
            }
        }
#pragma unroll
        for (int h = 0; h < NH; h++) red[warp][lane + 32 * h] = acc[h];
        __syncthreads();
        if (threadIdx.x < MAXRHS) {
            double2 t = make_double2(0, 0);
            for (int q = 0; q < 8; q++) { t.x += red[q][threadIdx.x].x; t.y += red[q][threadIdx.x].y; }
            part[((long long)blockIdx.x * (GM_KMAX + 1) + i) * MAXRHS + threadIdx.x] = t;
        }
        __syncthreads();
    }
}

// h[i][c] = sum_b part[b][i][c]
__global__ void k_mdot_reduce(int nblocks, int nv, const double2 *__restrict__ part, double2 *__restrict__ h)
{
    const int i = blockIdx.x, c = threadIdx.x;
    if (i >= nv || c >= MAXRHS) return;
    double2 t = make_double2(0, 0);
    for (int b = 0; b < nblocks; b++) {
        const double2 v = part[((long long)b * (GM_KMAX + 1) + i) * MAXRHS + c];
        t.x += v.x; t.y += v.y;
    }
    h[i * MAXRHS + c] = t;
}

// W[row, c] -= sum_{i < nv} coef[i][c] V_i[row, c]; with part != nullptr also
// part[b][c] = per-block sum of |W_new[row, c]|^2.
__global__ void __launch_bounds__(256) k_maxpy(long long n, int m, int nv, const double2 *__restrict__ V,
                                               long long vstride, const double2 *__restrict__ coef,
                                               double2 *__restrict__ W, double *__restrict__ part)
{
    __shared__ double red[256];
    const long long tot = n * MAXRHS;
    const long long stride = (long long)gridDim.x * blockDim.x;   // a multiple of MAXRHS: fixed column per thread
    const int c = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) % MAXRHS);
    double2 cf[GM_KMAX + 1];
#pragma unroll
    for (int i = 0; i <= GM_KMAX; i++) cf[i] = i < nv ? coef[i * MAXRHS + c] : make_double2(0, 0);
    double s2 = 0;
    if (c < m) {
        for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < tot; q += stride) {
            double2 w = W[q];
#pragma unroll
            for (int i = 0; i <= GM_KMAX; i++) {
                if (i >= nv) break;
                const double2 v = V[(long long)i * vstride + q];
                w.x -= cf[i].x * v.x - cf[i].y * v.y;
                w.y -= cf[i].x * v.y + cf[i].y * v.x;
            }
            W[q] = w;
            s2 += w.x * w.x + w.y * w.y;
        }
    }
    if (!part) return;
    red[threadIdx.x] = s2;
    __syncthreads();
    if (threadIdx.x < MAXRHS) {
        double t = 0;
        for (int q = threadIdx.x; q < 256; q += MAXRHS) t += red[q];
        part[(long long)blockIdx.x * MAXRHS + threadIdx.x] = t;
    }
}

__global__ void k_norm_reduce(int nblocks, const double *__restrict__ part, double *__restrict__ out)
{
    const int c = threadIdx.x;
    if (c >= MAXRHS) return;
    double t = 0;
    for (int b = 0; b < nblocks; b++) t += part[(long long)b * MAXRHS + c];
    out[c] = t;
}

// W[row, c] *= s[c]
__global__ void k_colscale(long long n, const double *__restrict__ sc, double2 *__restrict__ W)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n * MAXRHS) return;
    const double f = sc[q % MAXRHS];
    W[q].x *= f;
    W[q].y *= f;
}

// Spread sources: F[src_col[e] * n + 3 node[e] + comp[e]] += w[e] * sterm[e]
// (one thread per (source, weight) entry; entries of one source are distinct).
__global__ void k_put_sources(long long n, long long ne, const int *__restrict__ col, const long long *__restrict__ node,
                              const int *__restrict__ comp, const double *__restrict__ w,
                              const double2 *__restrict__ sterm, double2 *__restrict__ F)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const double2 s = sterm[col[e]];
    double2 *p = F + (long long)col[e] * n + 3 * node[e] + comp[e];
    p->x += w[e] * s.x;
    p->y += w[e] * s.y;
}

// Receivers: out[(j nrec + r) 3 + c] = sum_e w[e] U_j[3 node[e] + c] over the
// entries e of receiver r (rec_start[r] .. rec_start[r+1]).
__global__ void k_get_receivers(long long n, int m, int nrec, const int *__restrict__ rec_start,
                                const long long *__restrict__ node, const double *__restrict__ w,
                                const double2 *__restrict__ U, double2 *__restrict__ out)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long long)m * nrec * 3) return;
    const int c = (int)(q % 3), r = (int)((q / 3) % nrec), j = (int)(q / (3LL * nrec));
    double2 acc = make_double2(0, 0);
    for (int e = rec_start[r]; e < rec_start[r + 1]; e++) {
        const double2 u = U[(long long)j * n + 3 * node[e] + c];
        acc.x += w[e] * u.x;
        acc.y += w[e] * u.y;
    }
    out[q] = acc;
}

// Xs = S R (new ordering, engine precision); S the Jacobi scaling of the factor.
template <class T>
__global__ void k_gather_new(long long n, int m, const int *__restrict__ perm, const double *__restrict__ s,
                             const double2 *__restrict__ R, cx<T> *__restrict__ Xs)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n * m) return;
    long long i = q / m;
    int j = (int)(q % m);
    const long long o = perm[i];
    double2 v = R[o * MAXRHS + j];
    const double w = s[o];
    Xs[i * MAXRHS + j] = cx<T>((T)(v.x * w), (T)(v.y * w));
}

// Xn += S Xs (natural ordering, FP64 accumulate).
template <class T>
__global__ void k_scatter_add_nat(long long n, int m, const int *__restrict__ perm, const double *__restrict__ s,
                                  const cx<T> *__restrict__ Xs, double2 *__restrict__ Xn)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n * m) return;
    long long i = q / m;
    int j = (int)(q % m);
    cx<T> v = Xs[i * MAXRHS + j];
    const long long o = perm[i];
    const double w = s[o];
    double2 *d = Xn + o * MAXRHS + j;
    d->x += (double)v.re * w;
    d->y += (double)v.im * w;
}

__global__ void k_pw_expand(int nx, int ny, int nz, double dx, int m, const double2 *__restrict__ Uz,
                            const double2 *__restrict__ Wz, const double *__restrict__ kx,
                            const double *__restrict__ ky, const double *__restrict__ rx,
                            const double *__restrict__ ry, double2 *__restrict__ U0, int ld);
__global__ void k_hetfld(long long n, int m, const int *__restrict__ irptr, const int *__restrict__ jcptr,
                         const double2 *__restrict__ a, const double2 *__restrict__ abg,
                         const double2 *__restrict__ U0, int ld, double2 *__restrict__ F);
int haskgrn_host(const wt3d_layered1d &M, double omega, double ain, int s_wave, int nz, double dz, double zorig,
                 std::complex<double> *U, std::complex<double> *W);

__global__ void k_c64_to_c128(long long n, const float2 *__restrict__ s, double2 *__restrict__ d)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = make_double2(s[i].x, s[i].y);
}

// Values of an unsymmetric caller pattern into the stored A + A^T pattern
// (its other entries are zero): d[map[i]] = s[i].
__global__ void k_spread_c64(long long n, const float2 *__restrict__ s, const int *__restrict__ map,
                             double2 *__restrict__ d)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[map[i]] = make_double2(s[i].x, s[i].y);
}

__global__ void k_spread_c128(long long n, const double2 *__restrict__ s, const int *__restrict__ map,
                              double2 *__restrict__ d)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[map[i]] = s[i];
}

}  // namespace wt3d

using namespace wt3d;

namespace wt3d {
// Host analysis of one grid, shared by every handle of that grid: nested
// dissection + symbolic factorisation, the CSR -> front scatter map and the
// transposed CSR positions, and the factorisation workspaces of both
// precisions (alive while a handle uses them).
struct GridAnalysis {
    Symbolic sym;
    std::vector<long long> map;
    std::vector<int> tpos;
    std::mutex mu;
    // factorisation workspaces of this grid (up to wt3d_set_workspaces_per_grid)
    std::vector<std::weak_ptr<FactorWorkspace<float>>> ws32;
    std::vector<std::weak_ptr<FactorWorkspace<double>>> ws64;
};
}  // namespace wt3d

struct wt3d_solver {
    wt3d_grid grid{};
    int prec = WT3D_PREC_MIXED;
    bool general = false;                 // caller's pattern (wt3d_solver_create_csr), not the grid graph
    std::shared_ptr<GridAnalysis> ga;
    long long n = 0, nnz = 0;             // the (symmetrised) pattern the handle stores
    long long nnz_in = 0;                 // entries of the caller's pattern
    DevVec<int> irptr, jcptr, tpos, perm;
    DevVec<int> vmap;                     // caller entry -> stored entry (unsymmetric patterns only)
    DevVec<double2> a;
    DevVec<double2> da, mu;
    DevVec<double> ro;
    DevVec<float> vp, vs, rho;
    DevVec<float> qp, qs;                 // 1/Q per node (attenuation), optional
    double freqbase = 0;
    DevVec<double2> Bn, Xn, Rn, T1;
    DevVec<double2> abg, bgda, bgmu;      // background operator and Lame arrays
    DevVec<double> bgro;
    bool have_bg = false;
    double om_re = 0, om_im = 0;          // omega of the assembled operator
    DevVec<double> norms;
    DevVec<double> gscr;                  // per-row derivative records of the gradient
    DevVec<double2> batF, batX;           // caller batch buffers (wt3d_batch_buffers)
    StreamBuf<double2> gmV, gmZ;          // flexible GMRES: Krylov basis, preconditioned basis (per call)
    DevVec<double2> gmH;                  // flexible GMRES: projections
    DevVec<double2> gmPart;
    DevVec<double> gmNorm, gmScale;
    std::unique_ptr<Engine<float>> e32;
    std::unique_ptr<Engine<double>> e64;
    cudaStream_t st = nullptr;
    cudaStream_t sts = nullptr;           // substitution and refinement work, highest priority
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t evl = nullptr;            // marks the legacy default stream at entry to a device-buffer call
    bool have_model = false, have_values = false, have_factor = false;
    long long kernels_solve = 0;
    wt3d_stats stats{};
    ~wt3d_solver()
    {
        if (st) cudaStreamSynchronize(st);
        if (sts) cudaStreamSynchronize(sts);
        e32.reset();
        e64.reset();
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (evl) cudaEventDestroy(evl);
        if (st) cudaStreamDestroy(st);
        if (sts) cudaStreamDestroy(sts);
    }
};

namespace {

double ms_between(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

int check_grid(const wt3d_grid *g)
{
    if (!g || g->nx < 2 || g->ny < 2 || g->nz < 2 || !(g->dx > 0)) {
        set_error("invalid grid: need nx, ny, nz >= 2 and dx > 0");
        return WT3D_ERR_ARG;
    }
    long long nnz = wt3d_pattern_nnz(g->nx, g->ny, g->nz);
    if (nnz >= (1LL << 31)) {
        set_error("grid too large: nnz >= 2^31");
        return WT3D_ERR_ARG;
    }
    return WT3D_OK;
}

int have_gpu()
{
    int nd = 0;
    if (cudaGetDeviceCount(&nd) != cudaSuccess || nd == 0) {
        set_error("no CUDA device available");
        return WT3D_ERR_NOGPU;
    }
    return WT3D_OK;
}

// R = B - op(A) X (R = op(A) X when B is null), accumulating the squared
// column norms of R and B into h->norms: node-blocked rows for the grid
// pattern, one warp per row for a general pattern.
void residual(const wt3d_solver *h, cudaStream_t st, int m, const double2 *X, const double2 *B, double2 *R,
              bool adjoint)
{
    if (h->general)
        k_residual_rows<<<152 * 8, 256, 0, st>>>(h->n, m, h->irptr.p, h->jcptr.p, h->a.p, h->tpos.p, X, B, R,
                                                 h->norms.p, h->norms.p + MAXRHS, adjoint ? 1 : 0);
    else
        k_residual<<<152 * 8, 256, 0, st>>>(h->n, m, h->irptr.p, h->jcptr.p, h->a.p, h->tpos.p, X, B, R,
                                            h->norms.p, h->norms.p + MAXRHS, adjoint ? 1 : 0);
}

// Restarted flexible GMRES in FP64, right-preconditioned by the factorisation
// (z = M^-1 v is one substitution pass), over m columns.  On entry h->Xn holds
// the current iterate, h->Rn = B - op(A) Xn and bnorm2/rnorm2 the squared
// column norms of B and R; on exit Xn is the new iterate.  Classical
// Gram-Schmidt applied twice; Givens rotations and the small least-squares
// problems per column on the host.  The restart length is 8 unless the
// WT3D_GMRES_RESTART environment variable sets another (1..16); each Arnoldi
// vector costs 2 blocks of n x 32 complex128 while the call runs.
static int gmres_restart()
{
    static const int k = [] {
        const char *e = getenv("WT3D_GMRES_RESTART");
        const int v = e ? atoi(e) : 8;
        return v < 1 ? 1 : (v > GM_KMAX ? GM_KMAX : v);
    }();
    return k;
}

template <class T>
int fgmres(wt3d_solver *h, Engine<T> &E, Schedule<T> *sc, int m, bool adjoint, double tol, int maxit,
           const std::vector<double> &bnorm2, std::vector<double> &rnorm2, double *relres, int &it)
{
    cudaStream_t st = h->sts;
    const long long n = h->n, blk = n * MAXRHS;
    const int kr = gmres_restart();
    int rc;
    if (!h->gmH.p) {
        if ((rc = h->gmH.alloc((size_t)(GM_KMAX + 1) * MAXRHS)) ||
            (rc = h->gmPart.alloc((size_t)GM_BLOCKS * (GM_KMAX + 1) * MAXRHS)) ||
            (rc = h->gmNorm.alloc(MAXRHS)) || (rc = h->gmScale.alloc(MAXRHS)))
            return rc;
    }
    // the Krylov bases live for the call only (they are not part of a
    // handle's resident memory), in stream order on the handle's solve
    // stream, so that taking and returning them never waits for work of
    // other handles
    if ((rc = h->gmV.alloc((size_t)blk * (kr + 1), st)) || (rc = h->gmZ.alloc((size_t)blk * kr, st))) return rc;
    struct Release {
        wt3d_solver *h;
        ~Release() { h->gmV.release(); h->gmZ.release(); }
    } release{h};
    double2 *V = h->gmV.p, *Z = h->gmZ.p;
    const int th = 256;
    const unsigned nbm = (unsigned)ceil_div(n * m, th), nbb = (unsigned)ceil_div(blk, th);
    typedef std::complex<double> C;
    std::vector<double> sc_h(MAXRHS);
    std::vector<double2> hb((kr + 1) * MAXRHS), hb2((kr + 1) * MAXRHS), coef((kr + 1) * MAXRHS);
    std::vector<double> wn(MAXRHS);
    auto orth = [&](int nv, double2 *W, std::vector<double2> &out, bool norm) -> int {
        k_mdot<<<GM_BLOCKS, 256, 0, st>>>(n, m, nv, V, blk, W, h->gmPart.p);
        k_mdot_reduce<<<nv, MAXRHS, 0, st>>>(GM_BLOCKS, nv, h->gmPart.p, h->gmH.p);
        k_maxpy<<<GM_BLOCKS, 256, 0, st>>>(n, m, nv, V, blk, h->gmH.p, W, norm ? (double *)h->gmPart.p : nullptr);
        if (norm) k_norm_reduce<<<1, MAXRHS, 0, st>>>(GM_BLOCKS, (const double *)h->gmPart.p, h->gmNorm.p);
        WT_CUDA(cudaGetLastError());
        WT_CUDA(cudaMemcpyAsync(out.data(), h->gmH.p, sizeof(double2) * nv * MAXRHS, cudaMemcpyDeviceToHost, st));
        if (norm) WT_CUDA(cudaMemcpyAsync(wn.data(), h->gmNorm.p, sizeof(double) * MAXRHS, cudaMemcpyDeviceToHost, st));
        WT_CUDA(cudaStreamSynchronize(st));
        return WT3D_OK;
    };
    for (;;) {
        // ---- one cycle from the current residual ----
        std::vector<double> beta(m);
        std::vector<int> done(m, 0), len(m, 0);
        for (int c = 0; c < m; c++) {
            beta[c] = sqrt(rnorm2[c]);
            const double bn = sqrt(bnorm2[c]);
            done[c] = !(beta[c] > tol * (bn > 0 ? bn : 1.0));
            sc_h[c] = done[c] ? 0.0 : 1.0 / beta[c];
        }
        for (int c = m; c < MAXRHS; c++) sc_h[c] = 0.0;
        WT_CUDA(cudaMemcpyAsync(V, h->Rn.p, sizeof(double2) * blk, cudaMemcpyDeviceToDevice, st));
        WT_CUDA(cudaMemcpyAsync(h->gmScale.p, sc_h.data(), sizeof(double) * MAXRHS, cudaMemcpyHostToDevice, st));
        k_colscale<<<nbb, th, 0, st>>>(n, h->gmScale.p, V);
        std::vector<std::vector<C>> H(m, std::vector<C>((kr + 1) * kr, C(0)));
        std::vector<std::vector<C>> g(m, std::vector<C>(kr + 1, C(0))), cs(m, std::vector<C>(kr)),
            sn(m, std::vector<C>(kr));
        for (int c = 0; c < m; c++) g[c][0] = beta[c];
        int j = 0;
        for (; j < kr; j++) {
            bool all = true;
            for (int c = 0; c < m; c++) all = all && done[c];
            if (all || it >= maxit) break;
            // z_j = M^-1 v_j
            double2 *Vj = V + (long long)j * blk, *Zj = Z + (long long)j * blk, *W = V + (long long)(j + 1) * blk;
            k_gather_new<T><<<nbm, th, 0, st>>>(n, m, h->perm.p, E.scale.p, Vj, E.X.p);
            if ((rc = E.run(*sc, st))) return rc;
            WT_CUDA(cudaMemsetAsync(Zj, 0, sizeof(double2) * blk, st));
            k_scatter_add_nat<T><<<nbm, th, 0, st>>>(n, m, h->perm.p, E.scale.p, E.X.p, Zj);
            // w = op(A) z_j
            WT_CUDA(cudaMemsetAsync(h->norms.p, 0, sizeof(double) * 2 * MAXRHS, st));
            residual(h, st, m, Zj, nullptr, W, adjoint);
            h->kernels_solve += sc->kernels() + 11;
            if ((rc = orth(j + 1, W, hb, false)) || (rc = orth(j + 1, W, hb2, true))) return rc;
            it++;
            for (int c = 0; c < m; c++) {
                if (done[c]) { sc_h[c] = 0.0; continue; }
                std::vector<C> &Hc = H[c];
                for (int i = 0; i <= j; i++)
                    Hc[i * kr + j] = C(hb[i * MAXRHS + c].x + hb2[i * MAXRHS + c].x,
                                         hb[i * MAXRHS + c].y + hb2[i * MAXRHS + c].y);
                const double hn = sqrt(wn[c]);
                // earlier rotations, then a new one zeroing H[j+1][j]
                for (int i = 0; i < j; i++) {
                    const C a = Hc[i * kr + j], b = Hc[(i + 1) * kr + j];
                    Hc[i * kr + j] = std::conj(cs[c][i]) * a + std::conj(sn[c][i]) * b;
                    Hc[(i + 1) * kr + j] = -sn[c][i] * a + cs[c][i] * b;
                }
                const C a = Hc[j * kr + j];
                const double den = sqrt(std::norm(a) + hn * hn);
                cs[c][j] = den > 0 ? a / den : C(1);
                sn[c][j] = den > 0 ? C(hn / den) : C(0);
                Hc[j * kr + j] = den;
                g[c][j + 1] = -sn[c][j] * g[c][j];
                g[c][j] = std::conj(cs[c][j]) * g[c][j];
                len[c] = j + 1;
                const double bn = sqrt(bnorm2[c]);
                const double est = std::abs(g[c][j + 1]) / (bn > 0 ? bn : 1.0);
                if (relres) relres[c] = est;
                if (est <= 0.5 * tol || hn <= 1e-300) done[c] = 1;
                sc_h[c] = done[c] ? 0.0 : 1.0 / hn;
            }
            WT_CUDA(cudaMemcpyAsync(h->gmScale.p, sc_h.data(), sizeof(double) * MAXRHS, cudaMemcpyHostToDevice, st));
            k_colscale<<<nbb, th, 0, st>>>(n, h->gmScale.p, W);
        }
        // x += Z y, y = R^-1 g per column
        const int jmax = j;
        if (jmax > 0) {
            std::fill(coef.begin(), coef.end(), make_double2(0, 0));
            for (int c = 0; c < m; c++) {
                const int L = len[c];
                std::vector<C> y(L);
                for (int i = L - 1; i >= 0; i--) {
                    C t = g[c][i];
                    for (int q = i + 1; q < L; q++) t -= H[c][i * kr + q] * y[q];
                    y[i] = t / H[c][i * kr + i];
                }
                for (int i = 0; i < L; i++) coef[i * MAXRHS + c] = make_double2(-y[i].real(), -y[i].imag());
            }
            WT_CUDA(cudaMemcpyAsync(h->gmH.p, coef.data(), sizeof(double2) * jmax * MAXRHS, cudaMemcpyHostToDevice, st));
            k_maxpy<<<GM_BLOCKS, 256, 0, st>>>(n, m, jmax, Z, blk, h->gmH.p, h->Xn.p, nullptr);
        }
        // true residual
        std::vector<double> hn2(2 * MAXRHS);
        WT_CUDA(cudaMemsetAsync(h->norms.p, 0, sizeof(double) * 2 * MAXRHS, st));
        residual(h, st, m, h->Xn.p, h->Bn.p, h->Rn.p, adjoint);
        WT_CUDA(cudaGetLastError());
        WT_CUDA(cudaMemcpyAsync(hn2.data(), h->norms.p, sizeof(double) * 2 * MAXRHS, cudaMemcpyDeviceToHost, st));
        WT_CUDA(cudaStreamSynchronize(st));
        double worst = 0;
        for (int c = 0; c < m; c++) {
            rnorm2[c] = hn2[c];
            const double r = hn2[MAXRHS + c] > 0 ? sqrt(hn2[c] / hn2[MAXRHS + c]) : sqrt(hn2[c]);
            if (relres) relres[c] = r;
            worst = std::max(worst, r);
        }
        if (!(worst == worst)) return WT3D_ERR_NOCONV;
        if (worst <= tol) return WT3D_OK;
        if (it >= maxit || jmax == 0) return WT3D_ERR_NOCONV;
    }
}

// Plain refinement continues while a pass cuts the worst residual by at least
// this factor (WT3D_REFINE_SWITCH, default 0.08); otherwise the solve
// switches to the flexible GMRES, which reaches the tolerance in fewer
// passes once refinement converges more slowly than that.  The first pass
// counts as a refinement step from x = 0 (relative residual 1), so a
// preconditioner that leaves more than that fraction of the right-hand side
// goes to GMRES after one pass.
static double refine_switch()
{
    static const double v = [] {
        const char *e = getenv("WT3D_REFINE_SWITCH");
        const double x = e ? atof(e) : 0.08;
        return (x > 0 && x < 1) ? x : 0.08;
    }();
    return v;
}

// Refinement driver over m <= MAXRHS columns held in h->Bn; result in h->Xn.
// Plain iterative refinement while each step reduces the worst residual by
// the switch factor; flexible GMRES preconditioned by the same factors
// otherwise (a few near-singular modes of the preconditioned operator slow
// refinement down, and the Krylov solver removes them in a few steps).
template <class T>
int refine(wt3d_solver *h, Engine<T> &E, int m, bool adjoint, double tol, int maxit, double *relres, int *iters)
{
    cudaStream_t st = h->sts;
    const long long n = h->n;
    Schedule<T> *sc = E.solve_schedule(m, adjoint);
    if (!sc) return WT3D_ERR_NOMEM;
    WT_CUDA(cudaMemsetAsync(h->Xn.p, 0, sizeof(double2) * n * MAXRHS, st));
    // start from R = B
    WT_CUDA(cudaMemcpyAsync(h->Rn.p, h->Bn.p, sizeof(double2) * n * MAXRHS, cudaMemcpyDeviceToDevice, st));
    std::vector<double> hn(2 * MAXRHS);
    int it = 0, rc = WT3D_OK;
    // the first pass is a refinement step from x = 0, whose relative residual is 1
    double prev_worst = 1.0;
    const int th = 256;
    const unsigned nb = (unsigned)ceil_div(n * m, th);
    for (;;) {
        k_gather_new<T><<<nb, th, 0, st>>>(n, m, h->perm.p, E.scale.p, h->Rn.p, E.X.p);
        rc = E.run(*sc, st);
        if (rc) return rc;
        h->kernels_solve += sc->kernels() + 3;   // + gather, scatter-add, residual
        k_scatter_add_nat<T><<<nb, th, 0, st>>>(n, m, h->perm.p, E.scale.p, E.X.p, h->Xn.p);
        WT_CUDA(cudaMemsetAsync(h->norms.p, 0, sizeof(double) * 2 * MAXRHS, st));
        residual(h, st, m, h->Xn.p, h->Bn.p, h->Rn.p, adjoint);
        WT_CUDA(cudaGetLastError());
        WT_CUDA(cudaMemcpyAsync(hn.data(), h->norms.p, sizeof(double) * 2 * MAXRHS, cudaMemcpyDeviceToHost, st));
        WT_CUDA(cudaStreamSynchronize(st));
        double worst = 0;
        for (int j = 0; j < m; j++) {
            double r = hn[MAXRHS + j] > 0 ? sqrt(hn[j] / hn[MAXRHS + j]) : sqrt(hn[j]);
            if (relres) relres[j] = r;
            worst = std::max(worst, r);
        }
        if (!(worst == worst)) { rc = WT3D_ERR_NOCONV; break; }   // NaN
        if (worst <= tol) break;
        if (it >= maxit) { rc = WT3D_ERR_NOCONV; break; }
        if (worst > refine_switch() * prev_worst) {
            std::vector<double> bn2(hn.begin() + MAXRHS, hn.begin() + MAXRHS + m), rn2(hn.begin(), hn.begin() + m);
            it++;
            rc = fgmres<T>(h, E, sc, m, adjoint, tol, maxit, bn2, rn2, relres, it);
            break;
        }
        prev_worst = worst;
        it++;
    }
    if (iters) *iters = it;
    if (rc == WT3D_ERR_NOCONV) set_error("iterative refinement did not reach the requested tolerance");
    return rc;
}

// Entry points that take caller device buffers run on the handle's own
// non-blocking streams.  Callers (PyTorch among them) commonly fill or consume
// those buffers on the legacy default stream without synchronising, so each
// such entry point first makes its stream wait for everything already queued
// there.  Work the caller queued on other streams must be complete before the
// call.  Every entry point synchronises its stream before it returns.
static int after_legacy(wt3d_solver *h, cudaStream_t s)
{
    WT_CUDA(cudaEventRecord(h->evl, cudaStreamLegacy));
    WT_CUDA(cudaStreamWaitEvent(s, h->evl, 0));
    return WT3D_OK;
}

int solve_dev_cm(wt3d_solver *h, int nrhs, const double2 *d_B, double2 *d_X, double tol, int maxit, double *relres,
                 int *iters, bool adjoint)
{
    if (!h->have_factor) { set_error("solve before factor"); return WT3D_ERR_STATE; }
    if (int rc = after_legacy(h, h->sts)) return rc;
    const long long n = h->n;
    int worst_rc = WT3D_OK, maxits = 0;
    h->kernels_solve = 0;
    cudaEventRecord(h->ev0, h->sts);
    for (int c0 = 0; c0 < nrhs; c0 += MAXRHS) {
        int m = std::min(MAXRHS, nrhs - c0);
        k_cm_to_rm<<<ceil_div(n, 256), 256, 0, h->sts>>>(n, m, d_B + (long long)c0 * n, h->Bn.p);
        h->kernels_solve += 2;   // layout conversions in and out
        int its = 0, rc;
        if (h->e32) rc = refine<float>(h, *h->e32, m, adjoint, tol, maxit, relres ? relres + c0 : nullptr, &its);
        else rc = refine<double>(h, *h->e64, m, adjoint, tol, maxit, relres ? relres + c0 : nullptr, &its);
        if (rc && rc != WT3D_ERR_NOCONV) return rc;
        if (rc) worst_rc = rc;
        maxits = std::max(maxits, its);
        k_rm_to_cm<<<ceil_div(n, 256), 256, 0, h->sts>>>(n, m, h->Xn.p, d_X + (long long)c0 * n);
    }
    cudaEventRecord(h->ev1, h->sts);
    WT_CUDA(cudaStreamSynchronize(h->sts));
    if (int rc = h->e32 ? h->e32->check_tc_err() : h->e64->check_tc_err()) return rc;
    h->stats.t_solve_ms = ms_between(h->ev0, h->ev1);
    h->stats.kernels_solve = (int)h->kernels_solve;
    if (iters) *iters = maxits;
    return worst_rc;
}

std::mutex g_ana_mu;
std::map<std::array<int, 3>, std::shared_ptr<GridAnalysis>> g_ana;

// Symbolic analysis of an nx*ny*nz grid, computed once per process.
int grid_analysis(int nx, int ny, int nz, std::shared_ptr<GridAnalysis> &out)
{
    std::lock_guard<std::mutex> lk(g_ana_mu);
    auto &slot = g_ana[{nx, ny, nz}];
    if (!slot) {
        auto ga = std::make_shared<GridAnalysis>();
        int rc = symbolic_grid(nx, ny, nz, 64, ga->sym);
        if (rc) { g_ana.erase({nx, ny, nz}); return rc; }
        slot = ga;
    }
    out = slot;
    return WT3D_OK;
}

// Factorisation workspaces per grid: handles that share one factor one at a
// time; up to this many workspaces let handles of one grid factor at once.
std::atomic<int> g_ws_per_grid{1};

// A new handle's workspace: an unused slot of the grid's pool gets a new
// workspace (allocated at the handle's first factorisation set-up); with
// every slot in use, the workspace with the fewest handles is shared.
template <class T>
std::shared_ptr<FactorWorkspace<T>> pick_workspace(std::vector<std::weak_ptr<FactorWorkspace<T>>> &pool)
{
    const size_t n = (size_t)std::max(1, g_ws_per_grid.load());
    if (pool.size() < n) pool.resize(n);
    for (size_t i = 0; i < n; i++)
        if (pool[i].expired()) {
            auto w = std::make_shared<FactorWorkspace<T>>();
            pool[i] = w;
            return w;
        }
    std::shared_ptr<FactorWorkspace<T>> best;
    for (size_t i = 0; i < n; i++) {
        auto w = pool[i].lock();
        if (w && (!best || w.use_count() < best.use_count())) best = w;
    }
    return best;
}

// Device bytes a handle holds on its own once created and factored:
// out[0] always, out[1] more once plane-wave sources are built, out[2] the
// level-parity update buffers of the shared factorisation workspace.
void handle_bytes(const Symbolic &S, long long nnz, int prec, double *out)
{
    const double n = (double)S.n, nn = n / 3, sz = prec == WT3D_PREC_MIXED ? 8.0 : 16.0;
    long long npan = 0;
    for (const Front &F : S.fronts) npan += (F.p + KB - 1) / KB;
    const double engine = (double)S.fac_total * sz + n * MAXRHS * sz + (double)npan * 2 * KB * KB * sz + n * 4 +
                          (double)(S.border.size() + S.rel.size()) * 4 + (double)S.fronts.size() * sizeof(FrontDev) +
                          (double)nnz * 8 + n * 8;
    const double api = (n + 1) * 4 + (double)nnz * (4 + 16 + 4) + n * 4 + 3 * n * MAXRHS * 16 + nn * (12 + 32 + 8);
    out[0] = engine + api;
    out[1] = (double)nnz * 16 + nn * (32 + 8);
    out[2] = ((double)std::max<long long>(S.upd_size[0], 1) + (double)std::max<long long>(S.upd_size[1], 1)) * sz;
}

// Device bytes a handle currently holds (the shared workspace excluded).
double own_bytes(const wt3d_solver *h)
{
    double b = (double)(h->e32 ? h->e32->device_bytes() : h->e64->device_bytes());
    b += (double)(h->irptr.n + h->jcptr.n + h->tpos.n + h->perm.n + h->vmap.n) * 4;
    b += (double)(h->a.n + h->da.n + h->mu.n + h->Bn.n + h->Xn.n + h->Rn.n + h->T1.n + h->abg.n + h->bgda.n +
                  h->bgmu.n + h->batF.n + h->batX.n) * 16;
    b += (double)(h->ro.n + h->bgro.n + h->norms.n + h->gscr.n) * 8 +
         (double)(h->vp.n + h->vs.n + h->rho.n + h->qp.n + h->qs.n) * 4;
    return b;
}

}  // namespace

extern "C" {

const char *wt3d_last_error(void) { return g_err.c_str(); }

int wt3d_set_workspaces_per_grid(int n)
{
    if (n < 1 || n > 8) { set_error("wt3d_set_workspaces_per_grid: need 1 <= n <= 8"); return WT3D_ERR_ARG; }
    g_ws_per_grid.store(n);
    return WT3D_OK;
}

long long wt3d_pattern_nnz(int nx, int ny, int nz)
{
    return 9LL * (3LL * nx - 2) * (3LL * ny - 2) * (3LL * nz - 2);
}

int wt3d_pattern(int nx, int ny, int nz, int base, int *irptr, int *jcptr)
{
    if (nx < 2 || ny < 2 || nz < 2 || (base != 0 && base != 1) || !irptr || !jcptr) {
        set_error("wt3d_pattern: invalid arguments");
        return WT3D_ERR_ARG;
    }
    int rc = have_gpu();
    if (rc) return rc;
    long long nnz = wt3d_pattern_nnz(nx, ny, nz);
    long long n = 3LL * nx * ny * nz;
    int *di = nullptr, *dj = nullptr;
    WT_CUDA(cudaMalloc(&di, sizeof(int) * (n + 1)));
    if (cudaMalloc(&dj, sizeof(int) * nnz) != cudaSuccess) { cudaFree(di); set_error("cudaMalloc"); return WT3D_ERR_NOMEM; }
    rc = device_pattern(nx, ny, nz, base, di, dj, 0);
    if (!rc && (cudaMemcpy(irptr, di, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(jcptr, dj, sizeof(int) * nnz, cudaMemcpyDeviceToHost) != cudaSuccess)) {
        set_error("wt3d_pattern: copy back failed");
        rc = WT3D_ERR_CUDA;
    }
    cudaFree(di);
    cudaFree(dj);
    return rc;
}

int wt3d_assemble_device(const wt3d_grid *g, const float *d_vp, const float *d_vs, const float *d_rho,
                         double omega_re, double omega_im, const int *d_irptr, void *d_a, void *stream)
{
    int rc = check_grid(g);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    long long nn = (long long)g->nx * g->ny * g->nz;
    void *da = nullptr, *mu = nullptr;
    double *ro = nullptr;
    WT_CUDA(cudaMallocAsync(&da, sizeof(double2) * nn, st));
    WT_CUDA(cudaMallocAsync(&mu, sizeof(double2) * nn, st));
    WT_CUDA(cudaMallocAsync(&ro, sizeof(double) * nn, st));
    rc = device_lame(nn, d_vp, d_vs, d_rho, da, mu, ro, st);
    if (!rc) rc = device_assemble(*g, da, mu, ro, omega_re, omega_im, d_irptr, d_a, st);
    cudaFreeAsync(da, st);
    cudaFreeAsync(mu, st);
    cudaFreeAsync(ro, st);
    return rc;
}

int wt3d_assemble(const wt3d_grid *g, const float *vp, const float *vs, const float *rho, double omega_re,
                  double omega_im, double _Complex *a)
{
    int rc = check_grid(g);
    if (rc) return rc;
    if ((rc = have_gpu())) return rc;
    if (!vp || !vs || !rho || !a) { set_error("wt3d_assemble: null pointer"); return WT3D_ERR_ARG; }
    long long nn = (long long)g->nx * g->ny * g->nz, n = 3 * nn, nnz = wt3d_pattern_nnz(g->nx, g->ny, g->nz);
    DevVec<float> dvp, dvs, drho;
    DevVec<int> di, dj;
    DevVec<double2> da;
    if ((rc = dvp.alloc(nn)) || (rc = dvs.alloc(nn)) || (rc = drho.alloc(nn)) || (rc = di.alloc(n + 1)) ||
        (rc = dj.alloc(nnz)) || (rc = da.alloc(nnz)))
        return rc;
    WT_CUDA(cudaMemcpy(dvp.p, vp, sizeof(float) * nn, cudaMemcpyHostToDevice));
    WT_CUDA(cudaMemcpy(dvs.p, vs, sizeof(float) * nn, cudaMemcpyHostToDevice));
    WT_CUDA(cudaMemcpy(drho.p, rho, sizeof(float) * nn, cudaMemcpyHostToDevice));
    if ((rc = device_pattern(g->nx, g->ny, g->nz, 0, di.p, dj.p, 0))) return rc;
    if ((rc = wt3d_assemble_device(g, dvp.p, dvs.p, drho.p, omega_re, omega_im, di.p, da.p, nullptr))) return rc;
    WT_CUDA(cudaMemcpy(a, da.p, sizeof(double2) * nnz, cudaMemcpyDeviceToHost));
    return WT3D_OK;
}

// -------------------------------------------------------------------------
}  // extern "C"

namespace {

// Leaf fronts of a general pattern hold at most this many dofs (the grid's
// leaf boxes hold 64 nodes, 192 dofs).
constexpr long long GENERAL_LEAF_DOFS = 192;

// Entry points that build or use the grid's model, sources and receivers
// refuse handles of a general pattern.
int grid_only(const char *fn)
{
    set_error(std::string(fn) + ": needs a grid handle (wt3d_solver_create), not a general pattern");
    return WT3D_ERR_STATE;
}

// Streams and events of a new handle.
int handle_streams(wt3d_solver *h)
{
    WT_CUDA(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
    {
        // solves run ahead of other handles' factorisations: their kernels are
        // short and latency-bound, a factorisation's are long
        int least = 0, greatest = 0;
        WT_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        WT_CUDA(cudaStreamCreateWithPriority(&h->sts, cudaStreamNonBlocking, greatest));
    }
    WT_CUDA(cudaEventCreate(&h->ev0));
    WT_CUDA(cudaEventCreate(&h->ev1));
    WT_CUDA(cudaEventCreateWithFlags(&h->evl, cudaEventDisableTiming));
    return WT3D_OK;
}

// The rest of a new handle once its analysis (h->ga, with the scatter map and
// transposed positions) and its 0-based pattern on the device are in place:
// the permutation, the FP64 refinement blocks and the engine of the
// precision, over the factorisation workspace w32 or w64.
int handle_engine(wt3d_solver *h, int precision, std::shared_ptr<FactorWorkspace<float>> w32,
                  std::shared_ptr<FactorWorkspace<double>> w64, std::chrono::steady_clock::time_point t0)
{
    int rc;
    const GridAnalysis &ga = *h->ga;
    const Symbolic &sym = ga.sym;
    if ((rc = h->tpos.upload(ga.tpos))) return rc;
    if ((rc = h->perm.upload(sym.perm))) return rc;
    if ((rc = h->Bn.alloc((size_t)h->n * MAXRHS)) || (rc = h->Xn.alloc((size_t)h->n * MAXRHS)) ||
        (rc = h->Rn.alloc((size_t)h->n * MAXRHS)) || (rc = h->norms.alloc(2 * MAXRHS)))
        return rc;
    if (precision == WT3D_PREC_MIXED) {
        h->e32.reset(new Engine<float>());
        rc = h->e32->init(sym, ga.map, h->irptr.p, h->jcptr.p, w32);
    } else {
        h->e64.reset(new Engine<double>());
        rc = h->e64->init(sym, ga.map, h->irptr.p, h->jcptr.p, w64);
    }
    if (rc) return rc;
    auto t1 = std::chrono::steady_clock::now();
    h->stats.n = h->n;
    h->stats.nnz = h->nnz;
    h->stats.nfronts = (long long)sym.fronts.size();
    h->stats.factor_entries = sym.fac_total;
    h->stats.factor_flops = sym.flops;
    h->stats.factor_bytes = (double)sym.fac_total * (precision == WT3D_PREC_MIXED ? 8.0 : 16.0);
    h->stats.levels = (int)sym.levels.size();
    h->stats.t_analyse_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    h->stats.device_bytes = own_bytes(h);
    h->stats.workspace_bytes = (double)(h->e32 ? h->e32->workspace_bytes() : h->e64->workspace_bytes());
    return WT3D_OK;
}

std::vector<int> to_int(const std::vector<long long> &v)
{
    return std::vector<int>(v.begin(), v.end());
}

}  // namespace

extern "C" {

int wt3d_solver_create(wt3d_solver **out, const wt3d_grid *g, int precision)
{
    if (!out) { set_error("null handle pointer"); return WT3D_ERR_ARG; }
    *out = nullptr;
    int rc = check_grid(g);
    if (rc) return rc;
    if (precision != WT3D_PREC_MIXED && precision != WT3D_PREC_FP64) { set_error("bad precision"); return WT3D_ERR_ARG; }
    if ((rc = have_gpu())) return rc;
    auto t0 = std::chrono::steady_clock::now();
    std::unique_ptr<wt3d_solver> h(new wt3d_solver());
    h->grid = *g;
    h->prec = precision;
    if ((rc = grid_analysis(g->nx, g->ny, g->nz, h->ga))) return rc;
    GridAnalysis &ga = *h->ga;
    const Symbolic &sym = ga.sym;
    h->n = sym.n;
    h->nnz = wt3d_pattern_nnz(g->nx, g->ny, g->nz);
    if ((rc = handle_streams(h.get()))) return rc;
    if ((rc = h->irptr.alloc(h->n + 1)) || (rc = h->jcptr.alloc(h->nnz)) || (rc = h->a.alloc(h->nnz))) return rc;
    if ((rc = device_pattern(g->nx, g->ny, g->nz, 0, h->irptr.p, h->jcptr.p, h->st))) return rc;
    std::shared_ptr<FactorWorkspace<float>> w32;
    std::shared_ptr<FactorWorkspace<double>> w64;
    {
        std::lock_guard<std::mutex> lk(ga.mu);
        if (ga.map.empty()) {
            std::vector<int> hir(h->n + 1), hjc(h->nnz);
            WT_CUDA(cudaMemcpyAsync(hir.data(), h->irptr.p, sizeof(int) * (h->n + 1), cudaMemcpyDeviceToHost, h->st));
            WT_CUDA(cudaMemcpyAsync(hjc.data(), h->jcptr.p, sizeof(int) * h->nnz, cudaMemcpyDeviceToHost, h->st));
            WT_CUDA(cudaStreamSynchronize(h->st));
            std::vector<long long> map;
            if ((rc = scatter_map(sym, hir, hjc, map))) return rc;
            // transposed positions for the adjoint residual
            std::vector<int> tp = to_int(transpose_positions(h->n, hir.data(), hjc.data()));
            ga.map.swap(map);
            ga.tpos.swap(tp);
        }
        if (precision == WT3D_PREC_MIXED) w32 = pick_workspace(ga.ws32);
        else w64 = pick_workspace(ga.ws64);
    }
    if ((rc = handle_engine(h.get(), precision, w32, w64, t0))) return rc;
    *out = h.release();
    return WT3D_OK;
}

int wt3d_solver_create_csr(wt3d_solver **out, int n, long long nnz, const int *irptr, const int *jcptr, int base,
                           int precision)
{
    if (!out) { set_error("null handle pointer"); return WT3D_ERR_ARG; }
    *out = nullptr;
    if (precision != WT3D_PREC_MIXED && precision != WT3D_PREC_FP64) { set_error("bad precision"); return WT3D_ERR_ARG; }
    int rc = check_csr(n, nnz, irptr, jcptr, base, false);
    if (rc) return rc;
    if (nnz == 0) { set_error("CSR: the matrix has no entries"); return WT3D_ERR_PATTERN; }
    if ((rc = have_gpu())) return rc;
    auto t0 = std::chrono::steady_clock::now();
    std::unique_ptr<wt3d_solver> h(new wt3d_solver());
    h->general = true;
    h->prec = precision;
    h->ga = std::make_shared<GridAnalysis>();
    GridAnalysis &ga = *h->ga;
    std::vector<int> hir, hjc, vmap;
    try {   // host analysis: its only failure mode besides a bad pattern is host memory
        if ((rc = symmetrize(n, irptr, jcptr, base, hir, hjc, vmap))) return rc;
        if ((rc = symbolic_graph(n, hir.data(), hjc.data(), 0, GENERAL_LEAF_DOFS, ga.sym))) return rc;
        if ((rc = scatter_map(ga.sym, hir, hjc, ga.map))) return rc;
        ga.tpos = to_int(transpose_positions(n, hir.data(), hjc.data()));
    } catch (const std::bad_alloc &) {
        set_error("wt3d_solver_create_csr: out of host memory");
        return WT3D_ERR_NOMEM;
    }
    h->n = n;
    h->nnz = (long long)hjc.size();
    h->nnz_in = nnz;
    if ((rc = handle_streams(h.get()))) return rc;
    if ((rc = h->irptr.upload(hir)) || (rc = h->jcptr.upload(hjc)) || (rc = h->a.alloc(h->nnz))) return rc;
    if (!vmap.empty() && (rc = h->vmap.upload(vmap))) return rc;
    std::shared_ptr<FactorWorkspace<float>> w32;
    std::shared_ptr<FactorWorkspace<double>> w64;
    if (precision == WT3D_PREC_MIXED) w32 = pick_workspace(ga.ws32);
    else w64 = pick_workspace(ga.ws64);
    if ((rc = handle_engine(h.get(), precision, w32, w64, t0))) return rc;
    *out = h.release();
    return WT3D_OK;
}

int wt3d_solver_destroy(wt3d_solver *h)
{
    delete h;
    return WT3D_OK;
}

int wt3d_set_model(wt3d_solver *h, const float *vp, const float *vs, const float *rho)
{
    if (h && h->general) return grid_only("wt3d_set_model");
    if (!h || !vp || !vs || !rho) { set_error("wt3d_set_model: null pointer"); return WT3D_ERR_ARG; }
    long long nn = h->n / 3;
    int rc;
    if (!h->vp.p) {
        if ((rc = h->vp.alloc(nn)) || (rc = h->vs.alloc(nn)) || (rc = h->rho.alloc(nn)) || (rc = h->da.alloc(nn)) ||
            (rc = h->mu.alloc(nn)) || (rc = h->ro.alloc(nn)))
            return rc;
    }
    WT_CUDA(cudaMemcpyAsync(h->vp.p, vp, sizeof(float) * nn, cudaMemcpyHostToDevice, h->st));
    WT_CUDA(cudaMemcpyAsync(h->vs.p, vs, sizeof(float) * nn, cudaMemcpyHostToDevice, h->st));
    WT_CUDA(cudaMemcpyAsync(h->rho.p, rho, sizeof(float) * nn, cudaMemcpyHostToDevice, h->st));
    if ((rc = device_lame(nn, h->vp.p, h->vs.p, h->rho.p, h->da.p, h->mu.p, h->ro.p, h->st))) return rc;
    WT_CUDA(cudaStreamSynchronize(h->st));
    h->have_model = true;
    return WT3D_OK;
}

static int factor_values(wt3d_solver *h)
{
    int np = 0, rc;
    {
        // the update buffers are shared by the handles of this grid: one
        // factorisation at a time, until its kernels have finished
        std::lock_guard<std::mutex> lk(h->e32 ? h->e32->ws->mu : h->e64->ws->mu);
        cudaEventRecord(h->ev0, h->st);
        if (h->e32) rc = h->e32->factor(h->a.p, h->nnz, h->st, &np);
        else rc = h->e64->factor(h->a.p, h->nnz, h->st, &np);
        if (rc) return rc;
        cudaEventRecord(h->ev1, h->st);
        WT_CUDA(cudaStreamSynchronize(h->st));
    }
    if ((rc = h->e32 ? h->e32->check_tc_err() : h->e64->check_tc_err())) return rc;
    h->stats.t_factor_ms = ms_between(h->ev0, h->ev1);
    h->stats.perturbed_pivots = np;
    h->stats.kernels_factor = 2 + (h->e32 ? h->e32->fsched->kernels() : h->e64->fsched->kernels());
    h->stats.device_bytes = own_bytes(h);
    h->stats.workspace_bytes = (double)(h->e32 ? h->e32->workspace_bytes() : h->e64->workspace_bytes());
    h->have_factor = true;
    return WT3D_OK;
}

int wt3d_factor(wt3d_solver *h, double omega_re, double omega_im)
{
    if (h && h->general) return grid_only("wt3d_factor");
    if (!h) { set_error("null handle"); return WT3D_ERR_ARG; }
    if (!h->have_model) { set_error("wt3d_factor: no model set"); return WT3D_ERR_STATE; }
    h->have_factor = false;
    cudaEventRecord(h->ev0, h->st);
    int rc;
    // attenuation: Lame arrays dispersed to this frequency
    if (h->qp.p && (rc = device_lame_q(h->n / 3, h->vp.p, h->vs.p, h->rho.p, h->qp.p, h->qs.p, omega_re, h->freqbase,
                                       h->da.p, h->mu.p, h->ro.p, h->st)))
        return rc;
    rc = device_assemble(h->grid, h->da.p, h->mu.p, h->ro.p, omega_re, omega_im, h->irptr.p, h->a.p, h->st);
    if (rc) return rc;
    cudaEventRecord(h->ev1, h->st);
    WT_CUDA(cudaStreamSynchronize(h->st));
    h->stats.t_assemble_ms = ms_between(h->ev0, h->ev1);
    h->have_values = true;
    h->om_re = omega_re;
    h->om_im = omega_im;
    rc = factor_values(h);
    h->stats.kernels_factor += 1;   // the assembly kernel
    return rc;
}

int wt3d_set_attenuation(wt3d_solver *h, const float *qp_inv, const float *qs_inv, double freqbase)
{
    if (h && h->general) return grid_only("wt3d_set_attenuation");
    if (!h) { set_error("null handle"); return WT3D_ERR_ARG; }
    if (!qp_inv || !qs_inv) {   // back to an elastic model
        h->qp.free();
        h->qs.free();
        if (h->have_model) {
            int rc = device_lame(h->n / 3, h->vp.p, h->vs.p, h->rho.p, h->da.p, h->mu.p, h->ro.p, h->st);
            if (rc) return rc;
            WT_CUDA(cudaStreamSynchronize(h->st));
        }
        return WT3D_OK;
    }
    const long long nn = h->n / 3;
    int rc;
    if ((!h->qp.p && (rc = h->qp.alloc(nn))) || (!h->qs.p && (rc = h->qs.alloc(nn)))) return rc;
    WT_CUDA(cudaMemcpyAsync(h->qp.p, qp_inv, sizeof(float) * nn, cudaMemcpyHostToDevice, h->st));
    WT_CUDA(cudaMemcpyAsync(h->qs.p, qs_inv, sizeof(float) * nn, cudaMemcpyHostToDevice, h->st));
    WT_CUDA(cudaStreamSynchronize(h->st));
    h->freqbase = freqbase;
    return WT3D_OK;
}

int wt3d_set_background(wt3d_solver *h, const float *vp, const float *vs, const float *rho)
{
    if (h && h->general) return grid_only("wt3d_set_background");
    if (!h || !vp || !vs || !rho) { set_error("wt3d_set_background: null pointer"); return WT3D_ERR_ARG; }
    const long long nn = h->n / 3;
    int rc;
    if (!h->bgro.p && ((rc = h->bgda.alloc(nn)) || (rc = h->bgmu.alloc(nn)) || (rc = h->bgro.alloc(nn)))) return rc;
    StreamBuf<float> dvp, dvs, drho;   // per-call temporaries in stream order (see StreamBuf)
    if ((rc = dvp.alloc(nn, h->st)) || (rc = dvs.alloc(nn, h->st)) || (rc = drho.alloc(nn, h->st))) return rc;
    WT_CUDA(cudaMemcpyAsync(dvp.p, vp, sizeof(float) * nn, cudaMemcpyHostToDevice, h->st));
    WT_CUDA(cudaMemcpyAsync(dvs.p, vs, sizeof(float) * nn, cudaMemcpyHostToDevice, h->st));
    WT_CUDA(cudaMemcpyAsync(drho.p, rho, sizeof(float) * nn, cudaMemcpyHostToDevice, h->st));
    if ((rc = device_lame(nn, dvp.p, dvs.p, drho.p, h->bgda.p, h->bgmu.p, h->bgro.p, h->st))) return rc;
    WT_CUDA(cudaStreamSynchronize(h->st));
    h->have_bg = true;
    return WT3D_OK;
}

int wt3d_haskgrn(const wt3d_layered1d *m, double omega, double ain, int s_wave, int nz, double dz, double zorig,
                 double _Complex *U, double _Complex *W)
{
    if (!m || !U || !W || nz < 1) { set_error("wt3d_haskgrn: bad arguments"); return WT3D_ERR_ARG; }
    return haskgrn_host(*m, omega, ain, s_wave, nz, dz, zorig, reinterpret_cast<std::complex<double> *>(U),
                        reinterpret_cast<std::complex<double> *>(W));
}

int wt3d_rhs_planewave(wt3d_solver *h, const wt3d_layered1d *m, int nsrc, const double *ain, const double *baz,
                       const int *s_wave, void *d_F, void *d_U0)
{
    if (h && h->general) return grid_only("wt3d_rhs_planewave");
    if (!h || !m || nsrc < 1 || !ain || !baz || !d_F) { set_error("wt3d_rhs_planewave: bad arguments"); return WT3D_ERR_ARG; }
    if (int rc0 = after_legacy(h, h->st)) return rc0;
    if (!h->have_values || !h->have_bg) { set_error("wt3d_rhs_planewave: needs a factored operator and a background"); return WT3D_ERR_STATE; }
    const int nx = h->grid.nx, ny = h->grid.ny, nz = h->grid.nz;
    const long long n = h->n;
    int rc;
    if (!h->abg.p && (rc = h->abg.alloc(h->nnz))) return rc;
    if ((rc = device_assemble(h->grid, h->bgda.p, h->bgmu.p, h->bgro.p, h->om_re, h->om_im, h->irptr.p, h->abg.p,
                              h->st)))
        return rc;
    const int nl = m->nl;
    for (int c0 = 0; c0 < nsrc; c0 += MAXRHS) {
        const int mm = std::min(MAXRHS, nsrc - c0);
        std::vector<std::complex<double>> Uz((size_t)mm * nz), Wz((size_t)mm * nz);
        std::vector<double> kx(mm), ky(mm), rx(mm), ry(mm);
        for (int j = 0; j < mm; j++) {
            const int sw = s_wave ? s_wave[c0 + j] : 0;
            if ((rc = haskgrn_host(*m, h->om_re, ain[c0 + j], sw, nz, h->grid.dx, 0.0, &Uz[(size_t)j * nz],
                                   &Wz[(size_t)j * nz])))
                return rc;
            const double vh = sw ? m->vs[nl - 1] : m->vp[nl - 1];
            const double p = std::sin(ain[c0 + j]) / vh;
            rx[j] = -std::cos(baz[c0 + j]);
            ry[j] = -std::sin(baz[c0 + j]);
            kx[j] = h->om_re * p * rx[j];
            ky[j] = h->om_re * p * ry[j];
        }
        // per-call tables in stream order (see StreamBuf)
        StreamBuf<double2> dU, dW;
        StreamBuf<double> dkx, dky, drx, dry;
        std::vector<double2> hu(Uz.size()), hw(Wz.size());
        for (size_t i = 0; i < Uz.size(); i++) {
            hu[i] = make_double2(Uz[i].real(), Uz[i].imag());
            hw[i] = make_double2(Wz[i].real(), Wz[i].imag());
        }
        if ((rc = dU.upload(hu, h->st)) || (rc = dW.upload(hw, h->st)) || (rc = dkx.upload(kx, h->st)) ||
            (rc = dky.upload(ky, h->st)) || (rc = drx.upload(rx, h->st)) || (rc = dry.upload(ry, h->st)))
            return rc;
        k_pw_expand<<<ceil_div((n / 3) * mm, 256), 256, 0, h->st>>>(nx, ny, nz, h->grid.dx, mm, dU.p, dW.p, dkx.p,
                                                                     dky.p, drx.p, dry.p, h->Rn.p, MAXRHS);
        k_hetfld<<<152 * 8, 256, 0, h->st>>>(n, mm, h->irptr.p, h->jcptr.p, h->a.p, h->abg.p, h->Rn.p, MAXRHS,
                                             (double2 *)d_F + (long long)c0 * n);
        if (d_U0) k_rm_to_cm<<<ceil_div(n, 256), 256, 0, h->st>>>(n, mm, h->Rn.p, (double2 *)d_U0 + (long long)c0 * n);
        WT_CUDA(cudaGetLastError());
        WT_CUDA(cudaStreamSynchronize(h->st));
    }
    return WT3D_OK;
}

int wt3d_set_values_c64(wt3d_solver *h, const float _Complex *a)
{
    if (!h || !a) { set_error("null pointer"); return WT3D_ERR_ARG; }
    const long long nin = h->vmap.p ? h->nnz_in : h->nnz;   // caller entries
    StreamBuf<float2> tmp;   // per-call, in stream order (see StreamBuf)
    int rc = tmp.alloc(nin, h->st);
    if (rc) return rc;
    WT_CUDA(cudaMemcpyAsync(tmp.p, a, sizeof(float2) * nin, cudaMemcpyHostToDevice, h->st));
    if (h->vmap.p) {
        WT_CUDA(cudaMemsetAsync(h->a.p, 0, sizeof(double2) * h->nnz, h->st));
        k_spread_c64<<<ceil_div(nin, 256), 256, 0, h->st>>>(nin, tmp.p, h->vmap.p, h->a.p);
    } else {
        k_c64_to_c128<<<ceil_div(nin, 256), 256, 0, h->st>>>(nin, tmp.p, h->a.p);
    }
    WT_CUDA(cudaStreamSynchronize(h->st));
    h->have_values = true;
    h->have_factor = false;
    return WT3D_OK;
}

int wt3d_set_values_c128(wt3d_solver *h, const double _Complex *a)
{
    if (!h || !a) { set_error("null pointer"); return WT3D_ERR_ARG; }
    if (h->vmap.p) {
        StreamBuf<double2> tmp;
        int rc = tmp.alloc(h->nnz_in, h->st);
        if (rc) return rc;
        WT_CUDA(cudaMemcpyAsync(tmp.p, a, sizeof(double2) * h->nnz_in, cudaMemcpyHostToDevice, h->st));
        WT_CUDA(cudaMemsetAsync(h->a.p, 0, sizeof(double2) * h->nnz, h->st));
        k_spread_c128<<<ceil_div(h->nnz_in, 256), 256, 0, h->st>>>(h->nnz_in, tmp.p, h->vmap.p, h->a.p);
    } else {
        WT_CUDA(cudaMemcpyAsync(h->a.p, a, sizeof(double2) * h->nnz, cudaMemcpyHostToDevice, h->st));
    }
    WT_CUDA(cudaStreamSynchronize(h->st));
    h->have_values = true;
    h->have_factor = false;
    return WT3D_OK;
}

int wt3d_factor_values(wt3d_solver *h)
{
    if (!h || !h->have_values) { set_error("no operator values"); return WT3D_ERR_STATE; }
    return factor_values(h);
}

int wt3d_solve_device(wt3d_solver *h, int nrhs, const void *d_B, void *d_X, double tol, int maxit, double *relres,
                      int *iters, int adjoint)
{
    if (!h || nrhs < 1 || !d_B || !d_X) { set_error("wt3d_solve_device: bad arguments"); return WT3D_ERR_ARG; }
    return solve_dev_cm(h, nrhs, (const double2 *)d_B, (double2 *)d_X, tol, maxit, relres, iters, adjoint != 0);
}

static int solve_host(wt3d_solver *h, int nrhs, const double _Complex *B, double _Complex *X, double tol, int maxit,
                      double *relres, int *iters, bool adjoint)
{
    if (!h || nrhs < 1 || !B || !X) { set_error("wt3d_solve: bad arguments"); return WT3D_ERR_ARG; }
    if (!h->have_factor) { set_error("solve before factor"); return WT3D_ERR_STATE; }
    StreamBuf<double2> dB, dX;   // per-call, in the solve stream's order (see StreamBuf)
    int rc;
    if ((rc = dB.alloc((size_t)h->n * nrhs, h->sts)) || (rc = dX.alloc((size_t)h->n * nrhs, h->sts))) return rc;
    WT_CUDA(cudaMemcpyAsync(dB.p, B, sizeof(double2) * h->n * nrhs, cudaMemcpyHostToDevice, h->sts));
    rc = solve_dev_cm(h, nrhs, dB.p, dX.p, tol, maxit, relres, iters, adjoint);
    if (rc && rc != WT3D_ERR_NOCONV) return rc;
    WT_CUDA(cudaMemcpyAsync(X, dX.p, sizeof(double2) * h->n * nrhs, cudaMemcpyDeviceToHost, h->sts));
    WT_CUDA(cudaStreamSynchronize(h->sts));
    return rc;
}

int wt3d_solve(wt3d_solver *h, int nrhs, const double _Complex *B, double _Complex *X, double tol, int maxit,
               double *relres, int *iters)
{
    return solve_host(h, nrhs, B, X, tol, maxit, relres, iters, false);
}

int wt3d_solve_adjoint(wt3d_solver *h, int nrhs, const double _Complex *B, double _Complex *X, double tol, int maxit,
                       double *relres, int *iters)
{
    return solve_host(h, nrhs, B, X, tol, maxit, relres, iters, true);
}

int wt3d_apply(wt3d_solver *h, int nrhs, const double _Complex *X, double _Complex *Y)
{
    if (!h || nrhs < 1 || !X || !Y) { set_error("wt3d_apply: bad arguments"); return WT3D_ERR_ARG; }
    if (!h->have_values) { set_error("no operator"); return WT3D_ERR_STATE; }
    const long long n = h->n;
    StreamBuf<double2> dX;   // per-call, in stream order (see StreamBuf)
    int rc = dX.alloc((size_t)n * nrhs, h->st);
    if (rc) return rc;
    WT_CUDA(cudaMemcpyAsync(dX.p, X, sizeof(double2) * n * nrhs, cudaMemcpyHostToDevice, h->st));
    for (int c0 = 0; c0 < nrhs; c0 += MAXRHS) {
        int m = std::min(MAXRHS, nrhs - c0);
        k_cm_to_rm<<<ceil_div(n, 256), 256, 0, h->st>>>(n, m, dX.p + (long long)c0 * n, h->Xn.p);
        WT_CUDA(cudaMemsetAsync(h->Bn.p, 0, sizeof(double2) * n * MAXRHS, h->st));
        WT_CUDA(cudaMemsetAsync(h->norms.p, 0, sizeof(double) * 2 * MAXRHS, h->st));
        // R = 0 - A X
        residual(h, h->st, m, h->Xn.p, h->Bn.p, h->Rn.p, false);
        k_rm_to_cm<<<ceil_div(n, 256), 256, 0, h->st>>>(n, m, h->Rn.p, dX.p + (long long)c0 * n);
    }
    std::vector<std::complex<double>> tmp((size_t)n * nrhs);
    WT_CUDA(cudaMemcpyAsync(tmp.data(), dX.p, sizeof(double2) * n * nrhs, cudaMemcpyDeviceToHost, h->st));
    WT_CUDA(cudaStreamSynchronize(h->st));
    std::complex<double> *Yc = reinterpret_cast<std::complex<double> *>(Y);
    for (size_t i = 0; i < tmp.size(); i++) Yc[i] = -tmp[i];
    return WT3D_OK;
}

int wt3d_apply_device(wt3d_solver *h, int nrhs, const void *d_X, void *d_Y)
{
    if (!h || nrhs < 1 || !d_X || !d_Y) { set_error("wt3d_apply_device: bad arguments"); return WT3D_ERR_ARG; }
    if (int rc0 = after_legacy(h, h->st)) return rc0;
    if (!h->have_values) { set_error("no operator"); return WT3D_ERR_STATE; }
    const long long n = h->n;
    for (int c0 = 0; c0 < nrhs; c0 += MAXRHS) {
        int m = std::min(MAXRHS, nrhs - c0);
        k_cm_to_rm<<<ceil_div(n, 256), 256, 0, h->st>>>(n, m, (const double2 *)d_X + (long long)c0 * n, h->Xn.p);
        WT_CUDA(cudaMemsetAsync(h->Bn.p, 0, sizeof(double2) * n * MAXRHS, h->st));
        WT_CUDA(cudaMemsetAsync(h->norms.p, 0, sizeof(double) * 2 * MAXRHS, h->st));
        // R = 0 - A X, then Y = -R
        residual(h, h->st, m, h->Xn.p, h->Bn.p, h->Rn.p, false);
        k_rm_to_cm_neg<<<ceil_div(n, 256), 256, 0, h->st>>>(n, m, h->Rn.p, (double2 *)d_Y + (long long)c0 * n);
    }
    WT_CUDA(cudaGetLastError());
    WT_CUDA(cudaStreamSynchronize(h->st));
    return WT3D_OK;
}

int wt3d_update_operator(wt3d_solver *h)
{
    if (h && h->general) return grid_only("wt3d_update_operator");
    if (!h) { set_error("null handle"); return WT3D_ERR_ARG; }
    if (!h->have_model || !h->have_values) { set_error("wt3d_update_operator: needs a model and a factored operator"); return WT3D_ERR_STATE; }
    int rc;
    if (h->qp.p && (rc = device_lame_q(h->n / 3, h->vp.p, h->vs.p, h->rho.p, h->qp.p, h->qs.p, h->om_re, h->freqbase,
                                       h->da.p, h->mu.p, h->ro.p, h->st)))
        return rc;
    rc = device_assemble(h->grid, h->da.p, h->mu.p, h->ro.p, h->om_re, h->om_im, h->irptr.p, h->a.p, h->st);
    if (rc) return rc;
    WT_CUDA(cudaStreamSynchronize(h->st));
    return WT3D_OK;
}

int wt3d_gradient_contract(wt3d_solver *h, int nrhs, const void *d_U, const void *d_Lam, void *d_grad)
{
    if (h && h->general) return grid_only("wt3d_gradient_contract");
    if (!h || nrhs < 1 || !d_U || !d_Lam || !d_grad) { set_error("wt3d_gradient_contract: bad arguments"); return WT3D_ERR_ARG; }
    if (int rc0 = after_legacy(h, h->st)) return rc0;
    if (!h->have_model || !h->have_values) { set_error("wt3d_gradient_contract: needs a model and an assembled operator"); return WT3D_ERR_STATE; }
    if (h->qp.p) { set_error("wt3d_gradient_contract: the gradient is built for elastic models (no attenuation)"); return WT3D_ERR_STATE; }
    const long long nn = h->n / 3;
    int rc;
    if (!h->gscr.p && (rc = h->gscr.alloc((size_t)gradient_scratch_doubles(nn)))) return rc;
    cudaEventRecord(h->ev0, h->st);
    if ((rc = device_gradient(h->grid, h->da.p, h->mu.p, h->ro.p, h->vp.p, h->vs.p, h->rho.p, h->om_re, h->om_im,
                              nrhs, h->n, d_U, d_Lam, h->gscr.p, (double *)d_grad, h->st)))
        return rc;
    cudaEventRecord(h->ev1, h->st);
    WT_CUDA(cudaStreamSynchronize(h->st));
    h->stats.t_gradient_ms = ms_between(h->ev0, h->ev1);
    return WT3D_OK;
}

int wt3d_misfit_gradient(wt3d_solver *h, int nsrc, const void *d_F, const void *d_U0, int nrec,
                         const long long *rec_node, const double _Complex *dobs, double tol, int maxit, double *chi,
                         double *grad, double _Complex *dpred)
{
    if (h && h->general) return grid_only("wt3d_misfit_gradient");
    if (!h || nsrc < 1 || !d_F || nrec < 1 || !rec_node || !dobs || !chi || !grad) {
        set_error("wt3d_misfit_gradient: bad arguments");
        return WT3D_ERR_ARG;
    }
    if (!h->have_factor || !h->have_model) { set_error("wt3d_misfit_gradient: needs a model and a factor"); return WT3D_ERR_STATE; }
    if (int rc0 = after_legacy(h, h->st)) return rc0;
    const long long n = h->n, nn = n / 3;
    for (int r = 0; r < nrec; r++)
        if (rec_node[r] < 0 || rec_node[r] >= nn) { set_error("wt3d_misfit_gradient: receiver node out of range"); return WT3D_ERR_ARG; }
    const long long nd = (long long)nsrc * nrec * 3;
    DevVec<double2> X, S, Lm, dd, dp, dr;
    DevVec<long long> drec;
    DevVec<double> dg;
    int rc;
    if ((rc = X.alloc((size_t)n * nsrc)) || (rc = S.alloc((size_t)n * nsrc)) || (rc = Lm.alloc((size_t)n * nsrc)) ||
        (rc = dd.alloc(nd)) || (rc = dp.alloc(nd)) || (rc = dr.alloc(nd)) || (rc = drec.alloc(nrec)) ||
        (rc = dg.alloc(3 * nn)))
        return rc;
    WT_CUDA(cudaMemcpyAsync(drec.p, rec_node, sizeof(long long) * nrec, cudaMemcpyHostToDevice, h->st));
    WT_CUDA(cudaMemcpyAsync(dd.p, dobs, sizeof(double2) * nd, cudaMemcpyHostToDevice, h->st));
    // forward wavefields; the total field adds the background u0
    int rcf = solve_dev_cm(h, nsrc, (const double2 *)d_F, X.p, tol, maxit, nullptr, nullptr, false);
    if (rcf && rcf != WT3D_ERR_NOCONV) return rcf;
    if (d_U0 && (rc = device_add(n * nsrc, d_U0, X.p, h->st))) return rc;
    WT_CUDA(cudaMemsetAsync(S.p, 0, sizeof(double2) * n * nsrc, h->st));
    if ((rc = device_receivers(nsrc, nrec, n, drec.p, X.p, dd.p, dp.p, dr.p, S.p, h->st))) return rc;
    std::vector<double2> res(nd);
    WT_CUDA(cudaMemcpyAsync(res.data(), dr.p, sizeof(double2) * nd, cudaMemcpyDeviceToHost, h->st));
    if (dpred) WT_CUDA(cudaMemcpyAsync(dpred, dp.p, sizeof(double2) * nd, cudaMemcpyDeviceToHost, h->st));
    WT_CUDA(cudaStreamSynchronize(h->st));
    double c = 0;
    for (const double2 &e : res) c += e.x * e.x + e.y * e.y;
    *chi = 0.5 * c;
    // adjoint wavefields: A^H lam = R^T (R u - d), reusing the factors
    int rca = solve_dev_cm(h, nsrc, S.p, Lm.p, tol, maxit, nullptr, nullptr, true);
    if (rca && rca != WT3D_ERR_NOCONV) return rca;
    if ((rc = wt3d_gradient_contract(h, nsrc, X.p, Lm.p, dg.p))) return rc;
    WT_CUDA(cudaMemcpy(grad, dg.p, sizeof(double) * 3 * nn, cudaMemcpyDeviceToHost));
    return rcf ? rcf : rca;
}

int wt3d_batch_buffers(wt3d_solver *h, int ncols, void **d_F, void **d_X)
{
    if (!h || ncols < 1 || !d_F || !d_X) { set_error("wt3d_batch_buffers: bad arguments"); return WT3D_ERR_ARG; }
    const size_t need = (size_t)h->n * ncols;
    int rc;
    if (h->batF.n < need) {
        WT_CUDA(cudaStreamSynchronize(h->st));
        if ((rc = h->batF.alloc(need)) || (rc = h->batX.alloc(need))) return rc;
    }
    *d_F = h->batF.p;
    *d_X = h->batX.p;
    return WT3D_OK;
}

int wt3d_memcpy(wt3d_solver *h, void *dst, const void *src, long long bytes)
{
    if (!h || !dst || !src || bytes < 0) { set_error("wt3d_memcpy: bad arguments"); return WT3D_ERR_ARG; }
    if (int rc0 = after_legacy(h, h->st)) return rc0;
    WT_CUDA(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDefault, h->st));
    WT_CUDA(cudaStreamSynchronize(h->st));
    return WT3D_OK;
}

int wt3d_rhs_sources(wt3d_solver *h, int nsrc, const double *xyz, const int *comp, const double _Complex *sterm,
                     int ireg, double sprd, void *d_F)
{
    if (h && h->general) return grid_only("wt3d_rhs_sources");
    if (!h || nsrc < 1 || !xyz || !comp || !d_F) { set_error("wt3d_rhs_sources: bad arguments"); return WT3D_ERR_ARG; }
    if (int rc0 = after_legacy(h, h->st)) return rc0;
    const long long n = h->n;
    std::vector<int> col, cmp;
    std::vector<long long> nd;
    std::vector<double> w;
    std::vector<double2> st(nsrc);
    for (int j = 0; j < nsrc; j++) {
        if (comp[j] < 0 || comp[j] > 2) { set_error("wt3d_rhs_sources: component must be 0, 1 or 2"); return WT3D_ERR_ARG; }
        std::vector<long long> a;
        std::vector<double> b;
        int rc = source_weights(h->grid, xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2], ireg, sprd, a, b);
        if (rc) return rc;
        // merge repeated nodes (mirrored terms) so that the kernel's entries are distinct
        std::map<long long, double> acc;
        for (size_t e = 0; e < a.size(); e++) acc[a[e]] += b[e];
        for (auto &kv : acc) { col.push_back(j); nd.push_back(kv.first); w.push_back(kv.second); cmp.push_back(comp[j]); }
        const std::complex<double> v = sterm ? reinterpret_cast<const std::complex<double> *>(sterm)[j] : 1.0;
        st[j] = make_double2(v.real(), v.imag());
    }
    DevVec<int> dcol, dcmp;
    DevVec<long long> dnd;
    DevVec<double> dw;
    DevVec<double2> dst;
    int rc;
    if ((rc = dcol.upload(col)) || (rc = dcmp.upload(cmp)) || (rc = dnd.upload(nd)) || (rc = dw.upload(w)) ||
        (rc = dst.upload(st)))
        return rc;
    WT_CUDA(cudaMemsetAsync(d_F, 0, sizeof(double2) * n * nsrc, h->st));
    const long long ne = (long long)col.size();
    if (ne) k_put_sources<<<ceil_div(ne, 256), 256, 0, h->st>>>(n, ne, dcol.p, dnd.p, dcmp.p, dw.p, dst.p,
                                                                (double2 *)d_F);
    WT_CUDA(cudaGetLastError());
    WT_CUDA(cudaStreamSynchronize(h->st));
    return WT3D_OK;
}

int wt3d_sample_receivers(wt3d_solver *h, int nrhs, const void *d_U, int nrec, const double *xyz, int ireg,
                          double sprd, double _Complex *out)
{
    if (h && h->general) return grid_only("wt3d_sample_receivers");
    if (!h || nrhs < 1 || !d_U || nrec < 1 || !xyz || !out) { set_error("wt3d_sample_receivers: bad arguments"); return WT3D_ERR_ARG; }
    if (int rc0 = after_legacy(h, h->st)) return rc0;
    std::vector<int> start(1, 0);
    std::vector<long long> nd;
    std::vector<double> w;
    for (int r = 0; r < nrec; r++) {
        std::vector<long long> a;
        std::vector<double> b;
        int rc = source_weights(h->grid, xyz[3 * r], xyz[3 * r + 1], xyz[3 * r + 2], ireg, sprd, a, b);
        if (rc) return rc;
        nd.insert(nd.end(), a.begin(), a.end());
        w.insert(w.end(), b.begin(), b.end());
        start.push_back((int)nd.size());
    }
    DevVec<int> dstart;
    DevVec<long long> dnd;
    DevVec<double> dw;
    DevVec<double2> dout;
    const long long tot = (long long)nrhs * nrec * 3;
    int rc;
    if ((rc = dstart.upload(start)) || (rc = dnd.upload(nd)) || (rc = dw.upload(w)) || (rc = dout.alloc(tot))) return rc;
    k_get_receivers<<<ceil_div(tot, 256), 256, 0, h->st>>>(h->n, nrhs, nrec, dstart.p, dnd.p, dw.p,
                                                            (const double2 *)d_U, dout.p);
    WT_CUDA(cudaGetLastError());
    WT_CUDA(cudaMemcpyAsync(out, dout.p, sizeof(double2) * tot, cudaMemcpyDeviceToHost, h->st));
    WT_CUDA(cudaStreamSynchronize(h->st));
    return WT3D_OK;
}

int wt3d_sample_pressure(wt3d_solver *h, int nrhs, const void *d_U, int nrec, const double *xyz, int ireg,
                         double sprd, double _Complex *out)
{
    if (h && h->general) return grid_only("wt3d_sample_pressure");
    if (!h || nrhs < 1 || !d_U || nrec < 1 || !xyz || !out) { set_error("wt3d_sample_pressure: bad arguments"); return WT3D_ERR_ARG; }
    if (!h->have_model || !h->have_values) { set_error("wt3d_sample_pressure: needs a model and an assembled operator"); return WT3D_ERR_STATE; }
    const wt3d_grid &g = h->grid;
    const double d = g.dx;
    // six sampling points per hydrophone: x -+ dx (u), y -+ dy (v), z -+ dz (w) (makeuh.f:137-153)
    std::vector<double> pts((size_t)nrec * 6 * 3);
    for (int r = 0; r < nrec; r++)
        for (int a = 0; a < 3; a++)
            for (int sgn = 0; sgn < 2; sgn++) {
                double *q = &pts[((size_t)r * 6 + a * 2 + sgn) * 3];
                q[0] = xyz[3 * r]; q[1] = xyz[3 * r + 1]; q[2] = xyz[3 * r + 2];
                q[a] += sgn ? d : -d;
            }
    std::vector<std::complex<double>> smp((size_t)nrhs * nrec * 6 * 3);
    int rc = wt3d_sample_receivers(h, nrhs, d_U, nrec * 6, pts.data(), ireg, sprd,
                                   reinterpret_cast<double _Complex *>(smp.data()));
    if (rc) return rc;
    // Lame parameters at the hydrophone node INT(1.5 + x/dx), clamped (makeuh.f:130-136)
    std::vector<double2> lam(nrec), muv(nrec);
    for (int r = 0; r < nrec; r++) {
        int ix = (int)(1.5 + xyz[3 * r] / d), iy = (int)(1.5 + xyz[3 * r + 1] / d), iz = (int)(1.5 + xyz[3 * r + 2] / d);
        ix = std::min(std::max(ix, 1), g.nx);
        iy = std::min(std::max(iy, 1), g.ny);
        iz = std::min(std::max(iz, 1), g.nz);
        const long long node = (iz - 1) + (long long)g.nz * ((ix - 1) + (long long)g.nx * (iy - 1));
        WT_CUDA(cudaMemcpyAsync(&lam[r], h->da.p + node, sizeof(double2), cudaMemcpyDeviceToHost, h->st));
        WT_CUDA(cudaMemcpyAsync(&muv[r], h->mu.p + node, sizeof(double2), cudaMemcpyDeviceToHost, h->st));
    }
    WT_CUDA(cudaStreamSynchronize(h->st));
    const std::complex<double> cfact = std::complex<double>(0.0, -1.0) * std::complex<double>(h->om_re, h->om_im);
    std::complex<double> *o = reinterpret_cast<std::complex<double> *>(out);
    for (int j = 0; j < nrhs; j++)
        for (int r = 0; r < nrec; r++) {
            std::complex<double> div = 0;
            for (int a = 0; a < 3; a++) {
                const std::complex<double> um = smp[(((size_t)j * nrec + r) * 6 + a * 2) * 3 + a];
                const std::complex<double> up = smp[(((size_t)j * nrec + r) * 6 + a * 2 + 1) * 3 + a];
                div += -(up - um) / (2.0 * d * cfact);
            }
            const std::complex<double> L(lam[r].x, lam[r].y), M(muv[r].x, muv[r].y);
            o[(size_t)j * nrec + r] = (L + 2.0 * M / 3.0) * div;
        }
    return WT3D_OK;
}

int wt3d_mem_info(double *free_bytes, double *total_bytes)
{
    size_t f = 0, t = 0;
    WT_CUDA(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = (double)f;
    if (total_bytes) *total_bytes = (double)t;
    return WT3D_OK;
}

int wt3d_get_stats(const wt3d_solver *h, wt3d_stats *st)
{
    if (!h || !st) return WT3D_ERR_ARG;
    *st = h->stats;
    st->device_bytes = own_bytes(h);
    st->workspace_bytes = (double)(h->e32 ? h->e32->workspace_bytes() : h->e64->workspace_bytes());
    return WT3D_OK;
}

int wt3d_solver_bytes(const wt3d_grid *g, int precision, double *out)
{
    if (!out) { set_error("wt3d_solver_bytes: null output"); return WT3D_ERR_ARG; }
    int rc = check_grid(g);
    if (rc) return rc;
    std::shared_ptr<GridAnalysis> ga;
    if ((rc = grid_analysis(g->nx, g->ny, g->nz, ga))) return rc;
    handle_bytes(ga->sym, wt3d_pattern_nnz(g->nx, g->ny, g->nz), precision, out);
    return WT3D_OK;
}

// -------------------------------------------------------------------------
// strumpack_serial_finter drop-in (strumpack_finter.c:9-121)
// -------------------------------------------------------------------------
static wt3d_solver *g_sp = nullptr;
static bool g_sp_factored = false;
static std::mutex g_sp_mu;
// job 3's refinement target, iteration limit and the residual it last reached
static double g_sp_tol = 1e-10;
static int g_sp_maxit = 20;
static double g_sp_relres = 0.0;

int wt3d_finter_set_refinement(double tol, int maxit)
{
    if (!(tol > 0) || maxit < 0) {
        set_error("wt3d_finter_set_refinement: need tol > 0 and maxit >= 0");
        return WT3D_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_sp_mu);
    g_sp_tol = tol;
    g_sp_maxit = maxit;
    return WT3D_OK;
}

double wt3d_finter_last_relres(void)
{
    std::lock_guard<std::mutex> lock(g_sp_mu);
    return g_sp_relres;
}

void strumpack_serial_finter(int *job, int *nrows, int *nnz, int *irptr, int *jcptr, float _Complex *a,
                             float _Complex *rhs, float _Complex *sol, int *ierr)
{
    const char *fcnm = "strumpack_serial_finter";
    std::lock_guard<std::mutex> lock(g_sp_mu);
    *ierr = 0;
    if (*job == 1) {
        if (g_sp) { printf("%s: Error already initialized!\n", fcnm); *ierr = 1; return; }
        // the grid graph of srel3d + SPARSE_ADJ2CRS gets the geometric nested
        // dissection; any other structurally symmetric pattern the general one
        int nx, ny, nz, rc;
        if (!irptr || !jcptr || !nrows || !nnz) {
            printf("%s: Error reordering matrix!\n", fcnm);
            set_error("null pattern argument");
            *ierr = 1;
            return;
        }
        if (detect_grid(*nrows, *nnz, irptr, jcptr, nx, ny, nz) == WT3D_OK) {
            wt3d_grid g{nx, ny, nz, 1.0, 0.0, 0.0, 1, 1};
            rc = wt3d_solver_create(&g_sp, &g, WT3D_PREC_MIXED);
        } else {
            rc = wt3d_solver_create_csr(&g_sp, *nrows, *nnz, irptr, jcptr, 1, WT3D_PREC_MIXED);
        }
        if (rc != WT3D_OK) {
            printf("%s: Error reordering matrix! (%s)\n", fcnm, g_err.c_str());
            g_sp = nullptr;
            *ierr = 1;
        }
        g_sp_factored = false;
    } else if (*job == 2) {
        g_sp_factored = false;
        if (!g_sp) { printf("%s: Error not initialized!\n", fcnm); *ierr = 1; return; }
        if (wt3d_set_values_c64(g_sp, a) != WT3D_OK || wt3d_factor_values(g_sp) != WT3D_OK) {
            printf("%s: Error factoring matrix! (%s)\n", fcnm, g_err.c_str());
            *ierr = 1;
            return;
        }
        g_sp_factored = true;
    } else if (*job == 3) {
        if (!g_sp || !g_sp_factored) { printf("%s: Error matrix not factorized!\n", fcnm); *ierr = 1; return; }
        const long long n = g_sp->n;
        std::vector<std::complex<double>> b(n), x(n);
        const std::complex<float> *r = reinterpret_cast<const std::complex<float> *>(rhs);
        for (long long i = 0; i < n; i++) b[i] = std::complex<double>(r[i]);
        double rr = 0;
        int rc = wt3d_solve(g_sp, 1, reinterpret_cast<double _Complex *>(b.data()),
                            reinterpret_cast<double _Complex *>(x.data()), g_sp_tol, g_sp_maxit, &rr, nullptr);
        g_sp_relres = rr;
        if (rc != WT3D_OK && rc != WT3D_ERR_NOCONV) {
            printf("%s: Error in solution phase1\n", fcnm);
            *ierr = 1;
            return;
        }
        // the last iterate is returned either way; a solve that missed the
        // refinement target is a failed solve for the caller
        std::complex<float> *s = reinterpret_cast<std::complex<float> *>(sol);
        for (long long i = 0; i < n; i++) s[i] = std::complex<float>(x[i]);
        if (rc == WT3D_ERR_NOCONV) {
            printf("%s: Error in solution phase1: relative residual %.3e after %d refinement steps, target %.1e\n",
                   fcnm, rr, g_sp_maxit, g_sp_tol);
            *ierr = 1;
        }
    } else if (*job == -1) {
        if (g_sp) wt3d_solver_destroy(g_sp);
        g_sp = nullptr;
        g_sp_factored = false;
    }
}

}  // extern "C"

// ---------------------------------------------------------------------------
// host-only inspection of the analysis (no GPU needed)
// ---------------------------------------------------------------------------
static void analysis_info(const Symbolic &S, long long *info, double *flops)
{
    if (info) {
        info[0] = (long long)S.fronts.size();
        info[1] = S.fac_total;
        info[2] = (long long)S.levels.size();
        info[3] = S.max_p;
        info[4] = S.max_b;
        info[5] = (long long)S.border.size();
        info[6] = S.upd_size[0];
        info[7] = S.upd_size[1];
    }
    if (flops) *flops = S.flops;
}

static void analysis_export(const Symbolic &S, int *perm, int *fp, int *fb, int *ffirst, int *fparent, int *flevel,
                            int *border, int *rel)
{
    std::copy(S.perm.begin(), S.perm.end(), perm);
    for (size_t f = 0; f < S.fronts.size(); f++) {
        fp[f] = S.fronts[f].p;
        fb[f] = S.fronts[f].b;
        ffirst[f] = S.fronts[f].first;
        fparent[f] = S.fronts[f].parent;
        flevel[f] = S.fronts[f].level;
    }
    std::copy(S.border.begin(), S.border.end(), border);
    std::copy(S.rel.begin(), S.rel.end(), rel);
}

extern "C" int wt3d_analyse_info(int nx, int ny, int nz, int leaf_nodes, long long *info, double *flops)
{
    Symbolic S;
    int rc = symbolic_grid(nx, ny, nz, leaf_nodes > 0 ? leaf_nodes : 64, S);
    if (rc) return rc;
    analysis_info(S, info, flops);
    return WT3D_OK;
}

extern "C" int wt3d_analyse_export(int nx, int ny, int nz, int leaf_nodes, int *perm, int *fp, int *fb, int *ffirst,
                                   int *fparent, int *flevel, int *border, int *rel)
{
    Symbolic S;
    int rc = symbolic_grid(nx, ny, nz, leaf_nodes > 0 ? leaf_nodes : 64, S);
    if (rc) return rc;
    analysis_export(S, perm, fp, fb, ffirst, fparent, flevel, border, rel);
    return WT3D_OK;
}

// Host analysis of a caller pattern as wt3d_solver_create_csr does it:
// checked, symmetrised, ordered, and every entry mapped into its front.
static int csr_analysis(int n, long long nnz, const int *irptr, const int *jcptr, int base, int leaf_dofs,
                        Symbolic &S)
{
    int rc = check_csr(n, nnz, irptr, jcptr, base, false);
    if (rc) return rc;
    try {
        std::vector<int> hir, hjc, vmap;
        std::vector<long long> map;
        if ((rc = symmetrize(n, irptr, jcptr, base, hir, hjc, vmap)) ||
            (rc = symbolic_graph(n, hir.data(), hjc.data(), 0, leaf_dofs > 0 ? leaf_dofs : GENERAL_LEAF_DOFS, S)) ||
            (rc = scatter_map(S, hir, hjc, map)))
            return rc;
    } catch (const std::bad_alloc &) {
        set_error("host analysis: out of host memory");
        return WT3D_ERR_NOMEM;
    }
    return WT3D_OK;
}

extern "C" int wt3d_general_ordering_uses_metis(void) { return metis_linked() ? 1 : 0; }

extern "C" int wt3d_analyse_csr_info(int n, long long nnz, const int *irptr, const int *jcptr, int base,
                                     int leaf_dofs, long long *info, double *flops)
{
    Symbolic S;
    if (int rc = csr_analysis(n, nnz, irptr, jcptr, base, leaf_dofs, S)) return rc;
    analysis_info(S, info, flops);
    return WT3D_OK;
}

extern "C" int wt3d_analyse_csr_export(int n, long long nnz, const int *irptr, const int *jcptr, int base,
                                       int leaf_dofs, int *perm, int *fp, int *fb, int *ffirst, int *fparent,
                                       int *flevel, int *border, int *rel)
{
    Symbolic S;
    if (int rc = csr_analysis(n, nnz, irptr, jcptr, base, leaf_dofs, S)) return rc;
    analysis_export(S, perm, fp, fb, ffirst, fparent, flevel, border, rel);
    return WT3D_OK;
}

// Copy internal device state to the host for checks: what = 0 factor pool
// (complex entries of the engine precision), 1 pivot indices, 2 the two update
// buffers back to back.  count = elements to copy.
extern "C" void *wt3d_get_stream(wt3d_solver *h) { return h ? (void *)h->st : nullptr; }

extern "C" int wt3d_profile_factor(wt3d_solver *h, double *out)
{
    if (!h || !out || !h->have_values) return WT3D_ERR_STATE;
    int rc = h->e32 ? h->e32->profile_factor(h->a.p, h->nnz, h->st, out)
                    : h->e64->profile_factor(h->a.p, h->nnz, h->st, out);
    if (!rc) h->have_factor = true;
    return rc;
}

// One forward+backward pass over m right-hand sides (whatever X holds) with
// per-launch events; out as wt3d_profile_factor, plus out[11] = ms of one FP64
// residual over m columns.
extern "C" int wt3d_profile_solve(wt3d_solver *h, int m, double *out)
{
    if (!h || !out || !h->have_factor || m < 1 || m > MAXRHS) return WT3D_ERR_STATE;
    int rc;
    if (h->e32) {
        Schedule<float> *sc = h->e32->solve_schedule(m, false);
        if (!sc) return WT3D_ERR_NOMEM;
        rc = h->e32->profile_schedule(*sc, h->st, out);
    } else {
        Schedule<double> *sc = h->e64->solve_schedule(m, false);
        if (!sc) return WT3D_ERR_NOMEM;
        rc = h->e64->profile_schedule(*sc, h->st, out);
    }
    if (rc) return rc;
    cudaEventRecord(h->ev0, h->st);
    residual(h, h->st, m, h->Xn.p, h->Bn.p, h->Rn.p, false);
    cudaEventRecord(h->ev1, h->st);
    WT_CUDA(cudaStreamSynchronize(h->st));
    out[11] = ms_between(h->ev0, h->ev1);
    return WT3D_OK;
}

// Per-launch profile of the factor schedule (which = 0) or of one substitution
// pass over m columns (which = 1, forward + backward, whatever X holds):
// out[4i..4i+3] = kind (LaunchKind), ms, real flops, operand bytes; at most
// cap launches are written, *count receives the schedule's launch count.
extern "C" int wt3d_profile_launches(wt3d_solver *h, int which, int m, double *out, int cap, int *count)
{
    if (!h || !out || !count || !h->have_values || (which == 1 && (!h->have_factor || m < 1 || m > MAXRHS)))
        return WT3D_ERR_STATE;
    std::vector<float> ms;
    const std::vector<LaunchRec> *recs = nullptr;
    int rc;
    if (h->e32) {
        Engine<float> &E = *h->e32;
        if (which == 0) { rc = E.profile_factor_each(h->a.p, h->nnz, h->st, ms); recs = &E.fsched->launches; }
        else {
            Schedule<float> *sc = E.solve_schedule(m, false);
            if (!sc) return WT3D_ERR_NOMEM;
            rc = E.profile_each(*sc, h->st, ms);
            recs = &sc->launches;
        }
    } else {
        Engine<double> &E = *h->e64;
        if (which == 0) { rc = E.profile_factor_each(h->a.p, h->nnz, h->st, ms); recs = &E.fsched->launches; }
        else {
            Schedule<double> *sc = E.solve_schedule(m, false);
            if (!sc) return WT3D_ERR_NOMEM;
            rc = E.profile_each(*sc, h->st, ms);
            recs = &sc->launches;
        }
    }
    if (rc) return rc;
    if (which == 0) h->have_factor = true;
    *count = (int)ms.size();
    for (int i = 0; i < (int)ms.size() && i < cap; i++) {
        out[4 * i] = (*recs)[i].kind;
        out[4 * i + 1] = ms[i];
        out[4 * i + 2] = (*recs)[i].flops;
        out[4 * i + 3] = (*recs)[i].bytes;
    }
    return WT3D_OK;
}

extern "C" int wt3d_debug_fetch(wt3d_solver *h, int what, void *out, long long count)
{
    if (!h || !out) return WT3D_ERR_ARG;
    WT_CUDA(cudaStreamSynchronize(h->st));
    if (what == 0) {
        if (h->e32) WT_CUDA(cudaMemcpy(out, h->e32->fac.p, sizeof(cx<float>) * std::min<long long>(count, h->e32->fac.n), cudaMemcpyDeviceToHost));
        else WT_CUDA(cudaMemcpy(out, h->e64->fac.p, sizeof(cx<double>) * std::min<long long>(count, h->e64->fac.n), cudaMemcpyDeviceToHost));
    } else if (what == 1) {
        const int *p = h->e32 ? h->e32->ipiv.p : h->e64->ipiv.p;
        WT_CUDA(cudaMemcpy(out, p, sizeof(int) * std::min<long long>(count, h->n), cudaMemcpyDeviceToHost));
    } else {
        return WT3D_ERR_ARG;
    }
    return WT3D_OK;
}

// Select the CUDA device for the calling thread (multi-GPU replicas: one
// process per GPU).
extern "C" int wt3d_set_device(int dev)
{
    WT_CUDA(cudaSetDevice(dev));
    return WT3D_OK;
}
