// Multifrontal numeric kernels (templated on the real type T: float for the
// complex64 mixed-precision path, double for the complex128 oracle path).
//
// Front layout (row-major): the pivot rows P = F[0:p, 0:nf] (p x nf) are
// followed by the lower-left border block Lo = F[p:nf, 0:p] (b x p) in the
// factor pool; the Schur/update block F22 (b x b) lives in one of two
// level-parity update buffers.  Factorisation is right-looking blocked LU on
// the first p columns with KB-wide panels and partial pivoting restricted to
// the diagonal KB x KB tile; row interchanges are LINPACK style (applied to
// the columns right of the panel only), so the forward solve applies them
// block by block.
#pragma once
#include "common.cuh"

namespace wt3d {

constexpr int KB = 64;        // panel width
constexpr int MAXRHS = 32;    // right-hand sides per solve pass (a multiple of 32)

struct FrontDev {
    long long fac;     // P block offset in the factor pool (complex elements)
    long long upd;     // F22 offset in its parity buffer
    long long border;  // offset into the border index array
    int p, b, first, parity;
    int pan;           // index of the front's first KB panel (tile-inverse store)
};

struct PanelTask { int f, k; };
struct RowTask { int f, k, c0; };
struct ColTask { int f, k, r0, which; };
struct EATask { int child, parent; long long row0; };
// One CTA of a fused substitution step (k_sub_step): panel k of front f.
// role 0: flush the previous panel's solved rows (kprev >= 0) from the front's
// scratch slot into X, then store this panel's solved rows in the slot;
// role 1: update rows [r0, r1) with this panel's solved rows;
// role 3: as role 0 for a front with no update CTA in this step (its last
// panel of the block): the solved rows go straight into X.
struct StepTask { int f, k, r0, r1, role, kprev, slot; };

template <class T>
struct GemmTask {
    const cx<T> *A;
    const cx<T> *B;
    cx<T> *C;
    const int *brow;   // optional row gather for B
    const int *crow;   // optional row scatter for C (atomic)
    int lda, ldb, ldc, M, N, K;
    int tiles_n;
    long long tile0;
    int conjA;         // use conj(A^T): A is read as its conjugate transpose
    int atom;          // C -= A B with atomics (a K-chunk of a split task)
};

template <class T>
__device__ __forceinline__ void atomic_sub(cx<T> *p, cx<T> v)
{
    atomicAdd(&p->re, -v.re);
    atomicAdd(&p->im, -v.im);
}

template <class Task>
__device__ __forceinline__ int find_task(const Task *tasks, int ntasks, long long key)
{
    int lo = 0, hi = ntasks - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].tile0 <= key) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// original entries -> fronts
// ---------------------------------------------------------------------------
// One thread per CSR row: a_ij * s_i * s_j into the front that owns the entry.
// s is the symmetric Jacobi scaling 1/sqrt|a_ii| (natural ordering): Dirichlet
// rows carry unit diagonals next to O(1e8) stiffness rows, and equilibrating
// both sides keeps the complex64 fronts well scaled.
template <class T>
__global__ void k_scatter(long long n, const int *__restrict__ irptr, const int *__restrict__ jcptr,
                          const long long *__restrict__ map, const double2 *__restrict__ a,
                          const double *__restrict__ s, cx<T> *__restrict__ fac)
{
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const double sr = s[r];
    for (int k = irptr[r]; k < irptr[r + 1]; k++) {
        double2 v = a[k];
        double w = sr * s[jcptr[k]];
        fac[map[k]] = cx<T>((T)(v.x * w), (T)(v.y * w));
    }
}

static __global__ void k_jacobi_scale(long long n, const int *__restrict__ irptr, const int *__restrict__ jcptr,
                               const double2 *__restrict__ a, double *__restrict__ s)
{
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double d = 0;
    for (int k = irptr[r]; k < irptr[r + 1]; k++)
        if (jcptr[k] == r) d = sqrt(a[k].x * a[k].x + a[k].y * a[k].y);
    s[r] = (d > 0 && d < INFINITY) ? 1.0 / sqrt(d) : 1.0;
}

static __global__ void k_maxabs(long long n, const double2 *__restrict__ a, unsigned long long *out)
{
    double m = 0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        double2 v = a[k];
        m = fmax(m, v.x * v.x + v.y * v.y);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// ---------------------------------------------------------------------------
// extend-add: child update matrix into the parent front (one warp per row)
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_extend_add(const EATask *__restrict__ tasks, int ntasks, long long nrows,
                             const FrontDev *__restrict__ fr, const int *__restrict__ rel, cx<T> *__restrict__ fac,
                             cx<T> *__restrict__ upd0, cx<T> *__restrict__ upd1)
{
    long long gr = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (gr >= nrows) return;
    int lo = 0, hi = ntasks - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].row0 <= gr) lo = mid;
        else hi = mid - 1;
    }
    const EATask t = tasks[lo];
    const FrontDev C = fr[t.child], P = fr[t.parent];
    const int i = (int)(gr - t.row0);
    const int *rl = rel + C.border;   // rel shares the border indexing
    const cx<T> *src = (C.parity ? upd1 : upd0) + C.upd + (long long)i * C.b;
    const int R = rl[i];
    const int nfP = P.p + P.b;
    cx<T> *pf = fac + P.fac;
    cx<T> *p22 = (P.parity ? upd1 : upd0) + P.upd;
    for (int j = lane; j < C.b; j += 32) {
        const int Cc = rl[j];
        cx<T> v = src[j];
        cx<T> *dst;
        if (R < P.p) dst = pf + (long long)R * nfP + Cc;
        else if (Cc < P.p) dst = pf + (long long)P.p * nfP + (long long)(R - P.p) * P.p + Cc;
        else dst = p22 + (long long)(R - P.p) * P.b + (Cc - P.p);
        *dst = *dst + v;
    }
}

// Row order of panel k after its LINPACK-style interchanges: idx[i] is the
// stored row that lands at position i (the panel kernel stores it per panel
// in pord; identity when not pivoted).  Threads tid < KB write idx; callers
// synchronise before reading it.
__device__ __forceinline__ void panel_rows(const int *__restrict__ pord, int pan, int kb, bool pivoted, int *idx)
{
    const int tid = threadIdx.x;
    if (tid < KB) idx[tid] = (pivoted && tid < kb) ? pord[(long long)pan * KB + tid] : tid;
}

// ---------------------------------------------------------------------------
// panel: LU of the KB x KB diagonal tile with partial pivoting inside the tile
// ---------------------------------------------------------------------------
// Columns of L_D^{-1} (thread c < KB) and U_D^{-1} (KB <= c < 2 KB) of the
// factored kb x kb tile held in S (row stride KB + 1), padded to KB x KB with
// the identity, stored row-major into Li and Ui.  Scratch: 2 KB columns of
// KB + 1 elements after the tile.
template <class T>
__device__ __forceinline__ void tile_inverse_cols(const cx<T> *S, int kb, cx<T> *Li, cx<T> *Ui, int c)
{
    const int LD = KB + 1;
    const bool up = c >= KB;
    const int cc = up ? c - KB : c;
    cx<T> *x = const_cast<cx<T> *>(S) + KB * LD + c * (KB + 1);
    if (!up) {
        for (int i = 0; i < KB; i++) {
            cx<T> s = (i == cc) ? cx<T>(1) : cx<T>(0);
            if (i < kb && cc < kb)
                for (int l = cc; l < i; l++) s = s - S[i * LD + l] * x[l];
            x[i] = s;
        }
    } else {
        for (int i = KB - 1; i >= 0; i--) {
            cx<T> s = (i == cc) ? cx<T>(1) : cx<T>(0);
            if (i < kb && cc < kb) {
                for (int l = i + 1; l <= cc; l++) s = s - S[i * LD + l] * x[l];
                s = cdiv(s, S[i * LD + i]);
            }
            x[i] = s;
        }
    }
    cx<T> *dst = up ? Ui : Li;
    for (int i = 0; i < KB; i++) dst[i * KB + cc] = x[i];
}

// The stored row at each position after the tile's interchanges goes to the
// panel's slot of pord (the row band and the substitution passes read it).
template <class T>
__global__ void __launch_bounds__(256) k_panel(const PanelTask *__restrict__ tasks, const FrontDev *__restrict__ fr,
                                               cx<T> *__restrict__ fac, int *__restrict__ ipiv,
                                               const unsigned long long *__restrict__ amax2, double pivot_rel,
                                               int *__restrict__ npert, int *__restrict__ pord)
{
    // static-pivot threshold: pivot_rel * max |a_ij| of the assembled operator
    const T thresh = (T)(pivot_rel * sqrt(__longlong_as_double((long long)*amax2)));
    extern __shared__ __align__(16) unsigned char smraw[];
    cx<T> *S = reinterpret_cast<cx<T> *>(smraw);   // KB x (KB+1), then 2 KB scratch columns
    __shared__ int prow[KB];   // stored row at each position, as the interchanges go
    const PanelTask t = tasks[blockIdx.x];
    const FrontDev F = fr[t.f];
    const int nf = F.p + F.b, k = t.k, kb = min(KB, F.p - k);
    const int LD = KB + 1;
    cx<T> *D = fac + F.fac + (long long)k * nf + k;
    const int tid = threadIdx.x;
    #pragma unroll 8   // several loads in flight per thread
    for (int idx = tid; idx < kb * kb; idx += blockDim.x) {
        int i = idx / kb, j = idx % kb;
        S[i * LD + j] = D[(long long)i * nf + j];
    }
    if (tid < KB) prow[tid] = tid;
    __syncthreads();
    // Column j: warp 0 finds the pivot, swaps the two rows, applies the
    // static-pivot threshold and scales the column below the diagonal (one
    // block barrier); then all threads update the trailing block, thread
    // (tid / 16, tid % 16) taking every 16th row and column (a second one).
    const int ty = tid >> 4, tx = tid & 15;
    for (int j = 0; j < kb; j++) {
        if (tid < 32) {
            T best = -1; int bi = j;
            for (int i = j + tid; i < kb; i += 32) {
                T v = cabs2(S[i * LD + j]);
                if (v > best) { best = v; bi = i; }
            }
            for (int o = 16; o > 0; o >>= 1) {   // every lane ends with the same (best, bi)
                T ov = __shfl_xor_sync(0xffffffffu, best, o);
                int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
            }
            const int pv = bi;
            if (pv != j)
                for (int c = tid; c < kb; c += 32) {
                    cx<T> a = S[j * LD + c];
                    S[j * LD + c] = S[pv * LD + c];
                    S[pv * LD + c] = a;
                }
            __syncwarp();
            if (tid == 0) {
                ipiv[F.first + k + j] = k + pv;
                const int a = prow[j];
                prow[j] = prow[pv];
                prow[pv] = a;
                cx<T> d = S[j * LD + j];
                T m2 = cabs2(d);
                if (!(m2 >= thresh * thresh)) {   // also catches NaN
                    T m = sqrt(m2);
                    S[j * LD + j] = (m > 0 && m == m) ? d * (thresh / m) : cx<T>(thresh);
                    atomicAdd(npert, 1);
                }
            }
            __syncwarp();
            const cx<T> inv = cdiv(cx<T>(1), S[j * LD + j]);
            for (int i = j + 1 + tid; i < kb; i += 32) S[i * LD + j] = S[i * LD + j] * inv;
        }
        __syncthreads();
        for (int i = j + 1 + ty; i < kb; i += 16) {
            const cx<T> l = S[i * LD + j];
            for (int c = j + 1 + tx; c < kb; c += 16) S[i * LD + c] = S[i * LD + c] - l * S[j * LD + c];
        }
        __syncthreads();
    }
    for (int idx = tid; idx < kb * kb; idx += blockDim.x) {
        int i = idx / kb, j = idx % kb;
        D[(long long)i * nf + j] = S[i * LD + j];
    }
    if (tid < KB) pord[(long long)(F.pan + k / KB) * KB + tid] = prow[tid];
}

// ---------------------------------------------------------------------------
// Inverses of the unit-lower L_D and upper U_D factors of every factored tile,
// for the substitution passes of the solves (dense products instead of serial
// recurrences).  Run once after the factorisation over all panels: a tile is
// final once its panel step is done (later steps change only rows and columns
// to its right and below, and row interchanges are LINPACK style), so this
// work is off the factorisation's chain of dependent panel steps.
// Thread c < KB: column c of L_D^{-1}; KB <= c < 2 KB: column c - KB of
// U_D^{-1}.  Padded to KB x KB with the identity.
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(2 * KB) k_tile_inverse(const PanelTask *__restrict__ tasks,
                                                         const FrontDev *__restrict__ fr,
                                                         const cx<T> *__restrict__ fac, cx<T> *__restrict__ inv)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    cx<T> *S = reinterpret_cast<cx<T> *>(smraw);   // KB x (KB+1), then 2 KB scratch columns
    const int LD = KB + 1;
    const PanelTask t = tasks[blockIdx.x];
    const FrontDev F = fr[t.f];
    const int nf = F.p + F.b, k = t.k, kb = min(KB, F.p - k);
    const cx<T> *D = fac + F.fac + (long long)k * nf + k;
    const int tid = threadIdx.x;
    #pragma unroll 8   // several loads in flight per thread
    for (int idx = tid; idx < kb * kb; idx += blockDim.x) {
        const int i = idx / kb, j = idx % kb;
        S[i * LD + j] = D[(long long)i * nf + j];
    }
    __syncthreads();
    cx<T> *Li = inv + (long long)(F.pan + k / KB) * (2 * KB * KB);
    tile_inverse_cols<T>(S, kb, Li, Li + KB * KB, tid);
}

// ---------------------------------------------------------------------------
// row band right of the panel: swap rows, then L_D^{-1} (unit lower)
// ---------------------------------------------------------------------------
constexpr int TRW = 128;   // columns per CTA
template <class T>
__global__ void __launch_bounds__(TRW) k_trsm_row(const RowTask *__restrict__ tasks, const FrontDev *__restrict__ fr,
                                                  cx<T> *__restrict__ fac, const int *__restrict__ pord)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    cx<T> *L = reinterpret_cast<cx<T> *>(smraw);          // KB x (KB+1)
    cx<T> *Bt = L + KB * (KB + 1);                       // KB x (TRW+1)
    __shared__ int idx[KB];
    const RowTask t = tasks[blockIdx.x];
    const FrontDev F = fr[t.f];
    const int nf = F.p + F.b, k = t.k, kb = min(KB, F.p - k);
    const int c0 = t.c0, nc = min(TRW, nf - c0);
    const int tid = threadIdx.x;
    cx<T> *base = fac + F.fac + (long long)k * nf;
    #pragma unroll 8   // several loads in flight per thread
    for (int q = tid; q < kb * kb; q += blockDim.x) {
        int i = q / kb, j = q % kb;
        L[i * (KB + 1) + j] = base[(long long)i * nf + k + j];
    }
    panel_rows(pord, F.pan + k / KB, kb, true, idx);
    __syncthreads();
    #pragma unroll 8   // several loads in flight per thread
    for (int q = tid; q < kb * nc; q += blockDim.x) {
        int i = q / nc, c = q % nc;
        Bt[i * (TRW + 1) + c] = base[(long long)idx[i] * nf + c0 + c];
    }
    __syncthreads();
    if (tid < nc) {
        for (int i = 1; i < kb; i++) {
            cx<T> s = Bt[i * (TRW + 1) + tid];
            for (int l = 0; l < i; l++) s = s - L[i * (KB + 1) + l] * Bt[l * (TRW + 1) + tid];
            Bt[i * (TRW + 1) + tid] = s;
        }
    }
    __syncthreads();
    for (int q = tid; q < kb * nc; q += blockDim.x) {
        int i = q / nc, c = q % nc;
        base[(long long)i * nf + c0 + c] = Bt[i * (TRW + 1) + c];
    }
}

// ---------------------------------------------------------------------------
// column band below the panel: X <- X U_D^{-1}
// ---------------------------------------------------------------------------
constexpr int TCR = 128;   // rows per CTA
template <class T>
__global__ void __launch_bounds__(TCR) k_trsm_col(const ColTask *__restrict__ tasks, const FrontDev *__restrict__ fr,
                                                  cx<T> *__restrict__ fac)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    cx<T> *U = reinterpret_cast<cx<T> *>(smraw);          // KB x (KB+1)
    cx<T> *Xs = U + KB * (KB + 1);                        // TCR x (KB+1)
    __shared__ cx<T> invd[KB];
    const ColTask t = tasks[blockIdx.x];
    const FrontDev F = fr[t.f];
    const int nf = F.p + F.b, k = t.k, kb = min(KB, F.p - k);
    const int tid = threadIdx.x;
    const cx<T> *D = fac + F.fac + (long long)k * nf + k;
    #pragma unroll 8   // several loads in flight per thread
    for (int q = tid; q < kb * kb; q += blockDim.x) {
        int i = q / kb, j = q % kb;
        U[i * (KB + 1) + j] = D[(long long)i * nf + j];
    }
    cx<T> *xb;
    long long ld;
    int nr;
    if (t.which == 0) {
        xb = fac + F.fac + (long long)t.r0 * nf + k;
        ld = nf;
        nr = min(TCR, F.p - t.r0);
    } else {
        xb = fac + F.fac + (long long)F.p * nf + (long long)t.r0 * F.p + k;
        ld = F.p;
        nr = min(TCR, F.b - t.r0);
    }
    #pragma unroll 8   // several loads in flight per thread
    for (int q = tid; q < nr * kb; q += blockDim.x) {
        int r = q / kb, j = q % kb;
        Xs[r * (KB + 1) + j] = xb[(long long)r * ld + j];
    }
    __syncthreads();
    for (int j = tid; j < kb; j += blockDim.x) invd[j] = cdiv(cx<T>(1), U[j * (KB + 1) + j]);
    __syncthreads();
    if (tid < nr) {
        cx<T> *x = Xs + tid * (KB + 1);
        for (int j = 0; j < kb; j++) {
            cx<T> s = x[j];
            for (int l = 0; l < j; l++) s = s - x[l] * U[l * (KB + 1) + j];
            x[j] = s * invd[j];
        }
    }
    __syncthreads();
    for (int q = tid; q < nr * kb; q += blockDim.x) {
        int r = q / kb, j = q % kb;
        xb[(long long)r * ld + j] = Xs[r * (KB + 1) + j];
    }
}

// Asynchronous global -> shared copy of one complex element (8 or 16 bytes,
// naturally aligned), and the wait for all of a thread's copies.
template <class T>
__device__ __forceinline__ void cp_async_cx(cx<T> *dst, const cx<T> *src)
{
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    if constexpr (sizeof(cx<T>) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
}

// ---------------------------------------------------------------------------
// complex64 band solves by substitution, one column (row band) or one row
// (column band) per thread, in eight groups of eight unknowns.  For group G
// the thread solves its eight unknowns in registers with the diagonal 8 x 8
// block of the tile, writes them back to its own column (row) in shared
// memory, and then subtracts their multiples from every later group H, one
// 8 x 8 block of the tile at a time (the tile's rows are read as 16-byte
// broadcasts).  The loops over G and H are not unrolled, so the kernel's code
// stays small: fully unrolled, the 2,016 multiply-adds of a 64-vector are
// some 12k instructions per thread, and the warps then wait on instruction
// fetch (ncu: 1.7 cycles per issue stalled on no_instruction, 24 % issue
// activity).  The tile is padded with the identity beyond kb (a last,
// narrower panel).
// ---------------------------------------------------------------------------
constexpr int TG = 8;                       // unknowns per group
constexpr int LDT = KB + 2;                 // tile row stride: 16-byte-aligned rows
__host__ __device__ constexpr size_t band_row_smem() { return sizeof(cx<float>) * (KB * LDT + KB * (TRW + 1)); }
__host__ __device__ constexpr size_t band_col_smem() { return sizeof(cx<float>) * (KB * LDT + TCR * (KB + 1)); }

__device__ __forceinline__ void cfms(cx<float> &d, const cx<float> a, const cx<float> b)   // d -= a b
{
    d.re = fmaf(-a.re, b.re, fmaf(a.im, b.im, d.re));
    d.im = fmaf(-a.re, b.im, fmaf(-a.im, b.re, d.im));
}

// eight consecutive complex values of a 16-byte-aligned shared-memory row
__device__ __forceinline__ void lds8(const cx<float> *p, cx<float> (&a)[TG])
{
#pragma unroll
    for (int j = 0; j < TG; j += 2) {
        const float4 u = reinterpret_cast<const float4 *>(p)[j / 2];
        a[j] = cx<float>(u.x, u.y);
        a[j + 1] = cx<float>(u.z, u.w);
    }
}

// the KB x KB diagonal tile into shared memory (row stride LDT), identity
// beyond kb
__device__ __forceinline__ void load_tile_padded(cx<float> *T, const cx<float> *D, long long nf, int kb)
{
    for (int q = threadIdx.x; q < KB * KB; q += blockDim.x) {
        const int i = q / KB, j = q % KB;
        if (i < kb && j < kb) cp_async_cx(T + i * LDT + j, D + (long long)i * nf + j);
        else T[i * LDT + j] = cx<float>(i == j ? 1.f : 0.f, 0.f);
    }
}

template <int UNUSED = 0>
__global__ void __launch_bounds__(TRW) k_trsm_row_h(const RowTask *__restrict__ tasks, const FrontDev *__restrict__ fr,
                                                    cx<float> *__restrict__ fac, const int *__restrict__ pord)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    cx<float> *L = reinterpret_cast<cx<float> *>(smraw);   // KB x LDT
    cx<float> *Bt = L + KB * LDT;                         // KB x (TRW+1): band rows as stored
    __shared__ int idx[KB];
    const RowTask t = tasks[blockIdx.x];
    const FrontDev F = fr[t.f];
    const int nf = F.p + F.b, k = t.k, kb = min(KB, F.p - k);
    const int c0 = t.c0, nc = min(TRW, nf - c0);
    const int tid = threadIdx.x;
    cx<float> *base = fac + F.fac + (long long)k * nf;
    load_tile_padded(L, base + k, nf, kb);
    for (int q = tid; q < kb * nc; q += blockDim.x) {
        const int i = q / nc, c = q % nc;
        cp_async_cx(Bt + i * (TRW + 1) + c, base + (long long)i * nf + c0 + c);
    }
    panel_rows(pord, F.pan + k / KB, kb, true, idx);
    cp_async_wait_all();
    __syncthreads();
    // Row i of the result is kept in the stored slot idx[i] of the row it
    // came from: the slots of rows not yet read stay untouched.  Unknowns at
    // or beyond kb are zero and stay zero (identity padding).
    if (tid < nc) {
        cx<float> *col = Bt + tid;
        const int ng = (kb + TG - 1) / TG;
#pragma unroll 1
        for (int G = 0; G < ng; G++) {
            cx<float> b[TG];
#pragma unroll
            for (int i = 0; i < TG; i++) b[i] = TG * G + i < kb ? col[idx[TG * G + i] * (TRW + 1)] : cx<float>(0.f, 0.f);
#pragma unroll
            for (int i = 1; i < TG; i++) {
                cx<float> lr[TG];
                lds8(L + (TG * G + i) * LDT + TG * G, lr);
#pragma unroll
                for (int l = 0; l < i; l++) cfms(b[i], lr[l], b[l]);
            }
#pragma unroll
            for (int i = 0; i < TG; i++)
                if (TG * G + i < kb) col[idx[TG * G + i] * (TRW + 1)] = b[i];
#pragma unroll 1
            for (int H = G + 1; H < ng; H++) {
#pragma unroll
                for (int i = 0; i < TG; i++) {
                    const int row = TG * H + i;
                    if (row < kb) {
                        cx<float> lr[TG];
                        lds8(L + row * LDT + TG * G, lr);
                        cx<float> c = col[idx[row] * (TRW + 1)];
#pragma unroll
                        for (int l = 0; l < TG; l++) cfms(c, lr[l], b[l]);
                        col[idx[row] * (TRW + 1)] = c;
                    }
                }
            }
        }
    }
    __syncthreads();
    for (int q = tid; q < kb * nc; q += blockDim.x) {
        const int i = q / nc, c = q % nc;
        base[(long long)i * nf + c0 + c] = Bt[idx[i] * (TRW + 1) + c];
    }
}

template <int UNUSED = 0>
__global__ void __launch_bounds__(TCR) k_trsm_col_h(const ColTask *__restrict__ tasks, const FrontDev *__restrict__ fr,
                                                    cx<float> *__restrict__ fac)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    cx<float> *U = reinterpret_cast<cx<float> *>(smraw);   // KB x LDT
    cx<float> *Xs = U + KB * LDT;                         // TCR x (KB+1)
    __shared__ cx<float> invd[KB];
    const ColTask t = tasks[blockIdx.x];
    const FrontDev F = fr[t.f];
    const int nf = F.p + F.b, k = t.k, kb = min(KB, F.p - k);
    const int tid = threadIdx.x;
    load_tile_padded(U, fac + F.fac + (long long)k * nf + k, nf, kb);
    cx<float> *xb;
    long long ld;
    int nr;
    if (t.which == 0) {
        xb = fac + F.fac + (long long)t.r0 * nf + k;
        ld = nf;
        nr = min(TCR, F.p - t.r0);
    } else {
        xb = fac + F.fac + (long long)F.p * nf + (long long)t.r0 * F.p + k;
        ld = F.p;
        nr = min(TCR, F.b - t.r0);
    }
    for (int q = tid; q < nr * kb; q += blockDim.x) {
        const int r = q / kb, j = q % kb;
        cp_async_cx(Xs + r * (KB + 1) + j, xb + (long long)r * ld + j);
    }
    cp_async_wait_all();
    __syncthreads();
    for (int j = tid; j < KB; j += blockDim.x) invd[j] = cdiv(cx<float>(1.f, 0.f), U[j * LDT + j]);
    __syncthreads();
    if (tid < nr) {
        cx<float> *row = Xs + tid * (KB + 1);
        const int ng = (kb + TG - 1) / TG;
#pragma unroll 1
        for (int G = 0; G < ng; G++) {
            cx<float> x[TG];
#pragma unroll
            for (int j = 0; j < TG; j++) x[j] = TG * G + j < kb ? row[TG * G + j] : cx<float>(0.f, 0.f);
#pragma unroll
            for (int j = 0; j < TG; j++) {
                x[j] = x[j] * invd[TG * G + j];
                cx<float> ur[TG];
                lds8(U + (TG * G + j) * LDT + TG * G, ur);
#pragma unroll
                for (int j2 = j + 1; j2 < TG; j2++) cfms(x[j2], x[j], ur[j2]);
            }
#pragma unroll
            for (int j = 0; j < TG; j++)
                if (TG * G + j < kb) row[TG * G + j] = x[j];
#pragma unroll 1
            for (int H = G + 1; H < ng; H++) {
                cx<float> y[TG];
#pragma unroll
                for (int j = 0; j < TG; j++) y[j] = TG * H + j < kb ? row[TG * H + j] : cx<float>(0.f, 0.f);
#pragma unroll
                for (int l = 0; l < TG; l++) {
                    cx<float> ur[TG];
                    lds8(U + (TG * G + l) * LDT + TG * H, ur);
#pragma unroll
                    for (int j = 0; j < TG; j++) cfms(y[j], x[l], ur[j]);
                }
#pragma unroll
                for (int j = 0; j < TG; j++)
                    if (TG * H + j < kb) row[TG * H + j] = y[j];
            }
        }
    }
    __syncthreads();
    for (int q = tid; q < nr * kb; q += blockDim.x) {
        const int r = q / kb, j = q % kb;
        xb[(long long)r * ld + j] = Xs[r * (KB + 1) + j];
    }
}

// ---------------------------------------------------------------------------
// SIMT complex GEMM  C -= op(A) * B  (64x64 tiles, 4x4 per thread)
// ---------------------------------------------------------------------------
constexpr int GBM = 64, GBN = 64, GBK = 16;
template <class T>
__global__ void __launch_bounds__(256) k_gemm(const GemmTask<T> *__restrict__ tasks, int ntasks)
{
    __shared__ cx<T> As[GBK][GBM + 1];
    __shared__ cx<T> Bs[GBK][GBN];
    const int ti = find_task(tasks, ntasks, (long long)blockIdx.x);
    const GemmTask<T> t = tasks[ti];
    const long long lt = (long long)blockIdx.x - t.tile0;
    const int m0 = (int)(lt / t.tiles_n) * GBM, n0 = (int)(lt % t.tiles_n) * GBN;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    cx<T> acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = cx<T>(0);
    for (int k0 = 0; k0 < t.K; k0 += GBK) {
        if (!t.conjA) {
#pragma unroll
            for (int q = 0; q < (GBM * GBK) / 256; q++) {
                int idx = tid + q * 256;
                int i = idx / GBK, kk = idx % GBK;
                int r = m0 + i, c = k0 + kk;
                As[kk][i] = (r < t.M && c < t.K) ? t.A[(long long)r * t.lda + c] : cx<T>(0);
            }
        } else {
            // op(A)[r][c] = conj(A[c][r])
#pragma unroll
            for (int q = 0; q < (GBM * GBK) / 256; q++) {
                int idx = tid + q * 256;
                int kk = idx / GBM, i = idx % GBM;
                int r = m0 + i, c = k0 + kk;
                As[kk][i] = (r < t.M && c < t.K) ? conj(t.A[(long long)c * t.lda + r]) : cx<T>(0);
            }
        }
#pragma unroll
        for (int q = 0; q < (GBK * GBN) / 256; q++) {
            int idx = tid + q * 256;
            int kk = idx / GBN, j = idx % GBN;
            int r = k0 + kk, c = n0 + j;
            cx<T> v(0);
            if (r < t.K && c < t.N) {
                long long row = t.brow ? (long long)t.brow[r] : (long long)r;
                v = t.B[row * t.ldb + c];
            }
            Bs[kk][j] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GBK; kk++) {
            cx<T> a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    acc[i][j].re = fma(a[i].re, b[j].re, fma(-a[i].im, b[j].im, acc[i][j].re));
                    acc[i][j].im = fma(a[i].re, b[j].im, fma(a[i].im, b[j].re, acc[i][j].im));
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        int r = m0 + ty + 16 * i;
        if (r >= t.M) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            int c = n0 + tx + 16 * j;
            if (c >= t.N) continue;
            if (t.crow) {
                atomic_sub(t.C + (long long)t.crow[r] * t.ldc + c, acc[i][j]);
            } else {
                cx<T> *p = t.C + (long long)r * t.ldc + c;
                *p = *p - acc[i][j];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Tall-skinny SIMT complex GEMM  C -= op(A) * B  for N <= 32 (the right-hand
// side blocks of the substitution passes): 128 x 32 tiles, 4 x 4 complex
// outputs per thread, every A element read once per tile.
// ---------------------------------------------------------------------------
constexpr int TSBM = 128, TSBN = 32, TSBK = 16;   // TSBK: K granularity of split-K chunks
template <class T> struct TsCfg { static constexpr int BK = sizeof(T) == 4 ? 32 : 16; };

// 128 x 32 tile per CTA of 256 threads; thread (tx, ty) owns rows 4ty..4ty+3
// and columns 4tx..4tx+3 (16 complex accumulators).  The K loop stages
// BK-deep slices of A (transposed in shared memory) and B, prefetching the
// next slice into registers while the current one is consumed.
template <class T>
__global__ void __launch_bounds__(256, 2) k_gemm_ts(const GemmTask<T> *__restrict__ tasks, int ntasks)
{
    constexpr int BK = TsCfg<T>::BK;
    constexpr int AP = TSBM + 1;                       // padded row of the A^T slice
    constexpr int NA = TSBM * BK / 256, NB = BK * TSBN / 256;
    __shared__ cx<T> As[BK][AP];
    __shared__ cx<T> Bs[BK][TSBN];
    const int ti = find_task(tasks, ntasks, (long long)blockIdx.x);
    const GemmTask<T> t = tasks[ti];
    const int m0 = (int)((long long)blockIdx.x - t.tile0) * TSBM;
    const int tid = threadIdx.x, tx = tid & 7, ty = tid >> 3;
    cx<T> acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = cx<T>(0);
    cx<T> pa[NA], pb[NB];
    // A slice element q of this thread: non-conjugate A is read along K
    // (row-contiguous), the conjugate transpose along M.
    auto load = [&](int k0) {
#pragma unroll
        for (int q = 0; q < NA; q++) {
            const int idx = tid + q * 256;
            int i, kk;
            if (!t.conjA) { i = idx / BK; kk = idx % BK; }
            else { kk = idx / TSBM; i = idx % TSBM; }
            const int r = m0 + i, c = k0 + kk;
            cx<T> v(0);
            if (r < t.M && c < t.K) v = t.conjA ? conj(t.A[(long long)c * t.lda + r]) : t.A[(long long)r * t.lda + c];
            pa[q] = v;
        }
#pragma unroll
        for (int q = 0; q < NB; q++) {
            const int idx = tid + q * 256;
            const int kk = idx / TSBN, j = idx % TSBN;
            const int r = k0 + kk;
            cx<T> v(0);
            if (r < t.K && j < t.N) v = t.B[(t.brow ? (long long)t.brow[r] : (long long)r) * t.ldb + j];
            pb[q] = v;
        }
    };
    auto store = [&]() {
#pragma unroll
        for (int q = 0; q < NA; q++) {
            const int idx = tid + q * 256;
            int i, kk;
            if (!t.conjA) { i = idx / BK; kk = idx % BK; }
            else { kk = idx / TSBM; i = idx % TSBM; }
            As[kk][i] = pa[q];
        }
#pragma unroll
        for (int q = 0; q < NB; q++) {
            const int idx = tid + q * 256;
            Bs[idx / TSBN][idx % TSBN] = pb[q];
        }
    };
    load(0);
    for (int k0 = 0; k0 < t.K; k0 += BK) {
        store();
        __syncthreads();
        if (k0 + BK < t.K) load(k0 + BK);
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            cx<T> a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk][4 * ty + i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk][4 * tx + j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    acc[i][j].re = fma(a[i].re, b[j].re, fma(-a[i].im, b[j].im, acc[i][j].re));
                    acc[i][j].im = fma(a[i].re, b[j].im, fma(a[i].im, b[j].re, acc[i][j].im));
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int r = m0 + 4 * ty + i;
        if (r >= t.M) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int c = 4 * tx + j;
            if (c >= t.N) continue;
            if (t.crow) atomic_sub(t.C + (long long)t.crow[r] * t.ldc + c, acc[i][j]);
            else if (t.atom) atomic_sub(t.C + (long long)r * t.ldc + c, acc[i][j]);
            else {
                cx<T> *p = t.C + (long long)r * t.ldc + c;
                *p = *p - acc[i][j];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Fused substitution step: the diagonal-tile product of panel k and the update
// of the outer block's other rows, in one launch per panel step (the panel
// steps of a block form a dependent chain; one launch instead of two halves
// its latency).  Every CTA of a front computes the panel's solved rows
//   mode 0  Z = L_D^{-1} P y          mode 1  Z = U_D^{-1} y
//   mode 2  Z = U_D^{-H} y            mode 3  Z = P^T L_D^{-H} y
// from the panel rows y of X (which no CTA of the launch writes) into shared
// memory; update CTAs then subtract its contribution from their rows,
//   mode 0  y_r -= L[r, k:k2] Z       mode 1  y_r -= U[r, k:k2] Z
//   mode 2  y_r -= U[k:k2, r]^H Z     mode 3  y_r -= L[k:k2, r]^H Z
// (rows below the panel for the forward modes 0/2, above it for 1/3), and the
// role-0 CTA leaves Z in the front's scratch slot; the next step's role-0 CTA
// (or a flush) writes it into X once no CTA reads those rows any more.
// ---------------------------------------------------------------------------
constexpr int SUB_RB = 32;   // rows per update CTA

// Shared-memory layout of k_sub_step (complex elements).
__host__ __device__ constexpr int sub_step_smem_elems()
{
    return KB * KB + KB * (MAXRHS + 1) + KB * SUB_RB + SUB_RB * (MAXRHS + 1);
}

// d += a b and d += conj(a) b as four fused multiply-adds
template <class T>
__device__ __forceinline__ void cmac(cx<T> &d, const cx<T> a, const cx<T> b)
{
    d.re = fma(a.re, b.re, fma(-a.im, b.im, d.re));
    d.im = fma(a.re, b.im, fma(a.im, b.re, d.im));
}
template <class T>
__device__ __forceinline__ void cmac_conj(cx<T> &d, const cx<T> a, const cx<T> b)
{
    d.re = fma(a.re, b.re, fma(a.im, b.im, d.re));
    d.im = fma(a.re, b.im, fma(-a.im, b.re, d.im));
}

// four consecutive complex values from 16-byte-aligned shared memory
__device__ __forceinline__ void lds4(const cx<float> *p, cx<float> (&a)[4])
{
    const float4 u = reinterpret_cast<const float4 *>(p)[0], v = reinterpret_cast<const float4 *>(p)[1];
    a[0] = cx<float>(u.x, u.y); a[1] = cx<float>(u.z, u.w); a[2] = cx<float>(v.x, v.y); a[3] = cx<float>(v.z, v.w);
}
__device__ __forceinline__ void lds4(const cx<double> *p, cx<double> (&a)[4])
{
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const double2 u = reinterpret_cast<const double2 *>(p)[j];
        a[j] = cx<double>(u.x, u.y);
    }
}

// two consecutive complex values from 16-byte-aligned shared memory
__device__ __forceinline__ void lds2(const cx<float> *p, cx<float> (&a)[2])
{
    const float4 u = reinterpret_cast<const float4 *>(p)[0];
    a[0] = cx<float>(u.x, u.y); a[1] = cx<float>(u.z, u.w);
}
__device__ __forceinline__ void lds2(const cx<double> *p, cx<double> (&a)[2])
{
    const double2 u = reinterpret_cast<const double2 *>(p)[0], v = reinterpret_cast<const double2 *>(p)[1];
    a[0] = cx<double>(u.x, u.y); a[1] = cx<double>(v.x, v.y);
}

constexpr int SUB_THREADS = 512;   // 16 warps: each thread sums 4 rows of Z and 2 update rows
template <class T>
__global__ void __launch_bounds__(SUB_THREADS) k_sub_step(const StepTask *__restrict__ tasks, const FrontDev *__restrict__ fr,
                                                  const cx<T> *__restrict__ fac, const cx<T> *__restrict__ inv,
                                                  const int *__restrict__ pord, cx<T> *__restrict__ X, int ldx, int m,
                                                  int mode, cx<T> *__restrict__ zs)
{
    // Launched as a programmatic dependent of the previous step: the next
    // step may start as soon as every CTA of this one is running; it fetches
    // what no step writes (task, tile inverse, factor rows, row order) and
    // then waits for this grid's completion before it touches X or the slots.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    extern __shared__ __align__(16) unsigned char smraw[];
    // every input is fetched in one batch of asynchronous copies, laid out so
    // that the four rows a thread sums are adjacent: Ms[l][i] is the mode's
    // tile-inverse entry (i, l) (conjugated on read for modes 2, 3), As[l][r]
    // the update CTA's factor entry (r, l) (likewise)
    cx<T> *Ms = reinterpret_cast<cx<T> *>(smraw);   // KB x KB
    cx<T> *Ys = Ms + KB * KB;                       // KB x (MAXRHS+1): panel rows as stored, then Z
    cx<T> *As = Ys + KB * (MAXRHS + 1);             // KB x SUB_RB
    cx<T> *Yr = As + KB * SUB_RB;                   // SUB_RB x (MAXRHS+1): the update CTA's rows of X
    __shared__ int idx[KB];
    const StepTask t = tasks[blockIdx.x];
    const FrontDev F = fr[t.f];
    const int tid = threadIdx.x;
    const int nf = F.p + F.b;
    const int LY = MAXRHS + 1;
    cx<T> *Y = X + (long long)F.first * ldx;
    cx<T> *slot = zs + (long long)t.slot * (KB * MAXRHS);
    const int k = t.k, kb = min(KB, F.p - k);
    const cx<T> *Li = inv + (long long)(F.pan + k / KB) * (2 * KB * KB);
    const cx<T> *Mi = (mode == 0 || mode == 3) ? Li : Li + KB * KB;
    const bool herm = mode >= 2;
    const int nr = t.role == 1 ? t.r1 - t.r0 : 0;
    const cx<T> *P = fac + F.fac;
    // stored inverse entry q = (a, b): (i, l) = (a, b) transposed into Ms[l][i],
    // or (l, i) = (a, b) as stored for the conjugate transposes
    for (int q = tid; q < KB * KB; q += blockDim.x)
        cp_async_cx(herm ? Ms + q : Ms + (q & (KB - 1)) * KB + (q >> 6), Mi + q);
    if (nr) {
        if (mode == 0 || mode == 1) {   // A(r, l) = P[r0 + r][k + l]
            for (int q = tid; q < nr * KB; q += blockDim.x) {   // (row, column) = (q / KB, q % KB)
                const int r = q >> 6, l = q & (KB - 1);
                if (l < kb) cp_async_cx(As + l * SUB_RB + r, P + (long long)(t.r0 + r) * nf + k + l);
            }
        } else {                        // A(r, l) = conj(P[k + l][r0 + r])
            for (int q = tid; q < kb * SUB_RB; q += blockDim.x) {   // (column, row) = (q / SUB_RB, q % SUB_RB)
                const int l = q / SUB_RB, r = q % SUB_RB;
                if (r < nr) cp_async_cx(As + l * SUB_RB + r, P + (long long)(k + l) * nf + t.r0 + r);
            }
        }
    }
    panel_rows(pord, F.pan + k / KB, kb, mode == 0 || mode == 3, idx);
    // everything below reads or writes rows of X or the slots
    asm volatile("griddepcontrol.wait;" ::: "memory");
    // (row, column) loops run over MAXRHS columns (a power of two) and skip
    // those at or beyond m: no integer division per element
    for (int q = tid; q < kb * MAXRHS; q += blockDim.x) {
        const int i = q / MAXRHS, c = q % MAXRHS;
        if (c < m) cp_async_cx(Ys + i * LY + c, Y + (long long)(k + i) * ldx + c);
    }
    if (nr) {
        for (int q = tid; q < nr * MAXRHS; q += blockDim.x) {
            const int r = q / MAXRHS, c = q % MAXRHS;
            if (c < m) cp_async_cx(Yr + r * LY + c, Y + (long long)(t.r0 + r) * ldx + c);
        }
    }
    // while the copies fly: the previous panel's solved rows into X (roles
    // 0 and 3; no CTA of this launch reads those rows)
    if (t.role != 1 && t.kprev >= 0) {
        const int kbp = min(KB, F.p - t.kprev);
        #pragma unroll 8   // several loads in flight per thread
        for (int q = tid; q < kbp * MAXRHS; q += blockDim.x) {
            const int i = q / MAXRHS, c = q % MAXRHS;
            if (c < m) Y[(long long)(t.kprev + i) * ldx + c] = slot[i * MAXRHS + c];
        }
    }
    cp_async_wait_all();
    __syncthreads();
    // Z = M y: thread (lane c, warp w) owns rows 4w .. 4w+3 of column c; the
    // l loop runs outside, so its sums are independent chains (M entries are
    // warp broadcasts, two 16-byte loads per l for complex64)
    constexpr int NW = SUB_THREADS / 32, RPT = KB / NW, UPT = SUB_RB / NW;
    static_assert(RPT == 4 && UPT == 2, "four rows of Z, two update rows per thread");
    const int c = tid & 31, w = tid >> 5, i0 = RPT * w;
    cx<T> acc[RPT];
#pragma unroll
    for (int j = 0; j < RPT; j++) acc[j] = cx<T>(0);
    if (c < m) {
        if (!herm) {
            for (int l = 0; l < kb; l++) {
                const cx<T> y = Ys[(mode == 0 ? idx[l] : l) * LY + c];
                cx<T> a[4];
                lds4(Ms + l * KB + i0, a);
#pragma unroll
                for (int j = 0; j < RPT; j++) cmac(acc[j], a[j], y);
            }
        } else {
            for (int l = 0; l < kb; l++) {
                const cx<T> y = Ys[l * LY + c];
                cx<T> a[4];
                lds4(Ms + l * KB + i0, a);
#pragma unroll
                for (int j = 0; j < RPT; j++) cmac_conj(acc[j], a[j], y);
            }
        }
    }
    __syncthreads();
    // Z (with the output permutation of mode 3) replaces the panel rows
    if (c < m) {
#pragma unroll
        for (int j = 0; j < RPT; j++) {
            const int i = i0 + j;
            if (i < kb) Ys[(mode == 3 ? idx[i] : i) * LY + c] = acc[j];
        }
    }
    __syncthreads();
    if (t.role == 0 || t.role == 3) {
        // role 3: the front's last panel of the block, which no other CTA of
        // this launch reads: solved rows straight into X
        for (int q = tid; q < kb * MAXRHS; q += blockDim.x) {
            const int i = q / MAXRHS, cc = q % MAXRHS;
            if (cc >= m) continue;
            if (t.role == 0) slot[i * MAXRHS + cc] = Ys[i * LY + cc];
            else Y[(long long)(k + i) * ldx + cc] = Ys[i * LY + cc];
        }
        return;
    }
    // update rows 2w, 2w+1 of column c, independent sums as above
    if (c < m) {
        const int u0 = UPT * w;
        cx<T> u[UPT];
#pragma unroll
        for (int j = 0; j < UPT; j++) u[j] = cx<T>(0);
        if (!herm) {
            for (int l = 0; l < kb; l++) {
                const cx<T> z = Ys[l * LY + c];
                cx<T> a[UPT];
                lds2(As + l * SUB_RB + u0, a);
#pragma unroll
                for (int j = 0; j < UPT; j++) cmac(u[j], a[j], z);
            }
        } else {
            for (int l = 0; l < kb; l++) {
                const cx<T> z = Ys[l * LY + c];
                cx<T> a[UPT];
                lds2(As + l * SUB_RB + u0, a);
#pragma unroll
                for (int j = 0; j < UPT; j++) cmac_conj(u[j], a[j], z);
            }
        }
#pragma unroll
        for (int j = 0; j < UPT; j++) {
            const int r = u0 + j;
            if (r < nr) Y[(long long)(t.r0 + r) * ldx + c] = Yr[r * LY + c] - u[j];
        }
    }
}

}  // namespace wt3d
