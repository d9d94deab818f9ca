// Tall-skinny complex64 GEMM  C -= A B  on the tcgen05 tensor cores, for the
// substitution passes of the solve: A is a factor block (M x K, K-major rows
// in the front storage, any leading dimension) or, in the adjoint passes, the
// conjugate transpose of one, and B and C hold at most 32 right-hand sides.  Each factor entry is used for 32 complex multiply-adds
// only, so the kernel is meant to run at the speed of reading A from HBM.
//
// A is not copied or pre-split: front blocks start and stride at arbitrary
// 8-byte boundaries, which rules out TMA, so eight loader warps stream A with
// 8-byte asynchronous copies (cp.async, one 128-byte row segment per
// half-warp) into a ring of TS_RAW raw stages (~112 KB per SM in flight),
// then split every value into TF32 hi + lo (x = hi + lo to ~2^-24)
// and store both halves into the 128-byte-swizzled K-major tiles the MMA
// reads.  B is expanded once per
// launch into the 64 x 2K real matrix B~ (rows 2j, 2j+1 of column j, as in the
// square tensor-core GEMM), split into hi and lo, and fetched by TMA.  The
// complex product is the real product A_r B~^T into a 128 x 64 FP32 TMEM
// accumulator with D = Ahi Bhi + Ahi Blo + Alo Bhi.
//
// Work unit = (task, 128-row tile, K-chunk); persistent CTAs, one per SM.
// Warps 0-15 load and split A, warp 16 issues the TMA copies of B~ (and owns
// the TMEM allocation), warp 17 (one lane) issues the MMAs, warp 18 streams A
// by TMA in the variant for 16-byte-aligned blocks with even strides (the
// loaders then only convert), warps 19-22 drain the double-buffered
// accumulator: C -= D in place, or with atomics when the task is split along K
// or its rows are scattered (border updates).  Every mbarrier wait is bounded;
// on expiry the kernel records an error code and winds down as the square
// kernel does.
#include "tc_gemm.h"
#include "tc_ptx.cuh"
#include <cstring>

namespace wt3d {

constexpr int TS_BM = 128;                        // complex rows per tile (MMA M)
constexpr int TS_NR = 64;                         // real accumulator columns: 32 complex (MMA N)
constexpr int TS_KC = 16;                         // complex k per stage: one 128-byte swizzle row
constexpr int TS_STAGES = 2;                      // split A stages (hi + lo)
constexpr int TS_BSTAGES = 2;                     // B~ stages (TMA from L2)
constexpr int TS_A_BYTES = TS_BM * 128;           // 16 KB per split half
constexpr int TS_B_BYTES = TS_NR * 128;           // 8 KB per split half
constexpr int TS_ASTAGE_BYTES = 2 * TS_A_BYTES;
constexpr int TS_BSTAGE_BYTES = 2 * TS_B_BYTES;
constexpr int TS_RAW = 8;                         // raw A stages in flight (asynchronous copies)
constexpr int TS_RAW_BYTES = TS_BM * TS_KC * 8;   // 16 KB
constexpr int TS_B_OFF = TS_STAGES * TS_ASTAGE_BYTES;
constexpr int TS_RAW_OFF = TS_B_OFF + TS_BSTAGES * TS_BSTAGE_BYTES;
constexpr int TS_BAR_OFF = TS_RAW_OFF + TS_RAW * TS_RAW_BYTES;
constexpr int TS_SMEM = TS_BAR_OFF + 1024 + 512;
constexpr int TS_LOADERS = 16;                    // loader warps
constexpr int TS_WB = TS_LOADERS, TS_WM = TS_LOADERS + 1, TS_WA = TS_LOADERS + 2, TS_WE = TS_LOADERS + 3;
constexpr int TS_THREADS = (TS_LOADERS + 7) * 32; // + B producer, MMA, A producer (TMA variant), 4 epilogue warps
constexpr int TS_LT = TS_LOADERS * 32;            // loader threads
constexpr int TS_PER_THREAD = TS_BM * TS_KC / TS_LT;   // complex elements per loader thread per stage
constexpr int TS_QROWS = TS_LT / TS_KC;           // rows between a thread's elements
static_assert(TS_PER_THREAD * TS_LT == TS_BM * TS_KC && TS_QROWS % 8 == 0, "loader mapping");
static_assert((TS_LT / TS_BM) * TS_PER_THREAD == TS_KC, "conjugate-transposed loader mapping");

// Unit u of a launch: its task, first row, and K range [k0, k1).
__device__ __forceinline__ const TsTask *ts_unit(const TsTask *__restrict__ tasks, int ntasks, long long u, int &m0,
                                                 int &k0, int &k1)
{
    int lo = 0, hi = ntasks - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].unit0 <= u) lo = mid;
        else hi = mid - 1;
    }
    const TsTask *t = tasks + lo;
    const long long lt = u - t->unit0;
    m0 = (int)(lt / t->nkc) * TS_BM;
    k0 = (int)(lt % t->nkc) * t->kchunk;
    k1 = min(t->K, k0 + t->kchunk);
    return t;
}

// B~ of every task: 32 x 32 complex tiles (k x j) of B, rows gathered through
// brow when given, transposed through shared memory into rows 2j, 2j+1
// (hi and lo); columns j >= N and k >= K are zero.
__global__ void __launch_bounds__(256) k_ts_expand_b(const TsTask *__restrict__ tasks, int ntasks, long long total)
{
    __shared__ float2 tile[32][33];
    const long long q = blockIdx.x;
    if (q >= total) return;
    int lo = 0, hi = ntasks - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].b_work0 <= q) lo = mid;
        else hi = mid - 1;
    }
    const TsTask &t = tasks[lo];
    const int k0 = (int)(q - t.b_work0) * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int kk = ty; kk < 32; kk += 8) {
        const int k = k0 + kk;
        float2 v = make_float2(0.f, 0.f);
        if (k < t.K && tx < t.N) {
            const cx<float> b = t.B[(long long)(t.brow ? t.brow[k] : k) * t.ldb + tx];
            v = make_float2(b.re, b.im);
        }
        tile[kk][tx] = v;
    }
    __syncthreads();
    for (int j = ty; j < 32; j += 8) {
        const float2 b = tile[tx][j];   // k = k0 + tx
        float rh, rl, ih, il, nih, nil;
        split_tf32(b.x, rh, rl);
        split_tf32(b.y, ih, il);
        split_tf32(-b.y, nih, nil);
        const long long o0 = (long long)(2 * j) * t.Kr + 2 * (k0 + tx), o1 = o0 + t.Kr;
        *reinterpret_cast<float2 *>(t.bhi + o0) = make_float2(rh, nih);
        *reinterpret_cast<float2 *>(t.blo + o0) = make_float2(rl, nil);
        *reinterpret_cast<float2 *>(t.bhi + o1) = make_float2(ih, rh);
        *reinterpret_cast<float2 *>(t.blo + o1) = make_float2(il, rl);
    }
}

// Position of a CTA's loaders in its sequence of stages: unit u (every
// gridDim.x-th unit from blockIdx.x), its K range and stage i within it, with
// the per-thread quantities of the unit precomputed.  A stage is 128 rows x
// 16 k of the operand; loader thread l owns TS_PER_THREAD of its elements:
//   A as stored (row-major, K-major): row TS_QROWS q + l / 16, column l % 16:
//     a half-warp reads one contiguous 128-byte row segment, and all of a
//     thread's elements share one column;
//   A^H (conjugate transpose of a stored K x M block, MN-major): row l % 128,
//     column l / 128 + 4 q: a warp reads 32 consecutive stored entries of one
//     stored row, and all of a thread's elements share one row.
struct TsCursor {
    const TsTask *t;
    const cx<float> *src;   // element q = 0 of stage 0 of this thread
    long long u, qstep;     // complex elements between the thread's elements q and q + 1
    long long sstep;        // complex elements between consecutive stages
    int k0, k1, nsub, i;
    int nq;                 // A: elements in range (rows); A^H: 4 if the row is in range, else 0
    int kq;                 // first column of this thread within a stage
    bool valid, conj;
};

__device__ __forceinline__ void ts_cursor_at(TsCursor &c, const TsTask *__restrict__ tasks, int ntasks, long long nunits,
                                             long long u, int l)
{
    c.u = u;
    c.valid = u < nunits;
    if (!c.valid) return;
    int m0;
    c.t = ts_unit(tasks, ntasks, u, m0, c.k0, c.k1);
    c.nsub = (c.k1 - c.k0 + TS_KC - 1) / TS_KC;
    c.i = 0;
    const int M = c.t->M;
    const long long lda = c.t->lda;
    c.conj = c.t->conjA != 0;
    if (!c.conj) {
        const int r0 = m0 + (l >> 4);
        c.kq = l & 15;
        c.nq = r0 < M ? min(TS_PER_THREAD, (M - r0 + TS_QROWS - 1) / TS_QROWS) : 0;
        c.qstep = (long long)TS_QROWS * lda;
        c.sstep = TS_KC;
        c.src = c.t->A + (long long)r0 * lda + c.k0 + c.kq;
    } else {
        const int r = m0 + (l & (TS_BM - 1));
        c.kq = l / TS_BM;
        c.nq = r < M ? TS_PER_THREAD : 0;
        c.qstep = (long long)(TS_LT / TS_BM) * lda;
        c.sstep = (long long)TS_KC * lda;
        c.src = c.t->A + (long long)(c.k0 + c.kq) * lda + r;
    }
}

__device__ __forceinline__ void ts_cursor_next(TsCursor &c, const TsTask *__restrict__ tasks, int ntasks,
                                               long long nunits, int l)
{
    if (++c.i == c.nsub) ts_cursor_at(c, tasks, ntasks, nunits, c.u + gridDim.x, l);
}

// elements q < ts_count of the cursor's stage lie in the operand
__device__ __forceinline__ int ts_count(const TsCursor &c)
{
    const int kb = c.k0 + c.i * TS_KC + c.kq;   // column of element q = 0
    if (!c.conj) return kb < c.k1 ? c.nq : 0;
    constexpr int kstep = TS_LT / TS_BM;         // columns between a thread's elements
    return c.nq ? max(0, min(TS_PER_THREAD, (c.k1 - kb + kstep - 1) / kstep)) : 0;
}

// asynchronous 8-byte copies of the thread's elements into its slots raw[q][l]
__device__ __forceinline__ void ts_issue(const TsCursor &c, int l, uint32_t raw)
{
    const int n = ts_count(c);
    const cx<float> *src = c.src + c.i * c.sstep;
#pragma unroll
    for (int q = 0; q < TS_PER_THREAD; q++)
        if (q < n)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(raw + (uint32_t)((q * TS_LT + l) * 8)),
                         "l"(src + q * c.qstep)
                         : "memory");
}

// byte offset of element (row r, column k) of a stage in a 128-byte-swizzled
// K-major tile: 16-byte chunk c of row r sits at chunk c ^ (r mod 8)
__device__ __forceinline__ int ts_swz(int r, int k)
{
    return (r >> 3) * 1024 + (r & 7) * 128 + ((((k >> 1) ^ (r & 7))) << 4) + ((k & 1) << 3);
}

// hi = TF32 rounding of x (to nearest), lo = TF32 rounding of x - hi
__device__ __forceinline__ void split_cvt(float x, float &hi, float &lo)
{
    uint32_t h, lw;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
    hi = __uint_as_float(h);
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lw) : "f"(x - hi));
    lo = __uint_as_float(lw);
}

// TMA = false: loaders copy A with cp.async (any alignment, as stored or
// conjugate-transposed).  TMA = true: every task's A is 16-byte aligned with an
// even row stride, as stored; warp TS_WA streams raw 128 x 16 complex tiles of
// A into the ring by TMA and the loaders only convert.
template <bool TMA>
__global__ void __launch_bounds__(TS_THREADS, 1)
    k_tc_ts(const TsTask *__restrict__ tasks, int ntasks, long long nunits, const CUtensorMap *__restrict__ maps,
            int *err)
{
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + TS_BAR_OFF);   // split A stage written (8 loader warps)
    uint64_t *empty = full + TS_STAGES;                                  // split A stage consumed (MMA commit)
    uint64_t *bfull = empty + TS_STAGES;                                 // B~ stage landed (TMA)
    uint64_t *bempty = bfull + TS_BSTAGES;                               // B~ stage consumed (MMA commit)
    uint64_t *tfull = bempty + TS_BSTAGES;
    uint64_t *tempty = tfull + 2;
    uint64_t *drain = tempty + 2;
    uint64_t *rfull = drain + 1;                                         // raw A slot landed (TMA variant)
    uint64_t *rempty = rfull + TS_RAW;                                   // raw A slot converted (loader warps)
    uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(rempty + TS_RAW);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == TS_WB) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                     "r"(2 * TS_NR));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == TS_WM * 32) {
        for (int s = 0; s < TS_STAGES; s++) {
            mbar_init(&full[s], TS_LOADERS);
            mbar_init(&empty[s], 1);
        }
        for (int s = 0; s < TS_BSTAGES; s++) {
            mbar_init(&bfull[s], 1);
            mbar_init(&bempty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], 4);
        }
        mbar_init(drain, 1);
        for (int s = 0; s < TS_RAW; s++) {
            mbar_init(&rfull[s], 1);
            mbar_init(&rempty[s], TS_LOADERS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_holder;

    if (warp < TS_LOADERS) {
        // ---------------- A loaders: global -> raw ring -> split -> swizzled tiles ----------------
        // The copy cursor runs TS_RAW - 1 stages ahead of the conversion
        // cursor, across unit boundaries; one commit group per stage (empty
        // groups past the end keep the count uniform).
        const int l = threadIdx.x;
        uint8_t *rawb = smem + TS_RAW_OFF;
        const uint32_t raw0 = smem_u32(rawb);
        TsCursor cp, cs;
        ts_cursor_at(cs, tasks, ntasks, nunits, blockIdx.x, l);
        long long gc = 0, g = 0;
        if constexpr (!TMA) {
            ts_cursor_at(cp, tasks, ntasks, nunits, blockIdx.x, l);
            for (int p = 0; p < TS_RAW - 1; p++, gc++) {
                if (cp.valid) {
                    ts_issue(cp, l, raw0 + (uint32_t)((gc % TS_RAW) * TS_RAW_BYTES));
                    ts_cursor_next(cp, tasks, ntasks, nunits, l);
                }
                asm volatile("cp.async.commit_group;" ::: "memory");
            }
        }
        while (cs.valid) {
            const int slot = (int)(g % TS_RAW);
            if constexpr (!TMA) {
                if (cp.valid) {
                    ts_issue(cp, l, raw0 + (uint32_t)((gc % TS_RAW) * TS_RAW_BYTES));
                    ts_cursor_next(cp, tasks, ntasks, nunits, l);
                }
                asm volatile("cp.async.commit_group;" ::: "memory");
                gc++;
                asm volatile("cp.async.wait_group %0;" ::"n"(TS_RAW - 1) : "memory");   // stage g has landed
            } else {
                if (!mbar_wait(&rfull[slot], (uint32_t)((g / TS_RAW) & 1))) { atomicCAS(err, 0, 16); break; }
            }
            const uint8_t *rs = rawb + slot * TS_RAW_BYTES;
            const int s = (int)(g % TS_STAGES);
            const uint32_t ph = (uint32_t)((g / TS_STAGES) & 1) ^ 1u;
            if (!mbar_wait(&empty[s], ph)) { atomicCAS(err, 0, 11); break; }
            uint8_t *ahi = smem + s * TS_ASTAGE_BYTES, *alo = ahi + TS_A_BYTES;
            const int nq = ts_count(cs);
            const float ysign = cs.conj ? -1.f : 1.f;
#pragma unroll
            for (int q = 0; q < TS_PER_THREAD; q++) {
                float2 v = make_float2(0.f, 0.f);
                if (q < nq) {
                    if constexpr (TMA)   // the TMA box: row r of the stage at r * 128 bytes
                        v = *reinterpret_cast<const float2 *>(rs + (TS_QROWS * q + (l >> 4)) * 128 + (l & 15) * 8);
                    else                 // the thread's own slots raw[q][l]
                        v = reinterpret_cast<const float2 *>(rs)[q * TS_LT + l];
                }
                v.y *= ysign;
                const int off = cs.conj ? ts_swz(l & (TS_BM - 1), cs.kq + q * (TS_LT / TS_BM))
                                        : ts_swz(TS_QROWS * q + (l >> 4), l & 15);
                float h0, l0, h1, l1;
                split_cvt(v.x, h0, l0);
                split_cvt(v.y, h1, l1);
                *reinterpret_cast<float2 *>(ahi + off) = make_float2(h0, h1);
                *reinterpret_cast<float2 *>(alo + off) = make_float2(l0, l1);
            }
            // generic-proxy stores become visible to the tensor core's async proxy
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&full[s]);
                if constexpr (TMA) mbar_arrive(&rempty[slot]);
            }
            ts_cursor_next(cs, tasks, ntasks, nunits, l);
            g++;
        }
        if constexpr (!TMA) asm volatile("cp.async.wait_all;" ::: "memory");   // no copy into shared memory outlives the CTA
    } else if (warp == TS_WB && lane == 0) {
        // ---------------- B~ producer (TMA) ----------------
        long long g = 0;
        bool ok = true;
        for (long long u = blockIdx.x; u < nunits && ok; u += gridDim.x) {
            int m0, k0, k1;
            const TsTask *t = ts_unit(tasks, ntasks, u, m0, k0, k1);
            const CUtensorMap *mp = maps + t->map0;
            const int nsub = (k1 - k0 + TS_KC - 1) / TS_KC;
            for (int i = 0; i < nsub; i++, g++) {
                const int s = (int)(g % TS_BSTAGES);
                const uint32_t ph = (uint32_t)((g / TS_BSTAGES) & 1) ^ 1u;
                if (!mbar_wait(&bempty[s], ph)) { atomicCAS(err, 0, 12); ok = false; break; }
                uint8_t *st = smem + TS_B_OFF + s * TS_BSTAGE_BYTES;
                mbar_expect_tx(&bfull[s], 2 * TS_B_BYTES);
                const int x = 2 * (k0 + i * TS_KC);   // real column, a multiple of 32
                tma_load_2d(st, mp + 0, x, 0, &bfull[s]);
                tma_load_2d(st + TS_B_BYTES, mp + 1, x, 0, &bfull[s]);
            }
        }
        for (int s = 0; s < TS_BSTAGES; s++) {
            if (g <= s) continue;
            const long long last = g - 1 - ((g - 1 - s) % TS_BSTAGES);
            mbar_wait(&bfull[s], (uint32_t)((last / TS_BSTAGES) & 1));
        }
    } else if (TMA && warp == TS_WA && lane == 0) {
        // ---------------- raw A producer (TMA variant) ----------------
        uint8_t *rawb = smem + TS_RAW_OFF;
        long long g = 0;
        bool ok = true;
        for (long long u = blockIdx.x; u < nunits && ok; u += gridDim.x) {
            int m0, k0, k1;
            const TsTask *t = ts_unit(tasks, ntasks, u, m0, k0, k1);
            const CUtensorMap *mp = maps + t->map0 + 2;
            const int nsub = (k1 - k0 + TS_KC - 1) / TS_KC;
            for (int i = 0; i < nsub; i++, g++) {
                const int slot = (int)(g % TS_RAW);
                if (!mbar_wait(&rempty[slot], (uint32_t)((g / TS_RAW) & 1) ^ 1u)) { atomicCAS(err, 0, 17); ok = false; break; }
                mbar_expect_tx(&rfull[slot], TS_RAW_BYTES);
                // x: real column, a multiple of 32 floats (128 bytes); rows past M and columns
                // past K read as zeros
                tma_load_2d(rawb + slot * TS_RAW_BYTES, mp, 2 * (k0 + i * TS_KC), m0, &rfull[slot]);
            }
        }
        for (int s = 0; s < TS_RAW; s++) {
            if (g <= s) continue;
            const long long last = g - 1 - ((g - 1 - s) % TS_RAW);
            mbar_wait(&rfull[s], (uint32_t)((last / TS_RAW) & 1));
        }
    } else if (warp == TS_WM && lane == 0) {
        // ---------------- MMA issuer ----------------
        constexpr uint32_t idesc = tf32_idesc(TS_BM, TS_NR);
        long long g = 0;
        int it = 0;
        bool ok = true;
        for (long long u = blockIdx.x; u < nunits && ok; u += gridDim.x, it++) {
            int m0, k0, k1;
            ts_unit(tasks, ntasks, u, m0, k0, k1);
            const int nsub = (k1 - k0 + TS_KC - 1) / TS_KC;
            const int b = it & 1;
            const uint32_t use = (uint32_t)(it >> 1);
            if (!mbar_wait(&tempty[b], (use & 1u) ^ 1u)) { atomicCAS(err, 0, 14); ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t dacc = tmem + (uint32_t)(b * TS_NR);
            for (int i = 0; i < nsub; i++, g++) {
                const int s = (int)(g % TS_STAGES), sb = (int)(g % TS_BSTAGES);
                if (!mbar_wait(&full[s], (uint32_t)((g / TS_STAGES) & 1)) ||
                    !mbar_wait(&bfull[sb], (uint32_t)((g / TS_BSTAGES) & 1))) {
                    atomicCAS(err, 0, 13);
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t a_hi = smem_u32(smem + s * TS_ASTAGE_BYTES), a_lo = a_hi + TS_A_BYTES;
                const uint32_t b_hi = smem_u32(smem + TS_B_OFF + sb * TS_BSTAGE_BYTES), b_lo = b_hi + TS_B_BYTES;
#pragma unroll
                for (int kk = 0; kk < 4; kk++) {
                    const uint32_t off = kk * 32;   // 8 TF32 values along K
                    const uint64_t dah = sw128_desc(a_hi + off), dal = sw128_desc(a_lo + off);
                    const uint64_t dbh = sw128_desc(b_hi + off), dbl = sw128_desc(b_lo + off);
                    umma_tf32(dacc, dah, dbh, idesc, (i | kk) != 0);
                    umma_tf32(dacc, dah, dbl, idesc, 1);
                    umma_tf32(dacc, dal, dbh, idesc, 1);
                }
                umma_commit(&empty[s]);
                umma_commit(&bempty[sb]);
            }
            if (!ok) break;
            umma_commit(&tfull[b]);
        }
        umma_commit(drain);
        mbar_wait(drain, 0);
    } else if (warp >= TS_WE) {
        // ---------------- epilogue: C -= D ----------------
        // lane l of warp w owns accumulator row 32 (w mod 4) + l: its 32
        // complex values are one contiguous 256-byte row of C
        const int q = warp & 3;
        int it = 0;
        for (long long u = blockIdx.x; u < nunits; u += gridDim.x, it++) {
            int m0, k0, k1;
            const TsTask *t = ts_unit(tasks, ntasks, u, m0, k0, k1);
            const int b = it & 1;
            const uint32_t use = (uint32_t)(it >> 1);
            if (!mbar_wait(&tfull[b], use & 1u)) { atomicCAS(err, 0, 15); break; }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * TS_NR);
            const int r = m0 + 32 * q + lane;
            cx<float> *crow = nullptr;
            if (r < t->M) crow = t->C + (long long)(t->crow ? t->crow[r] : r) * t->ldc;
#pragma unroll 1
            for (int h = 0; h < 2; h++) {
                uint32_t v[32];
                TMEM_LD32(taddr + h * 32, v);
                asm volatile("tcgen05.wait::ld.sync.aligned;");
                if (crow) {
                    const int c0 = 16 * h, nc = min(16, t->N - c0);
                    cx<float> *p = crow + c0;
                    if (t->atom) {
#pragma unroll
                        for (int c = 0; c < 16; c++)
                            if (c < nc) {
                                atomicAdd(&p[c].re, -__uint_as_float(v[2 * c]));
                                atomicAdd(&p[c].im, -__uint_as_float(v[2 * c + 1]));
                            }
                    } else {
#pragma unroll
                        for (int g8 = 0; g8 < 16; g8 += 8) {   // 8 loads in flight per group
                            cx<float> cv[8];
#pragma unroll
                            for (int c = 0; c < 8; c++)
                                if (g8 + c < nc) cv[c] = p[g8 + c];
#pragma unroll
                            for (int c = 0; c < 8; c++)
                                if (g8 + c < nc)
                                    p[g8 + c] = cx<float>(cv[c].re - __uint_as_float(v[2 * (g8 + c)]),
                                                          cv[c].im - __uint_as_float(v[2 * (g8 + c) + 1]));
                        }
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[b]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == TS_WB) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TS_NR));
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int ts_sms()
{
    static const int n = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 1;
    }();
    return n;
}

bool ts_eligible(const GemmTask<float> &g)
{
    // large factor blocks of the substitution passes, as stored or conjugate-
    // transposed (adjoint passes)
    return g.N <= 32 && g.M >= TS_BM && g.K >= 256;
}

bool ts_tma_ok(const GemmTask<float> &g)
{
    // TMA needs a 16-byte-aligned start and a row stride that is a multiple of 16 bytes
    return !g.conjA && ((uintptr_t)g.A % 16) == 0 && (g.lda % 2) == 0;
}

static long long ts_kr(int K) { return align_up(2LL * K, 64); }   // whole 32-complex tiles of B~

long long ts_workspace_floats(const GemmTask<float> *g, int n)
{
    long long w = 0;
    for (int i = 0; i < n; i++) w += 2LL * TS_NR * ts_kr(g[i].K);
    return w;
}

int ts_build_launch(TsLaunch &L, const GemmTask<float> *g, int n, float *ws, bool tma)
{
    std::vector<TsTask> tasks(n);
    std::vector<CUtensorMap> maps(3 * n);
    memset(maps.data(), 0, maps.size() * sizeof(CUtensorMap));
    // K-chunk so that the launch has about four units per resident CTA
    double work = 0;
    for (int i = 0; i < n; i++) work += (double)((g[i].M + TS_BM - 1) / TS_BM) * g[i].K;
    const long long slots = ts_sms();   // one CTA per SM
    const int kchunk = (int)std::max<long long>(256, align_up((long long)std::ceil(work / (4.0 * slots)), TS_KC));
    long long off = 0, units = 0, bw = 0;
    for (int i = 0; i < n; i++) {
        TsTask &t = tasks[i];
        t.A = g[i].A; t.lda = g[i].lda;
        t.B = g[i].B; t.ldb = g[i].ldb; t.brow = g[i].brow;
        t.C = g[i].C; t.ldc = g[i].ldc; t.crow = g[i].crow;
        t.conjA = g[i].conjA;
        t.M = g[i].M; t.N = g[i].N; t.K = g[i].K;
        t.Kr = (int)ts_kr(t.K);
        t.kchunk = kchunk;
        t.nkc = (t.K + kchunk - 1) / kchunk;
        t.atom = (t.crow || t.nkc > 1 || g[i].atom) ? 1 : 0;
        t.bhi = ws + off; off += (long long)TS_NR * t.Kr;
        t.blo = ws + off; off += (long long)TS_NR * t.Kr;
        t.unit0 = units;
        units += (long long)((t.M + TS_BM - 1) / TS_BM) * t.nkc;
        t.b_work0 = bw;
        bw += t.Kr / 64;
        t.map0 = 3 * i;
        int rc;
        if ((rc = make_map(&maps[3 * i], t.bhi, TS_NR, t.Kr, TS_NR)) ||
            (rc = make_map(&maps[3 * i + 1], t.blo, TS_NR, t.Kr, TS_NR)))
            return rc;
        if (tma) {
            if (!ts_tma_ok(g[i])) { set_error("ts_build_launch: task not addressable by TMA"); return WT3D_ERR_ARG; }
            if ((rc = make_map_plain(&maps[3 * i + 2], reinterpret_cast<const float *>(t.A), t.M, 2LL * t.K,
                                     8LL * t.lda, TS_BM)))
                return rc;
        }
    }
    L.tma = tma;
    L.ntasks = n;
    L.units = units;
    L.b_tiles = bw;
    int rc;
    if ((rc = L.tasks.upload(tasks))) return rc;
    std::vector<unsigned char> raw(maps.size() * sizeof(CUtensorMap));
    memcpy(raw.data(), maps.data(), raw.size());
    if ((rc = L.maps.upload(raw))) return rc;
    return WT3D_OK;
}

void ts_expand(const TsLaunch &L, cudaStream_t st)
{
    if (L.ntasks == 0) return;
    k_ts_expand_b<<<(unsigned)L.b_tiles, 256, 0, st>>>(L.tasks.p, L.ntasks, L.b_tiles);
}

void ts_mma(const TsLaunch &L, int *err, cudaStream_t st)
{
    if (L.ntasks == 0) return;
    const long long grid = std::min<long long>(L.units, ts_sms());
    const CUtensorMap *maps = reinterpret_cast<const CUtensorMap *>(L.maps.p);
    if (L.tma) k_tc_ts<true><<<(unsigned)grid, TS_THREADS, TS_SMEM, st>>>(L.tasks.p, L.ntasks, L.units, maps, err);
    else k_tc_ts<false><<<(unsigned)grid, TS_THREADS, TS_SMEM, st>>>(L.tasks.p, L.ntasks, L.units, maps, err);
}

int ts_init()
{
    WT_CUDA(cudaFuncSetAttribute(k_tc_ts<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, TS_SMEM));
    WT_CUDA(cudaFuncSetAttribute(k_tc_ts<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, TS_SMEM));
    if (!encode_fn()) { set_error("cuTensorMapEncodeTiled unavailable"); return WT3D_ERR_CUDA; }
    return WT3D_OK;
}

}  // namespace wt3d
