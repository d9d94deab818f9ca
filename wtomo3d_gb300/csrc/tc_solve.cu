// Tall-skinny complex64 GEMM  C -= A B  on the tcgen05 tensor cores, for the
// substitution passes of the solve: A is a factor block (M x K, K-major rows
// in the front storage, any leading dimension) or, in the adjoint passes, the
// conjugate transpose of one, and B and C hold at most 32 right-hand sides.
// Each factor entry is used for 32 complex multiply-adds only, so the kernel
// is meant to run at the speed of reading A from HBM.
//
// A is not copied or pre-split.  It is streamed into a ring of TS_RAW raw
// stages in shared memory (128 rows x 16 complex k, 16 KB, in the 128-byte
// swizzle): by TMA when the task's block is 16-byte aligned with an even row
// stride, otherwise by 8-byte asynchronous copies of the loader warps (one
// 128-byte row segment per half-warp, or 32 consecutive stored entries per
// warp for the conjugate transpose).  The loader warps then split every value
// into TF32 hi + lo (x = hi + lo to ~2^-24) and store both halves into tensor
// memory: the MMA takes A from TMEM (row i of the tile in lane i), so the
// split operand never goes through shared memory, whose bandwidth bounded the
// kernel when it did.  B is expanded once per launch into the 64 x 2K real
// matrix B~ (rows 2j, 2j+1 of column j, as in the square tensor-core GEMM),
// split into hi and lo, and fetched by TMA.  The complex product is the real
// product A_r B~^T into a 128 x 64 FP32 TMEM accumulator with
// D = Ahi Bhi + Ahi Blo + Alo Bhi.
//
// Work unit = (task, 128-row tile, K-chunk); persistent CTAs, one per SM.
// Warps 0-15 convert A (warp w: TMEM lanes 32 (w mod 4) .., complex k
// 4 (w / 4) .. of each stage) and, in the copy variant, copy it; warp 16
// issues the TMA copies of B~ and owns the TMEM allocation; warp 17 (one lane)
// issues the MMAs; warp 18 streams A by TMA in the aligned variant; warps
// 19-22 drain the double-buffered accumulator: C -= D in place, or with
// atomics when the task is split along K or its rows are scattered (border
// updates).  Every mbarrier wait is bounded; on expiry the kernel records an
// error code and winds down as the square kernel does.
#include "tc_gemm.h"
#include "tc_ptx.cuh"
#include <cstring>

namespace wt3d {

constexpr int TS_BM = 128;                        // complex rows per tile (MMA M, TMEM lanes)
constexpr int TS_NR = 64;                         // real accumulator columns: 32 complex (MMA N)
constexpr int TS_KC = 16;                         // complex k per stage: one 128-byte swizzle row
constexpr int TS_TSTAGES = 4;                     // split A stages in TMEM (hi + lo: 64 columns each)
constexpr int TS_BSTAGES = 2;                     // B~ stages (TMA from L2)
constexpr int TS_B_BYTES = TS_NR * 128;           // 8 KB per split half
constexpr int TS_BSTAGE_BYTES = 2 * TS_B_BYTES;
constexpr int TS_RAW = 10;                        // raw A stages in flight
constexpr int TS_RAW_BYTES = TS_BM * TS_KC * 8;   // 16 KB
constexpr int TS_B_OFF = 0;
constexpr int TS_RAW_OFF = TS_B_OFF + TS_BSTAGES * TS_BSTAGE_BYTES;
constexpr int TS_BAR_OFF = TS_RAW_OFF + TS_RAW * TS_RAW_BYTES;
constexpr int TS_SMEM = TS_BAR_OFF + 1024 + 512;
constexpr int TS_ACC_COLS = 2 * TS_NR;            // TMEM columns of the two accumulators
constexpr int TS_TMEM_COLS = 512;                 // accumulators + TS_TSTAGES x 64 (power of two)
static_assert(TS_ACC_COLS + TS_TSTAGES * 64 <= TS_TMEM_COLS, "TMEM budget");
constexpr int TS_LOADERS = 16;                    // loader warps
constexpr int TS_WB = TS_LOADERS, TS_WM = TS_LOADERS + 1, TS_WA = TS_LOADERS + 2, TS_WE = TS_LOADERS + 3;
constexpr int TS_THREADS = (TS_LOADERS + 7) * 32; // + B producer, MMA, A producer (TMA variant), 4 epilogue warps
constexpr int TS_LT = TS_LOADERS * 32;            // loader threads
constexpr int TS_PER_THREAD = TS_BM * TS_KC / TS_LT;   // complex elements a loader thread copies per stage
constexpr int TS_QROWS = TS_LT / TS_KC;           // rows between a thread's copied elements
static_assert(TS_PER_THREAD * TS_LT == TS_BM * TS_KC && TS_QROWS % 8 == 0, "loader mapping");
static_assert((TS_LT / TS_BM) * TS_PER_THREAD == TS_KC, "conjugate-transposed loader mapping");
static_assert(TS_LOADERS == 16, "conversion mapping: 4 lane quarters x 4 k parts");

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

// byte offset of element (row r, complex column k) of a raw stage in the
// 128-byte swizzle: 16-byte chunk c of row r sits at chunk c ^ (r mod 8)
__device__ __forceinline__ int ts_swz(int r, int k)
{
    return r * 128 + ((((k >> 1) ^ (r & 7))) << 4) + ((k & 1) << 3);
}

// Position in the CTA's sequence of stages: unit u (every gridDim.x-th unit
// from blockIdx.x), its K range and stage i within it.
struct TsStage {
    const TsTask *t;
    long long u;
    int m0, k0, k1, nsub, i;
    int M;       // the task's row count and conjugation, kept in registers
    bool conj;
    bool valid;
};

__device__ __forceinline__ void ts_stage_at(TsStage &c, const TsTask *__restrict__ tasks, int ntasks, long long nunits,
                                            long long u)
{
    c.u = u;
    c.valid = u < nunits;
    if (!c.valid) return;
    c.t = ts_unit(tasks, ntasks, u, c.m0, c.k0, c.k1);
    c.nsub = (c.k1 - c.k0 + TS_KC - 1) / TS_KC;
    c.i = 0;
    c.M = c.t->M;
    c.conj = c.t->conjA != 0;
}

__device__ __forceinline__ void ts_stage_next(TsStage &c, const TsTask *__restrict__ tasks, int ntasks,
                                              long long nunits)
{
    if (++c.i == c.nsub) ts_stage_at(c, tasks, ntasks, nunits, c.u + gridDim.x);
}

// The loader thread l's asynchronous 8-byte copies of one stage into the
// swizzled raw slot at shared address raw:
//   A as stored (row-major, K-major): row TS_QROWS q + l / 16, column l % 16 -
//     a half-warp reads one contiguous 128-byte row segment;
//   A^H (conjugate transpose of a stored K x M block): row l % 128, column
//     l / 128 + 4 q - a warp reads 32 consecutive stored entries of one
//     stored row.
// Elements outside the operand are not copied; the conversion zeroes them.
__device__ __forceinline__ void ts_copy(const TsStage &c, int l, uint32_t raw)
{
    const TsTask *t = c.t;
    const int kb = c.k0 + c.i * TS_KC;
    const int M = t->M;
    const long long lda = t->lda;
    if (!t->conjA) {
        const int kc = l & 15, k = kb + kc;
        if (k >= c.k1) return;
#pragma unroll
        for (int q = 0; q < TS_PER_THREAD; q++) {
            const int r = TS_QROWS * q + (l >> 4);
            if (c.m0 + r < M)
                asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(raw + (uint32_t)ts_swz(r, kc)),
                             "l"(t->A + (long long)(c.m0 + r) * lda + k)
                             : "memory");
        }
    } else {
        const int r = l & (TS_BM - 1);
        if (c.m0 + r >= M) return;
#pragma unroll
        for (int q = 0; q < TS_PER_THREAD; q++) {
            const int kc = (l / TS_BM) + (TS_LT / TS_BM) * q, k = kb + kc;
            if (k < c.k1)
                asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(raw + (uint32_t)ts_swz(r, kc)),
                             "l"(t->A + (long long)k * lda + c.m0 + r)
                             : "memory");
        }
    }
}

// hi = TF32 rounding of x (to nearest, ties away from zero), lo = the same
// rounding of x - hi (exact in FP32), so x = hi + lo to ~2^-22 |x|.  The
// rounding is done on the bit pattern (add half a TF32 unit to the magnitude,
// clear the 13 low bits) on the integer pipe; finite inputs only.
__device__ __forceinline__ uint32_t rna_tf32_bits(uint32_t u) { return (u + 0x1000u) & 0xFFFFE000u; }
__device__ __forceinline__ void split_cvt(float x, uint32_t &hi, uint32_t &lo)
{
    hi = rna_tf32_bits(__float_as_uint(x));
    lo = rna_tf32_bits(__float_as_uint(x - __uint_as_float(hi)));
}

// The loader thread's part of a stage: tile row r = 32 (w mod 4) + lane,
// complex k 4 (w / 4) .. + 3, read from the raw slot, split and stored into
// TMEM columns col_hi + 0..7 (hi) and col_hi + 32 + 0..7 (lo) of the thread's
// lane.  COPY (the cp.async variant): the raw slot holds stale values outside
// the operand, which are zeroed, and A^H is conjugated.  The TMA variant needs
// neither: TMA fills outside the tensor with zeros and serves only blocks as
// stored.
template <bool COPY>
__device__ __forceinline__ void ts_convert(const TsStage &c, const uint8_t *rs, uint32_t tmem_lane, int col_hi,
                                           int r, int kpart)
{
    float4 a = *reinterpret_cast<const float4 *>(rs + r * 128 + (((2 * kpart) ^ (r & 7)) << 4));
    float4 b = *reinterpret_cast<const float4 *>(rs + r * 128 + (((2 * kpart + 1) ^ (r & 7)) << 4));
    if constexpr (COPY) {
        const int kbase = c.k0 + c.i * TS_KC + 4 * kpart;
        if (c.m0 + r >= c.M || kbase + 3 >= c.k1) {   // the operand's last rows or columns
            const bool rv = c.m0 + r < c.M;
            const bool k0v = rv && kbase < c.k1, k1v = rv && kbase + 1 < c.k1, k2v = rv && kbase + 2 < c.k1,
                       k3v = rv && kbase + 3 < c.k1;
            a = make_float4(k0v ? a.x : 0.f, k0v ? a.y : 0.f, k1v ? a.z : 0.f, k1v ? a.w : 0.f);
            b = make_float4(k2v ? b.x : 0.f, k2v ? b.y : 0.f, k3v ? b.z : 0.f, k3v ? b.w : 0.f);
        }
        if (c.conj) {
            a.y = -a.y; a.w = -a.w; b.y = -b.y; b.w = -b.w;
        }
    }
    uint32_t h[8], lw[8];
    split_cvt(a.x, h[0], lw[0]); split_cvt(a.y, h[1], lw[1]); split_cvt(a.z, h[2], lw[2]); split_cvt(a.w, h[3], lw[3]);
    split_cvt(b.x, h[4], lw[4]); split_cvt(b.y, h[5], lw[5]); split_cvt(b.z, h[6], lw[6]); split_cvt(b.w, h[7], lw[7]);
    const uint32_t th = tmem_lane + (uint32_t)col_hi, tl = th + 32;
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(th),
                 "r"(h[0]), "r"(h[1]), "r"(h[2]), "r"(h[3]), "r"(h[4]), "r"(h[5]), "r"(h[6]), "r"(h[7])
                 : "memory");
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(tl),
                 "r"(lw[0]), "r"(lw[1]), "r"(lw[2]), "r"(lw[3]), "r"(lw[4]), "r"(lw[5]), "r"(lw[6]), "r"(lw[7])
                 : "memory");
}

// D (+)= A B with A in tensor memory (kind::tf32, M = 128: row i in lane i)
__device__ __forceinline__ void umma_tf32_ta(uint32_t tmem_d, uint32_t tmem_a, uint64_t db, uint32_t idesc,
                                             uint32_t acc)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(tmem_d),
        "r"(tmem_a), "l"(db), "r"(idesc), "r"(acc));
}

// TMA = false: the loader warps copy A with cp.async (any alignment, as
// stored or conjugate-transposed).  TMA = true: every task's A is 16-byte
// aligned with an even row stride, as stored; warp TS_WA streams the raw
// 128 x 16 complex tiles by TMA.
template <bool TMA>
__global__ void __launch_bounds__(TS_THREADS, 1)
    k_tc_ts(const TsTask *__restrict__ tasks, int ntasks, long long nunits, const CUtensorMap *__restrict__ maps,
            int *err)
{
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + TS_BAR_OFF);   // TMEM A stage written (16 loader warps)
    uint64_t *empty = full + TS_TSTAGES;                                 // TMEM A stage consumed (MMA commit)
    uint64_t *bfull = empty + TS_TSTAGES;                                // B~ stage landed (TMA)
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
                     "r"(TS_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == TS_WM * 32) {
        for (int s = 0; s < TS_TSTAGES; s++) {
            mbar_init(&full[s], TMA ? TS_LOADERS / 2 : TS_LOADERS);   // the warps that convert a stage
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
            mbar_init(&rempty[s], TS_LOADERS / 2);
        }
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_holder;

    if (warp < TS_LOADERS) {
        // ---------------- A loaders: (copy) -> raw ring -> split -> TMEM ----------------
        // The copy cursor runs TS_RAW - 1 stages ahead of the conversion
        // cursor, across unit boundaries; one commit group per stage (empty
        // groups past the end keep the count uniform).  In the copy variant
        // the loaders read each other's copies, so every stage passes one
        // named barrier of the 512 loader threads; a loader whose wait timed
        // out keeps looping (without converting) so that none is left at it.
        // TMA variant: warps 0-7 convert the even stages and warps 8-15 the
        // odd ones, each thread two k parts of its row, so that two stages
        // are converted at once (one warp's stage is a chain of waits, shared
        // loads, the split, TMEM stores and their completion).  Copy variant:
        // all 16 warps every stage (they also copy it), one k part each.
        const int l = threadIdx.x;
        constexpr int NG = TMA ? 2 : 1, NKP = TMA ? 2 : 1;
        const int r = 32 * (warp & 3) + lane;
        const int kpa = TMA ? 2 * ((warp >> 2) & 1) : warp >> 2;   // first k part
        const uint32_t tlane = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
        uint8_t *rawb = smem + TS_RAW_OFF;
        const uint32_t raw0 = smem_u32(rawb);
        TsStage cp, cs;
        ts_stage_at(cs, tasks, ntasks, nunits, blockIdx.x);
        long long g = 0;
        if (TMA && (warp >> 3) == 1 && cs.valid) {   // the odd stages
            ts_stage_next(cs, tasks, ntasks, nunits);
            g = 1;
        }
        bool ok = true;
        if constexpr (!TMA) {
            ts_stage_at(cp, tasks, ntasks, nunits, blockIdx.x);
            for (int p = 0; p < TS_RAW - 1; p++) {
                if (cp.valid) {
                    ts_copy(cp, l, raw0 + (uint32_t)(p * TS_RAW_BYTES));
                    ts_stage_next(cp, tasks, ntasks, nunits);
                }
                asm volatile("cp.async.commit_group;" ::: "memory");
            }
        }
        while (cs.valid) {
            const int slot = (int)(g % TS_RAW);
            if constexpr (!TMA) {
                asm volatile("cp.async.wait_group %0;" ::"n"(TS_RAW - 2) : "memory");   // own copies of stage g
                asm volatile("bar.sync 1, %0;" ::"n"(TS_LT) : "memory");                // everyone's; slot g-1 free
                if (cp.valid) {
                    ts_copy(cp, l, raw0 + (uint32_t)(((g + TS_RAW - 1) % TS_RAW) * TS_RAW_BYTES));
                    ts_stage_next(cp, tasks, ntasks, nunits);
                }
                asm volatile("cp.async.commit_group;" ::: "memory");
            } else {
                if (ok && !mbar_wait(&rfull[slot], (uint32_t)((g / TS_RAW) & 1))) { atomicCAS(err, 0, 16); ok = false; }
            }
            const int s = (int)(g % TS_TSTAGES);
            if (ok && !mbar_wait(&empty[s], (uint32_t)((g / TS_TSTAGES) & 1) ^ 1u)) { atomicCAS(err, 0, 11); ok = false; }
            ok = __all_sync(0xffffffffu, ok);   // the tcgen05 stores below are warp-collective
            if (ok) {
                asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
                for (int kk = 0; kk < NKP; kk++)
                    ts_convert<!TMA>(cs, rawb + slot * TS_RAW_BYTES, tlane, TS_ACC_COLS + 64 * s + 8 * (kpa + kk), r,
                                     kpa + kk);
                asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                asm volatile("tcgen05.fence::before_thread_sync;");
            }
            __syncwarp();
            if (ok && lane == 0) {
                mbar_arrive(&full[s]);
                if constexpr (TMA) mbar_arrive(&rempty[slot]);
            }
            if (TMA && !ok) break;
#pragma unroll
            for (int i = 0; i < NG; i++) {
                ts_stage_next(cs, tasks, ntasks, nunits);
                g++;
                if (!cs.valid) break;
            }
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
                const int s = (int)(g % TS_TSTAGES), sb = (int)(g % TS_BSTAGES);
                if (!mbar_wait(&full[s], (uint32_t)((g / TS_TSTAGES) & 1)) ||
                    !mbar_wait(&bfull[sb], (uint32_t)((g / TS_BSTAGES) & 1))) {
                    atomicCAS(err, 0, 13);
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t a_hi = tmem + (uint32_t)(TS_ACC_COLS + 64 * s), a_lo = a_hi + 32;
                const uint32_t b_hi = smem_u32(smem + TS_B_OFF + sb * TS_BSTAGE_BYTES), b_lo = b_hi + TS_B_BYTES;
#pragma unroll
                for (int kk = 0; kk < 4; kk++) {   // 8 TF32 values along K: 8 TMEM columns, 32 bytes of B~
                    const uint64_t dbh = sw128_desc(b_hi + kk * 32), dbl = sw128_desc(b_lo + kk * 32);
                    umma_tf32_ta(dacc, a_hi + 8 * kk, dbh, idesc, (i | kk) != 0);
                    umma_tf32_ta(dacc, a_hi + 8 * kk, dbl, idesc, 1);
                    umma_tf32_ta(dacc, a_lo + 8 * kk, dbh, idesc, 1);
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
            const bool got = mbar_wait(&tfull[b], use & 1u);
            if (!__all_sync(0xffffffffu, got)) { atomicCAS(err, 0, 15); break; }   // warp-uniform: tcgen05.ld below
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
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TS_TMEM_COLS));
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
                                     8LL * t.lda, TS_BM, true)))
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
