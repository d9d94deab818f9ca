// Complex64 GEMM  C -= A * B  on the 5th-generation tensor cores (tcgen05) of
// sm_103a, accurate to FP32 through a three-term TF32 split.
//
// Complex product as one real GEMM: with A stored interleaved (row i =
// [re a_i0, im a_i0, re a_i1, ...], i.e. an M x 2K real matrix, K-major as
// stored) and B expanded to the 2N x 2K K-major real matrix
//     row 2j   = [ re b_0j, -im b_0j,  re b_1j, -im b_1j, ...]
//     row 2j+1 = [ im b_0j,  re b_0j,  im b_1j,  re b_1j, ...]
// the real product A_r * B~^T is the interleaved complex C (8 real flops per
// complex multiply-add, nothing wasted).
//
// Precision: each operand x is split as hi = rn_tf32(x), lo = rn_tf32(x - hi),
// both exact TF32 values with x = hi + lo to ~2^-24 relative;
// D = Ahi Bhi + Ahi Blo + Alo Bhi in an FP32 TMEM accumulator gives an
// FP32-class product (the dropped Alo Blo term is ~2^-24 relative).
//
// f16 mode (the default; WT3D_TC_F16=0 selects the TF32 split): every row of A
// and every complex column of B is multiplied by a power of two s that puts its
// largest |re|, |im| in [2^13, 2^14), and the scaled values are split as
// hi = rn_f16(x s), lo = rn_f16(x s - hi).  Entries within 2^16 of their row's
// (column's) largest keep 22 bits, like the TF32 split; smaller ones lose
// relative precision but stay far below the product's normwise rounding.  The
// same three products run as kind::f16 MMAs, at twice the TF32 rate and with
// half the operand bytes per K step; the epilogue multiplies each accumulator
// entry by 1/(s_row s_col) (exact: powers of two).
//
// Kernel structure (one 128 x 128-complex output tile per CTA, 10 warps):
//   warp 0      TMA producer (cp.async.bulk.tensor, SWIZZLE_128B tiles) and
//               TMEM allocator;
//   warp 1      single-thread tcgen05.mma issuer (kind::f16 or kind::tf32,
//               M=128, N=256), tcgen05.commit releases smem stages and
//               signals the epilogue;
//   warps 2..9  epilogue (two warps per TMEM lane quarter, half of the
//               columns each): tcgen05.ld of the 128 x 256 FP32 accumulator,
//               staged through shared memory, C -= D with coalesced 128-byte
//               warp accesses.
// Every mbarrier wait has an iteration limit; on expiry the kernel records an
// error code, skips ahead, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>
#include "tc_gemm.h"
#include "tc_ptx.cuh"
#include <atomic>
#include <cstring>

namespace wt3d {

constexpr int TC_BM = 128;                 // complex rows per tile
constexpr int TC_BNR = 256;                // real columns per tile (128 complex)
constexpr int TC_BK = 32;                  // real k per stage (128 bytes of FP32)
constexpr int TC_STAGES = 2;
constexpr int TC_A_BYTES = TC_BM * TC_BK * 4;     // 16 KB
constexpr int TC_B_BYTES = TC_BNR * TC_BK * 4;    // 32 KB
constexpr int TC_STAGE_BYTES = 2 * TC_A_BYTES + 2 * TC_B_BYTES;
constexpr int TC_EPI_WARPS = 8;            // two per TMEM lane quarter, each half of the columns
constexpr int TC_EPI_BYTES = TC_EPI_WARPS * 32 * 33 * 4;   // per epilogue warp a 32 x 33 float transpose buffer
constexpr int TC_SMEM = TC_STAGES * TC_STAGE_BYTES + 1024 + 256 + TC_EPI_BYTES;
static_assert(TC_SMEM <= 232448, "shared memory per CTA");
constexpr int TC_THREADS = 64 + 32 * TC_EPI_WARPS;
constexpr int TC_GROUP = 8;                 // column panels per rasterisation group

// ---------------------------------------------------------------------------
// operand split / expansion pre-pass
// ---------------------------------------------------------------------------
// Task of work item q, with tasks[i].*w the first item of task i (increasing):
// one binary search per block, by thread 0 for the block's first item, then
// each thread steps over the few task boundaries inside its block.  (A
// binary search per thread costs a chain of ~log2(ntasks) dependent loads.)
// Every thread of the block must call this.
__device__ __forceinline__ int block_task(const TcTask *__restrict__ tasks, int ntasks, long long q_first, long long q,
                                          long long TcTask::*w)
{
    __shared__ int s_t;
    if (threadIdx.x == 0) {
        int lo_t = 0, hi_t = ntasks - 1;
        while (lo_t < hi_t) {
            const int mid = (lo_t + hi_t + 1) >> 1;
            if (tasks[mid].*w <= q_first) lo_t = mid;
            else hi_t = mid - 1;
        }
        s_t = lo_t;
    }
    __syncthreads();
    int t = s_t;
    while (t + 1 < ntasks && tasks[t + 1].*w <= q) t++;
    return t;
}

// One thread per (row, complex k) of A: Ahi/Alo rows of Kr floats.
__global__ void k_split_a(const TcTask *__restrict__ tasks, int ntasks, long long total)
{
    const long long q0 = (long long)blockIdx.x * blockDim.x;
    long long q = q0 + threadIdx.x;
    const int ti = block_task(tasks, ntasks, q0, q < total ? q : total - 1, &TcTask::a_work0);
    if (q >= total) return;
    const TcTask &t = tasks[ti];
    const long long r = q - t.a_work0;
    const int kc = t.Kr / 2;
    const int i = (int)(r / kc), k = (int)(r % kc);
    cx<float> v(0.f, 0.f);
    if (k < t.K) v = t.A[(long long)i * t.lda + k];
    float h0, l0, h1, l1;
    split_tf32(v.re, h0, l0);
    split_tf32(v.im, h1, l1);
    const long long o = (long long)i * t.Kr + 2 * k;
    *reinterpret_cast<float2 *>(t.ahi + o) = make_float2(h0, h1);
    *reinterpret_cast<float2 *>(t.alo + o) = make_float2(l0, l1);
}

// 32 x 32 complex tiles of B (k x j) transposed through shared memory into the
// expanded K-major rows 2j, 2j+1 of B~.
__global__ void __launch_bounds__(256) k_split_b(const TcTask *__restrict__ tasks, int ntasks, long long total_tiles)
{
    __shared__ float2 tile[32][33];
    long long q = blockIdx.x;
    if (q >= total_tiles) return;
    int lo_t = 0, hi_t = ntasks - 1;
    while (lo_t < hi_t) {
        int mid = (lo_t + hi_t + 1) >> 1;
        if (tasks[mid].b_work0 <= q) lo_t = mid;
        else hi_t = mid - 1;
    }
    const TcTask &t = tasks[lo_t];
    const long long r = q - t.b_work0;
    const int kt = t.Kr / 64;                 // 32-complex k tiles
    const int j0 = (int)(r / kt) * 32, k0 = (int)(r % kt) * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
    for (int kk = ty; kk < 32; kk += 8) {
        int k = k0 + kk, j = j0 + tx;
        cx<float> v(0.f, 0.f);
        if (k < t.K && j < t.N) v = t.B[(long long)k * t.ldb + j];
        tile[kk][tx] = make_float2(v.re, v.im);
    }
    __syncthreads();
    for (int jj = ty; jj < 32; jj += 8) {
        const int j = j0 + jj;
        if (j >= t.N) continue;
        const float2 bt = tile[tx][jj];
        const cx<float> b(bt.x, bt.y);
        const int k = k0 + tx;
        float rh, rl, ih, il, nih, nil;
        split_tf32(b.re, rh, rl);
        split_tf32(b.im, ih, il);
        split_tf32(-b.im, nih, nil);
        const long long o0 = (long long)(2 * j) * t.Kr + 2 * k, o1 = o0 + t.Kr;
        *reinterpret_cast<float2 *>(t.bhi + o0) = make_float2(rh, nih);
        *reinterpret_cast<float2 *>(t.blo + o0) = make_float2(rl, nil);
        *reinterpret_cast<float2 *>(t.bhi + o1) = make_float2(ih, rh);
        *reinterpret_cast<float2 *>(t.blo + o1) = make_float2(il, rl);
    }
}

// ---- f16 mode ---------------------------------------------------------------
// Power of two that maps a largest magnitude m into [2^13, 2^14) (1 for m = 0,
// and for a non-finite m, whose NaN then propagates as with TF32).
__device__ __forceinline__ float f16_scale(unsigned mbits)
{
    const float m = __uint_as_float(mbits);
    if (!(m > 0.f) || !(m < INFINITY)) return 1.f;
    int e;
    frexpf(m, &e);                 // m in [2^(e-1), 2^e)
    return ldexpf(1.f, 14 - e);
}

__device__ __forceinline__ void split_f16(float x, __half &hi, __half &lo)
{
    hi = __float2half_rn(x);
    lo = __float2half_rn(x - __half2float(hi));
}

// Fused forms of the f16 split, one read of each operand from DRAM: a warp
// per row of A reads the row once for its largest magnitude and again (from
// L2) to split it; a block per 32 complex columns of B does the same over the
// column group, transposing 32 x 32 tiles of B through shared memory into the
// expanded K-major rows 2j, 2j+1 of B~.
__global__ void k_split_a_f16_rows(const TcTask *__restrict__ tasks, int ntasks, long long total_rows)
{
    const long long q0 = ((long long)blockIdx.x * blockDim.x) >> 5;
    const long long q = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int ti = block_task(tasks, ntasks, q0, q < total_rows ? q : total_rows - 1, &TcTask::a_row0);
    if (q >= total_rows) return;
    const TcTask &t = tasks[ti];
    const int i = (int)(q - t.a_row0);
    const cx<float> *row = t.A + (long long)i * t.lda;
    float m = 0.f;
    for (int k = lane; k < t.K; k += 32) {
        const cx<float> v = row[k];
        m = fmaxf(m, fmaxf(fabsf(v.re), fabsf(v.im)));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    const float sc = f16_scale(__float_as_uint(m));
    if (lane == 0) t.sa[i] = 1.f / sc;
    __half2 *hi = reinterpret_cast<__half2 *>(t.ahi) + ((long long)i * t.Kr >> 1);
    __half2 *lo = reinterpret_cast<__half2 *>(t.alo) + ((long long)i * t.Kr >> 1);
    const int kc = t.Kr / 2;
    for (int k = lane; k < kc; k += 32) {
        cx<float> v(0.f, 0.f);
        if (k < t.K) v = row[k];
        __half h0, l0, h1, l1;
        split_f16(v.re * sc, h0, l0);
        split_f16(v.im * sc, h1, l1);
        hi[k] = __halves2half2(h0, h1);
        lo[k] = __halves2half2(l0, l1);
    }
}

__global__ void __launch_bounds__(256) k_split_b_f16_cols(const TcTask *__restrict__ tasks, int ntasks,
                                                          long long total_groups)
{
    __shared__ float2 tile[32][33];
    __shared__ float red[8][33];
    const long long q = blockIdx.x;
    const int ti = block_task(tasks, ntasks, q, q, &TcTask::b_col0);
    if (q >= total_groups) return;
    const TcTask &t = tasks[ti];
    const int j0 = (int)(q - t.b_col0) * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
    const int jx = j0 + tx;
    float m = 0.f;
    if (jx < t.N)
        for (int k = ty; k < t.K; k += 8) {
            const cx<float> v = t.B[(long long)k * t.ldb + jx];
            m = fmaxf(m, fmaxf(fabsf(v.re), fabsf(v.im)));
        }
    red[ty][tx] = m;
    __syncthreads();
    if (ty == 0) {
        for (int y = 1; y < 8; y++) m = fmaxf(m, red[y][tx]);
        red[0][tx] = f16_scale(__float_as_uint(m));
        if (jx < t.N) t.sb[jx] = 1.f / red[0][tx];
    }
    __syncthreads();
    __half2 *bh = reinterpret_cast<__half2 *>(t.bhi), *bl = reinterpret_cast<__half2 *>(t.blo);
    for (int k0 = 0; k0 < t.Kr / 2; k0 += 32) {
        for (int kk = ty; kk < 32; kk += 8) {
            const int k = k0 + kk;
            cx<float> v(0.f, 0.f);
            if (k < t.K && jx < t.N) v = t.B[(long long)k * t.ldb + jx];
            tile[kk][tx] = make_float2(v.re, v.im);
        }
        __syncthreads();
        for (int jj = ty; jj < 32; jj += 8) {
            const int j = j0 + jj;
            if (j < t.N) {
                const float sc = red[0][jj];
                const float br = tile[tx][jj].x * sc, bi = tile[tx][jj].y * sc;
                const int k = k0 + tx;
                __half rh, rl, ih, il, nih, nil;
                split_f16(br, rh, rl);
                split_f16(bi, ih, il);
                split_f16(-bi, nih, nil);
                const long long o0 = ((long long)(2 * j) * t.Kr + 2 * k) >> 1, o1 = o0 + (t.Kr >> 1);
                bh[o0] = __halves2half2(rh, nih);
                bl[o0] = __halves2half2(rl, nil);
                bh[o1] = __halves2half2(ih, rh);
                bl[o1] = __halves2half2(il, rl);
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// the tensor-core kernel
// ---------------------------------------------------------------------------
// Tile gt of a launch: its task and the tile's first complex row and real column.
// Grouped rasterisation: consecutive tiles sweep a band of TC_GROUP column
// panels row panel by row panel, so the tiles in flight share a compact set of
// A and B panels in L2.  The expanded B operand (2N x 2K real) is twice the
// size of A, so B is the one kept resident while A panels stream.
__device__ __forceinline__ const TcTask *tc_tile(const TcTask *__restrict__ tasks, int ntasks, long long gt, int &m0,
                                                 int &n0r)
{
    int lo_t = 0, hi_t = ntasks - 1;
    while (lo_t < hi_t) {
        int mid = (lo_t + hi_t + 1) >> 1;
        if (tasks[mid].tile0 <= gt) lo_t = mid;
        else hi_t = mid - 1;
    }
    const TcTask *t = tasks + lo_t;
    const long long lt = gt - t->tile0;
    const int tiles_m = (t->M + TC_BM - 1) / TC_BM;
    const long long per_group = (long long)TC_GROUP * tiles_m;
    const int group = (int)(lt / per_group);
    const int first_n = group * TC_GROUP;
    const int gsize = min(t->tiles_n - first_n, TC_GROUP);
    const int in_group = (int)(lt % per_group);
    n0r = (first_n + in_group % gsize) * TC_BNR;
    m0 = (in_group / gsize) * TC_BM;
    return t;
}

// Persistent: one CTA per SM walks the launch's tiles gt = blockIdx.x,
// blockIdx.x + gridDim.x, ...  Warp 0 (one lane) streams the k-steps of all
// its tiles through the TC_STAGES-deep TMA pipeline; warp 1 (one lane) issues
// the MMAs into one of two TMEM accumulators (256 columns each) and commits
// the finished one; warps 2-5 drain a finished accumulator straight from TMEM
// into C -= D while the MMAs of the next tile run into the other one.  Every
// wait is bounded: a role that times out sets *err and stops, the others then
// time out in turn, and before TMEM is released the MMA lane waits for its
// issued MMAs and the producer for its issued copies.
template <bool F16>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_tc_gemm(const TcTask *__restrict__ tasks, int ntasks, long long ntiles, const CUtensorMap *__restrict__ maps,
              int *err)
{
    // elements of one 128-byte stage row: 32 TF32 or 64 FP16 values
    constexpr int EK = F16 ? 2 * TC_BK : TC_BK;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + TC_STAGES * TC_STAGE_BYTES);
    uint64_t *empty = full + TC_STAGES;
    uint64_t *tfull = empty + TC_STAGES;      // accumulator b written (MMA commit)
    uint64_t *tempty = tfull + 2;             // accumulator b read out (4 epilogue warps)
    uint64_t *drain = tempty + 2;
    uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(drain + 1);
    float *epi = reinterpret_cast<float *>(smem + TC_STAGES * TC_STAGE_BYTES + 256);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                     "r"(2 * TC_BNR));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 32) {
        for (int s = 0; s < TC_STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], TC_EPI_WARPS);
        }
        mbar_init(drain, 1);
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_holder;

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer ----------------
        long long gks = 0;
        bool ok = true;
        for (long long gt = blockIdx.x; gt < ntiles && ok; gt += gridDim.x) {
            int m0, n0r;
            const TcTask *t = tc_tile(tasks, ntasks, gt, m0, n0r);
            const CUtensorMap *mp = maps + t->map0;
            const int nk = t->Kr / EK;
            for (int ks = 0; ks < nk; ks++, gks++) {
                const int s = (int)(gks % TC_STAGES);
                const uint32_t ph = (uint32_t)((gks / TC_STAGES) & 1) ^ 1u;
                if (!mbar_wait(&empty[s], ph)) { atomicCAS(err, 0, 1); ok = false; break; }
                uint8_t *st = smem + s * TC_STAGE_BYTES;
                mbar_expect_tx(&full[s], TC_STAGE_BYTES);
                tma_load_2d(st, mp + 0, ks * EK, m0, &full[s]);
                tma_load_2d(st + TC_A_BYTES, mp + 1, ks * EK, m0, &full[s]);
                tma_load_2d(st + 2 * TC_A_BYTES, mp + 2, ks * EK, n0r, &full[s]);
                tma_load_2d(st + 2 * TC_A_BYTES + TC_B_BYTES, mp + 3, ks * EK, n0r, &full[s]);
            }
        }
        // the last copy issued into each stage has landed before the CTA exits
        for (int s = 0; s < TC_STAGES; s++) {
            if (gks <= s) continue;
            const long long last = gks - 1 - ((gks - 1 - s) % TC_STAGES);
            mbar_wait(&full[s], (uint32_t)((last / TC_STAGES) & 1));
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer ----------------
        constexpr uint32_t idesc = F16 ? f16_idesc(TC_BM, TC_BNR) : tf32_idesc(TC_BM, TC_BNR);
        long long gks = 0;
        int it = 0;
        bool ok = true;
        for (long long gt = blockIdx.x; gt < ntiles && ok; gt += gridDim.x, it++) {
            int m0, n0r;
            const TcTask *t = tc_tile(tasks, ntasks, gt, m0, n0r);
            const int nk = t->Kr / EK;
            const int b = it & 1;
            const uint32_t use = (uint32_t)(it >> 1);
            if (!mbar_wait(&tempty[b], (use & 1u) ^ 1u)) { atomicCAS(err, 0, 4); ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t dacc = tmem + (uint32_t)(b * TC_BNR);
            for (int ks = 0; ks < nk; ks++, gks++) {
                const int s = (int)(gks % TC_STAGES);
                const uint32_t ph = (uint32_t)((gks / TC_STAGES) & 1);
                if (!mbar_wait(&full[s], ph)) { atomicCAS(err, 0, 2); ok = false; break; }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t base = smem_u32(smem + s * TC_STAGE_BYTES);
                const uint32_t a_hi = base, a_lo = base + TC_A_BYTES;
                const uint32_t b_hi = base + 2 * TC_A_BYTES, b_lo = b_hi + TC_B_BYTES;
#pragma unroll
                for (int kk = 0; kk < TC_BK / 8; kk++) {
                    const uint32_t off = kk * 32;   // 32 bytes along K: 8 TF32 or 16 FP16 elements
                    const uint64_t dah = sw128_desc(a_hi + off), dal = sw128_desc(a_lo + off);
                    const uint64_t dbh = sw128_desc(b_hi + off), dbl = sw128_desc(b_lo + off);
                    if constexpr (F16) {
                        umma_f16(dacc, dah, dbh, idesc, (ks | kk) != 0);
                        umma_f16(dacc, dah, dbl, idesc, 1);
                        umma_f16(dacc, dal, dbh, idesc, 1);
                    } else {
                        umma_tf32(dacc, dah, dbh, idesc, (ks | kk) != 0);
                        umma_tf32(dacc, dah, dbl, idesc, 1);
                        umma_tf32(dacc, dal, dbh, idesc, 1);
                    }
                }
                umma_commit(&empty[s]);
            }
            if (!ok) break;
            umma_commit(&tfull[b]);
        }
        // no MMA of this CTA is in flight once the drain barrier completes
        umma_commit(drain);
        mbar_wait(drain, 0);
    } else if (warp >= 2) {
        // ---------------- epilogue ----------------
        // Lane l of warp w reads accumulator row 32 q + l (TMEM lane quarter
        // q = w mod 4) in 32-column chunks; each chunk goes through a 32 x 33
        // transpose buffer so that C is read-modified-written one row segment
        // (32 floats, 128 bytes) per warp instruction.  C does not depend on
        // the accumulator, so the loads of a tile's first two chunks are issued
        // before its MMAs are waited for, and every later chunk's loads one
        // chunk ahead of its stores (64 row segments in flight per warp).
        // Each lane also prefetches its row of the CTA's next C tile into L2
        // (128-byte lines, none outside the row's own span).
        // Warps 2-5 take the first half of the tile's columns (chunks 0-3),
        // warps 6-9 the second; warp w serves TMEM lane quarter w mod 4.
        constexpr int NCH = TC_BNR / 32 / 2;    // chunks per epilogue warp
        const int q = warp & 3, ch0 = NCH * ((warp - 2) >> 2);
        float *tb = epi + (warp - 2) * (32 * 33);
        auto prefetch_c = [&](long long g) {
            if (g >= ntiles) return;
            int pm0, pn0r;
            const TcTask *pt = tc_tile(tasks, ntasks, g, pm0, pn0r);
            const int r = pm0 + 32 * q + lane, c0 = (pn0r >> 1) + 16 * ch0;
            if (r >= pt->M || c0 >= pt->N) return;
            const char *p = reinterpret_cast<const char *>(pt->C + (long long)r * pt->ldc + c0);
            const int nb = 8 * min(16 * NCH, pt->N - c0);
            for (int off = 0; off < nb; off += 128) asm volatile("prefetch.global.L2 [%0];" ::"l"(p + off));
            asm volatile("prefetch.global.L2 [%0];" ::"l"(p + nb - 1));
        };
        prefetch_c(blockIdx.x);
        int it = 0;
        for (long long gt = blockIdx.x; gt < ntiles; gt += gridDim.x, it++) {
            prefetch_c(gt + gridDim.x);
            int m0, n0r;
            const TcTask *t = tc_tile(tasks, ntasks, gt, m0, n0r);
            const int b = it & 1;
            const uint32_t use = (uint32_t)(it >> 1);
            const int row0 = m0 + 32 * q;
            const int nr = min(32, t->M - row0);
            const long long ldf = 2LL * t->ldc;
            // this lane's real column of chunk 0 (real column = 2 * complex column + (re, im))
            float *cl = reinterpret_cast<float *>(t->C + (long long)row0 * t->ldc) + n0r + lane;
            const int cf0 = n0r + lane;
            auto load_c = [&](float(&cv)[32], int ch) {
                const bool colok = ((cf0 + 32 * ch) >> 1) < t->N;
#pragma unroll
                for (int r = 0; r < 32; r++) cv[r] = (colok && r < nr) ? cl[r * ldf + 32 * ch] : 0.f;
            };
            float ca[32], cb[32];
            load_c(ca, ch0);
            load_c(cb, ch0 + 1);
            // f16 mode: the row scales of the quarter's 32 rows in the transpose
            // buffer's spare column (read back as warp broadcasts)
            if constexpr (F16) tb[lane * 33 + 32] = lane < nr ? t->sa[row0 + lane] : 0.f;
            const bool got = mbar_wait(&tfull[b], use & 1u);
            if (!__all_sync(0xffffffffu, got)) { atomicCAS(err, 0, 3); break; }   // warp-uniform: tcgen05.ld below
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * TC_BNR);
            auto emit = [&](const float(&cv)[32], int ch) {
                uint32_t v[32];
                TMEM_LD32(taddr + ch * 32, v);
                asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
                for (int i = 0; i < 32; i++) tb[lane * 33 + i] = __uint_as_float(v[i]);
                __syncwarp();   // also orders the row scales written before the first chunk
                const int cf = cf0 + 32 * ch;
                if ((cf >> 1) < t->N) {
                    float *cp = cl + 32 * ch;
                    if constexpr (F16) {
                        // undo the row and column scales (powers of two: exact)
                        const float sbj = t->sb[cf >> 1];
#pragma unroll
                        for (int r = 0; r < 32; r++)
                            if (r < nr) cp[r * ldf] = cv[r] - tb[r * 33 + lane] * (tb[r * 33 + 32] * sbj);
                    } else {
#pragma unroll
                        for (int r = 0; r < 32; r++)
                            if (r < nr) cp[r * ldf] = cv[r] - tb[r * 33 + lane];
                    }
                }
                __syncwarp();
            };
#pragma unroll 1
            for (int ch = ch0; ch < ch0 + NCH; ch += 2) {
                emit(ca, ch);
                if (ch + 2 < ch0 + NCH) load_c(ca, ch + 2);
                emit(cb, ch + 1);
                if (ch + 3 < ch0 + NCH) load_c(cb, ch + 3);
            }
            // accumulator b may be overwritten by the tile after next
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[b]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_BNR));
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
long long tc_workspace_floats(const GemmTask<float> *g, int n)
{
    long long w = 0;
    for (int i = 0; i < n; i++) {
        const long long Kr = align_up(2LL * g[i].K, 2 * TC_BK);
        w += align_up((long long)g[i].M * Kr, 256) * 2 + align_up(2LL * g[i].N * Kr, 256) * 2;
    }
    return w;
}

bool tc_eligible(const GemmTask<float> &g)
{
    // large enough that the tensor-core tile (128 x 128 complex) is not mostly
    // padding; the narrow right-hand-side blocks of the solves stay on SIMT
    return !g.brow && !g.crow && !g.conjA && g.M >= 64 && g.N >= 96 && g.K >= 32;
}

// f16 mode unless WT3D_TC_F16=0 (then the TF32 split)
static bool tc_f16_mode()
{
    static const bool on = !(getenv("WT3D_TC_F16") && getenv("WT3D_TC_F16")[0] == '0');
    return on;
}

int tc_build_launch(TcLaunch &L, const GemmTask<float> *g, int n, float *ws)
{
    std::vector<TcTask> tasks(n);
    std::vector<CUtensorMap> maps(4 * n);
    const bool f16 = tc_f16_mode();
    long long off = 0, tiles = 0, aw = 0, bw = 0, arows = 0, bcols = 0;
    for (int i = 0; i < n; i++) {
        TcTask &t = tasks[i];
        t.A = g[i].A; t.lda = g[i].lda;
        t.B = g[i].B; t.ldb = g[i].ldb;
        t.C = g[i].C; t.ldc = g[i].ldc;
        t.M = g[i].M; t.N = g[i].N; t.K = g[i].K;
        t.Kr = (int)align_up(2LL * t.K, 2 * TC_BK);   // whole 32-complex tiles for the B transpose
        // operand sizes in floats (an FP16 pair takes one float's room)
        const long long asz = align_up((long long)t.M * t.Kr / (f16 ? 2 : 1), 256);
        const long long bsz = align_up(2LL * t.N * t.Kr / (f16 ? 2 : 1), 256);
        t.ahi = ws + off; off += asz;
        t.alo = ws + off; off += asz;
        t.bhi = ws + off; off += bsz;
        t.blo = ws + off; off += bsz;
        t.tiles_n = (int)((2LL * t.N + TC_BNR - 1) / TC_BNR);
        t.tile0 = tiles;
        tiles += (long long)((t.M + TC_BM - 1) / TC_BM) * t.tiles_n;
        t.a_work0 = aw;
        aw += (long long)t.M * (t.Kr / 2);
        t.b_work0 = bw;
        bw += (long long)((t.N + 31) / 32) * (t.Kr / 64);
        t.a_row0 = arows;
        arows += t.M;
        t.b_col0 = bcols;
        bcols += (t.N + 31) / 32;
        t.map0 = 4 * i;
        int rc;
        if (f16) {
            if ((rc = make_map_f16(&maps[4 * i + 0], t.ahi, t.M, t.Kr, TC_BM)) ||
                (rc = make_map_f16(&maps[4 * i + 1], t.alo, t.M, t.Kr, TC_BM)) ||
                (rc = make_map_f16(&maps[4 * i + 2], t.bhi, 2LL * t.N, t.Kr, TC_BNR)) ||
                (rc = make_map_f16(&maps[4 * i + 3], t.blo, 2LL * t.N, t.Kr, TC_BNR)))
                return rc;
        } else if ((rc = make_map(&maps[4 * i + 0], t.ahi, t.M, t.Kr, TC_BM)) ||
                   (rc = make_map(&maps[4 * i + 1], t.alo, t.M, t.Kr, TC_BM)) ||
                   (rc = make_map(&maps[4 * i + 2], t.bhi, 2LL * t.N, t.Kr, TC_BNR)) ||
                   (rc = make_map(&maps[4 * i + 3], t.blo, 2LL * t.N, t.Kr, TC_BNR))) {
            return rc;
        }
    }
    // f16 mode: the inverse scales of all tasks after the operands
    if (f16)
        for (auto &t : tasks) {
            t.sa = ws + off; off += align_up(t.M, 64);
            t.sb = ws + off; off += align_up(t.N, 64);
        }
    L.f16 = f16;
    L.ntasks = n;
    L.tiles = tiles;
    L.a_work = aw;
    L.b_tiles = bw;
    L.a_rows = arows;
    L.b_cols = bcols;
    int rc;
    if ((rc = L.tasks.upload(tasks))) return rc;
    std::vector<unsigned char> raw(maps.size() * sizeof(CUtensorMap));
    memcpy(raw.data(), maps.data(), raw.size());
    if ((rc = L.maps.upload(raw))) return rc;
    return WT3D_OK;
}

void tc_split(const TcLaunch &L, cudaStream_t st)
{
    if (L.ntasks == 0) return;
    if (L.f16) {
        k_split_a_f16_rows<<<ceil_div(L.a_rows * 32, 256), 256, 0, st>>>(L.tasks.p, L.ntasks, L.a_rows);
        k_split_b_f16_cols<<<(unsigned)L.b_cols, 256, 0, st>>>(L.tasks.p, L.ntasks, L.b_cols);
        return;
    }
    k_split_a<<<ceil_div(L.a_work, 256), 256, 0, st>>>(L.tasks.p, L.ntasks, L.a_work);
    k_split_b<<<(unsigned)L.b_tiles, 256, 0, st>>>(L.tasks.p, L.ntasks, L.b_tiles);
}

static int num_sms()
{
    static const int n = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 1;
    }();
    return n;
}

// SMs the persistent tensor-core kernel leaves to concurrent work (other
// handles' substitution passes): set through wt3d_set_sm_reserve.
static std::atomic<int> g_sm_reserve{0};

void tc_mma(const TcLaunch &L, int *err, cudaStream_t st)
{
    if (L.ntasks == 0) return;
    const int sms = std::max(1, num_sms() - g_sm_reserve.load());
    const long long grid = std::min<long long>(L.tiles, sms);
    const CUtensorMap *maps = reinterpret_cast<const CUtensorMap *>(L.maps.p);
    if (L.f16)
        k_tc_gemm<true><<<(unsigned)grid, TC_THREADS, TC_SMEM, st>>>(L.tasks.p, L.ntasks, L.tiles, maps, err);
    else
        k_tc_gemm<false><<<(unsigned)grid, TC_THREADS, TC_SMEM, st>>>(L.tasks.p, L.ntasks, L.tiles, maps, err);
}

int tc_init()
{
    // idempotent; safe to call from several threads
    WT_CUDA(cudaFuncSetAttribute(k_tc_gemm<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
    WT_CUDA(cudaFuncSetAttribute(k_tc_gemm<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
    if (!encode_fn()) { set_error("cuTensorMapEncodeTiled unavailable"); return WT3D_ERR_CUDA; }
    return WT3D_OK;
}

}  // namespace wt3d

// ---------------------------------------------------------------------------
// C ABI check entry: one GEMM C -= A B on host complex64 arrays (row-major),
// through the tensor-core path (path = 1), the SIMT path (path = 0) or the
// tall-skinny tensor-core kernel of the solves (path = 3; path = 4 with a row
// gather of B and a row scatter of C; path = 5 with C -= A^H B for A given as
// the K x M block, lda >= M); paths 3 and 4 stream A by TMA when it is
// 16-byte aligned with an even stride.  wt3d_bench_gemm also times path 2,
// the tall-skinny SIMT kernel, path 3, and path 6 (path 3 with A always
// copied by the loader warps).
// ---------------------------------------------------------------------------
using namespace wt3d;
extern "C" int wt3d_set_sm_reserve(int n)
{
    if (n < 0) { set_error("wt3d_set_sm_reserve: negative"); return WT3D_ERR_ARG; }
    g_sm_reserve.store(n);
    return WT3D_OK;
}

extern "C" int wt3d_debug_gemm(int path, int M, int N, int K, const void *A, int lda, const void *B, int ldb, void *C,
                               int ldc)
{
    DevVec<cx<float>> dA, dB, dC;
    int rc;
    const size_t arows = path == 5 ? (size_t)K : (size_t)M;   // path 5: A holds the K x M block whose A^H is used
    if ((rc = dA.alloc(arows * lda)) || (rc = dB.alloc((size_t)K * ldb)) || (rc = dC.alloc((size_t)M * ldc)))
        return rc;
    WT_CUDA(cudaMemcpy(dA.p, A, sizeof(cx<float>) * arows * lda, cudaMemcpyHostToDevice));
    WT_CUDA(cudaMemcpy(dB.p, B, sizeof(cx<float>) * K * ldb, cudaMemcpyHostToDevice));
    WT_CUDA(cudaMemcpy(dC.p, C, sizeof(cx<float>) * M * ldc, cudaMemcpyHostToDevice));
    GemmTask<float> g{};
    g.A = dA.p; g.B = dB.p; g.C = dC.p; g.lda = lda; g.ldb = ldb; g.ldc = ldc; g.M = M; g.N = N; g.K = K;
    g.tiles_n = (N + GBN - 1) / GBN;
    g.tile0 = 0;
    DevVec<int> err;
    if ((rc = err.alloc(1))) return rc;
    WT_CUDA(cudaMemset(err.p, 0, sizeof(int)));
    DevVec<int> drow, dcol;
    if (path == 1) {
        if ((rc = tc_init())) return rc;
        DevVec<float> ws;
        if ((rc = ws.alloc(tc_workspace_floats(&g, 1)))) return rc;
        TcLaunch L;
        if ((rc = tc_build_launch(L, &g, 1, ws.p))) return rc;
        tc_split(L, 0);
        tc_mma(L, err.p, 0);
    } else if (path >= 3 && path <= 5) {
        // tall-skinny tensor-core kernel; path 4 gathers B rows K-1-k and
        // scatters C rows M-1-r (atomic epilogue); path 5 uses A^H
        if (N > 32) { set_error("wt3d_debug_gemm: paths 3 to 5 need N <= 32"); return WT3D_ERR_ARG; }
        g.conjA = path == 5 ? 1 : 0;
        if (path == 4) {
            std::vector<int> br(K), cr(M);
            for (int k = 0; k < K; k++) br[k] = K - 1 - k;
            for (int r = 0; r < M; r++) cr[r] = M - 1 - r;
            if ((rc = drow.upload(br)) || (rc = dcol.upload(cr))) return rc;
            g.brow = drow.p;
            g.crow = dcol.p;
        }
        if ((rc = ts_init())) return rc;
        DevVec<float> ws;
        if ((rc = ws.alloc(ts_workspace_floats(&g, 1)))) return rc;
        TsLaunch L;
        if ((rc = ts_build_launch(L, &g, 1, ws.p, ts_tma_ok(g)))) return rc;
        ts_expand(L, 0);
        ts_mma(L, err.p, 0);
    } else {
        DevVec<GemmTask<float>> dt;
        std::vector<GemmTask<float>> v{g};
        if ((rc = dt.upload(v))) return rc;
        long long tiles = (long long)((M + GBM - 1) / GBM) * g.tiles_n;
        k_gemm<float><<<(unsigned)tiles, 256>>>(dt.p, 1);
    }
    WT_CUDA(cudaGetLastError());
    WT_CUDA(cudaDeviceSynchronize());
    int herr = 0;
    WT_CUDA(cudaMemcpy(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) { set_error("tensor-core GEMM barrier wait expired (code " + std::to_string(herr) + ")"); return WT3D_ERR_CUDA; }
    WT_CUDA(cudaMemcpy(C, dC.p, sizeof(cx<float>) * M * ldc, cudaMemcpyDeviceToHost));
    return WT3D_OK;
}

// Device-resident GEMM timing (operands filled on the device): avg ms of
// `iters` launches of C -= A B with M x K, K x N complex64 row-major operands.
static __global__ void k_fill(cx<float> *p, long long n, unsigned seed)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned h = (unsigned)(i * 2654435761u) ^ seed;
    h ^= h >> 13; h *= 0x5bd1e995u; h ^= h >> 15;
    p[i] = cx<float>((float)(h & 0xFFFF) / 65536.0f - 0.5f, (float)(h >> 16) / 65536.0f - 0.5f);
}

extern "C" int wt3d_bench_gemm(int path, int M, int N, int K, int iters, double *ms_out)
{
    DevVec<cx<float>> dA, dB, dC;
    int rc;
    if ((rc = dA.alloc((size_t)M * K)) || (rc = dB.alloc((size_t)K * N)) || (rc = dC.alloc((size_t)M * N))) return rc;
    k_fill<<<ceil_div((long long)M * K, 256), 256>>>(dA.p, (long long)M * K, 1);
    k_fill<<<ceil_div((long long)K * N, 256), 256>>>(dB.p, (long long)K * N, 2);
    k_fill<<<ceil_div((long long)M * N, 256), 256>>>(dC.p, (long long)M * N, 3);
    GemmTask<float> g{};
    g.A = dA.p; g.B = dB.p; g.C = dC.p; g.lda = K; g.ldb = N; g.ldc = N; g.M = M; g.N = N; g.K = K;
    g.tiles_n = (N + GBN - 1) / GBN;
    DevVec<int> err;
    if ((rc = err.alloc(1))) return rc;
    WT_CUDA(cudaMemset(err.p, 0, sizeof(int)));
    DevVec<float> ws;
    TcLaunch L;
    TsLaunch LT;
    DevVec<GemmTask<float>> dt;
    if (path == 1) {
        if ((rc = tc_init()) || (rc = ws.alloc(tc_workspace_floats(&g, 1))) || (rc = tc_build_launch(L, &g, 1, ws.p)))
            return rc;
        tc_split(L, 0);
    } else if (path == 3 || path == 6) {
        if (N > 32) { set_error("wt3d_bench_gemm: paths 3 and 6 need N <= 32"); return WT3D_ERR_ARG; }
        const bool tma = path == 3 && ts_tma_ok(g);
        if ((rc = ts_init()) || (rc = ws.alloc(ts_workspace_floats(&g, 1))) ||
            (rc = ts_build_launch(LT, &g, 1, ws.p, tma)))
            return rc;
        ts_expand(LT, 0);
    } else {
        std::vector<GemmTask<float>> v{g};
        if ((rc = dt.upload(v))) return rc;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const long long tiles = (long long)((M + GBM - 1) / GBM) * g.tiles_n;
    const long long ts_tiles = (M + TSBM - 1) / TSBM;   // path 2: tall-skinny kernel (N <= 32)
    if (path == 2 && N > TSBN) { set_error("wt3d_bench_gemm: path 2 needs N <= 32"); return WT3D_ERR_ARG; }
    auto launch = [&]() {
        if (path == 1) tc_mma(L, err.p, 0);
        else if (path == 3 || path == 6) ts_mma(LT, err.p, 0);
        else if (path == 2) k_gemm_ts<float><<<(unsigned)ts_tiles, 256>>>(dt.p, 1);
        else k_gemm<float><<<(unsigned)tiles, 256>>>(dt.p, 1);
    };
    for (int w = 0; w < 2; w++) launch();   // warm-up
    cudaEventRecord(e0);
    for (int i = 0; i < iters; i++) launch();
    cudaEventRecord(e1);
    WT_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    *ms_out = ms / iters;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    WT_CUDA(cudaGetLastError());
    int herr = 0;
    WT_CUDA(cudaMemcpy(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost));
    return herr ? WT3D_ERR_CUDA : WT3D_OK;
}
