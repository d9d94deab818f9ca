// Tall-skinny complex64 GEMM  C -= A B  on the tcgen05 tensor cores, for the
// substitution passes of the solve: A is a factor block (M x K, K-major rows
// in the front storage, any leading dimension), B and C hold at most 32
// right-hand sides.  Each factor entry is used for 32 complex multiply-adds
// only, so the kernel is meant to run at the speed of reading A from HBM.
//
// A is not copied or pre-split: front blocks start and stride at arbitrary
// 8-byte boundaries, which rules out TMA, so eight loader warps read A with
// plain 8-byte loads (one 128-byte row segment per half-warp), split every
// value into TF32 hi + lo (x = hi + lo to ~2^-24) and store both halves into
// the 128-byte-swizzled K-major tiles the MMA reads.  B is expanded once per
// launch into the 64 x 2K real matrix B~ (rows 2j, 2j+1 of column j, as in the
// square tensor-core GEMM), split into hi and lo, and fetched by TMA.  The
// complex product is the real product A_r B~^T into a 128 x 64 FP32 TMEM
// accumulator with D = Ahi Bhi + Ahi Blo + Alo Bhi.
//
// Work unit = (task, 128-row tile, K-chunk); persistent CTAs, two per SM.
// Warps 0-7 load and split A, warp 8 issues the TMA copies of B~ (and owns the
// TMEM allocation), warp 9 (one lane) issues the MMAs, warps 10-13 drain the
// double-buffered accumulator: C -= D in place, or with atomics when the task
// is split along K or its rows are scattered (border updates).  Every
// mbarrier wait is bounded; on expiry the kernel records an error code and
// winds down as the square kernel does.
#include "tc_gemm.h"
#include "tc_ptx.cuh"

namespace wt3d {

constexpr int TS_BM = 128;                        // complex rows per tile (MMA M)
constexpr int TS_NR = 64;                         // real accumulator columns: 32 complex (MMA N)
constexpr int TS_KC = 16;                         // complex k per stage: one 128-byte swizzle row
constexpr int TS_STAGES = 2;
constexpr int TS_A_BYTES = TS_BM * 128;           // 16 KB per split half
constexpr int TS_B_BYTES = TS_NR * 128;           // 8 KB per split half
constexpr int TS_STAGE_BYTES = 2 * TS_A_BYTES + 2 * TS_B_BYTES;
constexpr int TS_SMEM = TS_STAGES * TS_STAGE_BYTES + 1024 + 256;
constexpr int TS_LOADERS = 8;                     // loader warps
constexpr int TS_WB = TS_LOADERS, TS_WM = TS_LOADERS + 1, TS_WE = TS_LOADERS + 2;
constexpr int TS_THREADS = (TS_LOADERS + 6) * 32; // + B producer, MMA, 4 epilogue warps
constexpr int TS_PER_THREAD = TS_BM * TS_KC / (TS_LOADERS * 32);   // complex loads per loader thread per stage
static_assert(TS_PER_THREAD == 8, "loader mapping assumes 8 elements per thread");

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

// Loader thread l holds elements e = 256 i + l (i < 8) of a 128 x 16 complex
// stage: row e / 16, k e % 16, so a half-warp reads one contiguous 128-byte
// row segment.
__device__ __forceinline__ void ts_load(const TsTask *t, int m0, int kb, int k1, int l, float2 (&v)[TS_PER_THREAD])
{
#pragma unroll
    for (int i = 0; i < TS_PER_THREAD; i++) {
        const int e = i * (TS_LOADERS * 32) + l, r = m0 + (e >> 4), k = kb + (e & 15);
        v[i] = make_float2(0.f, 0.f);
        if (r < t->M && k < k1)
            v[i] = __ldg(reinterpret_cast<const float2 *>(t->A + (long long)r * t->lda + k));
    }
}

__global__ void __launch_bounds__(TS_THREADS, 2)
    k_tc_ts(const TsTask *__restrict__ tasks, int ntasks, long long nunits, const CUtensorMap *__restrict__ maps,
            int *err)
{
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + TS_STAGES * TS_STAGE_BYTES);
    uint64_t *empty = full + TS_STAGES;
    uint64_t *tfull = empty + TS_STAGES;
    uint64_t *tempty = tfull + 2;
    uint64_t *drain = tempty + 2;
    uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(drain + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == TS_WB) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                     "r"(2 * TS_NR));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == TS_WM * 32) {
        for (int s = 0; s < TS_STAGES; s++) {
            mbar_init(&full[s], TS_LOADERS + 1);   // 8 loader warps + the B copy's expect_tx arrival
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], 4);
        }
        mbar_init(drain, 1);
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_holder;

    if (warp < TS_LOADERS) {
        // ---------------- A loaders: global -> split -> swizzled tiles ----------------
        const int l = threadIdx.x;
        long long g = 0;
        bool ok = true;
        for (long long u = blockIdx.x; u < nunits && ok; u += gridDim.x) {
            int m0, k0, k1;
            const TsTask *t = ts_unit(tasks, ntasks, u, m0, k0, k1);
            const int nsub = (k1 - k0 + TS_KC - 1) / TS_KC;
            float2 nxt[TS_PER_THREAD];
            ts_load(t, m0, k0, k1, l, nxt);
            for (int i = 0; i < nsub; i++, g++) {
                float2 cur[TS_PER_THREAD];
#pragma unroll
                for (int q = 0; q < TS_PER_THREAD; q++) cur[q] = nxt[q];
                if (i + 1 < nsub) ts_load(t, m0, k0 + (i + 1) * TS_KC, k1, l, nxt);   // in flight meanwhile
                const int s = (int)(g % TS_STAGES);
                const uint32_t ph = (uint32_t)((g / TS_STAGES) & 1) ^ 1u;
                if (!mbar_wait(&empty[s], ph)) { atomicCAS(err, 0, 11); ok = false; break; }
                uint8_t *ahi = smem + s * TS_STAGE_BYTES, *alo = ahi + TS_A_BYTES;
#pragma unroll
                for (int q = 0; q < TS_PER_THREAD; q++) {
                    const int e = q * (TS_LOADERS * 32) + l, r = e >> 4, kc = e & 15;
                    // 128-byte swizzle: 16-byte chunk c of row r sits at chunk c ^ (r mod 8)
                    const int off = (r >> 3) * 1024 + (r & 7) * 128 + ((((kc >> 1) ^ (r & 7))) << 4) + ((kc & 1) << 3);
                    float h0, l0, h1, l1;
                    split_tf32(cur[q].x, h0, l0);
                    split_tf32(cur[q].y, h1, l1);
                    *reinterpret_cast<float2 *>(ahi + off) = make_float2(h0, h1);
                    *reinterpret_cast<float2 *>(alo + off) = make_float2(l0, l1);
                }
                // generic-proxy stores become visible to the tensor core's async proxy
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&full[s]);
            }
        }
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
                const int s = (int)(g % TS_STAGES);
                const uint32_t ph = (uint32_t)((g / TS_STAGES) & 1) ^ 1u;
                if (!mbar_wait(&empty[s], ph)) { atomicCAS(err, 0, 12); ok = false; break; }
                uint8_t *st = smem + s * TS_STAGE_BYTES + 2 * TS_A_BYTES;
                mbar_expect_tx(&full[s], 2 * TS_B_BYTES);
                const int x = 2 * (k0 + i * TS_KC);   // real column, a multiple of 32
                tma_load_2d(st, mp + 0, x, 0, &full[s]);
                tma_load_2d(st + TS_B_BYTES, mp + 1, x, 0, &full[s]);
            }
        }
        for (int s = 0; s < TS_STAGES; s++) {
            if (g <= s) continue;
            const long long last = g - 1 - ((g - 1 - s) % TS_STAGES);
            mbar_wait(&full[s], (uint32_t)((last / TS_STAGES) & 1));
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
                const int s = (int)(g % TS_STAGES);
                if (!mbar_wait(&full[s], (uint32_t)((g / TS_STAGES) & 1))) { atomicCAS(err, 0, 13); ok = false; break; }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t base = smem_u32(smem + s * TS_STAGE_BYTES);
                const uint32_t a_hi = base, a_lo = base + TS_A_BYTES;
                const uint32_t b_hi = base + 2 * TS_A_BYTES, b_lo = b_hi + TS_B_BYTES;
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
                        for (int c0 = 0; c0 < 16; c0 += 8) {   // 8 loads in flight per group
                            cx<float> cv[8];
#pragma unroll
                            for (int c = 0; c < 8; c++)
                                if (c0 + c < nc) cv[c] = p[c0 + c];
#pragma unroll
                            for (int c = 0; c < 8; c++)
                                if (c0 + c < nc)
                                    p[c0 + c] = cx<float>(cv[c].re - __uint_as_float(v[2 * (c0 + c)]),
                                                          cv[c].im - __uint_as_float(v[2 * (c0 + c) + 1]));
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
    // large factor blocks of the substitution passes; conjugate-transposed
    // blocks (adjoint solves) are MN-major and stay on the SIMT kernel
    return !g.conjA && g.N <= 32 && g.M >= TS_BM && g.K >= 256;
}

static long long ts_kr(int K) { return align_up(2LL * K, 64); }   // whole 32-complex tiles of B~

long long ts_workspace_floats(const GemmTask<float> *g, int n)
{
    long long w = 0;
    for (int i = 0; i < n; i++) w += 2LL * TS_NR * ts_kr(g[i].K);
    return w;
}

int ts_build_launch(TsLaunch &L, const GemmTask<float> *g, int n, float *ws)
{
    std::vector<TsTask> tasks(n);
    std::vector<CUtensorMap> maps(2 * n);
    // K-chunk so that the launch has about four units per resident CTA
    double work = 0;
    for (int i = 0; i < n; i++) work += (double)((g[i].M + TS_BM - 1) / TS_BM) * g[i].K;
    const long long slots = 2LL * ts_sms();
    const int kchunk = (int)std::max<long long>(256, align_up((long long)std::ceil(work / (4.0 * slots)), TS_KC));
    long long off = 0, units = 0, bw = 0;
    for (int i = 0; i < n; i++) {
        TsTask &t = tasks[i];
        t.A = g[i].A; t.lda = g[i].lda;
        t.B = g[i].B; t.ldb = g[i].ldb; t.brow = g[i].brow;
        t.C = g[i].C; t.ldc = g[i].ldc; t.crow = g[i].crow;
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
        t.map0 = 2 * i;
        int rc;
        if ((rc = make_map(&maps[2 * i], t.bhi, TS_NR, t.Kr, TS_NR)) ||
            (rc = make_map(&maps[2 * i + 1], t.blo, TS_NR, t.Kr, TS_NR)))
            return rc;
    }
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
    const long long grid = std::min<long long>(L.units, 2LL * ts_sms());
    k_tc_ts<<<(unsigned)grid, TS_THREADS, TS_SMEM, st>>>(L.tasks.p, L.ntasks, L.units,
                                                         reinterpret_cast<const CUtensorMap *>(L.maps.p), err);
}

int ts_init()
{
    WT_CUDA(cudaFuncSetAttribute(k_tc_ts, cudaFuncAttributeMaxDynamicSharedMemorySize, TS_SMEM));
    if (!encode_fn()) { set_error("cuTensorMapEncodeTiled unavailable"); return WT3D_ERR_CUDA; }
    return WT3D_OK;
}

}  // namespace wt3d
