// Allocation-free tensor-core GEMM entry point.
//
// wt3d_gemm_noalloc computes C -= A B (complex64, device pointers) with the
// same tcgen05 3xTF32 method as the front updates, but keeps its scratch (the
// TF32 hi/lo split of A and the real expansion of B) in a fixed array that is
// part of this library's device image instead of a cudaMalloc'd workspace.
// It is for callers that cannot allocate device memory themselves: a process
// whose device memory is owned by another allocator or budget (for example a
// Fortran driver or a serving loop that accounts for every byte of HBM), or a
// latency-critical path that must not pay for cudaMalloc/cudaFree and the
// device synchronisation they imply.
//
// The scratch array holds NOALLOC_MAX_FLOATS floats (64 MiB); every GPU on
// which this library is loaded keeps it for the life of the process.  All calls
// share it, so calls that overlap on the GPU (from different streams or
// threads) race: serialise them.  The error word that reports an expired
// pipeline wait is shared the same way: a call that overlaps another can
// report the other's timeout or clear it.  The first call on a device looks up the
// array's device address with that device current and caches it; make that
// first call before relying on the entry point elsewhere.  The kernels here are
// variants of the ones in tc_gemm.cu that take their single task and tensor
// maps as kernel parameters instead of device arrays.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <mutex>
#include "tc_gemm.h"

namespace wt3d {
namespace {

constexpr long long NOALLOC_MAX_FLOATS = 16LL << 20;   // 64 MiB of scratch
constexpr int NB_BM = 128, NB_BNR = 256, NB_BK = 32, NB_STAGES = 2, NB_THREADS = 192;
constexpr int NB_A_BYTES = NB_BM * NB_BK * 4, NB_B_BYTES = NB_BNR * NB_BK * 4;
constexpr int NB_STAGE_BYTES = 2 * NB_A_BYTES + 2 * NB_B_BYTES;
constexpr int NB_SMEM = NB_STAGES * NB_STAGE_BYTES + 1024 + 256;
constexpr unsigned NB_WAIT_LIMIT = 1u << 24;

__device__ __align__(256) float g_scratch[NOALLOC_MAX_FLOATS];
__device__ int g_err;

__device__ __forceinline__ uint32_t su32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool bar_wait(uint64_t *bar, uint32_t parity)
{
    for (unsigned it = 0; it < NB_WAIT_LIMIT; it++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(su32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ uint64_t desc_sw128(uint32_t a)
{
    return (uint64_t)((a & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ float tf32_rn(float x)
{
    uint32_t u = __float_as_uint(x);
    if ((u & 0x7F800000u) == 0x7F800000u) return x;
    u += 0xFFFu + ((u >> 13) & 1u);
    return __uint_as_float(u & 0xFFFFE000u);
}

__device__ __forceinline__ void split2(float x, float &hi, float &lo)
{
    hi = tf32_rn(x);
    lo = tf32_rn(x - hi);
}

__global__ void k_na_split_a(const TcTask t)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int kc = t.Kr / 2;
    if (q >= (long long)t.M * kc) return;
    const int i = (int)(q / kc), k = (int)(q % kc);
    cx<float> v(0.f, 0.f);
    if (k < t.K) v = t.A[(long long)i * t.lda + k];
    float h0, l0, h1, l1;
    split2(v.re, h0, l0);
    split2(v.im, h1, l1);
    const long long o = (long long)i * t.Kr + 2 * k;
    *reinterpret_cast<float2 *>(t.ahi + o) = make_float2(h0, h1);
    *reinterpret_cast<float2 *>(t.alo + o) = make_float2(l0, l1);
}

__global__ void __launch_bounds__(256) k_na_split_b(const TcTask t)
{
    __shared__ float2 tile[32][33];
    const int kt = t.Kr / 64;
    const int j0 = (int)(blockIdx.x / kt) * 32, k0 = (int)(blockIdx.x % kt) * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int kk = ty; kk < 32; kk += 8) {
        const int k = k0 + kk, j = j0 + tx;
        cx<float> v(0.f, 0.f);
        if (k < t.K && j < t.N) v = t.B[(long long)k * t.ldb + j];
        tile[kk][tx] = make_float2(v.re, v.im);
    }
    __syncthreads();
    for (int jj = ty; jj < 32; jj += 8) {
        const int j = j0 + jj;
        if (j >= t.N) continue;
        const float2 b = tile[tx][jj];
        const int k = k0 + tx;
        float rh, rl, ih, il, nih, nil;
        split2(b.x, rh, rl);
        split2(b.y, ih, il);
        split2(-b.y, nih, nil);
        const long long o0 = (long long)(2 * j) * t.Kr + 2 * k, o1 = o0 + t.Kr;
        *reinterpret_cast<float2 *>(t.bhi + o0) = make_float2(rh, nih);
        *reinterpret_cast<float2 *>(t.blo + o0) = make_float2(rl, nil);
        *reinterpret_cast<float2 *>(t.bhi + o1) = make_float2(ih, rh);
        *reinterpret_cast<float2 *>(t.blo + o1) = make_float2(il, rl);
    }
}

__global__ void __launch_bounds__(NB_THREADS, 1)
    k_na_tc_gemm(const TcTask t, const __grid_constant__ CUtensorMap mah, const __grid_constant__ CUtensorMap mal,
                 const __grid_constant__ CUtensorMap mbh, const __grid_constant__ CUtensorMap mbl)
{
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + NB_STAGES * NB_STAGE_BYTES);
    uint64_t *empty = full + NB_STAGES;
    uint64_t *accum = empty + NB_STAGES;
    uint64_t *drain = accum + 1;
    uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(drain + 1);
    int *epi_fail = reinterpret_cast<int *>(tmem_holder + 1);   // an epilogue warp's accumulator wait expired
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long lt = blockIdx.x;
    const int m0 = (int)(lt / t.tiles_n) * NB_BM, n0r = (int)(lt % t.tiles_n) * NB_BNR;
    const int nk = t.Kr / NB_BK;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_holder)),
                     "r"(256));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 32) {
        for (int s = 0; s < NB_STAGES; s++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&empty[s])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(accum)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(drain)));
        *epi_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_holder;
    if (warp == 0 && lane == 0) {
        const CUtensorMap *maps[4] = {&mah, &mal, &mbh, &mbl};
        int issued = 0;
        for (int ks = 0; ks < nk; ks++) {
            const int s = ks % NB_STAGES;
            // an expired wait stops the producer; the MMA lane then times out in turn
            if (!bar_wait(&empty[s], ((ks / NB_STAGES) & 1) ^ 1)) { atomicCAS(&g_err, 0, 1); break; }
            issued = ks + 1;
            uint8_t *st = smem + s * NB_STAGE_BYTES;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(&full[s])),
                         "r"(NB_STAGE_BYTES)
                         : "memory");
            const int x = ks * NB_BK;
            uint8_t *dst[4] = {st, st + NB_A_BYTES, st + 2 * NB_A_BYTES, st + 2 * NB_A_BYTES + NB_B_BYTES};
            const int y[4] = {m0, m0, n0r, n0r};
            for (int q = 0; q < 4; q++)
                asm volatile(
                    "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
                    "[%4];" ::"r"(su32(dst[q])),
                    "l"((uint64_t)maps[q]), "r"(x), "r"(y[q]), "r"(su32(&full[s]))
                    : "memory");
        }
        // the last copy issued into each stage has landed before the stage
        // memory is reused by the epilogue or the CTA exits
        for (int s = 0; s < NB_STAGES; s++) {
            if (issued <= s) continue;
            const int last = issued - 1 - ((issued - 1 - s) % NB_STAGES);
            bar_wait(&full[s], (last / NB_STAGES) & 1);
        }
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NB_BNR >> 3) << 17) |
                               ((uint32_t)(NB_BM >> 4) << 24);
        bool ok = true;
        for (int ks = 0; ks < nk; ks++) {
            const int s = ks % NB_STAGES;
            if (!bar_wait(&full[s], (ks / NB_STAGES) & 1)) { atomicCAS(&g_err, 0, 2); ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t base = su32(smem + s * NB_STAGE_BYTES);
            const uint32_t ah = base, al = base + NB_A_BYTES, bh = base + 2 * NB_A_BYTES, bl = bh + NB_B_BYTES;
            for (int kk = 0; kk < NB_BK / 8; kk++) {
                const uint32_t o = kk * 32;
                const uint64_t d[4] = {desc_sw128(ah + o), desc_sw128(al + o), desc_sw128(bh + o), desc_sw128(bl + o)};
                const int pairs[3][2] = {{0, 2}, {0, 3}, {1, 2}};
                for (int q = 0; q < 3; q++) {
                    const uint32_t acc = (q > 0 || ks > 0 || kk > 0) ? 1u : 0u;
                    asm volatile(
                        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                        "l"(d[pairs[q][0]]), "l"(d[pairs[q][1]]), "r"(idesc), "r"(acc));
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             su32(&empty[s]))
                         : "memory");
        }
        // the accumulator is complete only if every k-step was issued; on a
        // timeout it is never signalled and the epilogue gives up in turn
        if (ok)
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             su32(accum))
                         : "memory");
        // no MMA of this CTA is in flight once the drain barrier completes
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(drain))
                     : "memory");
        bar_wait(drain, 0);
    } else if (warp >= 2) {
        if (!bar_wait(accum, 0)) {
            atomicCAS(&g_err, 0, 3);
            atomicOr(epi_fail, 1);
        }
        __syncwarp();
        // every epilogue warp learns whether any of them gave up before the
        // staged rows (written by other warps) are read or C is touched
        asm volatile("bar.sync 1, 128;" ::: "memory");
        const bool epi_ok = *(volatile int *)epi_fail == 0;
        asm volatile("bar.sync 1, 128;" ::: "memory");
        asm volatile("tcgen05.fence::after_thread_sync;");
        const int q = warp & 3;
        const uint32_t tq = tmem + ((uint32_t)(32 * q) << 16);
        float *stage = reinterpret_cast<float *>(smem);
        constexpr int EP = NB_BNR + 4;
        float *myrow = stage + (32 * q + lane) * EP;
        for (int ch = 0; ch < NB_BNR / 32 && epi_ok; ch++) {
            uint32_t v[32];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,"
                "%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(tq + ch * 32));
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            for (int i = 0; i < 32; i += 4)
                *reinterpret_cast<float4 *>(myrow + ch * 32 + i) =
                    make_float4(__uint_as_float(v[i]), __uint_as_float(v[i + 1]), __uint_as_float(v[i + 2]),
                                __uint_as_float(v[i + 3]));
        }
        asm volatile("bar.sync 1, 128;" ::: "memory");
        const int c0 = n0r / 2, ew = warp - 2;
        for (int r = ew; r < NB_BM && epi_ok; r += 4) {
            const int row = m0 + r;
            if (row >= t.M) break;
            cx<float> *crow = t.C + (long long)row * t.ldc + c0;
            const float *srow = stage + r * EP;
            for (int j = 0; j < 4; j++) {
                const int c = lane + 32 * j;
                if (c0 + c < t.N) {
                    cx<float> o = crow[c];
                    const float2 d = *reinterpret_cast<const float2 *>(srow + 2 * c);
                    o.re -= d.x;
                    o.im -= d.y;
                    crow[c] = o;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256));
    }
}

long long up256(long long x) { return (x + 255) / 256 * 256; }

struct DeviceScratch {
    float *scratch = nullptr;
    int *err = nullptr;
    bool ready = false;
};
DeviceScratch g_dev[64];
std::mutex g_mu;

// Resolved once, under g_mu, by the first call on any device.
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int resolve_encode()
{
    if (g_encode) return WT3D_OK;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
        set_error("cuTensorMapEncodeTiled unavailable");
        return WT3D_ERR_CUDA;
    }
    g_encode = (PFN_cuTensorMapEncodeTiled_v12000)p;
    return WT3D_OK;
}

int encode(CUtensorMap *m, float *base, long long rows, int Kr, int box_rows)
{
    const PFN_cuTensorMapEncodeTiled_v12000 fn = g_encode;
    cuuint64_t gdim[2] = {(cuuint64_t)Kr, (cuuint64_t)rows};
    cuuint64_t gstr[1] = {(cuuint64_t)Kr * 4};
    cuuint32_t box[2] = {(cuuint32_t)NB_BK, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    if (fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, gdim, gstr, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
           CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
        CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed");
        return WT3D_ERR_CUDA;
    }
    return WT3D_OK;
}

}  // namespace
}  // namespace wt3d

using namespace wt3d;

extern "C" long long wt3d_gemm_noalloc_max_floats(void) { return NOALLOC_MAX_FLOATS; }

extern "C" int wt3d_gemm_noalloc(int M, int N, int K, const void *dA, int lda, const void *dB, int ldb, void *dC,
                                 int ldc, void *stream)
{
    if (M < 1 || N < 1 || K < 1 || !dA || !dB || !dC || lda < K || ldb < N || ldc < N) {
        set_error("wt3d_gemm_noalloc: invalid arguments");
        return WT3D_ERR_ARG;
    }
    const long long Kr = (2LL * K + 63) / 64 * 64;
    const long long need = 2 * up256((long long)M * Kr) + 2 * up256(2LL * N * Kr);
    if (need > NOALLOC_MAX_FLOATS) {
        set_error("wt3d_gemm_noalloc: problem needs " + std::to_string(need) + " scratch floats, limit is " +
                  std::to_string(NOALLOC_MAX_FLOATS) + " (2 M Kr + 4 N Kr with Kr = 2K rounded up to 64)");
        return WT3D_ERR_ARG;
    }
    int dev = 0;
    WT_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) { set_error("wt3d_gemm_noalloc: device index out of range"); return WT3D_ERR_ARG; }
    DeviceScratch &D = g_dev[dev];
    {
        // once per device, with that device current: the scratch array's
        // device address (its host-side name is only a stand-in)
        std::lock_guard<std::mutex> lk(g_mu);
        if (!D.ready) {
            if (int rc = resolve_encode()) return rc;
            WT_CUDA(cudaGetSymbolAddress((void **)&D.scratch, g_scratch));
            WT_CUDA(cudaGetSymbolAddress((void **)&D.err, g_err));
            WT_CUDA(cudaFuncSetAttribute(k_na_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, NB_SMEM));
            D.ready = true;
        }
    }
    cudaStream_t st = (cudaStream_t)stream;
    TcTask t{};
    t.A = (const cx<float> *)dA;
    t.B = (const cx<float> *)dB;
    t.C = (cx<float> *)dC;
    t.lda = lda; t.ldb = ldb; t.ldc = ldc; t.M = M; t.N = N; t.K = K; t.Kr = (int)Kr;
    float *w = D.scratch;
    t.ahi = w;
    t.alo = w + up256((long long)M * Kr);
    t.bhi = t.alo + up256((long long)M * Kr);
    t.blo = t.bhi + up256(2LL * N * Kr);
    t.tiles_n = (int)((2LL * N + NB_BNR - 1) / NB_BNR);
    CUtensorMap mah, mal, mbh, mbl;
    int rc;
    if ((rc = encode(&mah, t.ahi, M, t.Kr, NB_BM)) || (rc = encode(&mal, t.alo, M, t.Kr, NB_BM)) ||
        (rc = encode(&mbh, t.bhi, 2LL * N, t.Kr, NB_BNR)) || (rc = encode(&mbl, t.blo, 2LL * N, t.Kr, NB_BNR)))
        return rc;
    // the error word must start at zero; the split operands are fully rewritten
    WT_CUDA(cudaMemsetAsync(D.err, 0, sizeof(int), st));
    const long long awork = (long long)M * (Kr / 2);
    k_na_split_a<<<(unsigned)((awork + 255) / 256), 256, 0, st>>>(t);
    k_na_split_b<<<(unsigned)(((N + 31) / 32) * (Kr / 64)), 256, 0, st>>>(t);
    const long long tiles = (long long)((M + NB_BM - 1) / NB_BM) * t.tiles_n;
    k_na_tc_gemm<<<(unsigned)tiles, NB_THREADS, NB_SMEM, st>>>(t, mah, mal, mbh, mbl);
    WT_CUDA(cudaGetLastError());
    int herr = 0;
    WT_CUDA(cudaMemcpyAsync(&herr, D.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    WT_CUDA(cudaStreamSynchronize(st));
    if (herr) {
        set_error("wt3d_gemm_noalloc: tensor-core pipeline wait expired (code " + std::to_string(herr) + ")");
        return WT3D_ERR_CUDA;
    }
    return WT3D_OK;
}
