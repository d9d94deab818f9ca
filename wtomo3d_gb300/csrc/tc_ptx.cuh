// PTX helpers shared by the tcgen05 kernels (mbarriers, TMA, shared-memory
// matrix descriptors, kind::tf32 MMA, TMEM loads) and the TF32 operand split.
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cstdint>
#include <string>
#include "internal.h"

namespace wt3d {

constexpr unsigned TC_WAIT_LIMIT = 1u << 24;   // iterations of a bounded mbarrier wait

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Bounded wait for the phase with the given parity; returns false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
    const uint32_t a = smem_u32(bar);
    for (unsigned it = 0; it < TC_WAIT_LIMIT; it++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// K-major operand tile in the 128-byte-swizzle canonical layout: 8-row atoms
// of 128-byte rows, atoms 1024 bytes apart along M/N.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);        // start address
    d |= (uint64_t)1 << 16;                           // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;                 // stride byte offset between 8-row atoms
    d |= (uint64_t)1 << 46;                           // descriptor version (sm_100 family)
    d |= (uint64_t)2 << 61;                           // swizzle: 128B
    return d;
}

// kind::tf32 instruction descriptor: FP32 accumulate, TF32 A and B, both
// K-major, M = 128, N = 256.
__host__ __device__ constexpr uint32_t tf32_idesc(int M, int N)
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_tf32(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

// kind::f16 instruction descriptor: FP32 accumulate, FP16 A and B (type
// code 0), both K-major.
__host__ __device__ constexpr uint32_t f16_idesc(int M, int N)
{
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

#define TMEM_LD32(taddr, v)                                                                                       \
    asm volatile(                                                                                                 \
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18," \
        "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"                                            \
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),          \
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),   \
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), \
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])  \
        : "r"(taddr))

// Round to the nearest TF32 value (10 explicit mantissa bits), ties to even.
__device__ __forceinline__ float rn_tf32(float x)
{
    uint32_t u = __float_as_uint(x);
    if ((u & 0x7F800000u) == 0x7F800000u) return x;          // inf / nan unchanged
    u += 0xFFFu + ((u >> 13) & 1u);
    return __uint_as_float(u & 0xFFFFE000u);
}

// x = hi + lo + O(2^-24 |x|) with hi and lo both exact TF32 values, so the
// tensor core's reading of the operands loses nothing.
__device__ __forceinline__ void split_tf32(float x, float &hi, float &lo)
{
    hi = rn_tf32(x);
    lo = rn_tf32(x - hi);
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// ---------------------------------------------------------------------------
// host side: tensor maps
// ---------------------------------------------------------------------------
inline PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    // thread-safe one-time lookup (function-local static initialisation)
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return (PFN_cuTensorMapEncodeTiled_v12000)p;
        return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    }();
    return fn;
}

// 2-D FP32 tensor map of a rows x Kr K-major operand (Kr a multiple of 32),
// boxes of 32 floats (128 bytes) x box_rows in the 128-byte swizzle.
inline int make_map(CUtensorMap *m, float *base, long long rows, int Kr, int box_rows)
{
    auto fn = encode_fn();
    if (!fn) { set_error("cuTensorMapEncodeTiled unavailable"); return WT3D_ERR_CUDA; }
    cuuint64_t gdim[2] = {(cuuint64_t)Kr, (cuuint64_t)rows};
    cuuint64_t gstr[1] = {(cuuint64_t)Kr * 4};
    cuuint32_t box[2] = {32u, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, gdim, gstr, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
        return WT3D_ERR_CUDA;
    }
    return WT3D_OK;
}

// The same map over FP16 operand rows of Kr halves: 64-half (128-byte) boxes.
inline int make_map_f16(CUtensorMap *m, void *base, long long rows, int Kr, int box_rows)
{
    auto fn = encode_fn();
    if (!fn) { set_error("cuTensorMapEncodeTiled unavailable"); return WT3D_ERR_CUDA; }
    cuuint64_t gdim[2] = {(cuuint64_t)Kr, (cuuint64_t)rows};
    cuuint64_t gstr[1] = {(cuuint64_t)Kr * 2};
    cuuint32_t box[2] = {64u, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, base, gdim, gstr, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled (f16) failed: " + std::to_string((int)r));
        return WT3D_ERR_CUDA;
    }
    return WT3D_OK;
}

// 2-D FP32 tensor map of rows x width floats with a row stride in bytes (a
// multiple of 16), boxes of 32 floats x box_rows, in the 128-byte swizzle when
// swz128 (16-byte chunk c of box row r lands at chunk c ^ (r mod 8)), else
// unswizzled; reads outside the tensor return zeros.
inline int make_map_plain(CUtensorMap *m, const float *base, long long rows, long long width, long long stride_bytes,
                          int box_rows, bool swz128 = false)
{
    auto fn = encode_fn();
    if (!fn) { set_error("cuTensorMapEncodeTiled unavailable"); return WT3D_ERR_CUDA; }
    cuuint64_t gdim[2] = {(cuuint64_t)width, (cuuint64_t)rows};
    cuuint64_t gstr[1] = {(cuuint64_t)stride_bytes};
    cuuint32_t box[2] = {32u, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), gdim, gstr, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, swz128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
        return WT3D_ERR_CUDA;
    }
    return WT3D_OK;
}

inline long long align_up(long long x, long long a) { return (x + a - 1) / a * a; }

}  // namespace wt3d
