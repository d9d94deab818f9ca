// Shared definitions for the wtomo3d-gb300 native library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

namespace wt3d {

void set_error(const std::string &msg);

#define WT_CUDA(call)                                                              \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) {                                                   \
            ::wt3d::set_error(std::string(#call) + ": " + cudaGetErrorString(e_)); \
            return WT3D_ERR_CUDA;                                                  \
        }                                                                          \
    } while (0)

// Minimal complex arithmetic over a real type R, laid out as (re, im).
template <class R>
struct cx {
    R re, im;
    __host__ __device__ cx() {}
    __host__ __device__ constexpr cx(R r, R i = R(0)) : re(r), im(i) {}
};
template <class R> __host__ __device__ __forceinline__ cx<R> operator+(cx<R> a, cx<R> b) { return cx<R>(a.re + b.re, a.im + b.im); }
template <class R> __host__ __device__ __forceinline__ cx<R> operator-(cx<R> a, cx<R> b) { return cx<R>(a.re - b.re, a.im - b.im); }
template <class R> __host__ __device__ __forceinline__ cx<R> operator-(cx<R> a) { return cx<R>(-a.re, -a.im); }
template <class R> __host__ __device__ __forceinline__ cx<R> operator*(cx<R> a, cx<R> b) { return cx<R>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
template <class R> __host__ __device__ __forceinline__ cx<R> operator*(R s, cx<R> a) { return cx<R>(s * a.re, s * a.im); }
template <class R> __host__ __device__ __forceinline__ cx<R> operator*(cx<R> a, R s) { return cx<R>(s * a.re, s * a.im); }
template <class R> __host__ __device__ __forceinline__ cx<R> operator/(cx<R> a, R s) { return cx<R>(a.re / s, a.im / s); }
template <class R> __host__ __device__ __forceinline__ cx<R> cdiv(cx<R> a, cx<R> b)
{
    // Smith's algorithm (scaled division) for robustness.
    if (fabs(b.re) >= fabs(b.im)) {
        R r = b.im / b.re, d = b.re + b.im * r;
        return cx<R>((a.re + a.im * r) / d, (a.im - a.re * r) / d);
    } else {
        R r = b.re / b.im, d = b.im + b.re * r;
        return cx<R>((a.re * r + a.im) / d, (a.im * r - a.re) / d);
    }
}
template <class R> __host__ __device__ __forceinline__ cx<R> operator/(cx<R> a, cx<R> b) { return cdiv(a, b); }
template <class R> __host__ __device__ __forceinline__ R cabs2(cx<R> a) { return a.re * a.re + a.im * a.im; }
template <class R> __host__ __device__ __forceinline__ cx<R> conj(cx<R> a) { return cx<R>(a.re, -a.im); }

// Principal complex square root.
template <class R> __host__ __device__ __forceinline__ cx<R> csqrt_(cx<R> z)
{
    R m = sqrt(z.re * z.re + z.im * z.im);
    R sr = sqrt((m + z.re) * R(0.5));
    R si = sqrt((m - z.re) * R(0.5));
    if (z.im < 0) si = -si;
    return cx<R>(sr, si);
}

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace wt3d
